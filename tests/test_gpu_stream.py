"""The streamed graph build (ngia_stream_graph): records pass through a few
chunk slots of device memory; the edges must equal the resident path's and
the reference's."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
from ngia2_gb300 import synth

pytestmark = pytest.mark.gpu


def as_triples(e):
    return np.stack([e["rep"].astype(np.int64), e["tar"].astype(np.int64),
                     np.round(e["weight"].astype(np.float64) * 100).astype(np.int64)], axis=1) \
        if len(e) else np.zeros((0, 3), np.int64)


def pack(s):
    from gpu_util import build_db
    order = np.argsort(-s.lens, kind="stable")
    return build_db([s.seq(int(i)) for i in order])


@pytest.mark.parametrize("kind,identity,bands,pieces", [
    ("dna", 95, 64, 7), ("dna", 90, 3, 3), ("prot", 70, 64, 5), ("prot", 50, 3, 11)])
def test_stream_equals_resident(cuda, built, kind, identity, bands, pieces):
    s = (synth.dna_families(12_000, 1_200, seed=71) if kind == "dna"
         else synth.protein_families(8_000, 800, seed=72))
    packed, offs, lens = pack(s)
    # three chunk slots of planes, codes and recoded codes: chunks of ~1/pieces of the records
    chunk_bytes = 36 * (len(packed) // pieces + 2000)
    e_stream, st = ng.stream_graph(packed, offs, lens, identity, bands, chunk_bytes)
    assert st["chunks"] >= min(pieces, 3)
    with ng.Context() as ctx:
        ctx.load(packed, offs, lens)
        m, rst = ctx.group_align(identity, bands)
        e_res = ctx.edges(m)
    assert np.array_equal(as_triples(e_stream), as_triples(e_res))
    assert st["unique_pairs"] == rst["unique_pairs"]
    assert st["aligned_cells"] == rst["aligned_cells"]
    assert st["bytes_h2d_sketch"] >= 4 * len(lens)


def test_stream_golden_edges(cuda, built, golden):
    """The reference's own edge list for the golden protein set, with the
    records cut into many chunks."""
    from conftest import load_edges
    db = golden["prot"]["db"]
    want = load_edges("prot", 70, "fma")
    e, st = ng.stream_graph(db["packed"], db["offsets"], db["lens"], 70, 64,
                            36 * (len(db["packed"]) // 6 + 2000))
    assert st["chunks"] > 3
    assert np.array_equal(as_triples(e), np.asarray(want, np.int64))


def test_stream_refuses_records_larger_than_a_chunk(cuda, built):
    s = synth.protein_families(200, 20, seed=73)
    packed, offs, lens = pack(s)
    with pytest.raises(ng.NgiaError):
        ng.stream_graph(packed, offs, lens, 90, 3, 36 * 10)


def test_stream_from_page_locked_records(cuda, built):
    """Records in page-locked host memory are copied to the device in place
    (no host staging copy); the edges are the same as from pageable memory."""
    import torch
    s = synth.protein_families(8_000, 800, seed=74)
    packed, offs, lens = pack(s)
    chunk_bytes = 36 * (len(packed) // 5 + 2000)
    t = torch.empty(packed.nbytes, dtype=torch.uint8, pin_memory=True)
    pinned = t.numpy().view(np.uint32)
    pinned[:] = packed
    e_pin, st_pin = ng.stream_graph(pinned, offs, lens, 70, 64, chunk_bytes)
    e_page, st_page = ng.stream_graph(packed, offs, lens, 70, 64, chunk_bytes)
    assert st_pin["chunks"] >= 3
    assert np.array_equal(as_triples(e_pin), as_triples(e_page))
    assert st_pin["bytes_h2d_align"] == st_page["bytes_h2d_align"]
