"""ngia_ctx_run_host's pipelined load: the records go up in pieces while the
previous pieces are sketched under the code map of the context's previous
load.  Same edges as the resident path (load + group_align) whether the map
holds or not (another alphabet falls back to the ordinary sketch)."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
from ngia2_gb300 import synth

pytestmark = pytest.mark.gpu


def triples(e: np.ndarray) -> np.ndarray:
    return np.stack([e["rep"].astype(np.int64), e["tar"].astype(np.int64),
                     np.rint(e["weight"].astype(np.float64) * 100).astype(np.int64)], axis=1)


def database(seqs):
    from gpu_util import build_db
    seqs = sorted(seqs, key=len, reverse=True)
    packed, offs, lens = build_db(seqs)
    return np.ascontiguousarray(packed), np.ascontiguousarray(offs), np.ascontiguousarray(lens)


def dna(n, fam, seed, extra=()):
    s = synth.dna_families(n, fam, seed=seed)
    return database([s.seq(i) for i in range(len(s))] + list(extra))


def resident_edges(db, identity, bands=64):
    with ng.Context() as ctx:
        ctx.load(*db)
        m, _ = ctx.group_align(identity, bands)
        return triples(ctx.edges(m))


def host_edges(ctx, db, identity, bands=64):
    out = np.empty(64 * db[2].size + 16, ng.EDGE_DTYPE)
    m, st = ctx.run_host(db[0], db[1], db[2], identity, bands, out)
    return triples(out[:m]), st


def test_pipelined_load_matches_resident_path(cuda, built):
    db = dna(20_000, 2_000, 31)
    want = resident_edges(db, 90)
    assert len(want) > 0
    with ng.Context() as ctx:
        first, st0 = host_edges(ctx, db, 90)   # no previous map: sequential
        again, st1 = host_edges(ctx, db, 90)   # the same map: pipelined
        third, st2 = host_edges(ctx, db, 80, bands=16)
    assert st0["load_pipelined"] == 0
    assert st1["load_pipelined"] == 1 and st2["load_pipelined"] == 1
    assert np.array_equal(first, want)
    assert np.array_equal(again, want)
    assert np.array_equal(third, resident_edges(db, 80, 16))


def test_pipelined_load_falls_back_on_another_alphabet(cuda, built, golden):
    dna_db = dna(12_000, 1_200, 32)
    # an N: five codes, no table sketch; the assumed four-code map fails
    with_n = dna(12_000, 1_200, 33, extra=[b"ACGTNACGTACGTTGCA" * 40])
    prot = golden["prot"]["db"]
    prot_db = (np.ascontiguousarray(prot["packed"]), np.ascontiguousarray(prot["offsets"]),
               np.ascontiguousarray(prot["lens"]))
    with ng.Context() as ctx:
        host_edges(ctx, dna_db, 90)
        got_n, st_n = host_edges(ctx, with_n, 90)
        host_edges(ctx, dna_db, 90)
        got_p, st_p = host_edges(ctx, prot_db, 50)
        got_d, st_d = host_edges(ctx, dna_db, 90)
    assert st_n["load_pipelined"] == 0 and st_p["load_pipelined"] == 0
    assert st_d["load_pipelined"] == 0  # the previous load was the protein set
    assert np.array_equal(got_n, resident_edges(with_n, 90))
    assert np.array_equal(got_p, resident_edges(prot_db, 50))
    assert np.array_equal(got_d, resident_edges(dna_db, 90))


def test_pipelined_load_serves_a_subset_of_the_codes(cuda, built):
    """A database with only A, C, G after an A, C, G, T one: the assumed map is
    still one-to-one on the codes present, so the pipeline keeps it; the edges
    are the resident path's (which recodes to three codes)."""
    s = synth.dna_families(10_000, 1_000, seed=34)
    three = database([s.seq(i).replace(b"T", b"G") for i in range(len(s))])
    with ng.Context() as ctx:
        host_edges(ctx, dna(10_000, 1_000, 35), 90)
        host_edges(ctx, dna(10_000, 1_000, 35), 90)
        got, st = host_edges(ctx, three, 85)
    assert st["load_pipelined"] == 1
    assert np.array_equal(got, resident_edges(three, 85))
