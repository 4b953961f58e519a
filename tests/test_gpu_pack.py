"""Device packing (ngia_pack / ngia_pack_records) against the oracle's packer
and against makedb's packed records of the golden sets."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
import oracle

pytestmark = pytest.mark.gpu


def test_pack_matches_oracle_on_every_byte(cuda, built):
    rng = np.random.default_rng(5)
    lens = np.concatenate([np.arange(0, 70), rng.integers(1, 3000, size=200), [65534]])
    res = rng.integers(0, 256, size=int(lens.sum()), dtype=np.uint8)  # every byte value
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.uint64)
    packed, offs = ng.pack_records(res, starts, lens)
    for i in range(len(lens)):
        s, L = int(starts[i]), int(lens[i])
        want = oracle.pack_record(res[s:s + L].tobytes())
        o = int(offs[i])
        assert np.array_equal(packed[o:o + len(want)], want), i


@pytest.mark.parametrize("name", ["prot", "dna", "edge"])
def test_pack_reproduces_makedb_records(cuda, built, golden, name):
    """The packed file's FASTA area holds every read in index order; packing those
    residues gives the file's packed records word for word."""
    db = golden[name]["db"]
    raw = np.fromfile(golden[name]["packed"], dtype=np.uint8)
    n = db["n"]
    starts = (db["fasta_off"] + db["name_lens"].astype(np.uint64) + np.uint64(1)).astype(np.uint64)
    packed, offs = ng.pack_records(raw, starts, db["lens"])
    assert np.array_equal(offs, db["offsets"][:n])
    assert np.array_equal(packed, db["packed"][: len(packed)])
