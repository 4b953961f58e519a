"""The 8-mer hash table of four-letter databases: the same signatures as the
hashing sketch and as the oracle, short records included."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
import oracle
from ngia2_gb300 import synth

pytestmark = pytest.mark.gpu


def dna_db(extra: list[bytes]):
    from gpu_util import build_db
    s = synth.dna_families(3000, 300, seed=81)
    seqs = [s.seq(i) for i in range(len(s))] + extra
    seqs.sort(key=len, reverse=True)
    return build_db(seqs)


def random_dna(lengths, seed):
    rng = np.random.default_rng(seed)
    return [bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), size=n)) for n in lengths]


@pytest.mark.parametrize("extra", [
    [b"ACGT"[: k % 4 + 1] * (k % 9) for k in range(1, 40)],   # lengths 0..8 included
    # both sides of the rank walk's minimum span (512 signed positions = length
    # 519; 256 = length 263 under the build option), a record of four 8-mers
    # repeated (the longest walks), and long ones
    random_dna(list(range(255, 272)) + list(range(511, 528)) + [20_000, 60_000], 5)
    + [b"ACGTACGT" * 400],
    [b"ACGTNACGTACGT" * 5],                                    # an N: five codes, no table
])
def test_table_sketch_equals_hashing(cuda, built, extra):
    packed, offs, lens = dna_db(extra)
    four_letters = not any(b"N" in x for x in extra)
    with ng.Context() as ctx:
        ctx.load(packed, offs, lens)
        assert ctx.sketch_table_active() == four_letters
        ctx.sketch_bucket(64)
        with_table = ctx.sigs()
        ctx.use_sketch_table(False)
        assert not ctx.sketch_table_active()
        ctx.sketch_bucket(64)
        hashed = ctx.sigs()
    assert np.array_equal(with_table, hashed)
    rng = np.random.default_rng(2)
    for i in list(rng.choice(len(lens), size=200, replace=False)) + \
            [int(j) for j in np.nonzero(lens < 9)[0]]:
        o = int(offs[i])
        rec = packed[o:o + 1 + ((int(lens[i]) + 31) // 32) * 4]
        assert np.array_equal(with_table[:, i], oracle.sketch_record(rec)), i
