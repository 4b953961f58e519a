"""The candidate collection's warp-wide decoupled look-back
(collect_scan_kernel, csrc/pairs.cu) replayed on the host: a block's warp
reads the status words of its 32 nearest predecessors at once (lane l: block
j - l; before block 0 an inclusive 0), sums the lanes up to the nearest
inclusive prefix and steps 32 blocks back while none is inclusive.  For every
mix of published aggregates and inclusive prefixes the block's exclusive
prefix must be the sum of all earlier blocks' counts.  No GPU."""
from __future__ import annotations

import numpy as np
import pytest

AGG, INCL = 1, 2


def look_back(blk: int, flags: np.ndarray, values: np.ndarray) -> int:
    """Exclusive prefix of block blk from its predecessors' status words."""
    excl, j = 0, blk - 1
    lanes = np.arange(32)
    while True:
        q = j - lanes
        flag = np.where(q >= 0, flags[np.maximum(q, 0)], INCL)
        val = np.where(q >= 0, values[np.maximum(q, 0)], 0)
        incl = [int(l) for l in lanes if flag[l] == INCL]
        upto = incl[0] if incl else 31  # the nearest inclusive lane
        excl += int(val[: upto + 1].sum())
        if incl:
            return excl
        j -= 32


@pytest.mark.parametrize("nblocks", [1, 2, 31, 32, 33, 64, 65, 200, 1000])
@pytest.mark.parametrize("p_incl", [0.0, 0.05, 0.5, 1.0])
def test_look_back_gives_the_exclusive_prefix(nblocks, p_incl):
    rng = np.random.default_rng(nblocks * 101 + int(p_incl * 100))
    counts = rng.integers(0, 5000, nblocks).astype(np.int64)
    prefix = np.concatenate([[0], np.cumsum(counts)])  # prefix[b] = sum of counts[:b]
    for _ in range(4):  # several publication states
        flags = np.where(rng.random(nblocks) < p_incl, INCL, AGG)
        flags[0] = INCL  # block 0 publishes its inclusive prefix at once
        values = np.where(flags == INCL, prefix[1:], counts)
        for blk in range(nblocks):
            assert look_back(blk, flags, values) == prefix[blk], (blk, flags[:blk][-40:])
