"""The radix scatter's in-tile ranking (rs_scatter_kernel, csrc/sort.cu)
replayed lane by lane on the host: warp-private digit masks set with one
shared-memory OR per run of equal digits, three mask buffers in rotation with
each entry cleared one round after it was used, the leaders' running counts,
then the per-(warp, digit) slots.  Every tile -- full and partial, random
digits, one digit, runs, alternations, sorted and reversed -- must come out
as the stable sort of its keys by digit.  No GPU."""
from __future__ import annotations

import numpy as np
import pytest

K_TILE, WARPS = 4096, 8
WARP_KEYS = K_TILE // WARPS
ROUNDS = WARP_KEYS // 32
MASK_BUFS = 3
FULL = 0xFFFFFFFF
LANES = np.arange(32, dtype=np.int64)


def popc(x: np.ndarray) -> np.ndarray:
    return np.array([bin(int(v)).count("1") for v in x], np.int64)


def ffs(x: int) -> int:
    return (x & -x).bit_length()  # 1-based, 0 for 0


def scatter_tile(keys: np.ndarray, shift: int) -> np.ndarray:
    """The tile as the kernel leaves it in shared memory (sorted by digit)."""
    cnt = len(keys)
    count = np.zeros((WARPS, 256), np.int64)
    ranks = np.zeros((WARPS, ROUNDS, 32), np.int64)
    for w in range(WARPS):
        masks = np.zeros((MASK_BUFS, 256), np.int64)
        w0 = w * WARP_KEYS
        mine = np.maximum(cnt - w0 - LANES, 0)
        clear = [None] * 32  # (buffer, digit) each lane cleared one round later
        for r in range(ROUNDS):
            valid = 32 * r < mine
            idx = np.minimum(w0 + 32 * r + LANES, max(cnt - 1, 0))
            key = np.where(valid, keys[idx] if cnt else 0, 0)
            d = (key >> shift) & 255
            b = r % MASK_BUFS
            m = masks[b]
            dprev = np.concatenate([[d[0]], d[:-1]])  # shfl_up: lane 0 keeps its own
            start = valid & ((LANES == 0) | (dprev != d))
            starts = sum(1 << int(l) for l in LANES[start])
            vmask = sum(1 << int(l) for l in LANES[valid])
            for l in LANES[start]:
                above = starts & ~(((2 << int(l)) & FULL) - 1) & FULL
                end = ffs(above) - 1 if above else 32
                upto = FULL if end == 32 else (1 << end) - 1
                lt = (1 << int(l)) - 1
                m[d[l]] |= upto & ~lt & vmask & FULL
            peers = np.where(valid, m[d], 0)
            leader = np.array([ffs(int(p)) - 1 if p else int(l) for p, l in zip(peers, LANES)])
            seen = np.where(valid & (leader == LANES), count[w][d], 0)
            base = seen[leader]
            for l in range(32):  # last round's entries, now read by every lane
                if clear[l] is not None:
                    cb, cd = clear[l]
                    masks[cb][cd] = 0
                clear[l] = None
            lt_masks = (1 << LANES) - 1
            for l in range(32):
                if valid[l] and (int(peers[l]) & int(lt_masks[l])) == 0:
                    count[w][d[l]] = base[l] + bin(int(peers[l])).count("1")
                    clear[l] = (b, int(d[l]))
            ranks[w, r] = base + popc(peers & lt_masks)
        # every entry was cleared one round after its use, but the last round's
        others = [x for x in range(MASK_BUFS) if x != (ROUNDS - 1) % MASK_BUFS]
        assert not masks[others].any()
    # tile-local slot of each (warp, digit): digits in order, warps in order
    tot = count.sum(axis=0)
    first = np.concatenate([[0], np.cumsum(tot)[:-1]])
    slot0 = first[None, :] + np.concatenate([np.zeros((1, 256), np.int64),
                                             np.cumsum(count, axis=0)[:-1]], axis=0)
    out = np.full(cnt, -1, np.int64)
    for w in range(WARPS):
        for r in range(ROUNDS):
            for l in range(32):
                i = w * WARP_KEYS + 32 * r + l
                if i < cnt:
                    d = (int(keys[i]) >> shift) & 255
                    s = ranks[w, r, l] + slot0[w, d]
                    assert out[s] == -1, "two keys in one slot"
                    out[s] = keys[i]
    return out


def stable_by_digit(keys: np.ndarray, shift: int) -> np.ndarray:
    d = (keys >> shift) & 255
    return keys[np.argsort(d, kind="stable")]


def tiles():
    rng = np.random.default_rng(7)
    yield "random", rng.integers(0, 2**32, K_TILE, dtype=np.uint64).astype(np.int64)
    yield "one digit", np.full(K_TILE, 0x1234, np.int64) + np.arange(K_TILE) * 256
    yield "sorted", np.sort(rng.integers(0, 2**32, K_TILE, dtype=np.uint64)).astype(np.int64)
    yield "reversed", np.sort(rng.integers(0, 2**32, K_TILE, dtype=np.uint64))[::-1].astype(
        np.int64).copy()
    yield "alternating", np.where(np.arange(K_TILE) % 2 == 0, 5, 250).astype(np.int64)
    runs = np.repeat(rng.integers(0, 4, 200), rng.integers(1, 40, 200))[:K_TILE]
    yield "runs of few digits", np.resize(runs, K_TILE).astype(np.int64)
    for n in (1, 2, 31, 32, 33, 511, 512, 513, 600, 4095):
        yield f"partial {n}", rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.int64)
    yield "partial runs 700", np.repeat(np.arange(7), 100).astype(np.int64)


@pytest.mark.parametrize("name,keys", list(tiles()), ids=[t[0] for t in tiles()])
@pytest.mark.parametrize("shift", [0, 8])
def test_scatter_tile_is_the_stable_sort_by_digit(name, keys, shift):
    keys = keys if shift == 0 else (keys << 8) & FULL  # u32 keys
    got = scatter_tile(keys, shift)
    assert np.array_equal(got, stable_by_digit(keys, shift)), name
