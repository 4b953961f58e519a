"""The group aligner's early exit (align_group.cuh): G lanes hold slices of K
row words, slice q at column block tau - q of group step tau, so lower slices
run ahead.  Every fourth step the lanes bound the pair's final LCS by

    max over rows j of  prefix(j) + min(columns left, Lr - j)

where prefix(j) sums, in row order, the zeros of every slice through row j,
each slice read after its own latest block, and the columns left are counted
from the column of slice qhi + 1 (one block behind the highest slice with
rows in the band): at that column no row above slice qhi is in the band, so
the mixed counts bound the banded LCS there.  The lanes find row order from
their slice indices alone: the slices held are G consecutive indices, and the
lowest is the one whose ring neighbour below does not hold q - 1.

This restates the banded recurrence (rows i - ls .. i + rs of column block i,
retired rows frozen), replays the group's lanes on its per-block states -- the
slice walk, the retirements, the ring-neighbour test, the ballot, the suffix
scan by rank -- and checks at every step that the bound never falls below the
final LCS, and never rises above the whole-band bound it replaces.  The replay
also checks the binning's premise: within a class's limit every slice with rows
in the band is the one its lane holds.  No GPU."""
from __future__ import annotations

import math

import numpy as np
import pytest

FULL = (1 << 32) - 1
SHAPES = [(8, 3), (8, 4), (16, 4), (16, 6), (32, 4), (32, 6), (32, 8), (32, 16)]  # (G, K) of the group classes
# the widest classes as they run, one block of four warps per pair
# (align_group_cta.cuh): (32, 8) as (128, 2), (32, 16) as (128, 4)
CTA_SHAPES = [(128, 2), (128, 4)]


def band(lr: int, lt: int, t: float):
    """ls, rs, nr, nc in blocks (the reference's lsft / rsft in fp32)."""
    t32 = np.float32(t)
    dl = np.float32(np.float32(lt) - np.float32(np.float32(lt) * t32))
    dr = np.float32(np.float32(lr) - np.float32(np.float32(lt) * t32))
    lsft = (max(0, math.ceil(dl)) + 31) & ~31
    rsft = max(0, math.ceil(dr)) + 32
    return lsft >> 5, (rsft + 31) >> 5, (lr + 31) >> 5, (lt + 31) >> 5


def zeros(w: int) -> int:
    return 32 - bin(w).count("1")


def states(rep: np.ndarray, tar: np.ndarray, ls: int, rs: int, nr: int, nc: int):
    """Every row word after each column block (frozen words keep their value)."""
    masks = {}
    for c in np.unique(rep):
        masks[int(c)] = int("".join("1" if x else "0" for x in (rep == c)[::-1]), 2)
    words, frozen, out = {}, {}, []
    lt = len(tar)
    for i in range(nc):
        j0 = i - ls if i > ls else 0
        j1 = min(i + rs, nr)
        if i > ls and (j0 - 1) in words:
            frozen[j0 - 1] = words.pop(j0 - 1)
        for j in range(j0, j1):
            words.setdefault(j, FULL)
        for col in range(32):
            p = 32 * i + col
            code = int(tar[p]) if p < lt else -1
            whole = masks.get(code, 0)
            carry = 0
            for j in range(j0, j1):
                v = words[j]
                u = v & (whole >> (32 * j)) & FULL
                s = v + u + carry
                carry, s = s >> 32, s & FULL
                words[j] = s | (v ^ u)
        snap = dict(frozen)
        snap.update(words)
        out.append(snap)
    return out


def replay(rep, tar, t, G, K):
    """Final LCS and, per group step, the row-aware bound as the lanes compute
    it and as the slices in row order give it, the whole-band bound at the same
    column, and the whole-band bound at the top slice's own column; None on
    steps where no slice has rows in the band."""
    lr, lt = len(rep), len(tar)
    ls, rs, nr, nc = band(lr, lt, t)
    st = states(rep, tar, ls, rs, nr, nc)
    final = sum(zeros(w) for w in st[-1].values())
    top = min(nc + rs - 1, nr)
    ns = (top + K - 1) // K
    word = lambda i, w: st[i].get(w, FULL)  # noqa: E731
    q = list(range(G))
    zret = [0] * G
    e = [0] * G
    r = [0] * G
    V = [[FULL] * K for _ in range(G)]
    out = []
    for tau in range(nc + ns - 1):
        for l in range(G):  # the slice walk and this step's block
            while q[l] < ns and tau >= q[l]:
                i = tau - q[l]
                j0 = i - ls if i > ls else 0
                if i < nc and (q[l] + 1) * K > j0:
                    break
                zret[l] += sum(zeros(v) for v in V[l])
                V[l] = [FULL] * K
                e[l] = r[l] = 0
                q[l] += G
            if q[l] < ns and tau >= q[l]:
                i = tau - q[l]
                j0 = i - ls if i > ls else 0
                j1 = min(i + rs, nr)
                lo = q[l] * K
                if lo < j1:
                    rr = min(j0 - lo, K) if j0 > lo else 0
                    for m in range(r[l], max(rr, r[l])):
                        zret[l] += zeros(V[l][m])
                        V[l][m] = FULL
                    r[l] = max(r[l], rr)
                    e[l] = max(e[l], min(j1 - lo, K))
                    for m in range(r[l], e[l]):
                        V[l][m] = word(i, lo + m)
        # one live slice per lane: every slice with rows in the band at its
        # block is the one its lane holds (the class limits guarantee it)
        for s in range(ns):
            i = tau - s
            if 0 <= i < nc:
                j0 = i - ls if i > ls else 0
                if max(j0, s * K) < min(i + rs, nr, s * K + K):
                    assert q[s % G] == s, (tau, s, q)
        live = [sum(zeros(v) for v in V[l]) for l in range(G)]
        S = sum(zret) + sum(live)
        qhi1 = max((q[l] + 1) if (q[l] < ns and e[l] > 0) else 0 for l in range(G))
        # the slices held are G consecutive indices
        assert sorted(q) == list(range(min(q), min(q) + G))
        lowest = [q[(l - 1) % G] != q[l] - 1 for l in range(G)]
        low = [l for l in range(G) if lowest[l]]
        assert len(low) == 1 and q[low[0]] == min(q)
        rank = [(l + G - low[0]) % G for l in range(G)]
        above = list(live)  # inclusive suffix sums by rank, Hillis-Steele
        o = 1
        while o < G:
            got = [above[(l + o) % G] for l in range(G)]
            above = [above[l] + (got[l] if rank[l] + o < G else 0) for l in range(G)]
            o <<= 1
        # the block-wide kernel's form: suffix sums in lane order, rotated by
        # the lowest lane (align_group_cta.cuh)
        suf = list(np.cumsum(live[::-1])[::-1])
        total, sl = sum(live), suf[low[0]]
        rotated = [suf[l] + total - sl if l >= low[0] else suf[l] - sl for l in range(G)]
        assert rotated == above
        if not qhi1:
            out.append(None)
            continue
        cols = min(32 * (tau + 1 - qhi1), lt)
        left = lt - cols
        ub = 0  # as the lanes compute it
        for l in range(G):
            acc = S - above[l]  # zeros of every row below this slice
            best = acc + min(left, lr) if rank[l] == 0 else 0
            for m in range(K):
                acc += zeros(V[l][m])
                row = 32 * (q[l] * K + m)
                best = max(best, acc + min(left, max(lr - row, 0)))
            ub = max(ub, best)
        # the same bound straight from the slices in row order
        acc = sum(zret)
        direct = acc + min(left, lr)
        for l in sorted(range(G), key=lambda x: q[x]):
            for m in range(K):
                acc += zeros(V[l][m])
                direct = max(direct, acc + min(left, max(lr - 32 * (q[l] * K + m), 0)))
        top_left = lt - min(32 * (tau + 2 - qhi1), lt)  # at the top slice's own column
        out.append((ub, direct, S + left, S + top_left))
    return final, out


def mutate(rng, s, sub, indel):
    out = []
    for ch in s:
        x = rng.random()
        if x < indel / 2:
            continue
        if x < indel:
            out.append(int(rng.integers(1, 5)))
        out.append(int(rng.integers(1, 5)) if rng.random() < sub else int(ch))
    return np.array(out, dtype=np.int64)


def test_top_slice_column_is_not_a_bound():
    """The target a suffix of its rep just above the identity cut: after the
    first block only slice 0 has run while rs words are in the band, so the
    zeros counted plus the columns after the top slice's own column fall
    below the final LCS -- and below the identity test, which would end a
    pair that passes.  Counted from the next slice's column they do not."""
    rng = np.random.default_rng(912)
    rep = rng.integers(1, 5, size=298)
    tar = rep[146:].copy()
    t = 0.5
    final, out = replay(rep, tar, t, 16, 1)
    assert final == len(tar)
    den = len(rep) + len(tar)
    passes = lambda x: np.float32(x) > np.float32(np.float32(den - x) * np.float32(t))  # noqa: E731
    assert passes(final)
    first = out[0]
    assert first is not None
    ub, _, whole, whole_top = first
    assert whole_top < final and not passes(whole_top)
    assert whole >= final and ub >= final


@pytest.mark.parametrize("seed", range(6))
def test_group_row_aware_bound_never_below_final_lcs(seed):
    rng = np.random.default_rng(700 + seed)
    pairs = steps = tighter = 0
    for k in range(14):
        t = float(rng.choice([0.1, 0.3, 0.5, 0.7, 0.9]))
        n = int(rng.integers(250, 900))
        a = rng.integers(1, 5, size=n)
        kind = k % 4
        if kind == 0:
            b = rng.integers(1, 5, size=max(1, int(n * rng.uniform(0.5, 1.6))))
        elif kind == 1:
            b = mutate(rng, a, rng.uniform(0, 0.3), rng.uniform(0, 0.1))
        elif kind == 2:
            b = a[int(rng.integers(0, n // 3)):].copy()
        else:
            b = np.concatenate([mutate(rng, a, 0.05, 0.02),
                                rng.integers(1, 5, size=int(rng.integers(0, 200)))])
        rep, tar = (a, b) if len(a) >= len(b) else (b, a)
        if len(tar) == 0 or np.float32(len(tar)) < np.float32(len(rep)) * np.float32(t):
            continue  # the length filter: never aligned
        ls, rs, nr, nc = band(len(rep), len(tar), t)
        shapes = [(G, K) for G, K in SHAPES + CTA_SHAPES
                  if (nr + K - 1) // K <= G or ls + rs <= (G - 1) * K + G]
        if not shapes:
            continue
        G, K = shapes[int(rng.integers(0, len(shapes)))]
        final, out = replay(rep, tar, t, G, K)
        for step in out:
            if step is None:
                continue
            ub, direct, whole, _ = step
            assert ub == direct
            assert ub >= final, (len(rep), len(tar), t, G, K, final, ub)
            assert ub <= whole
            tighter += ub < whole
            steps += 1
        pairs += 1
    assert pairs > 0 and steps > 0 and tighter > 0


@pytest.mark.parametrize("G,K,t", [(128, 2, 0.9), (128, 4, 0.7)])
def test_block_wide_group_wraps_its_ring(G, K, t):
    """A pair long enough that its slices wrap the block's ring of 128 lanes
    (slice q + 128 on the lane of slice q): one live slice per lane, the
    lanes' bound equal to the row-order bound and never below the final LCS."""
    rng = np.random.default_rng(G + K)
    a = rng.integers(1, 5, size=9000 if K == 2 else 17500)
    b = mutate(rng, a, 0.02, 0.004)
    rep, tar = (a, b) if len(a) >= len(b) else (b, a)
    ls, rs, nr, nc = band(len(rep), len(tar), t)
    assert (nr + K - 1) // K > G, "no wrap"
    assert ls + rs <= (G - 1) * K + G
    final, out = replay(rep, tar, t, G, K)
    steps = 0
    for step in out:
        if step is None:
            continue
        ub, direct, _, _ = step
        assert ub == direct and ub >= final
        steps += 1
    assert steps > 0
