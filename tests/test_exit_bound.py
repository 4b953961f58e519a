"""The streaming aligner's early exit (align_stream.cuh, columns_dispatch):
after each column block it bounds the pair's final LCS by

    max over rows j of  L(j) + min(columns left, Lr - j)

taken at word granularity (zeros through a word's end, rows above its
start) plus a term for the retired rows, and stops when that bound cannot
pass the identity test.  The pair's score is 0 either way only if the bound
never falls below the final LCS.  This restates the banded bit-parallel
recurrence with the kernel's window (rows i - ls .. i - ls + W - 1 at column
block i, retired rows counted and frozen, entering rows all ones) and checks
the bound against the final LCS at every block, for random and related pairs
of all length ratios.  No GPU."""
from __future__ import annotations

import math

import numpy as np
import pytest

FULL = (1 << 32) - 1


def band(lr: int, lt: int, t: float):
    """ls, rs, nr, nc in blocks (the reference's lsft / rsft in fp32)."""
    t32 = np.float32(t)
    dl = np.float32(np.float32(lt) - np.float32(np.float32(lt) * t32))
    dr = np.float32(np.float32(lr) - np.float32(np.float32(lt) * t32))
    lsft = (max(0, math.ceil(dl)) + 31) & ~31
    rsft = max(0, math.ceil(dr)) + 32
    return lsft >> 5, (rsft + 31) >> 5, (lr + 31) >> 5, (lt + 31) >> 5


def run(rep: np.ndarray, tar: np.ndarray, t: float):
    """Final banded LCS and the exit bound after every column block."""
    lr, lt = len(rep), len(tar)
    ls, rs, nr, nc = band(lr, lt, t)
    width = ls + min(rs, nr)
    masks = {}  # code -> bit mask of the rep's rows with that code
    for c in np.unique(rep):
        masks[int(c)] = int("".join("1" if x else "0" for x in (rep == c)[::-1]), 2)
    words = {}
    retired = 0
    bounds, simple = [], []
    for i in range(nc):
        j0 = i - ls if i > ls else 0
        j1 = min(i + rs, nr)
        if i > ls:
            w = words.pop(j0 - 1, FULL)
            retired += 32 - bin(w).count("1")
        for j in range(j0, j1):
            words.setdefault(j, FULL)
        for col in range(32):
            p = 32 * i + col
            code = int(tar[p]) if p < lt else -1
            whole = masks.get(code, 0)
            carry = 0
            for j in range(j0, j1):
                v = words[j]
                m = (whole >> (32 * j)) & FULL
                u = v & m
                s = v + u + carry
                carry, s = s >> 32, s & FULL
                words[j] = s | (v ^ u)
        left = max(lt - 32 * (i + 1), 0)
        acc = retired
        best = retired + min(left, lr)
        for m in range(width):  # window words in row order, virtual ones included
            rb = i - ls + m
            if 0 <= rb < nr and rb in words:
                acc += 32 - bin(words[rb]).count("1")
            best = max(best, acc + min(left, max(lr - 32 * rb, 0)))
        bounds.append(best)
        simple.append(acc + left)  # LCS so far + columns left
    final = retired + sum(32 - bin(w).count("1") for w in words.values())
    return final, bounds, simple


def mutate(rng, s, sub, indel):
    out = []
    for ch in s:
        r = rng.random()
        if r < indel / 2:
            continue
        if r < indel:
            out.append(int(rng.integers(1, 5)))
        out.append(int(rng.integers(1, 5)) if rng.random() < sub else int(ch))
    return np.array(out, dtype=np.int64)


@pytest.mark.parametrize("seed", range(8))
def test_row_aware_bound_never_below_final_lcs(seed):
    rng = np.random.default_rng(100 + seed)
    checked = tighter = 0
    for k in range(40):
        t = float(rng.choice([0.5, 0.7, 0.9, 0.95]))
        n = int(rng.integers(20, 700))
        a = rng.integers(1, 5, size=n)
        kind = k % 4
        if kind == 0:
            b = rng.integers(1, 5, size=max(1, int(n * rng.uniform(0.5, 1.6))))
        elif kind == 1:
            b = mutate(rng, a, rng.uniform(0, 0.15), rng.uniform(0, 0.05))
        elif kind == 2:
            b = a.copy()
        else:
            b = np.concatenate([mutate(rng, a, 0.02, 0.01),
                                rng.integers(1, 5, size=int(rng.integers(0, 80)))])
        if len(b) == 0:
            continue
        rep, tar = (a, b) if len(a) >= len(b) else (b, a)
        if np.float32(len(tar)) < np.float32(len(rep)) * np.float32(t):
            continue  # the length filter: never aligned
        final, bounds, simple = run(rep, tar, t)
        assert all(ub >= final for ub in bounds), (len(rep), len(tar), t, final, min(bounds))
        assert all(ub <= sb for ub, sb in zip(bounds, simple))
        tighter += sum(ub < sb for ub, sb in zip(bounds, simple))
        checked += 1
    assert checked > 0 and tighter > 0  # the row terms do bite
