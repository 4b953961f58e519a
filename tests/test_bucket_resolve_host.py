"""A CPU replay of the bucketing (bucket.cu): the stable partition of each
band's (signature, index) pairs by the signature's low bits (as many 8-bit
radix passes as bucket.cu takes for n), then, per sorted entry, the scan back
through its bucket to the nearest entry with the same signature -- against
the oracle's grouping (oracle.bucket_band: the reference's stable sort and
predecessor chain).  Runs of equal signatures across the scan, buckets whose
low bits collide, and the empty read's all-ones signature included.  No GPU."""
from __future__ import annotations

import numpy as np
import pytest

import oracle


def partition_passes(n: int) -> int:
    return 1 if n <= 1 << 10 else 2 if n <= 1 << 18 else 3 if n <= 1 << 26 else 4


def resolve_replay(sig: np.ndarray, passes: int) -> np.ndarray:
    low_mask = 0xFFFFFFFF if passes >= 4 else (1 << (8 * passes)) - 1
    order = np.argsort(sig & low_mask, kind="stable")  # the stable partition
    sk, sv = sig[order].astype(np.int64), order.astype(np.int64)
    rep = np.empty(len(sig), np.int64)
    for e in range(len(sig)):
        r = sv[e]
        for q in range(e - 1, -1, -1):
            if (sk[q] & low_mask) != (sk[e] & low_mask):
                break
            if sk[q] == sk[e]:
                r = sv[q]
                break
        rep[sv[e]] = r
    return rep


def family_sigs(rng, n, families, spread):
    """Signatures of one band: members of a family often share one."""
    fam = rng.integers(0, families, n)
    base = rng.integers(0, 1 << 32, families, dtype=np.uint64)
    own = rng.integers(0, 1 << 32, n, dtype=np.uint64)
    share = rng.random(n) < spread
    return np.where(share, base[fam], own).astype(np.uint32)


@pytest.mark.parametrize("n,families,spread,passes", [
    (900, 90, 0.6, None),     # one pass (n <= 1024)
    (20000, 2000, 0.7, None),  # two passes
    (20000, 2000, 0.7, 1),     # fewer passes than bucket.cu takes: larger buckets
    (5000, 10, 0.95, None),    # a few huge signature groups
])
def test_resolve_replay_equals_reference_grouping(n, families, spread, passes):
    rng = np.random.default_rng(n + families)
    sig = family_sigs(rng, n, families, spread)
    sig[:7] = 0xFFFFFFFF  # an empty read's signature
    sig[100:130] = sig[99]  # a run of equal signatures
    got = resolve_replay(sig, passes or partition_passes(n))
    assert np.array_equal(got, oracle.bucket_band(sig).astype(np.int64))


def test_resolve_replay_low_bits_collide():
    """Many distinct signatures with the same low 16 bits."""
    rng = np.random.default_rng(7)
    n = 3000
    sig = ((rng.integers(0, 200, n).astype(np.uint32) << 16) | 0x5A5A).astype(np.uint32)
    got = resolve_replay(sig, 2)
    assert np.array_equal(got, oracle.bucket_band(sig).astype(np.int64))
