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


def two_phase_replay(sk, sv, n, bands, low_mask, tile, steps):
    """bucket.cu's resolve as it runs: tiles of `tile` sorted entries, each
    entry scanning back at most `steps` entries inside its tile and band; the
    rest listed and resolved by the warp-per-entry pass, which tests sixteen
    chunks of 32 entries a step and takes the nearest stop."""
    total = n * bands
    rep = np.full(total, -1, np.int64)
    slow = []
    for t0 in range(0, total, tile):
        for e in range(t0, min(t0 + tile, total)):
            first = e // n * n
            lo = max(first, t0)
            room = e - lo
            reach = min(room, steps)
            sig, bkt, r, settled = sk[e], sk[e] & low_mask, sv[e], False
            for d in range(1, reach + 1):
                s = sk[e - d]
                if (s & low_mask) != bkt:
                    settled = True
                    break
                if s == sig:
                    r, settled = sv[e - d], True
                    break
            if not settled and reach == room and lo == first:
                settled = True
            if settled:
                rep[first + sv[e]] = r
            else:
                slow.append(e)
    for e in slow:  # one warp per entry, sixteen chunks of 32 lanes a step
        first = e // n * n
        sig, bkt, r = sk[e], sk[e] & low_mask, sv[e]
        base, done = e, False
        while base > first and not done:
            for j in range(16):
                for l in range(32):
                    q = base - 1 - 32 * j - l
                    if q < first or (sk[q] & low_mask) != bkt:
                        done = True
                        break
                    if sk[q] == sig:
                        r, done = sv[q], True
                        break
                if done:
                    break
            base = base - 512 if base >= first + 512 else first
        rep[first + sv[e]] = r
    return rep, len(slow)


@pytest.mark.parametrize("tile,steps", [(64, 4), (100, 1), (4096, 64)])
def test_two_phase_resolve_equals_reference_grouping(tile, steps):
    """Three bands of family signatures with a long run of one signature whose
    low 16 bits collide with another's (a far predecessor), band boundaries
    inside tiles."""
    rng = np.random.default_rng(tile + steps)
    n, bands = 3000, 3
    rows = []
    for b in range(bands):
        sig = family_sigs(rng, n, 300, 0.7)
        sig[500:2500:7] = 0x12345A5A                  # a long run of one signature ...
        sig[[499, 2600, 2900]] = 0x77775A5A           # ... and one with the same low bits
        rows.append(sig)
    sk_parts, sv_parts = [], []
    for sig in rows:
        order = np.argsort(sig & 0xFFFF, kind="stable")
        sk_parts.append(sig[order].astype(np.int64))
        sv_parts.append(order.astype(np.int64))
    sk, sv = np.concatenate(sk_parts), np.concatenate(sv_parts)
    rep, far = two_phase_replay(sk, sv, n, bands, 0xFFFF, tile, steps)
    assert far > 0
    for b, sig in enumerate(rows):
        assert np.array_equal(rep[b * n:(b + 1) * n], oracle.bucket_band(sig).astype(np.int64))
