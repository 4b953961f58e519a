"""ngia_bucket_noalloc: the bucketing stage for callers that cannot allocate
device memory while they run.  Its rep rows must equal ngia_bucket's on the
same signatures, call after call (the shared fixed scratch keeps the previous
call's contents), and inputs beyond its fixed limit must be refused.

This file is collected last so that a run stopping at the first failure has
run every other test first; it also passes on its own in a fresh process."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
from gpu_util import dev_empty, from_dev, stream, to_dev

pytestmark = pytest.mark.gpu

MAX_ELEMS = 1 << 20


def signatures(n: int, bands: int, seed: int) -> np.ndarray:
    """Band-major signatures with many repeats, like real minhash buckets."""
    rng = np.random.default_rng(seed)
    pool = rng.integers(0, 2**32, size=max(4, n // 5), dtype=np.uint64).astype(np.uint32)
    sigs = pool[rng.integers(0, len(pool), size=(bands, n))]
    sigs[:, : n // 50] = 0xFFFFFFFF  # empty records sign nothing
    return np.ascontiguousarray(sigs)


def run(fn, sigs: np.ndarray, bands: int) -> np.ndarray:
    n = sigs.shape[1]
    d_sigs = to_dev(sigs)
    d_rep = dev_empty(bands * n * 4)
    fn(d_sigs.data_ptr(), n, bands, d_rep.data_ptr(), stream())
    return from_dev(d_rep, np.uint32, bands * n).reshape(bands, n)


def test_noalloc_matches_bucket_on_consecutive_calls(cuda, built):
    cases = [(16_384, 64, 1), (5_000, 7, 2), (MAX_ELEMS, 1, 3)]
    for n, bands, seed in cases:  # consecutive calls share the fixed scratch
        sigs = signatures(n, bands, seed)
        want = run(ng.bucket, sigs, bands)
        got = run(ng.bucket_noalloc, sigs, bands)
        assert np.array_equal(got, want), (n, bands)
        again = run(ng.bucket_noalloc, sigs, bands)
        assert np.array_equal(again, want), (n, bands)


def test_noalloc_refuses_inputs_beyond_its_limit(cuda, built):
    d = dev_empty(16)
    L = ng.lib()
    assert L.ngia_bucket_noalloc(d.data_ptr(), 16_385, 64, d.data_ptr(), 0) == -1
    assert L.ngia_bucket_noalloc(d.data_ptr(), MAX_ELEMS + 1, 1, d.data_ptr(), 0) == -1
    assert L.ngia_bucket_noalloc(d.data_ptr(), 10, 65, d.data_ptr(), 0) == -1
