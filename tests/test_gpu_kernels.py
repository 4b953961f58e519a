"""GPU parity of the four hot-path stages through the C ABI, against the
golden fixtures (outputs of the reference) and the CPU oracle.  Bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
import oracle
from conftest import GOLDEN, IDENTITIES, SETS, load_pairs
from gpu_util import (align_jobs_on_gpu, build_db, dev_empty, from_dev,
                      reference_rep_rows, stream, to_dev)

pytestmark = pytest.mark.gpu


def gpu_sketch(db) -> np.ndarray:
    n = db["n"]
    d_packed, d_offs = to_dev(db["packed"]), to_dev(db["offsets"])
    d_sigs = dev_empty(64 * n * 4)
    ng.sketch(d_packed.data_ptr(), d_offs.data_ptr(), n, d_sigs.data_ptr(), stream())
    return from_dev(d_sigs, np.uint32).reshape(64, n)


def gpu_bucket(sigs_band_major: np.ndarray, bands: int) -> np.ndarray:
    n = sigs_band_major.shape[1]
    d_sigs = to_dev(sigs_band_major)
    d_rep = dev_empty(bands * n * 4)
    ng.bucket(d_sigs.data_ptr(), n, bands, d_rep.data_ptr(), stream())
    return from_dev(d_rep, np.uint32, bands * n).reshape(bands, n)


@pytest.mark.parametrize("name", SETS)
def test_sketch_matches_reference(cuda, built, golden, name):
    sigs = np.load(GOLDEN / f"{name}.sigs.npy")
    assert np.array_equal(gpu_sketch(golden[name]["db"]), sigs.T)


@pytest.mark.parametrize("name", SETS)
def test_bucket_matches_reference(cuda, built, golden, name):
    sigs = np.ascontiguousarray(np.load(GOLDEN / f"{name}.sigs.npy").T)
    rep = golden[name]["db"]["rep"]
    assert np.array_equal(gpu_bucket(sigs, 64), rep)
    assert np.array_equal(gpu_bucket(sigs, 3), rep[:3])


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_align_pairs_matches_reference(cuda, built, golden, name, identity):
    db = golden[name]["db"]
    pairs, s_split, s_fma, _ = load_pairs(name, identity)
    if len(pairs) == 0:
        pytest.skip("no candidate pairs")
    got_fma = align_jobs_on_gpu(db["packed"], db["offsets"], pairs, identity, "fma")
    got_split = align_jobs_on_gpu(db["packed"], db["offsets"], pairs, identity, "split")
    assert np.array_equal(got_fma, s_fma)
    assert np.array_equal(got_split, s_split)


def random_pair_set(rng, count, max_len):
    """Related and unrelated protein pairs of varied lengths, rep >= tar."""
    seqs, pairs = [], []
    for k in range(count):
        lr = int(rng.integers(0, max_len + 1))
        lt = int(rng.integers(0, lr + 1)) if rng.random() < 0.8 else lr
        a = bytes(ng_alphabet()[rng.integers(0, 20, size=lr)])
        if rng.random() < 0.7 and lr:
            b = bytearray(a[:lt])
            for p in rng.integers(0, max(lt, 1), size=lt // 10):
                if lt:
                    b[int(p)] = ng_alphabet()[rng.integers(0, 20)]
            b = bytes(b)
        else:
            b = bytes(ng_alphabet()[rng.integers(0, 20, size=lt)])
        seqs += [a, b]
        pairs.append((2 * k, 2 * k + 1))
    return seqs, np.array(pairs, np.uint32)


def ng_alphabet():
    from ngia2_gb300 import synth
    return synth.AMINO


@pytest.mark.parametrize("identity", [1, 30, 50, 70, 90, 95, 99])
def test_align_random_pairs_matches_oracle(cuda, built, identity):
    rng = np.random.default_rng(1000 + identity)
    seqs, pairs = random_pair_set(rng, 400, 1200)
    seqs2, pairs2 = random_pair_set(rng, 6, 9000)  # wide bands: general path
    pairs2 = pairs2 + len(seqs)
    packed, offs, _ = build_db(seqs + seqs2)
    allp = np.concatenate([pairs, pairs2])
    for mode, m in (("fma", oracle.ROUND_FMA), ("split", oracle.ROUND_SPLIT)):
        want = oracle.align_pairs(packed, offs, allp, identity, m)
        got = align_jobs_on_gpu(packed, offs, allp, identity, mode)
        assert np.array_equal(got, want), mode


def test_align_keeps_score_word_when_length_filter_fails(cuda, built):
    seqs = [b"ACDEFGHIKL" * 20, b"ACDEFGHIKL" * 2]
    packed, offs, _ = build_db(seqs)
    jobs = np.array([[0, 1, 77]], np.uint32)
    d_packed, d_offs, d_jobs = to_dev(packed), to_dev(offs), to_dev(jobs)
    ng.align_pairs(d_packed.data_ptr(), d_offs.data_ptr(), d_jobs.data_ptr(), 1, 90, stream())
    assert from_dev(d_jobs, np.uint32)[2] == 77


def test_emit_edges(cuda, built):
    rng = np.random.default_rng(5)
    count = 50_000
    jobs = np.zeros((count, 3), np.uint32)
    jobs[:, 0] = rng.integers(0, 1000, count)
    jobs[:, 1] = rng.integers(0, 1000, count)
    jobs[:, 2] = np.where(rng.random(count) < 0.3, rng.integers(1, 101, count), 0)
    d_jobs = to_dev(jobs)
    d_edges = dev_empty(count * 12)
    d_n = dev_empty(4)
    ng.emit_edges(d_jobs.data_ptr(), count, d_edges.data_ptr(), d_n.data_ptr(), stream())
    m = int(from_dev(d_n, np.uint32)[0])
    hit = jobs[:, 2] > 0
    assert m == int(hit.sum())
    e = from_dev(d_edges, ng.EDGE_DTYPE, m)
    assert np.array_equal(e["rep"], jobs[hit, 0].astype(np.int32))
    assert np.array_equal(e["tar"], jobs[hit, 1].astype(np.int32))
    assert np.array_equal(e["weight"], jobs[hit, 2].astype(np.float32) / np.float32(100))


def test_sort_unique_edges(cuda, built):
    rng = np.random.default_rng(6)
    m = 30_000
    e = np.zeros(m, ng.EDGE_DTYPE)
    e["rep"] = rng.integers(0, 500, m)
    e["tar"] = rng.integers(0, 500, m)
    e["weight"] = rng.integers(1, 101, m).astype(np.float32) / np.float32(100)
    e[m // 2:] = e[: m - m // 2]  # duplicates
    d = to_dev(e)
    k = ng.sort_unique_edges(d.data_ptr(), m, 500, stream())
    got = from_dev(d, ng.EDGE_DTYPE, k)
    want = np.unique(e)  # structured: lexicographic (rep, tar, weight)
    assert k == len(want)
    assert np.array_equal(got, want)


def test_sketch_bucket_at_scale(cuda, built):
    """50,000 DNA sequences: the sketch matches the oracle on a sample, and the
    rep rows match an independent numpy restatement of the bucketing on all
    bands."""
    from ngia2_gb300 import synth
    s = synth.dna_families(50_000, 5_000, seed=9)
    order = np.argsort(-s.lens, kind="stable")
    seqs = [s.seq(int(i)) for i in order]
    packed, offs, lens = build_db(seqs)
    db = {"n": len(seqs), "packed": packed, "offsets": offs}
    sigs = gpu_sketch(db)
    rng = np.random.default_rng(3)
    for i in rng.choice(len(seqs), size=300, replace=False):
        o = int(offs[i])
        rec = packed[o:o + 1 + ((int(lens[i]) + 31) // 32) * 4]
        assert np.array_equal(sigs[:, i], oracle.sketch_record(rec)), i
    rep = gpu_bucket(sigs, 64)
    assert np.array_equal(rep, reference_rep_rows(sigs))


@pytest.mark.parametrize("n,bands", [(400_000, 2), (140_000, 3), (1, 1)])
def test_bucket_long_segments(cuda, built, n, bands):
    """Segments whose digit counts outgrow one scan block (more than 32 tiles
    of 4096) take the chunked scan; same rep rows as the numpy restatement.
    Signatures from a small range, so buckets hold many members."""
    rng = np.random.default_rng(n + bands)
    sigs = rng.integers(0, 5000, size=(bands, n), dtype=np.uint32)
    sigs[:, ::7] = rng.integers(0, 2**32, size=sigs[:, ::7].shape, dtype=np.uint64)
    assert np.array_equal(gpu_bucket(sigs, bands), reference_rep_rows(sigs))
