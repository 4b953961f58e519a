"""The CPU oracle pinned against the reference's own outputs (golden fixtures
made by running the reference's makedb / kernel / buildGraph code)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, IDENTITIES, SETS, load_edges, load_pairs


def records(db):
    for i in range(db["n"]):
        o = int(db["offsets"][i])
        yield db["packed"][o:o + 1 + ((int(db["lens"][i]) + 31) // 32) * 4]


def fasta_records(path):
    """(name, residues) of the FASTA records makedb keeps, in file order."""
    data = path.read_bytes()
    out = []
    for rec in data.split(b"\n>"):
        lines = rec.split(b"\n")
        name = lines[0] if lines[0].startswith(b">") else b">" + lines[0]
        seq = b"".join(lines[1:])
        out.append((name, seq))
    return out


@pytest.mark.parametrize("name", SETS)
def test_pack_matches_reference(built, golden, name):
    db = golden[name]["db"]
    recs = [r for r in fasta_records(golden[name]["fa"]) if len(r[1]) < 0xFFFF]
    # makedb order: stable by length descending
    order = sorted(range(len(recs)), key=lambda i: -len(recs[i][1]))
    assert db["n"] == len(recs)
    for i, rec in zip(order, records(db)):
        assert np.array_equal(oracle.pack_record(recs[i][1]), rec)


@pytest.mark.parametrize("name", SETS)
def test_sketch_matches_reference(built, golden, name):
    db = golden[name]["db"]
    sigs = np.load(GOLDEN / f"{name}.sigs.npy")
    mine = oracle.sketch_all(db["packed"], db["offsets"], db["lens"])
    assert np.array_equal(mine, sigs.T)


@pytest.mark.parametrize("name", SETS)
def test_bucket_matches_reference(built, golden, name):
    db = golden[name]["db"]
    sigs = np.load(GOLDEN / f"{name}.sigs.npy")
    for b in range(64):
        assert np.array_equal(oracle.bucket_band(sigs[:, b]), db["rep"][b]), b


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_align_matches_reference(built, golden, name, identity):
    db = golden[name]["db"]
    pairs, s_split, s_fma, _ = load_pairs(name, identity)
    assert np.array_equal(oracle.align_pairs(db["packed"], db["offsets"], pairs, identity,
                                             oracle.ROUND_SPLIT), s_split)
    assert np.array_equal(oracle.align_pairs(db["packed"], db["offsets"], pairs, identity,
                                             oracle.ROUND_FMA), s_fma)


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_graph_matches_reference(built, golden, name, identity):
    db = golden[name]["db"]
    for mode, tag in ((oracle.ROUND_SPLIT, "split"), (oracle.ROUND_FMA, "fma")):
        e, total = oracle.graph_edges(db["packed"], db["offsets"], db["lens"], db["rep"],
                                      identity, 64, mode)
        assert np.array_equal(e, load_edges(name, identity, tag))
    assert total == load_pairs(name, identity)[3]


def test_known_answer_lcs(built):
    """Full-band cases: the banded bit-parallel LCS equals the textbook DP."""
    z = np.load(GOLDEN / "known_answer.npz")
    ra = np.concatenate([[0], np.cumsum(z["rep_lens"])])
    ta = np.concatenate([[0], np.cumsum(z["tar_lens"])])
    for k in range(len(z["lcs"])):
        a = z["reps"][ra[k]:ra[k + 1]].tobytes()
        b = z["tars"][ta[k]:ta[k + 1]].tobytes()
        got = oracle.banded_lcs(oracle.pack_record(a), oracle.pack_record(b), 1)
        assert got == z["lcs"][k], (a, b)


def test_identity_formula(built):
    # identical 40-residue sequences: LCS 40, identity 40*100/(40+40-40) = 100
    s = b"ACDEFGHIKLMNPQRSTVWY" * 2
    r = oracle.pack_record(s)
    assert oracle.align_records(r, r, 90) == 100
    # disjoint codes: LCS 0 -> 0
    assert oracle.align_records(oracle.pack_record(b"A" * 40), oracle.pack_record(b"C" * 40),
                                1) == 0
    # code-0 residues never match, even against themselves
    x = oracle.pack_record(b"X" * 40)
    assert oracle.align_records(x, x, 1) == 0
    # half of a 40-mer: LCS 20 of 40 vs 20 -> 20*100/(40+20-20) = 50
    assert oracle.align_records(oracle.pack_record(s), oracle.pack_record(s[:20]), 40) == 50


def test_round_modes_differ_where_expected(built):
    # t = 0.9f: 320 - 320*t is exactly 32 after rounding the product, but
    # slightly above 32 when fused, which moves both band edges by one block.
    assert oracle.band_bounds(320, 320, 90, oracle.ROUND_SPLIT) == (32, 64)
    assert oracle.band_bounds(320, 320, 90, oracle.ROUND_FMA) == (64, 65)
    assert oracle.band_blocks(320, 320, 90, oracle.ROUND_SPLIT) < \
        oracle.band_blocks(320, 320, 90, oracle.ROUND_FMA)
    # at 300 the right bound differs by one residue but not in whole blocks
    assert oracle.band_bounds(300, 300, 90, oracle.ROUND_SPLIT) == (32, 62)
    assert oracle.band_bounds(300, 300, 90, oracle.ROUND_FMA) == (32, 63)
    assert oracle.band_blocks(300, 300, 90, oracle.ROUND_SPLIT) == \
        oracle.band_blocks(300, 300, 90, oracle.ROUND_FMA)
    # the length filter rejects Lt < Lr * t
    assert oracle.band_bounds(100, 89, 90) is None


def test_align_matches_reference_kernel_on_random_pairs(built):
    """The C restatement of the banded LCS against the reference's own
    kernel_dynamic (its host build), pair by pair, on random related and
    unrelated pairs over the whole identity range and both roundings --
    including lengths at the FMA-sensitive multiples of 10 and 32."""
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    rng = np.random.default_rng(31337)
    amino = np.frombuffer(b"ACDEFGHIKLMNPQRSTVWYX", np.uint8)
    seqs, pairs = [], []
    lengths = list(rng.integers(1, 3000, size=240)) + [10, 20, 32, 64, 320, 640, 1000, 2560]
    for L in lengths:
        L = int(L)
        a = rng.choice(amino, size=L)
        if rng.random() < 0.6:
            b = a.copy()
            at = rng.random(L) < rng.uniform(0.0, 0.4)
            b[at] = rng.choice(amino, size=int(at.sum()))
            keep = rng.random(L) >= rng.uniform(0.0, 0.05)  # deletions
            b = b[keep] if keep.any() else b[:1]
        else:
            b = rng.choice(amino, size=max(1, int(L * rng.uniform(0.5, 1.0))))
        seqs += [bytes(a), bytes(b)] if a.size >= b.size else [bytes(b), bytes(a)]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    recs = [oracle.pack_record(s) for s in seqs]
    offs = np.concatenate([[0], np.cumsum([len(r) for r in recs])[:-1]]).astype(np.uint64)
    packed = np.concatenate(recs).astype(np.uint32)
    pairs = np.array(pairs, np.uint32)
    hits = 0
    for identity in (1, 10, 30, 50, 70, 80, 90, 95, 99):
        for mode in (oracle.ROUND_SPLIT, oracle.ROUND_FMA):
            want = oracle.ref_align_jobs(packed, offs, pairs, identity, mode)
            got = oracle.align_pairs(packed, offs, pairs, identity, mode)
            assert np.array_equal(got, want), (identity, mode, np.nonzero(got != want)[0][:5])
            hits += int((want > 0).sum())
    assert hits > 0


def random_reads_fasta(tmp_path, seed: int = 2024):
    """Random protein and nucleotide reads of 0 to 4,000 residues (every tenth
    under 12), 40 % of them followed by a near copy (2 % substitutions)."""
    rng = np.random.default_rng(seed)
    amino = np.frombuffer(b"ACDEFGHIKLMNPQRSTVWYXBZ*", np.uint8)
    acgt = np.frombuffer(b"ACGTN", np.uint8)
    reads = []
    for k in range(400):
        letters = amino if k % 2 else acgt
        L = int(rng.integers(0, 12)) if k % 10 == 0 else int(rng.integers(0, 4000))
        r = rng.choice(letters, size=L)
        reads.append(r)
        if L and rng.random() < 0.4:  # a near copy
            c = r.copy()
            at = rng.random(L) < 0.02
            c[at] = rng.choice(letters, size=int(at.sum()))
            reads.append(c)
    fa = tmp_path / "random.fa"
    fa.write_bytes(b"".join(b">s%d\n" % i + bytes(r) + b"\n" for i, r in enumerate(reads)))
    return reads, fa


def test_pack_sketch_bucket_match_reference_makedb_on_random_reads(built, tmp_path):
    """The restated pack, sketch and grouping against the reference's own
    makedb (its host build) on random protein and nucleotide reads of 0 to
    4,000 residues -- lengths under 8 included -- with near copies so that
    bands group: the planes, the seq-major signatures (makedb without its
    grouping step) and the rep rows (with it)."""
    import ngia2_gb300 as ng
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    reads, fa = random_reads_fasta(tmp_path)
    seq_major, grouped = tmp_path / "nogroup.packed", tmp_path / "group.packed"
    assert oracle.ref_makedb(fa, seq_major, group=False) == 0
    assert oracle.ref_makedb(fa, grouped, group=True) == 0
    db = ng.read_packed(grouped)
    n = db["n"]
    assert n == len(reads)
    order = sorted(range(n), key=lambda i: -len(reads[i]))  # stable, length descending
    for i, o in zip(order, db["offsets"]):
        rec = db["packed"][int(o):int(o) + 1 + ((len(reads[i]) + 31) // 32) * 4]
        assert np.array_equal(oracle.pack_record(bytes(reads[i])), rec), i
    sigs = oracle.sketch_all(db["packed"], db["offsets"], db["lens"])
    raw = np.fromfile(seq_major, np.uint8)
    ref_sigs = raw[4 + 24 * n:4 + 24 * n + 256 * n].view(np.uint32).reshape(n, 64)
    assert np.array_equal(sigs, ref_sigs.T)
    for b in range(64):
        assert np.array_equal(oracle.bucket_band(sigs[b]), db["rep"][b]), b


def test_graph_matches_reference_build_graph_on_random_reads(built, tmp_path):
    """Candidate collection, scores and edge emission restated, against the
    reference's own readData + buildGraph on the grouped random reads, at
    identities 50 to 95, 64 and 7 bands, both roundings."""
    import ngia2_gb300 as ng
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    _, fa = random_reads_fasta(tmp_path, seed=77)
    packed = tmp_path / "group.packed"
    assert oracle.ref_makedb(fa, packed, group=True) == 0
    db = ng.read_packed(packed)
    edges = 0
    split, fma = oracle.ROUND_SPLIT, oracle.ROUND_FMA
    for identity, bands, mode in ((50, 64, fma), (80, 7, split), (90, 64, split),
                                  (90, 64, fma), (95, 64, fma), (95, 7, split)):
        mine, _ = oracle.graph_edges(db["packed"], db["offsets"], db["lens"], db["rep"],
                                     identity, bands, mode)
        rep, tar, w = oracle.ref_build_graph(packed, identity, bands, 4096, mode)
        ref = np.stack([rep.astype(np.int64), tar.astype(np.int64),
                        np.rint(w.astype(np.float64) * 100).astype(np.int64)], axis=1)
        ref = ref[np.lexsort((ref[:, 1], ref[:, 0]))]
        assert np.array_equal(mine, ref), (identity, bands, mode)
        edges += len(mine)
    assert edges > 0


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_fast_cluster_matches_reference(built, golden, name, identity):
    """The restated fast mode against the reference's own fast clusters
    (golden fixtures from its FastClustering::cluster)."""
    db = golden[name]["db"]
    got = oracle.fast_cluster(db["packed"], db["offsets"], db["rep"], identity, 64)
    assert np.array_equal(got, np.load(GOLDEN / f"{name}.fast_{identity}.npy"))


def test_fast_cluster_matches_reference_on_random_reads(built, tmp_path):
    """The restated fast mode against the reference's host build on the
    grouped random reads, several identities and band counts."""
    import ngia2_gb300 as ng
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    _, fa = random_reads_fasta(tmp_path, seed=5)
    packed = tmp_path / "group.packed"
    assert oracle.ref_makedb(fa, packed, group=True) == 0
    db = ng.read_packed(packed)
    merged = 0
    for identity, bands in ((50, 64), (90, 64), (95, 9)):
        got = oracle.fast_cluster(db["packed"], db["offsets"], db["rep"], identity, bands)
        want = oracle.ref_fast_cluster(packed, identity, bands, db["n"])
        assert np.array_equal(got, want), (identity, bands)
        merged += int((got != np.arange(db["n"])).sum())
    assert merged > 0
