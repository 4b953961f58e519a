"""GPU parity of the whole drop-in: makedb file bytes, the device graph build,
fast mode, and the result files of `-m clustering` / `-m fast`, against the
reference's outputs (golden fixtures)."""
from __future__ import annotations

import gzip
import hashlib
import subprocess

import numpy as np
import pytest

import ngia2_gb300 as ng
from conftest import GOLDEN, IDENTITIES, SETS, load_edges, load_pairs, result_sha

pytestmark = pytest.mark.gpu


def as_triples(e: np.ndarray) -> np.ndarray:
    return np.stack([e["rep"].astype(np.int64), e["tar"].astype(np.int64),
                     np.rint(e["weight"].astype(np.float64) * 100).astype(np.int64)], axis=1)


@pytest.mark.parametrize("name", SETS)
def test_makedb_file_is_byte_identical(cuda, built, golden, tmp_path, name):
    out = tmp_path / "mine.packed"
    n = ng.makedb(golden[name]["fa"], out)
    assert n == golden[name]["db"]["n"]
    with gzip.open(GOLDEN / f"{name}.packed.gz", "rb") as f:
        want = f.read()
    assert out.read_bytes() == want


@pytest.mark.parametrize("name", SETS)
def test_device_rep_rows_match_reference(cuda, built, golden, name):
    db = golden[name]["db"]
    with ng.Context() as ctx:
        ctx.load(db["packed"], db["offsets"], db["lens"])
        ctx.sketch_bucket(64)
        assert np.array_equal(ctx.rep_rows(64), db["rep"])


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_build_graph_matches_reference(cuda, built, golden, name, identity):
    db = golden[name]["db"]
    pairs, _, _, candidates = load_pairs(name, identity)
    with ng.Context() as ctx:
        ctx.load(db["packed"], db["offsets"], db["lens"], db["rep"], 64)
        e, st = ctx.graph(identity, 64)
        assert np.array_equal(as_triples(e), load_edges(name, identity, "fma"))
        assert st["candidate_pairs"] == candidates
        assert st["unique_pairs"] == len(pairs)
        # fewer bands: prefix of the rep rows
        e3, _ = ctx.graph(identity, 3)
        e3_ref, _ = ctx_free_graph(db, identity, 3)
        assert np.array_equal(as_triples(e3), e3_ref)


def ctx_free_graph(db, identity, bands):
    import oracle
    return oracle.graph_edges(db["packed"], db["offsets"], db["lens"], db["rep"], identity,
                              bands, oracle.ROUND_FMA)


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_fast_mode_matches_reference(cuda, built, golden, name, identity):
    db = golden[name]["db"]
    with ng.Context() as ctx:
        ctx.load(db["packed"], db["offsets"], db["lens"], db["rep"], 64)
        got = ctx.fast_cluster(identity, 64)
    assert np.array_equal(got, np.load(GOLDEN / f"{name}.fast_{identity}.npy"))


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_result_files_are_byte_identical(cuda, built, golden, tmp_path, name, identity):
    want = result_sha(name, identity)
    for kind, fast in (("leiden", False), ("fast", True)):
        out = tmp_path / f"{kind}.txt"
        ng.cluster_file(golden[name]["packed"], out, identity, 64, fast=fast)
        assert hashlib.sha256(out.read_bytes()).hexdigest() == want[kind], kind


@pytest.mark.parametrize("identity", [30, 50, 70, 90, 95])
def test_batched_aligner_on_chosen_pairs(cuda, built, identity):
    """Arbitrary pair sets through the batched path (every width class): rep
    rows are written so that target i's candidates are chosen partners j < i,
    and the sorted edge list must equal the oracle's."""
    import oracle
    from ngia2_gb300 import synth
    from gpu_util import build_db
    rng = np.random.default_rng(400 + identity)
    seqs = []
    for k in range(120):  # families of related sequences of varied length
        root = synth._draw(rng, synth.AMINO, synth.AMINO_FREQ,
                           int(rng.integers(20, 3000 if k % 10 else 6000))).tobytes()
        for _ in range(5):
            b = bytearray(root[: max(1, int(len(root) * rng.uniform(0.88, 1.0)))])
            for p in rng.integers(0, len(b), size=int(len(b) * rng.uniform(0, 0.12))):
                b[int(p)] = synth.AMINO[rng.integers(0, 20)]
            seqs.append(bytes(b))
    seqs.sort(key=len, reverse=True)  # index order = length descending
    packed, offs, lens = build_db(seqs)
    n = len(seqs)
    rep = np.tile(np.arange(n, dtype=np.uint32), (8, 1))
    for b in range(8):
        for i in range(1, n):
            if rng.random() < 0.7:
                rep[b, i] = rng.integers(max(0, i - 12), i)
    with ng.Context() as ctx:
        ctx.load(packed, offs, lens, rep, 8)
        e, st = ctx.graph(identity, 8)
    want, total = oracle.graph_edges(packed, offs, lens, rep, identity, 8, oracle.ROUND_FMA)
    assert st["candidate_pairs"] == total
    assert np.array_equal(as_triples(e), want)


def test_cli_end_to_end(cuda, built, golden, tmp_path):
    packed = tmp_path / "p.packed"
    r = subprocess.run([str(ng.CLI_PATH), "-m", "makedb", "-f", str(golden["prot"]["fa"]), "-p",
                        str(packed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for identity in IDENTITIES["prot"]:
        res = tmp_path / f"r{identity}.txt"
        r = subprocess.run([str(ng.CLI_PATH), "cluster", "-i", str(identity), "-p", str(packed),
                            "-r", str(res)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert hashlib.sha256(res.read_bytes()).hexdigest() == result_sha("prot", identity)["leiden"]
        fres = tmp_path / f"f{identity}.txt"
        r = subprocess.run([str(ng.CLI_PATH), "-m", "fast", "-p", str(packed), "-r", str(fres),
                            "-i", str(identity)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert hashlib.sha256(fres.read_bytes()).hexdigest() == result_sha("prot", identity)["fast"]


def test_run_host_matches_resident_path(cuda, built, golden):
    db = golden["prot"]["db"]
    out = np.empty(64 * db["n"], ng.EDGE_DTYPE)
    with ng.Context() as ctx:
        m, st = ctx.run_host(np.ascontiguousarray(db["packed"]),
                             np.ascontiguousarray(db["offsets"]), np.ascontiguousarray(db["lens"]),
                             50, 64, out)
        assert np.array_equal(as_triples(out[:m]), load_edges("prot", 50, "fma"))
        # a second call reuses the context's device buffers
        m2, _ = ctx.run_host(np.ascontiguousarray(db["packed"]),
                             np.ascontiguousarray(db["offsets"]),
                             np.ascontiguousarray(db["lens"]), 70, 64, out)
        assert np.array_equal(as_triples(out[:m2]), load_edges("prot", 70, "fma"))


def test_makedb_at_the_length_limit_is_byte_identical(cuda, built, tmp_path):
    """Reads of 65,534 residues kept (signed over 65,527 positions, grouped
    with their near copies), 65,535 and longer dropped: the device makedb's
    file equals the reference's own makedb byte for byte."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    rng = np.random.default_rng(65534)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    root = rng.choice(acgt, size=65534)
    near = root.copy()
    near[rng.integers(0, near.size, 40)] = rng.choice(acgt, size=40)
    reads = [rng.choice(acgt, size=120), rng.choice(acgt, size=65535), root,
             rng.choice(acgt, size=70000), near, rng.choice(acgt, size=65533),
             np.zeros(0, np.uint8), rng.choice(acgt, size=3000)]
    fa = tmp_path / "limit.fa"
    fa.write_bytes(b"".join(b">r%d\n" % i + bytes(r) + b"\n" for i, r in enumerate(reads)))
    mine, ref = tmp_path / "mine.packed", tmp_path / "ref.packed"
    assert ng.makedb(fa, mine) == sum(1 for r in reads if r.size < 0xFFFF)
    assert oracle.ref_makedb(fa, ref) == 0
    assert mine.read_bytes() == ref.read_bytes()


def test_makedb_unusual_records_byte_identical(cuda, built, tmp_path):
    """Lower case, ambiguity and stop letters, digits, tabs and spaces in reads,
    empty reads and reads over several lines: the device makedb's file equals
    the reference's own makedb byte for byte (planes, signatures, rep rows)."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    fa = tmp_path / "unusual.fa"
    fa.write_bytes(b">a desc with spaces\nacgtNNNNacgt\nACGT\n"
                   b">b\nMKV*LAX-UBZJOx\n"
                   b">c\n\n\n"
                   b">d\n" + b"ACGT" * 5 + b"\n" + b"acgu" * 3 + b"\n"
                   b">e 123\n12345 ACGT\tTT\n"
                   b">f\nACGTACGT\n")
    mine, ref = tmp_path / "mine.packed", tmp_path / "ref.packed"
    assert ng.makedb(fa, mine) == 6
    assert oracle.ref_makedb(fa, ref) == 0
    assert mine.read_bytes() == ref.read_bytes()
