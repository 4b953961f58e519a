"""Host-side parts of the drop-in that need no GPU: the C-ABI library loads and
exports every entry point of include/ngia.h; Leiden and the result file are
bit-exact with the reference; the CLI's argument handling."""
from __future__ import annotations

import hashlib
import re
import subprocess
import sys

import numpy as np
import pytest

import ngia2_gb300 as ng
from conftest import GOLDEN, IDENTITIES, ROOT, SETS, load_edges, result_sha


def header_symbols() -> set[str]:
    text = (ROOT / "include" / "ngia.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(ngia_[a-z0-9_]+)\s*\(", text))


def test_library_exports_every_declared_symbol(built):
    L = ng.lib()
    declared = header_symbols()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(L, name), name
    assert declared == set(ng.exported_symbols())
    assert b"sm_103a" in L.ngia_version()


def test_status_strings(built):
    L = ng.lib()
    assert L.ngia_status_string(0) == b"ok"
    assert L.ngia_status_string(-1) == b"invalid argument"
    assert L.ngia_status_string(-2) == b"CUDA error"


def test_argument_errors_need_no_gpu(built):
    L = ng.lib()
    assert L.ngia_align_pairs(0, 0, 0, 0, 90, 0) == 0  # empty batch is a no-op
    assert L.ngia_align_pairs(0, 0, 0, 5, 0, 0) == -1  # identity out of range
    assert L.ngia_align_pairs(0, 0, 0, 5, 100, 0) == -1
    assert L.ngia_bucket(0, 10, 65, 0, 0) == -1  # bands out of range
    assert L.ngia_sketch(0, 0, 10, 0, 0) == -1  # NULL pointers


def edges_struct(e: np.ndarray) -> np.ndarray:
    out = np.zeros(len(e), ng.EDGE_DTYPE)
    out["rep"] = e[:, 0]
    out["tar"] = e[:, 1]
    out["weight"] = e[:, 2].astype(np.float32) / np.float32(100)
    return out


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_leiden_matches_reference(built, golden, name, identity):
    n = golden[name]["db"]["n"]
    clu = ng.leiden(edges_struct(load_edges(name, identity)), n, ng.leiden_resolution(identity))
    assert np.array_equal(clu, np.load(GOLDEN / f"{name}.leiden_{identity}.npy"))


def test_leiden_resolution(built):
    assert ng.leiden_resolution(50) == 1.0
    assert abs(ng.leiden_resolution(90) - 0.2) < 1e-7
    assert abs(ng.leiden_resolution(95) - 0.1) < 1e-7
    assert abs(ng.leiden_resolution(1) - 0.02) < 1e-7


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_result_file_matches_reference(built, golden, tmp_path, name, identity):
    want = result_sha(name, identity)
    for kind, arr in (("leiden", np.load(GOLDEN / f"{name}.leiden_{identity}.npy")),
                      ("fast", np.load(GOLDEN / f"{name}.fast_{identity}.npy"))):
        out = tmp_path / f"{kind}.txt"
        ng.save_result(arr, golden[name]["packed"], out)
        assert hashlib.sha256(out.read_bytes()).hexdigest() == want[kind], kind


def test_read_packed_layout(golden):
    for name in SETS:
        db = golden[name]["db"]
        n = db["n"]
        assert np.all(np.diff(db["lens"].astype(np.int64)) <= 0)  # length-descending
        assert int(db["pack_off"][0]) == 4 + 24 * n + 256 * n
        words = 1 + ((db["lens"].astype(np.int64) + 31) // 32) * 4
        assert np.array_equal(np.diff(db["offsets"].astype(np.int64)), words[:-1])
        assert np.all(db["packed"][db["offsets"].astype(np.int64)] == db["lens"])
        last = n - 1
        size = int(db["fasta_off"][last]) + int(db["name_lens"][last]) + int(db["lens"][last]) + 2
        assert size == db["raw"].size
        rep = db["rep"].astype(np.int64)
        assert np.all(rep <= np.arange(n))


def test_read_packed_without_records(tmp_path):
    path = tmp_path / "empty.packed"
    path.write_bytes(np.zeros(1, np.uint32).tobytes())
    db = ng.read_packed(path)
    assert db["n"] == 0 and db["packed"].size == 0 and db["offsets"].size == 0
    assert db["rep"].shape == (ng.BANDS, 0)


def run_cli(*args):
    return subprocess.run([str(ng.CLI_PATH), *args], capture_output=True, text=True,
                          timeout=60)


def test_cli_usage_paths(built, tmp_path):
    r = run_cli()
    assert r.returncode == 0 and "usage" in r.stdout
    r = run_cli("-m", "clustering", "-p", str(tmp_path / "missing.packed"), "-r",
                str(tmp_path / "r.txt"))
    assert r.returncode == 0 and "does not exists" in r.stdout and "Usage" in r.stdout
    r = run_cli("-m", "makedb", "-f", str(tmp_path / "missing.fa"), "-p", str(tmp_path / "x"))
    assert r.returncode == 0 and "Usage" in r.stdout
    bad = tmp_path / "bad.fa"
    bad.write_bytes(b">a\r\nACGT\n")
    r = run_cli("-m", "makedb", "-f", str(bad), "-p", str(tmp_path / "x"))
    assert r.returncode == 0 and "\\r" in r.stdout
    bad.write_bytes(b">a\nACGT")
    r = run_cli("-m", "makedb", "-f", str(bad), "-p", str(tmp_path / "x"))
    assert r.returncode == 0 and "end with" in r.stdout
    r = run_cli("-m", "nonsense")
    assert r.returncode == 0 and "makedb/clustering/fast" in r.stdout


def test_cli_checks_identity_and_bands(built, golden, tmp_path):
    packed = str(golden["prot"]["packed"])
    for flags in (("-i", "0"), ("-i", "100"), ("-i", "abc"), ("-b", "0"), ("-b", "65")):
        r = run_cli("-m", "clustering", "-p", packed, "-r", str(tmp_path / "r.txt"), *flags)
        assert r.returncode == 0 and "Usage" in r.stdout, flags
    # README spelling: cluster -i -p -r goes to the same checks
    r = run_cli("cluster", "-i", "100", "-p", packed, "-r", str(tmp_path / "r.txt"))
    assert r.returncode == 0 and "identity should be 1-99" in r.stdout


def _cli_essentials(out: str, prog: str) -> list[str]:
    """The lines of a command-line run that carry its outcome: messages and
    usage text, without dates, timers and the settings the reference echoes."""
    import re
    keep = []
    for line in out.splitlines():
        s = line.strip()
        if (not s or "Consuming" in s or re.match(r"^[A-Z][a-z]{2} [A-Z][a-z]{2} +\d", s)
                or re.match(r"^(use gpu|packed file|result file|fasta file|fasta|packed|"
                            r"thread|identity|rounds|bands):", s)):
            continue
        keep.append(line.replace(prog, "PROG"))
    return keep


def test_cli_parser_quirks_match_the_reference(built, golden, tmp_path):
    """Argument handling against the reference's own command line (its host
    build): a later flag overrides an earlier one, the last token is never
    read as a flag name, invalid identity or bands and a missing file print
    the usage and exit 0 -- the same messages and exit codes."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    ref = str(oracle.ref_cli())
    packed = str(golden["prot"]["packed"])
    out = str(tmp_path / "r.txt")
    cases = [
        ["-m", "clustering", "-p", packed, "-r", out, "-i", "95", "-i", "0"],
        ["-m", "clustering", "-p", packed, "-r", out, "-b", "64", "-b", "65"],
        ["-m", "clustering", "-p", packed, "-r", out, "-i", "0", "-i"],
        ["-m", "clustering", "-i", "0", "-p", packed, "-r"],
        ["-m", "fast", "-p", packed, "-r", out, "-i", "100"],
        ["-m", "fast", "-p", packed, "-r", out, "-b", "0"],
        ["-m", "clustering", "-p", str(tmp_path / "missing"), "-r", out],
        ["-m", "makedb", "-f", str(tmp_path / "missing.fa"), "-p", out],
        ["-p", packed, "-r", out, "-m"],
        ["-m", "nonsense"],
        [],
    ]
    for args in cases:
        a = subprocess.run([ref, *args], capture_output=True, text=True, timeout=60)
        b = run_cli(*args)
        assert a.returncode == b.returncode == 0, args
        assert _cli_essentials(a.stdout, ref) == _cli_essentials(b.stdout, str(ng.CLI_PATH)), \
            args


def planted_graph(rng, n: int, groups: int, p_in: float, out_edges: int) -> np.ndarray:
    """Edges (rep < tar, sorted, unique) of a graph with planted groups, as
    the graph build emits them, weights score / 100 for scores 50..100."""
    label = rng.integers(0, groups, n)
    pairs = set()
    for g in range(groups):
        members = np.nonzero(label == g)[0]
        for i in range(len(members)):
            for j in range(i + 1, len(members)):
                if rng.random() < p_in:
                    pairs.add((int(members[i]), int(members[j])))
    for _ in range(out_edges):
        a, b = (int(x) for x in rng.integers(0, n, 2))
        if a != b:
            pairs.add((min(a, b), max(a, b)))
    e = np.array(sorted(pairs), np.int64).reshape(-1, 2)
    out = np.zeros(len(e), ng.EDGE_DTYPE)
    out["rep"], out["tar"] = e[:, 0], e[:, 1]
    out["weight"] = rng.integers(50, 101, len(e)).astype(np.float32) / np.float32(100)
    return out


@pytest.mark.parametrize("n,groups,p_in,out_edges", [
    (300, 40, 0.6, 100), (2000, 150, 0.3, 3000), (5000, 60, 0.05, 20000), (4000, 4000, 0.0, 0),
])
def test_leiden_matches_reference_on_planted_graphs(built, n, groups, p_in, out_edges):
    """The host Leiden against the reference's own LeidenOmp (its host build,
    same seed, same threads) on graphs with planted groups, sparse to dense,
    isolated nodes included, at the three resolutions the command line uses."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    rng = np.random.default_rng(n + groups)
    e = planted_graph(rng, n, groups, p_in, out_edges)
    for resolution in (0.1, 0.2, 1.0):
        for iterations in (1, 2):
            want = oracle.ref_leiden(e["rep"].astype(np.int32), e["tar"].astype(np.int32),
                                     e["weight"], n, resolution, 42, iterations)
            got = ng.leiden(e, n, resolution, 42, iterations)
            assert np.array_equal(got, want), (resolution, iterations)


LEIDEN_THREADS_CHECK = r'''
import sys
sys.path[:0] = [sys.argv[1], sys.argv[1] + "/tests"]
import numpy as np, oracle, ngia2_gb300 as ng
from test_host import planted_graph
e = planted_graph(np.random.default_rng(7), 3000, 100, 0.3, 5000)
want = oracle.ref_leiden(e["rep"].astype(np.int32), e["tar"].astype(np.int32), e["weight"],
                         3000, 0.2, 42, 1)
got = ng.leiden(e, 3000, 0.2, 42, 1)
import hashlib
print(int(np.array_equal(got, want)), hashlib.sha256(want.tobytes()).hexdigest())
'''


def test_leiden_follows_the_reference_at_each_thread_count(built):
    """The reference's LeidenOmp run with 1, 2 and 3 OpenMP threads: the host
    Leiden equals it at each, and the reference's clusters do not change with
    the thread count."""
    import os
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    seen = set()
    for threads in (1, 2, 3):
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        r = subprocess.run([sys.executable, "-c", LEIDEN_THREADS_CHECK, str(ROOT)], env=env,
                           capture_output=True, text=True, timeout=300, check=True)
        same, head = r.stdout.split()
        assert same == "1", threads
        seen.add(head)
    assert len(seen) == 1


def test_result_file_matches_reference_on_any_clustering(built, golden, tmp_path):
    """SaveResult against the reference's own (its host build) on clusterings
    the golden sets do not hold: all singletons, one cluster, fast-mode root
    ids, ids numbered in an arbitrary order, and ids larger than n."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    packed = golden["prot"]["packed"]
    n = golden["prot"]["db"]["n"]
    rng = np.random.default_rng(99)
    roots = np.arange(n, dtype=np.uint32)
    for i in range(1, n):
        if rng.random() < 0.7:
            roots[i] = roots[rng.integers(0, i)]
    labels = rng.integers(0, 37, n).astype(np.uint32)
    cases = {
        "singletons": np.arange(n, dtype=np.uint32),
        "one cluster": np.zeros(n, np.uint32),
        "roots": roots,
        "arbitrary order": rng.permutation(37).astype(np.uint32)[labels],
        "large ids": (labels * 1_000_003 + 7).astype(np.uint32),
    }
    for name, cluster in cases.items():
        mine, ref = tmp_path / "mine.txt", tmp_path / "ref.txt"
        ng.save_result(cluster, packed, mine)
        oracle.ref_save(cluster, packed, ref)
        assert mine.read_bytes() == ref.read_bytes(), name


C_CALLER = r'''
#include <stdio.h>
#include "ngia.h"
int main(void) {
  ngia_stats st;
  (void)st;
  printf("%s|%s|%d\n", ngia_version(), ngia_status_string(NGIA_ERR_ARG),
         ngia_bucket(0, 0, 65, 0, 0));
  return 0;
}
'''


@pytest.mark.parametrize("compiler,flags", [("gcc", ["-std=c99", "-x", "c"]),
                                            ("g++", ["-std=c++11", "-x", "c++"])])
def test_header_builds_a_plain_c_and_cpp_caller(built, tmp_path, compiler, flags):
    """include/ngia.h compiles warning-free as C99 and as C++11 (-Wall -Wextra
    -pedantic -Werror), and a caller links libngia.so and calls it without a
    GPU (argument checks only)."""
    import shutil
    cc = shutil.which(compiler)
    if cc is None:
        pytest.skip(f"{compiler} not available")
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    lib = ROOT / "ngia2_gb300" / "lib"
    subprocess.run([cc, *flags, "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                    str(ROOT / "include"), str(src), "-x", "none", "-o", str(exe),
                    "-L", str(lib), "-lngia", f"-Wl,-rpath,{lib}"],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60,
                         check=True).stdout.strip().split("|")
    assert out[0] and out[1] and int(out[2]) == ng.ERR_ARG
