"""The host half of makedb (index, layout, header and cleaned FASTA records,
written into the mapped packed file) against the reference's packed files
for the golden sets: every byte outside the signature area and the planes
(which the device fills) equal, those two areas still zero.  A small C++
driver links libngia.so and calls the host steps only; no GPU."""
from __future__ import annotations

import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, SETS

PROGRAM = r'''
#include <cstdio>
#include "host.hpp"
int main(int argc, char **argv) {
  ngia::Makedb m;
  int st = ngia::makedb_prepare(argv[1], argv[2], m);
  if (st == NGIA_OK) st = ngia::makedb_finish(m);
  std::printf("%d %llu %u\n", st, (unsigned long long)m.scanned, m.n);
  return 0;
}
'''


@pytest.fixture(scope="module")
def driver(built, tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("makedb_host")
    src = d / "drv.cpp"
    src.write_text(PROGRAM)
    exe = d / "drv"
    lib = ROOT / "ngia2_gb300" / "lib"
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", str(ROOT / "include"),
                    "-I", str(ROOT / "ngia2_gb300" / "csrc"), str(src), "-o", str(exe),
                    "-L", str(lib), "-lngia", f"-Wl,-rpath,{lib}", "-pthread"],
                   check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("name", SETS)
def test_host_half_of_makedb_matches_reference(driver, golden, tmp_path, name):
    out = tmp_path / "host.packed"
    r = subprocess.run([str(driver), str(golden[name]["fa"]), str(out)], capture_output=True,
                       text=True, check=True)
    st, scanned, n = map(int, r.stdout.split())
    assert st == 0
    want = golden[name]["packed"].read_bytes()
    got = out.read_bytes()
    assert len(got) == len(want)
    (nw,) = struct.unpack_from("<I", want, 0)
    assert n == nw
    sig0, pack0 = 4 + 24 * n, 4 + 280 * n
    fasta0 = struct.unpack_from("<Q", want, 4 + 16 * n)[0]
    assert got[:sig0] == want[:sig0], "header differs"
    assert got[fasta0:] == want[fasta0:], "FASTA area differs"
    assert not np.frombuffer(got[sig0:fasta0], np.uint8).any(), "device areas not left zero"
    fa = golden[name]["fa"].read_bytes()
    assert scanned == fa.count(b"\n>") + (1 if fa.startswith(b">") else 0)


def test_index_handles_wrapped_lines_and_stray_records(driver, tmp_path):
    """Reads wrapped over several lines, an empty read, a record before any
    '>' line, and equal lengths kept in file order."""
    fa = tmp_path / "w.fa"
    fa.write_bytes(b"ACGT\nAC\n>a\nAAAA\nCC\n\nGG\n>b\n>c\nACGTACGT\n>d\nTTTT\nTTTT\n")
    out = tmp_path / "w.packed"
    r = subprocess.run([str(driver), str(fa), str(out)], capture_output=True, text=True,
                       check=True)
    st, scanned, n = map(int, r.stdout.split())
    assert (st, scanned, n) == (0, 5, 5)
    b = out.read_bytes()
    name_lens = struct.unpack_from("<5I", b, 4)
    lens = struct.unpack_from("<5I", b, 24)
    # records: "ACGT"(AC) len 2, a: 8, b: 0, c: 8, d: 8 -> a, c, d, first, b
    assert lens == (8, 8, 8, 2, 0)
    assert name_lens == (2, 2, 2, 4, 2)
    fasta0 = struct.unpack_from("<Q", b, 4 + 16 * 5)[0]
    assert b[fasta0:] == b">a\nAAAACCGG\n>c\nACGTACGT\n>d\nTTTTTTTT\nACGT\nAC\n>b\n\n"


def test_length_filter_matches_reference(driver, tmp_path):
    """Reads at the format's limit: 65,534 residues kept, 65,535 and longer
    dropped (their records absent from the index and the FASTA area), against
    the reference's own makedb on the same file."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference's host build is not available")
    rng = np.random.default_rng(0xFFFF)
    lengths = [120, 65535, 65534, 70000, 8, 65533, 65534, 0, 65536, 3000]
    fa = tmp_path / "limit.fa"
    with open(fa, "wb") as f:
        for i, n in enumerate(lengths):
            f.write(b">r%d\n" % i + bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), size=n))
                    + b"\n")
    out = tmp_path / "host.packed"
    r = subprocess.run([str(driver), str(fa), str(out)], capture_output=True, text=True,
                       check=True)
    st, scanned, n = map(int, r.stdout.split())
    assert (st, scanned) == (0, len(lengths))
    assert n == sum(1 for x in lengths if x < 0xFFFF)
    ref = tmp_path / "ref.packed"
    assert oracle.ref_makedb(fa, ref) == 0  # status
    want = ref.read_bytes()
    got = out.read_bytes()
    assert len(got) == len(want)
    sig0 = 4 + 24 * n
    fasta0 = struct.unpack_from("<Q", want, 4 + 16 * n)[0]
    assert got[:sig0] == want[:sig0], "header differs"
    assert got[fasta0:] == want[fasta0:], "FASTA area differs"
    lens = struct.unpack_from(f"<{n}I", got, 4 + 4 * n)
    assert lens == tuple(sorted((x for x in lengths if x < 0xFFFF), reverse=True))


def test_unusual_records_match_reference(driver, tmp_path):
    """Lower case, ambiguity and stop letters, digits, tabs and spaces in reads,
    description text in names, empty reads and reads over several lines:
    the index and the FASTA area equal the reference's own makedb."""
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
    out, ref = tmp_path / "host.packed", tmp_path / "ref.packed"
    r = subprocess.run([str(driver), str(fa), str(out)], capture_output=True, text=True,
                       check=True)
    st, scanned, n = map(int, r.stdout.split())
    assert (st, scanned, n) == (0, 6, 6)
    assert oracle.ref_makedb(fa, ref) == 0  # status
    want, got = ref.read_bytes(), out.read_bytes()
    assert len(got) == len(want)
    sig0 = 4 + 24 * n
    fasta0 = struct.unpack_from("<Q", want, 4 + 16 * n)[0]
    assert got[:sig0] == want[:sig0], "header differs"
    assert got[fasta0:] == want[fasta0:], "FASTA area differs"
