"""The command line end to end against the reference's own GPU build (its
src/main.cu built unmodified by nvcc, run on the same GPU), on the small
protein configuration: 20,000 synthetic proteins from 2,000 families
(log-normal roots of median 300, 5-35 % substitutions, 2 % indels, seed 1),
and on 20,000 DNA sequences of the DNA generator (seed 2).  The packed files
of both makedbs, and the result files of -m clustering and -m fast at each
identity, must be byte-identical; so must the files of the one-process
modes (makedb+clustering, makedb+fast)."""
from __future__ import annotations

import hashlib
import subprocess

import pytest

import ngia2_gb300 as ng
import oracle
from ngia2_gb300 import synth

pytestmark = pytest.mark.gpu

REF = oracle.ref_gpu_cli()
CASES = {"protein": (lambda: synth.protein_families(20_000, 2_000, 1), (50, 70, 90)),
         "dna": (lambda: synth.dna_families(20_000, 2_000, 2), (80, 95))}


def sha(p) -> str:
    return hashlib.sha256(p.read_bytes()).hexdigest()


def run(cmd) -> str:
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, f"{cmd[0]}: {r.stdout[-2000:]}{r.stderr[-2000:]}"
    return r.stdout


@pytest.fixture(scope="module", params=sorted(CASES))
def dataset(request, tmp_path_factory, cuda):
    assert REF.exists(), "the reference GPU build is missing (oracle/build.sh)"
    kind = request.param
    make, identities = CASES[kind]
    d = tmp_path_factory.mktemp(f"refcli_{kind}")
    fa = d / "in.fa"
    make().write_fasta(fa)
    run([REF, "-m", "makedb", "-f", fa, "-p", d / "ref.packed"])
    run([ng.CLI_PATH, "-m", "makedb", "-f", fa, "-p", d / "ours.packed"])
    return kind, d, fa, identities


def test_packed_file_identical_to_reference_gpu_build(dataset):
    _, d, _, _ = dataset
    assert sha(d / "ours.packed") == sha(d / "ref.packed")


@pytest.mark.parametrize("mode", ["clustering", "fast"])
def test_result_files_identical_to_reference_gpu_build(dataset, mode):
    _, d, _, identities = dataset
    for identity in identities:
        args = ["-m", mode, "-i", str(identity), "-b", "64"]
        run([REF, *args, "-p", d / "ref.packed", "-r", d / f"ref_{mode}_{identity}.txt"])
        run([ng.CLI_PATH, *args, "-p", d / "ours.packed", "-r", d / f"ours_{mode}_{identity}.txt"])
        assert sha(d / f"ours_{mode}_{identity}.txt") == sha(d / f"ref_{mode}_{identity}.txt"), \
            f"{mode} at identity {identity}"


@pytest.mark.parametrize("mode", ["clustering", "fast"])
def test_one_process_mode_identical_to_reference_gpu_build(dataset, mode):
    _, d, fa, identities = dataset
    identity = identities[0]
    ref_out = d / f"ref_{mode}_{identity}_b.txt"
    run([REF, "-m", mode, "-i", str(identity), "-b", "64", "-p", d / "ref.packed",
         "-r", ref_out])
    one_packed, one_out = d / f"one_{mode}.packed", d / f"one_{mode}.txt"
    out = run([ng.CLI_PATH, "-m", f"makedb+{mode}", "-f", fa, "-p", one_packed, "-r", one_out,
               "-i", str(identity), "-b", "64"])
    assert "valid:" in out
    assert sha(one_packed) == sha(d / "ref.packed")
    assert sha(one_out) == sha(ref_out)
