"""The product kernel against the reference's own CUDA kernel
(BuildGraph::kernel_dynamic built unmodified by nvcc), pair by pair on the
same GPU.  Includes pairs crafted so that the two roundings of the band
bounds (fused multiply-add or not) give different scores; this pins which
rounding the reference's GPU build uses."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

import oracle
from conftest import IDENTITIES, SETS, load_pairs
from gpu_util import align_jobs_on_gpu, build_db

pytestmark = pytest.mark.gpu

REF_ALIGN = oracle.ref_gpu_align()


def run_reference_kernel(tmp_path, packed, offs, pairs, identity) -> np.ndarray:
    jobs = np.zeros((len(pairs), 3), np.uint32)
    jobs[:, :2] = pairs
    files = {k: tmp_path / f"{k}.bin" for k in ("packed", "offs", "jobs", "out")}
    np.ascontiguousarray(packed, np.uint32).tofile(files["packed"])
    np.ascontiguousarray(offs, np.uint64).tofile(files["offs"])
    jobs.tofile(files["jobs"])
    r = subprocess.run([str(REF_ALIGN), str(files["packed"]), str(files["offs"]),
                        str(files["jobs"]), str(identity), str(files["out"])],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return np.fromfile(files["out"], np.uint32).reshape(-1, 3)[:, 2]


def crafted_pairs(identity: int, count: int, seed: int):
    """Pairs whose band bounds differ between the two roundings and whose
    content (a shifted middle segment) makes the extra band blocks matter."""
    from ngia2_gb300 import synth
    rng = np.random.default_rng(seed)
    seqs, pairs = [], []
    tries = 0
    while len(pairs) < count and tries < 20000:
        tries += 1
        lt = int(rng.integers(32, 2500))
        lr = int(rng.integers(lt, int(lt * 1.08) + 2))
        if oracle.band_blocks(lr, lt, identity, oracle.ROUND_SPLIT) == \
                oracle.band_blocks(lr, lt, identity, oracle.ROUND_FMA):
            continue
        a = synth._draw(rng, synth.AMINO, synth.AMINO_FREQ, lr).tobytes()
        shift = int(rng.integers(20, 80))
        cut = int(rng.integers(0, max(1, lt - shift)))
        b = (a[:cut] + synth._draw(rng, synth.AMINO, synth.AMINO_FREQ, shift).tobytes()
             + a[cut:])[:lt]
        k = len(seqs)
        seqs += [a, b]
        pairs.append((k, k + 1))
    return seqs, np.array(pairs, np.uint32)


@pytest.fixture(scope="module")
def ref_kernel():
    if not REF_ALIGN.exists():
        pytest.skip("reference GPU build not available (oracle/_ref/ref_gpu_align)")
    return REF_ALIGN


@pytest.mark.parametrize("identity", [50, 80, 90, 95])
def test_crafted_rounding_pairs(cuda, built, ref_kernel, tmp_path, identity):
    seqs, pairs = crafted_pairs(identity, 300, 77 + identity)
    packed, offs, _ = build_db(seqs)
    split = oracle.align_pairs(packed, offs, pairs, identity, oracle.ROUND_SPLIT)
    fused = oracle.align_pairs(packed, offs, pairs, identity, oracle.ROUND_FMA)
    ref = run_reference_kernel(tmp_path, packed, offs, pairs, identity)
    mine = align_jobs_on_gpu(packed, offs, pairs, identity)  # default rounding
    differ = int((split != fused).sum())
    assert np.array_equal(mine, ref), (
        f"default rounding disagrees with the reference GPU kernel on "
        f"{int((mine != ref).sum())} of {len(ref)} pairs; reference equals fused on "
        f"{int((ref == fused).sum())}, split on {int((ref == split).sum())}; "
        f"{differ} pairs distinguish the roundings")
    assert np.array_equal(ref, fused)


@pytest.mark.parametrize("name,identity", [(s, i) for s in SETS for i in IDENTITIES[s]])
def test_golden_pairs_against_reference_kernel(cuda, built, ref_kernel, golden, tmp_path, name,
                                               identity):
    db = golden[name]["db"]
    pairs, _, _, _ = load_pairs(name, identity)
    if len(pairs) == 0:
        pytest.skip("no candidate pairs")
    ref = run_reference_kernel(tmp_path, db["packed"], db["offsets"], pairs, identity)
    mine = align_jobs_on_gpu(db["packed"], db["offsets"], pairs, identity)
    assert np.array_equal(mine, ref)
