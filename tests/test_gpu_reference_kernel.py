"""The product kernel against the reference's own CUDA kernel
(BuildGraph::kernel_dynamic built unmodified by nvcc), pair by pair on the
same GPU.  Includes pairs whose band geometry differs between the two
roundings of the band bounds (fused multiply-add or not).  Scores rarely
differ between the roundings, since the band is wide enough for every path
that passes the threshold; the pin is that the reference kernel equals the
fused rounding on every pair."""
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
    """Pairs whose band bounds differ between the two roundings (one more row
    block at an edge of the band), with targets derived from the rep by
    substitutions and indels of up to the band's half-width, so that some
    paths run near the band edges."""
    from ngia2_gb300 import synth
    rng = np.random.default_rng(seed)
    t = identity / 100.0
    shapes = [(lr, lt) for lt in range(32, 3000) for lr in range(lt, lt + lt // 8 + 2)
              if oracle.band_blocks(lr, lt, identity, oracle.ROUND_SPLIT)
              != oracle.band_blocks(lr, lt, identity, oracle.ROUND_FMA)]
    assert shapes, f"no lengths distinguish the roundings at identity {identity}"

    def draw(k):
        return synth._draw(rng, synth.AMINO, synth.AMINO_FREQ, k).tobytes()

    seqs, pairs = [], []
    for _ in range(count):
        lr, lt = shapes[int(rng.integers(0, len(shapes)))]
        a = draw(lr)
        b = bytearray(a)
        for _ in range(int(rng.integers(0, 6))):
            g = int(rng.integers(1, max(2, int(lt * (1 - t)) + 1)))
            p = int(rng.integers(0, max(1, len(b) - g)))
            if rng.random() < 0.5:
                del b[p:p + g]
            else:
                b[p:p] = draw(g)
        b = b[:lt]
        b += draw(lt - len(b))
        for p in rng.integers(0, lt, size=int(lt * rng.random() * (1 - t))):
            b[int(p)] = synth.AMINO[rng.integers(0, 20)]
        k = len(seqs)
        seqs += [a, bytes(b)]
        pairs.append((k, k + 1))
    return seqs, np.array(pairs, np.uint32)


@pytest.fixture(scope="module")
def ref_kernel():
    if not REF_ALIGN.exists():
        pytest.skip("reference GPU build not available (oracle/_ref/ref_gpu_align)")
    return REF_ALIGN


@pytest.mark.parametrize("identity", [70, 84, 90, 95])
def test_crafted_rounding_pairs(cuda, built, ref_kernel, tmp_path, identity):
    seqs, pairs = crafted_pairs(identity, 4000, 77 + identity)
    packed, offs, _ = build_db(seqs)
    ref = run_reference_kernel(tmp_path, packed, offs, pairs, identity)
    fused = align_jobs_on_gpu(packed, offs, pairs, identity, "fma")
    split = align_jobs_on_gpu(packed, offs, pairs, identity, "split")
    mine = align_jobs_on_gpu(packed, offs, pairs, identity)  # default rounding
    assert np.array_equal(mine, fused)
    assert np.array_equal(ref, fused), (
        f"reference kernel differs from the fused rounding on {int((ref != fused).sum())} of "
        f"{len(ref)} pairs (from the split rounding on {int((ref != split).sum())})")
    # spot-check the GPU scores of both roundings against the oracle
    sample = np.arange(0, len(pairs), 20)
    assert np.array_equal(fused[sample], oracle.align_pairs(packed, offs, pairs[sample], identity,
                                                            oracle.ROUND_FMA))
    assert np.array_equal(split[sample], oracle.align_pairs(packed, offs, pairs[sample], identity,
                                                            oracle.ROUND_SPLIT))


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
