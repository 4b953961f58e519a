"""Shared fixtures.  Tests marked `gpu` need a CUDA GPU (GB300) and the built
libngia.so; everything else runs on a CPU-only machine."""
from __future__ import annotations

import gzip
import shutil
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))

SETS = ("prot", "dna", "edge")
IDENTITIES = {"prot": (50, 70, 90), "dna": (80, 90, 95), "edge": (30, 50, 90)}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libngia.so")


@pytest.fixture(scope="session")
def built():
    """Builds (or reuses) libngia.so and the oracle libraries."""
    from ngia2_gb300 import build as b
    import oracle
    b.build()
    if not (oracle.REF / "liboracle.so").exists():
        oracle.build(no_gpu=True)
    return True


@pytest.fixture(scope="session")
def golden(tmp_path_factory):
    """Decompressed golden inputs: name -> {'fa': path, 'packed': path, 'db': dict}."""
    import ngia2_gb300 as ng
    d = tmp_path_factory.mktemp("golden")
    out = {}
    for name in SETS:
        fa = d / f"{name}.fa"
        packed = d / f"{name}.packed"
        with gzip.open(GOLDEN / f"{name}.fa.gz", "rb") as f:
            fa.write_bytes(f.read())
        with gzip.open(GOLDEN / f"{name}.packed.gz", "rb") as f:
            packed.write_bytes(f.read())
        out[name] = {"fa": fa, "packed": packed, "db": ng.read_packed(packed)}
    return out


def load_pairs(name: str, identity: int):
    z = np.load(GOLDEN / f"{name}.pairs_{identity}.npz")
    return z["pairs"], z["score_split"], z["score_fma"], int(z["candidates"])


def load_edges(name: str, identity: int, mode: str = "fma") -> np.ndarray:
    return np.load(GOLDEN / f"{name}.edges_{identity}_{mode}.npy")


def result_sha(name: str, identity: int) -> dict:
    out = {}
    for line in (GOLDEN / f"{name}.result_{identity}.sha256").read_text().splitlines():
        h, kind = line.split()
        out[kind] = h
    return out


@pytest.fixture(scope="session")
def cuda():
    """The CUDA device; fails (does not skip) when absent, so a GPU run that
    lost its GPU shows up as a failure."""
    import torch
    assert torch.cuda.is_available(), "a CUDA GPU is required for tests marked gpu"
    return torch.device("cuda:0")
