"""Builds libngia.so (CUDA kernels + C ABI + host code) and the ngia2 CLI.

Everything is compiled in-tree for sm_103a only:
    ngia2_gb300/lib/libngia.so   the C-ABI library (include/ngia.h)
    ngia2_gb300/lib/ngia2        the drop-in command line
Objects go to _build/ (git-ignored).  Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIBDIR = PKG / "lib"
OBJDIR = ROOT / "_build" / "ngia"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["sketch.cu", "sort.cu", "bucket.cu", "align.cu", "pairs.cu", "edges.cu", "ctx.cu",
              "round.cu", "serve.cu", "stream.cu", "pack.cu", "probe.cu"]
CPP_SOURCES = ["packed_io.cpp", "leiden.cpp", "cluster.cpp", "device_session.cpp"]
CLI_SOURCES = ["cli.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libngia")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _newer(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile the library and CLI; returns the path of libngia.so."""
    OBJDIR.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) + [INCLUDE / "ngia.h"]
    nv = nvcc()
    inc = ["-I", str(INCLUDE), "-I", str(CSRC)]
    jobs = []
    for src in CU_SOURCES:
        out = OBJDIR / (src + ".o")
        cmd = [nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "--expt-relaxed-constexpr", *inc, *os.environ.get("NGIA_NVCC_FLAGS", "").split(),
               "-c", str(CSRC / src), "-o", str(out)]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((out, [CSRC / src, *headers], cmd))
    for src in CPP_SOURCES + CLI_SOURCES:
        out = OBJDIR / (src + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
               "-I", "/usr/local/cuda/include", *inc, "-c", str(CSRC / src), "-o", str(out)]
        jobs.append((out, [CSRC / src, *headers], cmd))
    todo = [(o, c) for o, deps, c in jobs if force or ptxas_info or not _newer(o, deps)]
    with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4) or 1) as ex:
        for r in ex.map(lambda oc: _run(oc[1]) if not verbose else _run_verbose(oc[1]), todo):
            pass
    lib = LIBDIR / "libngia.so"
    lib_objs = [OBJDIR / (s + ".o") for s in CU_SOURCES + CPP_SOURCES]
    if force or todo or not _newer(lib, lib_objs):
        tmp = LIBDIR / "libngia.so.tmp"
        _run([nv, *ARCH, "-shared", "-o", str(tmp), *map(str, lib_objs), "-lpthread"])
        os.replace(tmp, lib)
    cli = LIBDIR / "ngia2"
    cli_obj = OBJDIR / "cli.cpp.o"
    if force or todo or not _newer(cli, [cli_obj, lib]):
        _run(["g++", "-o", str(cli), str(cli_obj), "-L", str(LIBDIR), "-lngia",
              "-Wl,-rpath,$ORIGIN", "-pthread"])
    return lib


def _run_verbose(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    sys.stdout.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd))


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv,
          ptxas_info="--ptxas-info" in sys.argv)
    print(LIBDIR / "libngia.so")
