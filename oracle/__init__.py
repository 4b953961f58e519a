"""CPU oracle (TEST INFRASTRUCTURE ONLY).

ctypes bindings for
  * oracle/_ref/liboracle.so      -- the C restatement (ngia_oracle.c);
  * oracle/_ref/libngia_ref*.so   -- the reference's own makedb / alignment /
                                     Leiden / save code built as a host
                                     program (ref_build via build.sh);
  * oracle/_ref/ngia2_gpu, ref_gpu_align -- the reference's GPU build.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this package.  Build everything with oracle/build.sh.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"
ROUND_SPLIT, ROUND_FMA = 0, 1

_u32 = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64 = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")

_lib = None
_ref_libs: dict[int, C.CDLL] = {}


def build(no_gpu: bool = False) -> None:
    cmd = ["bash", str(HERE / "build.sh")] + (["--no-gpu"] if no_gpu else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = REF / "liboracle.so"
        if not path.exists():
            build(no_gpu=True)
        L = C.CDLL(str(path))
        L.ngo_residue_code.restype = C.c_uint32
        L.ngo_residue_code.argtypes = [C.c_ubyte]
        L.ngo_record_words.restype = C.c_size_t
        L.ngo_record_words.argtypes = [C.c_uint32]
        L.ngo_pack_record.restype = None
        L.ngo_pack_record.argtypes = [C.c_char_p, C.c_uint32, _u32]
        L.ngo_sketch_record.restype = None
        L.ngo_sketch_record.argtypes = [_u32, _u32]
        L.ngo_bucket_band.restype = None
        L.ngo_bucket_band.argtypes = [C.c_void_p, C.c_size_t, C.c_uint32, _u32]
        L.ngo_band_bounds.restype = C.c_int
        L.ngo_band_bounds.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int,
                                      C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.ngo_align.restype = C.c_uint32
        L.ngo_align.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int]
        L.ngo_banded_lcs.restype = C.c_uint32
        L.ngo_banded_lcs.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int]
        L.ngo_band_blocks.restype = C.c_uint64
        L.ngo_band_blocks.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]
        L.ngo_collect_band.restype = C.c_size_t
        L.ngo_collect_band.argtypes = [_u32, _u32, C.c_uint32, C.c_uint32, _u32]
        L.ngo_align_many.restype = None
        L.ngo_align_many.argtypes = [_u32, _u64, _u32, C.c_size_t, C.c_uint32, C.c_int, _u32]
        _lib = L
    return _lib


# ---- C restatement ------------------------------------------------------------------
def residue_code(ch: int) -> int:
    return int(lib().ngo_residue_code(ch))


def pack_record(seq: bytes) -> np.ndarray:
    rec = np.zeros(lib().ngo_record_words(len(seq)), np.uint32)
    lib().ngo_pack_record(seq, len(seq), rec)
    return rec


def sketch_record(rec: np.ndarray) -> np.ndarray:
    out = np.empty(64, np.uint32)
    lib().ngo_sketch_record(np.ascontiguousarray(rec, np.uint32), out)
    return out


def sketch_all(packed: np.ndarray, offsets: np.ndarray, lens: np.ndarray) -> np.ndarray:
    """Signatures band-major [64][n]."""
    n = len(offsets)
    out = np.empty((64, n), np.uint32)
    one = np.empty(64, np.uint32)
    for i in range(n):
        o = int(offsets[i])
        rec = np.ascontiguousarray(packed[o:o + 1 + ((int(lens[i]) + 31) // 32) * 4])
        lib().ngo_sketch_record(rec, one)
        out[:, i] = one
    return out


def bucket_band(sig_row: np.ndarray) -> np.ndarray:
    sig_row = np.ascontiguousarray(sig_row, np.uint32)
    rep = np.empty(sig_row.size, np.uint32)
    lib().ngo_bucket_band(sig_row.ctypes.data, 1, sig_row.size, rep)
    return rep


def band_bounds(lr: int, lt: int, identity: int, mode: int = ROUND_FMA):
    a, b = C.c_uint32(), C.c_uint32()
    ok = lib().ngo_band_bounds(lr, lt, identity, mode, C.byref(a), C.byref(b))
    return (a.value, b.value) if ok else None


def band_blocks(lr: int, lt: int, identity: int, mode: int = ROUND_FMA) -> int:
    return int(lib().ngo_band_blocks(lr, lt, identity, mode))


def align_records(rep: np.ndarray, tar: np.ndarray, identity: int,
                  mode: int = ROUND_FMA) -> int:
    rep = np.ascontiguousarray(rep, np.uint32)
    tar = np.ascontiguousarray(tar, np.uint32)
    return int(lib().ngo_align(rep.ctypes.data, tar.ctypes.data, identity, mode))


def banded_lcs(rep: np.ndarray, tar: np.ndarray, identity: int, mode: int = ROUND_FMA) -> int:
    rep = np.ascontiguousarray(rep, np.uint32)
    tar = np.ascontiguousarray(tar, np.uint32)
    return int(lib().ngo_banded_lcs(rep.ctypes.data, tar.ctypes.data, identity, mode))


def align_pairs(packed: np.ndarray, offsets: np.ndarray, pairs: np.ndarray, identity: int,
                mode: int = ROUND_FMA) -> np.ndarray:
    pairs = np.ascontiguousarray(pairs, np.uint32).reshape(-1, 2)
    out = np.zeros(len(pairs), np.uint32)
    lib().ngo_align_many(np.ascontiguousarray(packed, np.uint32),
                         np.ascontiguousarray(offsets, np.uint64), pairs, len(pairs),
                         identity, mode, out)
    return out


def collect_band(rep_row: np.ndarray, lens: np.ndarray, identity: int) -> np.ndarray:
    n = len(lens)
    out = np.empty(2 * n, np.uint32)
    k = lib().ngo_collect_band(np.ascontiguousarray(rep_row, np.uint32),
                               np.ascontiguousarray(lens, np.uint32), n, identity, out)
    return out[:2 * k].reshape(-1, 2)


def graph_edges(packed, offsets, lens, rep, identity: int, bands: int,
                mode: int = ROUND_FMA):
    """buildGraph restated: all bands' candidates, scores, sorted unique edges
    (rep, tar, score) as an int64 array of shape (m, 3); also the candidate
    count with duplicates."""
    cand = [collect_band(rep[b], lens, identity) for b in range(bands)]
    total = sum(len(c) for c in cand)
    allp = np.concatenate(cand) if total else np.zeros((0, 2), np.uint32)
    uniq = np.unique(allp, axis=0) if total else allp
    scores = align_pairs(packed, offsets, uniq, identity, mode) if len(uniq) else \
        np.zeros(0, np.uint32)
    hit = scores > 0
    e = np.stack([uniq[hit, 0].astype(np.int64), uniq[hit, 1].astype(np.int64),
                  scores[hit].astype(np.int64)], axis=1) if hit.any() else \
        np.zeros((0, 3), np.int64)
    return e, total


def fast_cluster(packed, offsets, rep, identity: int, bands: int,
                 mode: int = ROUND_FMA) -> np.ndarray:
    """Fast mode restated (FastClustering::cluster, src/fastClustering.hpp:249-352).
    Bands in order; in band b every record i whose rep is not itself and that
    no earlier band assigned (the list is fixed before the band's alignments)
    is aligned against rep[b][i] with the kernel's scoring, and a hit makes
    that rep its parent.  A record's cluster id is its root: itself when it
    has no parent, else its parent's root (parents have lower indices)."""
    n = rep.shape[1] if rep.ndim == 2 else 0
    free = np.uint32(0xFFFFFFFF)
    parent = np.full(n, free, np.uint32)
    idx = np.arange(n, dtype=np.uint32)
    for b in range(bands):
        row = np.ascontiguousarray(rep[b], np.uint32)
        tar = np.nonzero((row != idx) & (parent == free))[0]
        if len(tar) == 0:
            continue
        pairs = np.stack([row[tar], tar.astype(np.uint32)], axis=1)
        hit = align_pairs(packed, offsets, pairs, identity, mode) > 0
        parent[tar[hit]] = row[tar[hit]]
    root = np.empty(n, np.uint32)
    for i in range(n):
        p = parent[i]
        root[i] = i if p == free else root[p]
    return root


# ---- the reference itself, built as a host program -------------------------------------
def ref_available() -> bool:
    return (REF / "libngia_ref.so").exists()


def ref_lib(mode: int = ROUND_FMA) -> C.CDLL:
    if mode not in _ref_libs:
        name = "libngia_ref_fma.so" if mode == ROUND_FMA else "libngia_ref.so"
        L = C.CDLL(str(REF / name))
        L.ref_align_jobs.restype = C.c_int
        L.ref_align_jobs.argtypes = [_u32, _u64, _u32, C.c_uint32, C.c_uint32]
        L.ref_makedb.restype = C.c_int
        L.ref_makedb.argtypes = [C.c_char_p, C.c_char_p]
        L.ref_makedb_nogroup.restype = C.c_int
        L.ref_makedb_nogroup.argtypes = [C.c_char_p, C.c_char_p]
        L.ref_build_graph.restype = C.c_long
        L.ref_build_graph.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32, _i32, _i32, _f32,
                                      C.c_long]
        L.ref_leiden.restype = C.c_int
        L.ref_leiden.argtypes = [_i32, _i32, _f32, C.c_long, C.c_int, C.c_float, C.c_uint,
                                 C.c_int, _u32]
        L.ref_fast_cluster.restype = C.c_int
        L.ref_fast_cluster.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32, _u32, C.c_uint32]
        L.ref_save.restype = C.c_int
        L.ref_save.argtypes = [_u32, C.c_uint32, C.c_char_p, C.c_char_p]
        _ref_libs[mode] = L
    return _ref_libs[mode]


def ref_align_jobs(packed, offsets, pairs, identity: int, mode: int = ROUND_FMA) -> np.ndarray:
    pairs = np.asarray(pairs, np.uint32).reshape(-1, 2)
    jobs = np.zeros((len(pairs), 3), np.uint32)
    jobs[:, :2] = pairs
    jobs = np.ascontiguousarray(jobs.reshape(-1))
    ref_lib(mode).ref_align_jobs(np.ascontiguousarray(packed, np.uint32),
                                 np.ascontiguousarray(offsets, np.uint64), jobs, len(pairs),
                                 identity)
    return jobs.reshape(-1, 3)[:, 2].copy()


def ref_makedb(fasta, packed, group: bool = True) -> int:
    L = ref_lib()
    fn = L.ref_makedb if group else L.ref_makedb_nogroup
    return fn(os.fsencode(fasta), os.fsencode(packed))


def ref_build_graph(packed, identity: int, bands: int, cap: int, mode: int = ROUND_FMA):
    rep = np.empty(cap, np.int32)
    tar = np.empty(cap, np.int32)
    w = np.empty(cap, np.float32)
    m = ref_lib(mode).ref_build_graph(os.fsencode(packed), identity, bands, rep, tar, w, cap)
    if m < 0:
        raise RuntimeError(f"ref_build_graph failed ({m})")
    if m > cap:
        return ref_build_graph(packed, identity, bands, m, mode)
    return rep[:m], tar[:m], w[:m]


def ref_leiden(rep, tar, w, n: int, resolution: float, seed: int = 42,
               iterations: int = 1) -> np.ndarray:
    out = np.empty(n, np.uint32)
    rc = ref_lib().ref_leiden(np.ascontiguousarray(rep, np.int32),
                              np.ascontiguousarray(tar, np.int32),
                              np.ascontiguousarray(w, np.float32), len(rep), n, resolution,
                              seed, iterations, out)
    if rc:
        raise RuntimeError("ref_leiden failed")
    return out


def ref_fast_cluster(packed, identity: int, bands: int, n: int,
                     mode: int = ROUND_FMA) -> np.ndarray:
    out = np.empty(n, np.uint32)
    rc = ref_lib(mode).ref_fast_cluster(os.fsencode(packed), identity, bands, out, n)
    if rc:
        raise RuntimeError(f"ref_fast_cluster failed ({rc})")
    return out


def ref_save(cluster, packed, result) -> None:
    ref_lib().ref_save(np.ascontiguousarray(cluster, np.uint32), len(cluster),
                       os.fsencode(packed), os.fsencode(result))


def ref_cli(mode: int = ROUND_FMA) -> Path:
    return REF / ("ngia2_cpu_fma" if mode == ROUND_FMA else "ngia2_cpu")


def ref_gpu_cli() -> Path:
    return REF / "ngia2_gpu"


def ref_gpu_align() -> Path:
    return REF / "ref_gpu_align"
