"""ngia2_gb300 -- GB300-native group-then-align hot path of nGIA2.

Python host mirror of the C ABI in include/ngia.h (libngia.so, loaded with
ctypes).  The compute path is the library's CUDA kernels; this module only
marshals arguments.  There is no CPU fallback: if the library is not built or
no GPU is present, the calls fail.

Main entry points
    makedb(fasta, packed)                      src/main.cu:54-83
    cluster_file(packed, result, identity, bands, fast=False)
                                               src/main.cu:86-156
    Context                                    a device-resident database:
        .load(...) / .load_packed_file(...)    BuildGraph::readData
        .sketch_bucket(bands)                  MakeDB pack signing + groupSignatures
        .build_graph(identity, bands)          BuildGraph::buildGraph
        .fast_cluster(identity, bands)         FastClustering::cluster
        .run_host(...)                         all of the above on host buffers
    align_pairs / sketch / bucket / emit_edges raw device-pointer entry points
    leiden(edges, n, resolution, seed, iters)  LeidenOmp::cluster
    read_packed(path)                          the packed file as numpy arrays
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libngia.so"
CLI_PATH = PKG / "lib" / "ngia2"
BANDS = 64

EDGE_DTYPE = np.dtype([("rep", "<i4"), ("tar", "<i4"), ("weight", "<f4")])

STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "out of memory",
          -4: "I/O error", -5: "malformed input", -6: "call out of order"}
OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_IO, ERR_FORMAT, ERR_STATE = 0, -1, -2, -3, -4, -5, -6


class NgiaError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)}")


class Stats(C.Structure):
    _fields_ = [("candidate_pairs", C.c_uint64), ("unique_pairs", C.c_uint64),
                ("aligned_cells", C.c_uint64), ("edges", C.c_uint64),
                ("ms_sketch", C.c_double), ("ms_bucket", C.c_double),
                ("ms_pairs", C.c_double), ("ms_align", C.c_double), ("ms_emit", C.c_double),
                ("computed_cells", C.c_uint64), ("load_pipelined", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


GROUP_SHAPES = [(8, 3), (8, 4), (16, 4), (16, 6), (32, 4), (32, 6), (32, 8), (32, 16)]  # (lanes, words)
# class numbers of the batched aligner (align.cuh): 11 one-pair-per-lane
# windows, the group classes, the general kernel, then the length-filter skip
FIRST_GROUP_CLASS = 11
GENERAL_CLASS = FIRST_GROUP_CLASS + len(GROUP_SHAPES)
SKIP_CLASS = GENERAL_CLASS + 1


class Plan(C.Structure):
    """ngia_plan: the widest one-pair-per-lane window and the widest band each
    group class (GROUP_SHAPES) takes (0 = unused)."""
    _fields_ = [("stream_max", C.c_uint32), ("group_limit", C.c_uint32 * len(GROUP_SHAPES))]

    def as_dict(self) -> dict:
        return {"stream_max": int(self.stream_max),
                "group_limit": [int(x) for x in self.group_limit]}

    @classmethod
    def from_dict(cls, d: dict) -> "Plan":
        p = cls()
        p.stream_max = int(d["stream_max"])
        for g, v in enumerate(d["group_limit"]):
            p.group_limit[g] = int(v)
        return p


NEW_CLUSTER = 0xFFFFFFFF


class StreamStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("chunks", "chunk_loads", "bytes_h2d_sketch",
                                          "bytes_h2d_align", "candidate_pairs", "unique_pairs",
                                          "aligned_cells", "computed_cells", "edges")] + \
               [(k, C.c_double) for k in ("ms_sketch", "ms_bucket", "ms_pairs", "ms_align",
                                          "ms_emit", "ms_total")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("identity", C.c_uint32), ("slots", C.c_uint32), ("max_queries", C.c_uint32),
                ("max_words", C.c_uint64), ("hbm_budget", C.c_uint64), ("plain", C.c_int),
                ("small_queries", C.c_uint32), ("small_slots", C.c_uint32)]


class RequestStats(C.Structure):
    _fields_ = [("queue_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double),
                ("queries", C.c_uint32), ("assigned", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
edgep = np.ctypeslib.ndpointer(EDGE_DTYPE, flags="C_CONTIGUOUS")

_SIGNATURES = {
    "ngia_status_string": (C.c_char_p, [C.c_int]),
    "ngia_last_cuda_error": (C.c_int, []),
    "ngia_version": (C.c_char_p, []),
    "ngia_kernel_launches": (C.c_ulonglong, []),
    "ngia_set_round_mode": (C.c_int, [C.c_int]),
    "ngia_sketch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "ngia_bucket": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]),
    "ngia_bucket_noalloc": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                      C.c_void_p]),
    "ngia_align_pairs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                   C.c_uint32, C.c_void_p]),
    "ngia_emit_edges": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ngia_sort_unique_edges": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.c_uint32,
                                         C.c_void_p]),
    "ngia_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p]),
    "ngia_ctx_destroy": (None, [C.c_void_p]),
    "ngia_ctx_load": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                C.c_uint32, C.c_void_p, C.c_uint32]),
    "ngia_ctx_load_packed_file": (C.c_int, [C.c_void_p, C.c_char_p, C.c_uint32, C.c_int]),
    "ngia_ctx_sketch_bucket": (C.c_int, [C.c_void_p, C.c_uint32]),
    "ngia_ctx_build_graph": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32,
                                       C.POINTER(C.c_uint64), C.POINTER(Stats)]),
    "ngia_ctx_group_align": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32,
                                       C.POINTER(C.c_uint64), C.POINTER(Stats)]),
    "ngia_ctx_edges": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "ngia_ctx_build_graph_part": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                            C.c_uint32, C.c_void_p, C.POINTER(C.c_uint64),
                                            C.POINTER(Stats)]),
    "ngia_ctx_test_lookback_timeout": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32,
                                                 C.c_uint32]),
    "ngia_ctx_align_pairs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                       C.c_void_p, C.POINTER(Stats)]),
    "ngia_ctx_align_pairs_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                            C.c_void_p, C.POINTER(Stats)]),
    "ngia_ctx_use_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "ngia_ctx_get_plan": (C.c_int, [C.c_void_p, C.POINTER(Plan)]),
    "ngia_ctx_set_plan": (C.c_int, [C.c_void_p, C.POINTER(Plan)]),
    "ngia_ctx_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int,
                                    C.POINTER(Plan), C.POINTER(C.c_double)]),
    "ngia_int32_peak": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ngia_server_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_void_p,
                                     C.POINTER(ServerConfig)]),
    "ngia_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                     C.c_uint32, C.POINTER(C.c_uint64)]),
    "ngia_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p,
                                   C.POINTER(RequestStats)]),
    "ngia_server_destroy": (None, [C.c_void_p]),
    "ngia_pack": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                            C.c_void_p, C.c_void_p]),
    "ngia_pack_records": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint32,
                                    C.c_void_p, C.c_uint64, C.c_void_p]),
    "ngia_stream_graph": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint32,
                                    C.c_uint32, C.c_uint32, C.c_uint64, C.c_void_p, C.c_uint64,
                                    C.POINTER(C.c_uint64), C.POINTER(StreamStats)]),
    "ngia_ctx_fast_cluster": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                        C.POINTER(Stats)]),
    "ngia_ctx_rep_rows": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "ngia_ctx_sigs": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ngia_ctx_use_sketch_table": (C.c_int, [C.c_void_p, C.c_int]),
    "ngia_ctx_sketch_table_active": (C.c_int, [C.c_void_p]),
    "ngia_sketch_table_bands": (C.c_int, []),
    "ngia_ctx_run_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                    C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                    C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64),
                                    C.POINTER(Stats)]),
    "ngia_makedb": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_uint32)]),
    "ngia_leiden": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_float, C.c_uint32,
                              C.c_int, C.c_void_p]),
    "ngia_leiden_resolution": (C.c_float, [C.c_uint32]),
    "ngia_save_result": (C.c_int, [C.c_void_p, C.c_uint32, C.c_char_p, C.c_char_p]),
    "ngia_cluster_file": (C.c_int, [C.c_char_p, C.c_char_p, C.c_uint32, C.c_uint32, C.c_int,
                                    C.POINTER(Stats)]),
}


def exported_symbols() -> list[str]:
    """Every entry point include/ngia.h declares (the binding table)."""
    return sorted(_SIGNATURES)


def lib() -> C.CDLL:
    """The loaded libngia.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int, what: str) -> None:
    if status != 0:
        raise NgiaError(status, what)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None else 0


def kernel_launches() -> int:
    """Kernels launched by libngia in this process so far."""
    return int(lib().ngia_kernel_launches())


def int32_peak(stream: int = 0) -> float:
    """Measured lop3 lane-operations per second of the current device."""
    v = C.c_double()
    _check(lib().ngia_int32_peak(stream, C.byref(v)), "ngia_int32_peak")
    return float(v.value)


def set_round_mode(mode: str) -> str:
    """'fma' (default) or 'split' band-bound rounding; returns the previous."""
    old = lib().ngia_set_round_mode({"split": 0, "fma": 1}[mode])
    return "fma" if old == 1 else "split"


# ---- raw device-pointer entry points (pointers as ints, e.g. tensor.data_ptr()) ----
def sketch(d_packed: int, d_offsets: int, n: int, d_sigs: int, stream: int = 0) -> None:
    _check(lib().ngia_sketch(d_packed, d_offsets, n, d_sigs, stream), "ngia_sketch")


def bucket(d_sigs: int, n: int, bands: int, d_rep: int, stream: int = 0) -> None:
    _check(lib().ngia_bucket(d_sigs, n, bands, d_rep, stream), "ngia_bucket")


def bucket_noalloc(d_sigs: int, n: int, bands: int, d_rep: int, stream: int = 0) -> None:
    """ngia_bucket with its scratch in the library's fixed device array (no
    allocation; n * bands <= 1,048,576; calls must not overlap on the GPU)."""
    _check(lib().ngia_bucket_noalloc(d_sigs, n, bands, d_rep, stream), "ngia_bucket_noalloc")


def align_pairs(d_packed: int, d_offsets: int, d_jobs: int, count: int, identity: int,
                stream: int = 0) -> None:
    _check(lib().ngia_align_pairs(d_packed, d_offsets, d_jobs, count, identity, stream),
           "ngia_align_pairs")


def emit_edges(d_jobs: int, count: int, d_edges: int, d_n_edges: int, stream: int = 0) -> None:
    _check(lib().ngia_emit_edges(d_jobs, count, d_edges, d_n_edges, stream), "ngia_emit_edges")


def sort_unique_edges(d_edges: int, m: int, n_nodes: int, stream: int = 0) -> int:
    k = C.c_uint32(m)
    _check(lib().ngia_sort_unique_edges(d_edges, C.byref(k), n_nodes, stream),
           "ngia_sort_unique_edges")
    return k.value


# ---- context ------------------------------------------------------------------------
class Context:
    """A device-resident database and its graph-build workspace (ngia_ctx)."""

    def __init__(self, stream: int = 0):
        h = C.c_void_p()
        _check(lib().ngia_ctx_create(C.byref(h), stream), "ngia_ctx_create")
        self._h = h
        self.n = 0

    def close(self) -> None:
        if self._h:
            lib().ngia_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def load(self, packed: np.ndarray, offsets: np.ndarray, lens: np.ndarray,
             rep: np.ndarray | None = None, bands: int = BANDS) -> None:
        packed = np.ascontiguousarray(packed, np.uint32)
        offsets = np.ascontiguousarray(offsets, np.uint64)
        lens = np.ascontiguousarray(lens, np.uint32)
        if rep is not None:
            rep = np.ascontiguousarray(rep, np.uint32)
        _check(lib().ngia_ctx_load(self._h, _ptr(packed), packed.size, _ptr(offsets), _ptr(lens),
                                   lens.size, _ptr(rep), bands), "ngia_ctx_load")
        self.n = int(lens.size)

    def load_packed_file(self, path, bands: int = BANDS, use_file_rep_rows: bool = True) -> None:
        _check(lib().ngia_ctx_load_packed_file(self._h, os.fsencode(path), bands,
                                               1 if use_file_rep_rows else 0),
               "ngia_ctx_load_packed_file")
        with open(path, "rb") as f:
            self.n = int(np.frombuffer(f.read(4), np.uint32)[0])

    def sketch_bucket(self, bands: int = BANDS) -> None:
        _check(lib().ngia_ctx_sketch_bucket(self._h, bands), "ngia_ctx_sketch_bucket")

    def sigs(self) -> np.ndarray:
        """The 64 signatures of every record, band-major [64][n]."""
        out = np.empty((BANDS, self.n), np.uint32)
        _check(lib().ngia_ctx_sigs(self._h, _ptr(out)), "ngia_ctx_sigs")
        return out

    def sketch_table_active(self) -> bool:
        return lib().ngia_ctx_sketch_table_active(self._h) == 1

    def use_sketch_table(self, on: bool) -> bool:
        """Sketch 4-letter databases through the 8-mer hash table; returns the old setting."""
        r = lib().ngia_ctx_use_sketch_table(self._h, 1 if on else 0)
        if r < 0:
            _check(r, "ngia_ctx_use_sketch_table")
        return bool(r)

    def rep_rows(self, bands: int = BANDS) -> np.ndarray:
        out = np.empty((bands, self.n), np.uint32)
        _check(lib().ngia_ctx_rep_rows(self._h, _ptr(out), bands), "ngia_ctx_rep_rows")
        return out

    def build_graph(self, identity: int, bands: int = BANDS) -> tuple[int, dict]:
        m = C.c_uint64()
        st = Stats()
        _check(lib().ngia_ctx_build_graph(self._h, identity, bands, C.byref(m), C.byref(st)),
               "ngia_ctx_build_graph")
        return int(m.value), st.as_dict()

    def build_graph_part(self, identity: int, part: int, parts: int,
                         bands: int = BANDS) -> tuple[int, dict, tuple[int, int]]:
        """This device's share (part of parts, by band cells) of build_graph:
        the edge count, the stats and the range of distinct pairs aligned."""
        m = C.c_uint64()
        st = Stats()
        rng = (C.c_uint64 * 2)()
        _check(lib().ngia_ctx_build_graph_part(self._h, identity, bands, part, parts, rng,
                                               C.byref(m), C.byref(st)),
               "ngia_ctx_build_graph_part")
        return int(m.value), st.as_dict(), (int(rng[0]), int(rng[1]))

    def group_align(self, identity: int, bands: int = BANDS) -> tuple[int, dict]:
        """Sketch + bucket + graph build on the resident planes."""
        m = C.c_uint64()
        st = Stats()
        _check(lib().ngia_ctx_group_align(self._h, identity, bands, C.byref(m), C.byref(st)),
               "ngia_ctx_group_align")
        return int(m.value), st.as_dict()

    def edges(self, m: int) -> np.ndarray:
        out = np.empty(m, EDGE_DTYPE)
        _check(lib().ngia_ctx_edges(self._h, _ptr(out), m), "ngia_ctx_edges")
        return out

    def graph(self, identity: int, bands: int = BANDS) -> tuple[np.ndarray, dict]:
        m, st = self.build_graph(identity, bands)
        return self.edges(m), st

    def align_pairs(self, pairs: np.ndarray, identity: int) -> tuple[np.ndarray, dict]:
        """Batched alignment of (rep, tar) index pairs [count, 2] from host
        memory; returns the u32 scores and the stats."""
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        out = np.zeros(len(pairs), np.uint32)
        st = Stats()
        _check(lib().ngia_ctx_align_pairs_host(self._h, _ptr(pairs), len(pairs), identity,
                                               _ptr(out), C.byref(st)),
               "ngia_ctx_align_pairs_host")
        return out, st.as_dict()

    def plan(self) -> dict:
        p = Plan()
        _check(lib().ngia_ctx_get_plan(self._h, C.byref(p)), "ngia_ctx_get_plan")
        return p.as_dict()

    def set_plan(self, plan: dict) -> None:
        p = Plan.from_dict(plan)
        _check(lib().ngia_ctx_set_plan(self._h, C.byref(p)), "ngia_ctx_set_plan")

    def autotune(self, d_pairs: int, count: int, identity: int, reps: int = 2) -> tuple[dict, float]:
        """Picks the binning plan on `count` device pairs; returns it and its time (ms)."""
        p, ms = Plan(), C.c_double()
        _check(lib().ngia_ctx_autotune(self._h, d_pairs, count, identity, reps, C.byref(p),
                                       C.byref(ms)), "ngia_ctx_autotune")
        return p.as_dict(), float(ms.value)

    def use_graphs(self, on: bool) -> bool:
        """Capture/replay the batched round as a CUDA graph; returns the old setting."""
        r = lib().ngia_ctx_use_graphs(self._h, 1 if on else 0)
        if r < 0:
            _check(r, "ngia_ctx_use_graphs")
        return bool(r)

    def align_pairs_device(self, d_pairs: int, count: int, identity: int,
                           d_scores: int) -> dict:
        """Batched alignment of `count` device (rep, tar) pairs into d_scores."""
        st = Stats()
        _check(lib().ngia_ctx_align_pairs(self._h, d_pairs, count, identity, d_scores,
                                          C.byref(st)), "ngia_ctx_align_pairs")
        return st.as_dict()

    def fast_cluster(self, identity: int, bands: int = BANDS) -> np.ndarray:
        out = np.empty(self.n, np.uint32)
        st = Stats()
        _check(lib().ngia_ctx_fast_cluster(self._h, identity, bands, _ptr(out), C.byref(st)),
               "ngia_ctx_fast_cluster")
        return out

    def run_host(self, packed: np.ndarray, offsets: np.ndarray, lens: np.ndarray,
                 identity: int, bands: int, edges_out: np.ndarray) -> tuple[int, dict]:
        """Host buffers in, host edges out (edges_out sized for the worst case)."""
        m = C.c_uint64()
        st = Stats()
        _check(lib().ngia_ctx_run_host(self._h, _ptr(packed), packed.size, _ptr(offsets),
                                       _ptr(lens), lens.size, identity, bands, _ptr(edges_out),
                                       edges_out.size, C.byref(m), C.byref(st)),
               "ngia_ctx_run_host")
        self.n = int(lens.size)
        return int(m.value), st.as_dict()


# ---- serving --------------------------------------------------------------------------
class Server:
    """Query batches assigned to a resident database's clusters
    (ngia_server_*): submit() queues a request, wait() returns its cluster ids
    (NEW_CLUSTER for a query that opens a new cluster) and timings."""

    def __init__(self, ctx: "Context", cluster: np.ndarray, identity: int = 90, slots: int = 4,
                 max_queries: int = 50_000, max_words: int = 16 << 20,
                 hbm_budget: int = 8 << 30, plain: bool = False, small_queries: int = 0,
                 small_slots: int = 0):
        cluster = np.ascontiguousarray(cluster, dtype=np.uint32)
        cfg = ServerConfig(identity, slots, max_queries, max_words, hbm_budget, 1 if plain else 0,
                           small_queries, small_slots)
        h = C.c_void_p()
        _check(lib().ngia_server_create(C.byref(h), ctx._h, _ptr(cluster), C.byref(cfg)),
               "ngia_server_create")
        self._h = h

    def submit(self, packed: np.ndarray, offsets: np.ndarray, lens: np.ndarray) -> int:
        packed = np.ascontiguousarray(packed, dtype=np.uint32)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        lens = np.ascontiguousarray(lens, dtype=np.uint32)
        t = C.c_uint64()
        _check(lib().ngia_server_submit(self._h, _ptr(packed), packed.size, _ptr(offsets),
                                        _ptr(lens), lens.size, C.byref(t)), "ngia_server_submit")
        return int(t.value)

    def wait(self, ticket: int, count: int) -> tuple[np.ndarray, dict]:
        out = np.empty(count, np.uint32)
        st = RequestStats()
        _check(lib().ngia_server_wait(self._h, ticket, _ptr(out), C.byref(st)),
               "ngia_server_wait")
        return out, st.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().ngia_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def pack_records(residues: np.ndarray, starts: np.ndarray, lens: np.ndarray):
    """Pack residues (uint8 ASCII; record i at starts[i], lens[i] bytes) on the
    device into back-to-back packed records: (packed words, word offsets)."""
    residues = np.ascontiguousarray(residues, dtype=np.uint8)
    starts = np.ascontiguousarray(starts, dtype=np.uint64)
    lens = np.ascontiguousarray(lens, dtype=np.uint32)
    words = int((1 + 4 * ((lens.astype(np.int64) + 31) // 32)).sum())
    packed = np.empty(max(words, 1), np.uint32)
    offs = np.empty(max(lens.size, 1), np.uint64)
    _check(lib().ngia_pack_records(_ptr(residues), residues.size, _ptr(starts), _ptr(lens),
                                   lens.size, _ptr(packed), words, _ptr(offs)),
           "ngia_pack_records")
    return packed[:words], offs[: lens.size]


def stream_graph(packed: np.ndarray, offsets: np.ndarray, lens: np.ndarray, identity: int,
                 bands: int, chunk_bytes: int, cap: int | None = None) -> tuple[np.ndarray, dict]:
    """The graph build of a database held in host memory, with at most
    chunk_bytes of device memory for its records (ngia_stream_graph): the
    sorted unique edges and per-stage stats."""
    packed = np.ascontiguousarray(packed, dtype=np.uint32)
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    lens = np.ascontiguousarray(lens, dtype=np.uint32)
    cap = int(cap if cap is not None else max(1, lens.size * bands))
    edges = np.empty(cap, EDGE_DTYPE)
    m, st = C.c_uint64(), StreamStats()
    _check(lib().ngia_stream_graph(_ptr(packed), packed.size, _ptr(offsets), _ptr(lens),
                                   lens.size, identity, bands, chunk_bytes, _ptr(edges), cap,
                                   C.byref(m), C.byref(st)), "ngia_stream_graph")
    return edges[: m.value].copy(), st.as_dict()


# ---- host-side drop-in pieces ---------------------------------------------------------
def makedb(fasta, packed) -> int:
    n = C.c_uint32()
    _check(lib().ngia_makedb(os.fsencode(fasta), os.fsencode(packed), C.byref(n)), "ngia_makedb")
    return int(n.value)


def cluster_file(packed, result, identity: int = 95, bands: int = BANDS,
                 fast: bool = False) -> dict:
    st = Stats()
    _check(lib().ngia_cluster_file(os.fsencode(packed), os.fsencode(result), identity, bands,
                                   1 if fast else 0, C.byref(st)), "ngia_cluster_file")
    return st.as_dict()


def leiden_resolution(identity: int) -> float:
    return float(lib().ngia_leiden_resolution(identity))


def leiden(edges: np.ndarray, n: int, resolution: float, seed: int = 42,
           iterations: int = 1) -> np.ndarray:
    edges = np.ascontiguousarray(edges, EDGE_DTYPE)
    out = np.empty(n, np.uint32)
    _check(lib().ngia_leiden(_ptr(edges), edges.size, n, resolution, seed, iterations,
                             _ptr(out)), "ngia_leiden")
    return out


def save_result(cluster: np.ndarray, packed, result) -> None:
    cluster = np.ascontiguousarray(cluster, np.uint32)
    _check(lib().ngia_save_result(_ptr(cluster), cluster.size, os.fsencode(packed),
                                  os.fsencode(result)), "ngia_save_result")


def read_packed(path) -> dict:
    """Parse a packed file (src/makedb.hpp:1-21) into numpy arrays."""
    raw = np.fromfile(path, dtype=np.uint8)
    n = int(raw[:4].view(np.uint32)[0])
    o = 4
    name_lens = raw[o:o + 4 * n].view(np.uint32); o += 4 * n
    lens = raw[o:o + 4 * n].view(np.uint32); o += 4 * n
    pack_off = raw[o:o + 8 * n].view(np.uint64); o += 8 * n
    fasta_off = raw[o:o + 8 * n].view(np.uint64); o += 8 * n
    rep = raw[o:o + 4 * BANDS * n].view(np.uint32).reshape(BANDS, n); o += 4 * BANDS * n
    if n == 0:  # a database with no records: the count and nothing else
        packed, offsets = np.zeros(0, np.uint32), np.zeros(0, np.uint64)
    else:
        p0, f0 = int(pack_off[0]), int(fasta_off[0])
        packed = raw[p0:f0].view(np.uint32)
        offsets = ((pack_off - np.uint64(p0)) // np.uint64(4)).astype(np.uint64)
    return {"n": n, "name_lens": name_lens, "lens": lens, "pack_off": pack_off,
            "fasta_off": fasta_off, "rep": rep, "packed": packed, "offsets": offsets,
            "raw": raw}
