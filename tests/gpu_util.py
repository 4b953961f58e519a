"""Helpers for the GPU tests: raw device buffers through torch (plumbing
only; every computation goes through libngia's C ABI)."""
from __future__ import annotations

import numpy as np
import torch

import ngia2_gb300 as ng


def to_dev(a: np.ndarray) -> torch.Tensor:
    """Copy an array's bytes to a device uint8 tensor."""
    b = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
    return torch.from_numpy(b.copy()).to("cuda")


def dev_empty(nbytes: int) -> torch.Tensor:
    return torch.empty(max(nbytes, 16), dtype=torch.uint8, device="cuda")


def from_dev(t: torch.Tensor, dtype, count: int | None = None) -> np.ndarray:
    torch.cuda.synchronize()
    a = t.cpu().numpy().view(dtype)
    return a if count is None else a[:count]


def stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def align_jobs_on_gpu(packed: np.ndarray, offsets: np.ndarray, pairs: np.ndarray,
                      identity: int, mode: str = "fma") -> np.ndarray:
    """Scores of (rep, tar) pairs through ngia_align_pairs (one launch)."""
    pairs = np.asarray(pairs, np.uint32).reshape(-1, 2)
    jobs = np.zeros((len(pairs), 3), np.uint32)
    jobs[:, :2] = pairs
    d_packed, d_offs, d_jobs = to_dev(packed), to_dev(np.asarray(offsets, np.uint64)), to_dev(jobs)
    old = ng.set_round_mode(mode)
    try:
        ng.align_pairs(d_packed.data_ptr(), d_offs.data_ptr(), d_jobs.data_ptr(), len(pairs),
                       identity, stream())
        out = from_dev(d_jobs, np.uint32).reshape(-1, 3)[:, 2].copy()
    finally:
        ng.set_round_mode(old)
    return out


def build_db(seqs: list[bytes]):
    """Pack sequences (already in the order wanted) into a packed region with
    word offsets, using the oracle's packer."""
    import oracle
    recs = [oracle.pack_record(s) for s in seqs]
    offs = np.concatenate([[0], np.cumsum([len(r) for r in recs])[:-1]]).astype(np.uint64)
    packed = np.concatenate(recs).astype(np.uint32) if recs else np.zeros(1, np.uint32)
    lens = np.array([len(s) for s in seqs], np.uint32)
    return packed, offs, lens


def reference_rep_rows(sigs_band_major: np.ndarray) -> np.ndarray:
    """rep[b][i] = largest j < i with equal signature, else i (numpy)."""
    bands, n = sigs_band_major.shape
    out = np.empty((bands, n), np.uint32)
    idx = np.arange(n, dtype=np.uint32)
    for b in range(bands):
        s = sigs_band_major[b]
        order = np.lexsort((idx, s))
        ss = s[order]
        prev = np.empty(n, np.uint32)
        prev[0] = order[0]
        same = ss[1:] == ss[:-1]
        prev[1:] = np.where(same, order[:-1], order[1:])
        out[b, order] = prev
    return out
