"""One database's graph built by several devices (one process per device):
each rank aligns a share of the distinct candidate pairs cut by band cells
(ngia_ctx_build_graph_part), then the compacted edge lists are gathered and
merged into the one sorted edge list that Leiden reads.  The reference runs
on one device (src/buildGraph.hpp:101-102); the exchange is this one gather,
before the host's sort (src/buildGraph.hpp:357-358).

    cut_points(blocks, parts)  the ranges' boundaries, the rule the library
                               applies on the device (for tests and planning)
    gather_edges(edges, pg)    every rank's edges, concatenated in rank order
    merge_edges(lists)         the sorted, unique union
"""
from __future__ import annotations

import numpy as np

from . import EDGE_DTYPE


def cut_points(blocks: np.ndarray, parts: int) -> np.ndarray:
    """Boundaries of `parts` contiguous ranges of pairs with about equal band
    blocks: range k starts at the first pair whose exclusive prefix of blocks
    reaches total * k // parts (0 and len(blocks) at the ends)."""
    blocks = np.asarray(blocks, np.uint64)
    prefix = np.concatenate([[0], np.cumsum(blocks, dtype=np.uint64)[:-1]]).astype(np.uint64) \
        if len(blocks) else np.zeros(0, np.uint64)
    total = int(blocks.sum()) if len(blocks) else 0
    cuts = [0]
    for k in range(1, parts):
        target = total // parts * k + (total % parts) * k // parts
        cuts.append(int(np.searchsorted(prefix, np.uint64(target), side="left")))
    cuts.append(len(blocks))
    return np.asarray(cuts, np.int64)


def merge_edges(lists) -> np.ndarray:
    """Union of the ranks' edge lists, sorted by (rep, tar, weight), unique
    (the reference's sort + unique of the whole list)."""
    lists = [np.asarray(x, EDGE_DTYPE) for x in lists]
    e = np.concatenate(lists) if lists else np.zeros(0, EDGE_DTYPE)
    if len(e) == 0:
        return e
    order = np.lexsort((e["weight"], e["tar"], e["rep"]))
    e = e[order]
    keep = np.ones(len(e), bool)
    keep[1:] = (e["rep"][1:] != e["rep"][:-1]) | (e["tar"][1:] != e["tar"][:-1]) | \
               (e["weight"][1:] != e["weight"][:-1])
    return e[keep]


def gather_edges(edges: np.ndarray, pg=None, device: str = "cpu") -> list[np.ndarray]:
    """Every rank's edge list (torch.distributed: all-gather of the counts,
    then of the lists padded to the longest), in rank order.  device: where
    the collective's tensors live ('cpu' for gloo, 'cuda' for NCCL)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(pg)
    raw = np.ascontiguousarray(edges, EDGE_DTYPE).view(np.int32).reshape(-1, 3)
    n = torch.tensor([len(raw)], dtype=torch.int64, device=device)
    counts = [torch.zeros(1, dtype=torch.int64, device=device) for _ in range(world)]
    dist.all_gather(counts, n, group=pg)
    counts = [int(c.item()) for c in counts]
    cap = max(1, max(counts))
    mine = torch.zeros((cap, 3), dtype=torch.int32, device=device)
    if len(raw):
        mine[:len(raw)] = torch.from_numpy(raw).to(device)
    bufs = [torch.zeros((cap, 3), dtype=torch.int32, device=device) for _ in range(world)]
    dist.all_gather(bufs, mine, group=pg)
    return [b[:c].cpu().numpy().copy().view(EDGE_DTYPE).reshape(-1)
            for b, c in zip(bufs, counts)]
