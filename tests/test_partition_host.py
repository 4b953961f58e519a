"""One database's graph split over two ranks (gloo, world size 2, CPU): the
distinct candidate pairs cut by band cells (partition.cut_points, the rule
the library applies on the device), each rank aligning its range, the
edges gathered (partition.gather_edges) and merged (partition.merge_edges)
-- the merged list must equal the reference's edge list on the golden sets.
The aligner here is the oracle (no GPU on this machine); the split, the
collective and the merge are the product's."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from conftest import load_edges

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def distinct_pairs(db, rep, identity):
    """Every band's candidates (the oracle's collection), each distinct pair
    once, grouped by target in index order."""
    import oracle
    cand = [oracle.collect_band(rep[b], db["lens"], identity) for b in range(64)]
    allp = np.concatenate(cand)
    uniq = np.unique(allp, axis=0)
    return uniq[np.lexsort((uniq[:, 0], uniq[:, 1]))]


def rank_main(rank, world, port, packed_path, identity, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    import ngia2_gb300 as ng
    import oracle
    from ngia2_gb300 import partition
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        db = ng.read_packed(packed_path)
        pairs = distinct_pairs(db, db["rep"], identity)
        lens = db["lens"]
        blocks = np.array([oracle.band_blocks(int(lens[a]), int(lens[b]), identity)
                           for a, b in pairs], np.uint64)
        cuts = partition.cut_points(blocks, world)
        mine = pairs[cuts[rank]:cuts[rank + 1]]
        scores = oracle.align_pairs(db["packed"], db["offsets"], mine, identity)
        hit = scores > 0
        e = np.zeros(int(hit.sum()), ng.EDGE_DTYPE)
        e["rep"], e["tar"] = mine[hit, 0], mine[hit, 1]
        e["weight"] = scores[hit].astype(np.float32) / np.float32(100)
        lists = partition.gather_edges(e)
        merged = partition.merge_edges(lists)
        np.save(os.path.join(out_dir, f"merged_{rank}.npy"), merged)
        np.save(os.path.join(out_dir, f"cuts_{rank}.npy"), cuts)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,identity", [("prot", 50), ("dna", 80), ("edge", 30)])
def test_two_ranks_merge_to_the_reference_edges(built, golden, tmp_path, name, identity):
    port = free_port()
    mp.start_processes(rank_main, args=(2, port, str(golden[name]["packed"]), identity,
                                        str(tmp_path)),
                       nprocs=2, join=True, start_method="spawn")
    want = load_edges(name, identity)
    for rank in range(2):
        got = np.load(tmp_path / f"merged_{rank}.npy")
        e = np.stack([got["rep"], got["tar"],
                      np.rint(got["weight"].astype(np.float64) * 100)], axis=1).astype(np.int64)
        assert np.array_equal(e, want), f"rank {rank}"
    c0, c1 = np.load(tmp_path / "cuts_0.npy"), np.load(tmp_path / "cuts_1.npy")
    assert np.array_equal(c0, c1) and c0[0] == 0 and c0[1] > 0


def test_cut_points_balance_cells():
    from ngia2_gb300 import partition
    rng = np.random.default_rng(3)
    blocks = rng.integers(0, 1000, 10_000).astype(np.uint64)
    blocks[5000:5010] = 10**7  # a few heavy pairs
    for parts in (1, 2, 3, 8):
        c = partition.cut_points(blocks, parts)
        assert c[0] == 0 and c[-1] == len(blocks) and np.all(np.diff(c) >= 0)
        share = [int(blocks[c[k]:c[k + 1]].sum()) for k in range(parts)]
        assert sum(share) == int(blocks.sum())
        assert max(share) <= int(blocks.sum()) // parts + 10**7 + 1000
    assert list(partition.cut_points(np.zeros(0, np.uint64), 4)) == [0, 0, 0, 0, 0]


def test_merge_edges_sorts_and_dedups():
    import ngia2_gb300 as ng
    from ngia2_gb300 import partition
    a = np.zeros(3, ng.EDGE_DTYPE)
    a["rep"], a["tar"], a["weight"] = [5, 1, 1], [9, 3, 2], [0.5, 0.9, 0.7]
    b = np.zeros(2, ng.EDGE_DTYPE)
    b["rep"], b["tar"], b["weight"] = [1, 0], [3, 4], [0.9, 0.6]
    m = partition.merge_edges([a, b])
    assert [(int(x["rep"]), int(x["tar"])) for x in m] == [(0, 4), (1, 2), (1, 3), (5, 9)]
