"""Host-side logic of bench.py: rank bookkeeping over gloo (world size 2, CPU)
and the algorithmic unit counts."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      LOCAL_RANK=str(rank), WORLD_SIZE=str(world))

    class Args:
        impl = "reference"  # the gloo path (the reference arm runs on host cores)

    w, r, local, pg = bench.dist_setup(Args)
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(pg)
    # the slowest rank's step time decides the whole-job throughput
    out[rank] = bench.max_over_ranks(pg, 10.0 + rank)
    pg.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = free_port()
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        assert dict(out) == {0: 11.0, 1: 11.0}


def test_single_rank_needs_no_process_group():
    class Args:
        impl = "ours"
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    w, r, local, pg = bench.dist_setup(Args)
    assert (w, r, local, pg) == (1, 0, 0, None)
    assert bench.max_over_ranks(None, 3.5) == 3.5


def test_signed_positions():
    # L >= 8 signs L - 7 positions; 1..7 signs one; an empty record none
    lens = np.array([0, 1, 7, 8, 9, 100])
    assert bench.signed_positions(lens) == 0 + 1 + 1 + 1 + 2 + 93


@pytest.mark.parametrize("steps,warmup", [(60, 3), (5, 3), (1000, 10)])
def test_reference_arm_sample_is_bounded(steps, warmup):
    fam = bench.reference_sample_families(steps, warmup)
    assert 50 <= fam <= bench.CPU_SAMPLE_FAMILIES
    # whole run within a few minutes at the rate the sample is sized from
    assert (steps + warmup) * fam / bench.CPU_FAMILIES_PER_S <= 240
