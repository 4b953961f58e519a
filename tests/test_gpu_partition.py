"""The graph build split into shares by band cells (ngia_ctx_build_graph_part),
the shares run one after another on this GPU as the ranks of a multi-GPU
build would: their ranges tile the distinct pairs in order, and their edges,
merged (partition.merge_edges), equal the whole build's and the reference's
golden edges."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
from conftest import IDENTITIES, SETS, load_edges
from ngia2_gb300 import partition

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", SETS)
@pytest.mark.parametrize("parts", [2, 3, 8])
def test_shares_merge_to_the_whole_graph(cuda, golden, name, parts):
    db = golden[name]["db"]
    identity = IDENTITIES[name][0]
    with ng.Context() as ctx:
        ctx.load(db["packed"], db["offsets"], db["lens"], db["rep"], 64)
        whole, st = ctx.graph(identity)
        lists, ranges = [], []
        for part in range(parts):
            m, pst, rng = ctx.build_graph_part(identity, part, parts)
            lists.append(ctx.edges(m))
            ranges.append(rng)
            assert pst["unique_pairs"] == rng[1] - rng[0]
    assert ranges[0][0] == 0 and ranges[-1][1] == st["unique_pairs"]
    assert all(ranges[k][1] == ranges[k + 1][0] for k in range(parts - 1))
    merged = partition.merge_edges(lists)
    assert np.array_equal(merged, whole)
    e = np.stack([merged["rep"], merged["tar"],
                  np.rint(merged["weight"].astype(np.float64) * 100)], axis=1).astype(np.int64)
    assert np.array_equal(e, load_edges(name, identity))


def test_shares_balance_band_cells(cuda, golden):
    db = golden["prot"]["db"]
    with ng.Context() as ctx:
        ctx.load(db["packed"], db["offsets"], db["lens"], db["rep"], 64)
        _, st = ctx.build_graph(50)
        cells = [ctx.build_graph_part(50, k, 4)[1]["aligned_cells"] for k in range(4)]
    assert sum(cells) == st["aligned_cells"]
    assert max(cells) < 0.5 * sum(cells)
