"""Databases of a handful of records, loaded one after another into one
context with a larger one between them: the device signatures, rep rows and
graph equal the oracle's each time, so the cached bucketing graph (captured
again whenever the record count changes) follows every load.  One record,
two equal records, records of 0, 1, 7 and 9 residues, a DNA family and a
protein family."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
import oracle
from gpu_util import build_db, reference_rep_rows
from ngia2_gb300 import synth

pytestmark = pytest.mark.gpu


def family(seed: int, n: int, length: int, letters: bytes) -> list[bytes]:
    rng = np.random.default_rng(seed)
    alphabet = np.frombuffer(letters, np.uint8)
    root = rng.choice(alphabet, size=length)
    out = [bytes(root)]
    for _ in range(1, n):
        s = root.copy()
        at = rng.choice(length, size=max(1, length // 60), replace=False)
        s[at] = rng.choice(alphabet, size=at.size)
        out.append(bytes(s))
    return out


def by_length(seqs: list[bytes]) -> list[bytes]:
    return sorted(seqs, key=len, reverse=True)  # stable: the packed file's order


CASES = [
    ("one record", [b"ACGTACGTAC"]),
    ("two equal records", [b"MKVLAAGIVGLLA" * 3] * 2),
    ("0, 1, 7 and 9 residues", [b"ACGTACGTA", b"ACGTACG", b"A", b""]),
    ("DNA family", family(3, 5, 700, b"ACGT")),
    ("protein family", family(4, 6, 260, b"ACDEFGHIKLMNPQRSTVWY")),
]


def as_triples(e: np.ndarray) -> np.ndarray:
    return np.stack([e["rep"].astype(np.int64), e["tar"].astype(np.int64),
                     np.rint(e["weight"].astype(np.float64) * 100).astype(np.int64)], axis=1)


def check(ctx: ng.Context, seqs: list[bytes], identity: int) -> None:
    packed, offs, lens = build_db(by_length(seqs))
    ctx.load(packed, offs, lens)
    ctx.sketch_bucket(64)
    sigs = oracle.sketch_all(packed, offs, lens)
    assert np.array_equal(ctx.sigs(), sigs)
    rep = reference_rep_rows(sigs)
    assert np.array_equal(ctx.rep_rows(64), rep)
    for bands in (64, 3):
        got, _ = ctx.graph(identity, bands)
        want, _ = oracle.graph_edges(packed, offs, lens, rep, identity, bands)
        assert np.array_equal(as_triples(got), want), bands


def test_small_databases_one_after_another(cuda, built):
    s = synth.dna_families(2000, 200, seed=17)
    larger = [s.seq(i) for i in range(len(s))]
    with ng.Context() as ctx:
        for name, seqs in CASES[:3]:
            check(ctx, seqs, 90)
        check(ctx, larger, 95)
        for name, seqs in CASES[2:]:
            check(ctx, seqs, 90)
        check(ctx, CASES[0][1], 90)


def test_launch_count_includes_graph_replays(cuda, built):
    """ngia_kernel_launches counts a cached graph's kernels at every replay
    and once for the call that captures it: the bucketing inside a graph
    build and a batched round count the same replayed, captured or launched
    directly."""
    s = synth.dna_families(3000, 300, seed=23)
    packed, offs, lens = build_db(by_length([s.seq(i) for i in range(len(s))]))
    rng = np.random.default_rng(23)
    a, b = rng.integers(0, 1500, 4000), rng.integers(0, 1500, 4000)
    pairs = np.stack([np.minimum(a, b), np.maximum(a, b)], axis=1).astype(np.uint32)
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]

    def count(fn) -> int:
        before = ng.kernel_launches()
        fn()
        return ng.kernel_launches() - before

    with ng.Context() as ctx:
        ctx.load(packed, offs, lens)
        calls = {  # (first key, another key)
            "graph build": (lambda: ctx.group_align(95, 64), lambda: ctx.group_align(95, 32)),
            "round": (lambda: ctx.align_pairs(pairs, 70), lambda: ctx.align_pairs(pairs, 80)),
        }
        got = {}
        for name, (first, other) in calls.items():
            ctx.use_graphs(True)
            first()  # captured (and the load's one-time work done)
            got[name, "replayed"] = count(first)
            got[name, "captured"] = count(other)
            ctx.use_graphs(False)
            got[name, "direct"] = count(first)
            got[name, "direct other"] = count(other)
    for name in calls:
        assert got[name, "replayed"] == got[name, "direct"] > 0, got
        assert got[name, "captured"] == got[name, "direct other"] > 0, got
