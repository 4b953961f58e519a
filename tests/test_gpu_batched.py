"""The batched aligner on caller-given pairs (ngia_ctx_align_pairs): every
width class -- one pair per lane for narrow bands, groups of 8, 16 and 32
lanes for wide ones, the general kernel beyond -- against the oracle, pair by pair,
and against the drop-in one-thread-per-pair kernel."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
import oracle
from ngia2_gb300 import synth

GROUP_SHAPES = ng.GROUP_SHAPES


def width_class(lr: int, lt: int, identity: int) -> int:
    """The class the library bins a pair into (align.cuh width_class)."""
    bb = oracle.band_bounds(lr, lt, identity, oracle.ROUND_FMA)
    if bb is None:
        return ng.SKIP_CLASS
    lsft, rsft = bb
    ls, rs, nr = lsft // 32, (rsft + 31) // 32, (lr + 31) // 32
    ws = ls + min(rs, nr)
    if ws <= 16:
        return 0 if ws <= 4 else ws - 4 if ws <= 12 else 9 if ws <= 14 else 10
    for c, (g, k) in enumerate(GROUP_SHAPES, start=ng.FIRST_GROUP_CLASS):
        if (nr + k - 1) // k <= g or ls + rs <= (g - 1) * k + g:
            return c
    return ng.GENERAL_CLASS


def mutate(rng, s: bytes, sub: float, indel: float) -> bytes:
    b = bytearray(s)
    for p in rng.integers(0, len(b), size=int(len(b) * sub)):
        b[int(p)] = synth.AMINO[rng.integers(0, 20)]
    out = bytearray()
    for ch in b:
        r = rng.random()
        if r < indel / 2:
            continue  # deletion
        out.append(ch)
        if r > 1 - indel / 2:
            out += bytes(synth.AMINO[rng.integers(0, 20, size=int(rng.integers(1, 4)))])
    return bytes(out) or b"A"


def pair_set(identity: int, seed: int):
    """Pairs of related and unrelated protein sequences whose bands cover the
    width classes at this identity."""
    rng = np.random.default_rng(seed)
    seqs: list[bytes] = []
    pairs = []
    lengths = list(np.exp(rng.uniform(np.log(20), np.log(12000), size=160)).astype(int))
    lengths += [int(x) for x in rng.integers(15000, 36000, size=4)]
    for L in lengths:
        root = synth._draw(rng, synth.AMINO, synth.AMINO_FREQ, int(L)).tobytes()
        related = rng.random() < 0.7
        if related:
            other = mutate(rng, root, rng.uniform(0.0, 0.3), rng.uniform(0.0, 0.03))
        else:
            m = max(1, int(L * rng.uniform(0.85, 1.0)))
            other = synth._draw(rng, synth.AMINO, synth.AMINO_FREQ, m).tobytes()
        a, b = (root, other) if len(root) >= len(other) else (other, root)
        seqs += [a, b]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    return seqs, np.array(pairs, np.uint32)


@pytest.mark.gpu
@pytest.mark.parametrize("identity", [30, 50, 70, 90, 95])
def test_batched_pairs_match_oracle(cuda, built, identity):
    from gpu_util import align_jobs_on_gpu, build_db
    seqs, pairs = pair_set(identity, 900 + identity)
    packed, offs, lens = build_db(seqs)
    want = oracle.align_pairs(packed, offs, pairs, identity, oracle.ROUND_FMA)
    with ng.Context() as ctx:
        ctx.load(packed, offs, lens)
        got, st = ctx.align_pairs(pairs, identity)  # captures the round as a graph
        # replayed with other contents: queues and counters start over
        again, _ = ctx.align_pairs(pairs[::-1], identity)
        ctx.use_graphs(False)
        eager, st_eager = ctx.align_pairs(pairs, identity)
    assert np.array_equal(eager, got)
    assert st_eager["computed_cells"] == st["computed_cells"]
    assert st_eager["aligned_cells"] == st["aligned_cells"]
    classes = {width_class(int(lens[r]), int(lens[t]), identity) for r, t in pairs}
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, [(int(pairs[i, 0]), int(pairs[i, 1]), int(lens[pairs[i, 0]]),
                            int(lens[pairs[i, 1]]), int(got[i]), int(want[i]),
                            width_class(int(lens[pairs[i, 0]]), int(lens[pairs[i, 1]]),
                                        identity)) for i in bad[:10]]
    assert np.array_equal(again[::-1], want)
    assert np.array_equal(align_jobs_on_gpu(packed, offs, pairs, identity), want)
    assert st["unique_pairs"] == len(pairs)
    assert (want > 0).any() and (want == 0).any()
    # the set reaches the group kernels at every identity
    assert classes & set(range(ng.FIRST_GROUP_CLASS, ng.GENERAL_CLASS)), sorted(classes)


@pytest.mark.gpu
@pytest.mark.parametrize("identity", [50, 90])
def test_group_exit_when_the_path_runs_high(cuda, built, identity):
    """Targets that are a suffix of their rep, just above the identity cut:
    the LCS path runs Lr - Lt rows above the diagonal, near the band's upper
    edge, where rows enter the band before the slice holding them has run its
    first block.  The early exit must not end such pairs: scores equal the
    oracle's with the default plan and with narrow bands sent to the group
    classes."""
    from gpu_util import build_db
    rng = np.random.default_rng(4242 + identity)
    seqs: list[bytes] = []
    pairs = []
    for _ in range(400):
        lr = int(rng.integers(200, 1500))
        lt = min(lr, int(np.ceil(lr * identity / 100 * rng.uniform(1.005, 1.08))))
        rep = synth._draw(rng, synth.AMINO, synth.AMINO_FREQ, lr).tobytes()
        seqs += [rep, rep[lr - lt:]]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    pairs = np.array(pairs, np.uint32)
    packed, offs, lens = build_db(seqs)
    want = oracle.align_pairs(packed, offs, pairs, identity, oracle.ROUND_FMA)
    assert (want > 0).mean() > 0.9
    with ng.Context() as ctx:
        ctx.load(packed, offs, lens)
        default = ctx.plan()
        for plan in (default, {"stream_max": 4, "group_limit": default["group_limit"]}):
            ctx.set_plan(plan)
            got, _ = ctx.align_pairs(pairs, identity)
            bad = np.nonzero(got != want)[0]
            assert len(bad) == 0, (plan["stream_max"], [
                (int(lens[pairs[i, 0]]), int(lens[pairs[i, 1]]), int(got[i]), int(want[i]))
                for i in bad[:8]])


def test_every_group_class_is_covered(built):
    """Across the identities above, every class is reached (host-side check
    of the test data, no GPU)."""
    seen = set()
    for identity in (30, 50, 70, 90, 95):
        seqs, pairs = pair_set(identity, 900 + identity)
        lens = [len(s) for s in seqs]
        seen |= {width_class(lens[r], lens[t], identity) for r, t in pairs}
    assert set(range(ng.FIRST_GROUP_CLASS, ng.GENERAL_CLASS)) <= seen, sorted(seen)
    assert {0, ng.GENERAL_CLASS} <= seen, sorted(seen)


@pytest.mark.gpu
def test_plans_change_binning_not_scores(cuda, built):
    """Every plan -- narrow per-lane windows, group classes switched off, the
    autotuner's pick -- gives the same scores; plans beyond a class's band
    limit are refused."""
    from gpu_util import build_db, to_dev
    seqs, pairs = pair_set(70, 977)
    packed, offs, lens = build_db(seqs)
    want = oracle.align_pairs(packed, offs, pairs, 70, oracle.ROUND_FMA)
    with ng.Context() as ctx:
        ctx.load(packed, offs, lens)
        default = ctx.plan()
        assert default["stream_max"] == 16
        limits = default["group_limit"]
        assert limits == [(g - 1) * k + g for g, k in ng.GROUP_SHAPES]
        for plan in ({"stream_max": 8, "group_limit": limits},
                     {"stream_max": 4, "group_limit": [0, limits[1], 0, limits[3], 0, 0,
                                                      limits[6], 0]},
                     {"stream_max": 12, "group_limit": [0] * len(limits)}):
            ctx.set_plan(plan)
            assert ctx.plan() == plan
            got, _ = ctx.align_pairs(pairs, 70)
            assert np.array_equal(got, want), plan
        with pytest.raises(ng.NgiaError):
            ctx.set_plan({"stream_max": 18, "group_limit": limits})
        with pytest.raises(ng.NgiaError):
            ctx.set_plan({"stream_max": 16, "group_limit": [limits[0] + 1] + limits[1:]})
        d_pairs = to_dev(pairs)
        plan, ms = ctx.autotune(d_pairs.data_ptr(), len(pairs), 70, 1)
        assert ctx.plan() == plan and ms > 0
        got, _ = ctx.align_pairs(pairs, 70)
        assert np.array_equal(got, want)


@pytest.mark.gpu
def test_host_pairs_are_checked(cuda, built):
    from gpu_util import build_db
    packed, offs, lens = build_db([b"ACDEFGHIKL", b"ACDEFGHIKV"])
    with ng.Context() as ctx:
        ctx.load(packed, offs, lens)
        with pytest.raises(ng.NgiaError):
            ctx.align_pairs(np.array([[0, 2]], np.uint32), 90)
        s, _ = ctx.align_pairs(np.array([[0, 1]], np.uint32), 80)
        assert s[0] == oracle.align_pairs(packed, offs, np.array([[0, 1]], np.uint32), 80)[0]


@pytest.mark.gpu
def test_replayed_round_follows_a_new_database(cuda, built):
    """The round's cached graph is keyed on the database's alphabet and
    buffers: a four-letter nucleotide database (five-entry tables), then the
    same sequences with a few N (eight-entry tables) loaded into the same
    context -- the same buffers, lengths, device pairs and scores arrays; each
    round's scores must be its own database's."""
    from gpu_util import build_db, to_dev
    rng = np.random.default_rng(11)
    s = synth.dna_families(2_000, 200, seed=12)
    order = np.argsort(-s.lens, kind="stable")
    seqs = [s.seq(int(i)) for i in order]
    with_n = []
    for q in seqs:
        b = bytearray(q)
        for p in rng.integers(0, len(b), size=max(1, len(b) // 200)):
            b[int(p)] = ord("N")
        with_n.append(bytes(b))
    a = rng.integers(0, 800, 3000)
    b = rng.integers(0, 800, 3000)
    pairs = np.stack([np.minimum(a, b), np.maximum(a, b)], axis=1).astype(np.uint32)
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    d_pairs = to_dev(pairs)
    import torch
    d_scores = torch.zeros(len(pairs), dtype=torch.int32, device="cuda")
    with ng.Context() as ctx:
        for db in (build_db(seqs), build_db(with_n)):
            packed, offs, lens = db
            ctx.load(packed, offs, lens)
            ctx.align_pairs_device(d_pairs.data_ptr(), len(pairs), 70, d_scores.data_ptr())
            got = d_scores.cpu().numpy().view(np.uint32)
            want = oracle.align_pairs(packed, offs, pairs, 70, oracle.ROUND_FMA)
            assert np.array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,identities", [("protein", (30, 50, 90, 99)), ("dna", (50, 95))])
def test_pairs_at_the_longest_record(cuda, built, kind, identities):
    """Records of the format's longest read (65,534 residues; the packed file
    drops 65,535 and above) and just below it, close and distant relatives and
    an unrelated one, every pair: the batched round (the general kernel at low
    identities) and the drop-in kernel both equal the oracle."""
    from gpu_util import align_jobs_on_gpu, build_db
    rng = np.random.default_rng(65534 if kind == "protein" else 65533)
    alphabet = (np.asarray(synth.AMINO, np.uint8) if kind == "protein"
                else np.frombuffer(b"ACGT", np.uint8))
    top = 65534

    def draw(n):
        return bytes(rng.choice(alphabet, size=n))

    def subst(s, rate):
        a = np.frombuffer(s, np.uint8).copy()
        at = rng.random(a.size) < rate
        a[at] = rng.choice(alphabet, size=int(at.sum()))
        return bytes(a)

    root = draw(top)
    seqs = [root, subst(root, 0.03), subst(root, 0.4)[: top - 1000], draw(top - 7)]
    seqs.sort(key=len, reverse=True)
    packed, offs, lens = build_db(seqs)
    assert int(lens[0]) == top
    pairs = np.array([(r, t) for r in range(4) for t in range(r + 1, 4)], np.uint32)
    with ng.Context() as ctx:
        ctx.load(packed, offs, lens)
        for identity in identities:
            want = oracle.align_pairs(packed, offs, pairs, identity, oracle.ROUND_FMA)
            got, _ = ctx.align_pairs(pairs, identity)
            assert np.array_equal(got, want), identity
            assert np.array_equal(align_jobs_on_gpu(packed, offs, pairs, identity), want), identity
    classes = {width_class(int(lens[r]), int(lens[t]), 30) for r, t in pairs}
    if kind == "protein":
        assert ng.GENERAL_CLASS in classes, sorted(classes)
