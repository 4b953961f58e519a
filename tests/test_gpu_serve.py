"""The serving engine (ngia_server_*): queries assigned against a resident
database by fast mode's first-band rule, checked against a restatement with
the oracle's sketch and aligner; the same result alone and in a mix of
concurrent requests; the plain one-slot form; admission under a small budget."""
from __future__ import annotations

import numpy as np
import pytest

import ngia2_gb300 as ng
import oracle
from ngia2_gb300 import synth

pytestmark = pytest.mark.gpu

IDENTITY = 90


def database(seed: int = 31):
    """A protein database (index order = length descending) and held-out
    queries: members of the same families plus unrelated sequences."""
    from gpu_util import build_db
    # close relatives (0-4 % substitutions), so that identity 90 finds clusters
    fam = synth.families(2400, 240, synth.AMINO, synth.AMINO_FREQ,
                         synth._lognormal_roots(300, 0.5, 50, 1500), 0.0, 0.04, 0.005, 2.0,
                         seed, prefix=b"srv")
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(fam))
    db_ids, q_ids = idx[:2000], idx[2000:]
    db = sorted((fam.seq(int(i)) for i in db_ids), key=len, reverse=True)
    queries = [fam.seq(int(i)) for i in q_ids]
    queries += [synth._draw(rng, synth.AMINO, synth.AMINO_FREQ, int(L)).tobytes()
                for L in rng.integers(50, 1500, size=60)]
    return build_db(db), build_db(queries)


def expected_clusters(dbr, qr, cluster):
    """The rule restated: per band, the latest database record with the query's
    signature; the first band whose pair (longer record as rep) scores > 0."""
    (dp, do, dl), (qp, qo, ql) = dbr, qr
    n = len(dl)
    dsig = oracle.sketch_all(dp, do, dl)
    qsig = oracle.sketch_all(qp, qo, ql)
    last = [{int(s): i for i, s in enumerate(dsig[b])} for b in range(64)]  # later wins
    packed = np.concatenate([dp, qp])
    offs = np.concatenate([do, qo + len(dp)]).astype(np.uint64)
    lens = np.concatenate([dl, ql])
    cands, pairs = [], []
    for qi in range(len(ql)):
        row = [last[b].get(int(qsig[b, qi]), -1) for b in range(64)]
        cands.append(row)
        g = n + qi
        for j in dict.fromkeys(x for x in row if x >= 0):
            pairs.append((j, g) if lens[j] >= lens[g] else (g, j))
    scores = dict(zip(pairs, oracle.align_pairs(packed, offs, np.array(pairs, np.uint32),
                                                IDENTITY, oracle.ROUND_FMA))) if pairs else {}
    out = np.full(len(ql), ng.NEW_CLUSTER, np.uint32)
    for qi, row in enumerate(cands):
        g = n + qi
        for j in row:
            if j < 0:
                continue
            pr = (j, g) if lens[j] >= lens[g] else (g, j)
            if scores[pr] > 0:
                out[qi] = cluster[j]
                break
    return out


def slice_requests(qr, sizes):
    """Cut the query records into requests of the given sizes (packed,
    offsets relative to each request, lengths)."""
    qp, qo, ql = qr
    out, k = [], 0
    for s in sizes:
        sel = range(k, k + s)
        recs = [qp[int(qo[i]):int(qo[i]) + 1 + 4 * ((int(ql[i]) + 31) // 32)] for i in sel]
        offs = np.concatenate([[0], np.cumsum([len(r) for r in recs])[:-1]]).astype(np.uint64)
        out.append((np.concatenate(recs).astype(np.uint32), offs, ql[k:k + s].copy(), k))
        k += s
    return out


@pytest.fixture(scope="module")
def served(cuda, built):
    dbr, qr = database()
    with ng.Context() as ctx:
        ctx.load(*dbr)
        ctx.sketch_bucket(64)
        cluster = ctx.fast_cluster(IDENTITY)
        want = expected_clusters(dbr, qr, cluster)
        yield ctx, cluster, qr, want


def test_server_matches_the_rule(served):
    ctx, cluster, qr, want = served
    nq = len(qr[2])
    reqs = slice_requests(qr, [1, 7, 50, nq - 58])
    with ng.Server(ctx, cluster, IDENTITY, slots=4) as srv:
        tickets = [(srv.submit(p, o, l), len(l), k) for p, o, l, k in reqs]
        got = np.empty(nq, np.uint32)
        for t, c, k in tickets:
            res, st = srv.wait(t, c)
            got[k:k + c] = res
            assert st["queries"] == c and st["total_ms"] >= st["run_ms"] >= 0
    assert np.array_equal(got, want)
    # held-out family members find clusters; unrelated sequences open new ones
    assert (want[:-60] != ng.NEW_CLUSTER).any()
    assert (want[-60:] == ng.NEW_CLUSTER).all()


def test_same_result_alone_and_in_the_mix(served):
    ctx, cluster, qr, want = served
    reqs = slice_requests(qr, [120, 33, 150, 90, 1, 60])
    with ng.Server(ctx, cluster, IDENTITY, slots=3) as srv:
        p, o, l, k = reqs[0]
        alone, _ = srv.wait(srv.submit(p, o, l), len(l))
        tickets = [srv.submit(p2, o2, l2) for p2, o2, l2, _ in reqs] + [srv.submit(p, o, l)]
        mixed = [srv.wait(t, len(r[2]))[0] for t, r in zip(tickets, reqs + [reqs[0]])]
    assert np.array_equal(alone, mixed[0]) and np.array_equal(alone, mixed[-1])
    for (_, _, l2, k2), res in zip(reqs, mixed):
        assert np.array_equal(res, want[k2:k2 + len(l2)])


def test_plain_server_and_small_budget(served):
    ctx, cluster, qr, want = served
    reqs = slice_requests(qr, [64, 64, 64])
    for kw in ({"plain": True}, {"slots": 4, "hbm_budget": 1}):  # budget 1: one at a time
        with ng.Server(ctx, cluster, IDENTITY, **kw) as srv:
            tickets = [srv.submit(p, o, l) for p, o, l, _ in reqs]
            for t, (_, _, l, k) in zip(tickets, reqs):
                res, _ = srv.wait(t, len(l))
                assert np.array_equal(res, want[k:k + len(l)]), kw


def test_submit_checks_its_records(served):
    ctx, cluster, qr, _ = served
    p, o, l, _ = slice_requests(qr, [4])[0]
    with ng.Server(ctx, cluster, IDENTITY, slots=1, max_queries=3) as srv:
        with pytest.raises(ng.NgiaError):
            srv.submit(p, o, l)  # more queries than a request may hold
    with ng.Server(ctx, cluster, IDENTITY, slots=1) as srv:
        bad = o.copy()
        bad[1] = len(p) + 5
        with pytest.raises(ng.NgiaError):
            srv.submit(p, bad, l)


def test_small_requests_first_same_results(served):
    """Small requests admitted ahead of large ones, on slots reserved for
    them: every request still gets the rule's answer, whatever the order."""
    ctx, cluster, qr, want = served
    sizes = [150, 3, 1, 140, 8, 2, 100, 5]  # 409 of the 460 queries
    reqs = slice_requests(qr, sizes)
    with ng.Server(ctx, cluster, IDENTITY, slots=3, small_queries=16, small_slots=1) as srv:
        tickets = [srv.submit(p, o, l) for p, o, l, _ in reqs]
        for t, (_, _, l, k) in zip(tickets, reqs):
            res, st = srv.wait(t, len(l))
            assert np.array_equal(res, want[k:k + len(l)])
    with pytest.raises(ng.NgiaError):  # every slot reserved: large requests never run
        ng.Server(ctx, cluster, IDENTITY, slots=2, small_queries=16, small_slots=2)


def test_server_follows_its_device(served):
    """A server created while device 1 is current runs there (its dispatcher
    thread makes that device current)."""
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("one GPU")
    ctx0, cluster, qr, want = served
    torch.cuda.set_device(1)
    try:
        dbr, _ = database()
        with ng.Context() as ctx:
            ctx.load(*dbr)
            ctx.sketch_bucket(64)
            reqs = slice_requests(qr, [50])
            with ng.Server(ctx, cluster, IDENTITY, slots=2) as srv:
                p, o, l, k = reqs[0]
                res, _ = srv.wait(srv.submit(p, o, l), len(l))
        assert np.array_equal(res, want[k:k + len(l)])
    finally:
        torch.cuda.set_device(0)
