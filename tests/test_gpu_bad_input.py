"""Caller-built databases that do not hold together are refused, and the
candidate collection's bounded wait gives up with an error the host reads:
  * a record offset or read length that puts a record past the end of the
    packed region -> NGIA_ERR_ARG from the host check, before any copy or
    launch (ngia_ctx_load, ngia_ctx_run_host, ngia_stream_graph);
  * a record whose length word is not its read length -> NGIA_ERR_FORMAT
    from the first layout kernel, which lays such records out empty (the
    pieced upload of ngia_ctx_run_host and the streamed build sketch before
    they read the flag);
  * the look-back of the one-pass candidate collection with a predecessor
    that never publishes -> NGIA_ERR_CUDA after a short poll limit.
After each, the same context loads the good database and builds the same
graph as a fresh one."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import ngia2_gb300 as ng

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prot(golden):
    return golden["prot"]["db"]


def edges_of(ctx, db, identity=50):
    ctx.load(db["packed"], db["offsets"], db["lens"])
    ctx.sketch_bucket(64)
    e, _ = ctx.graph(identity)
    return e


def raw_load(ctx, packed, offs, lens):
    packed = np.ascontiguousarray(packed, np.uint32)
    offs = np.ascontiguousarray(offs, np.uint64)
    lens = np.ascontiguousarray(lens, np.uint32)
    return ng.lib().ngia_ctx_load(ctx._h, packed.ctypes.data, packed.size, offs.ctypes.data,
                                  lens.ctypes.data, lens.size, None, 64)


def test_records_outside_the_region_are_refused(cuda, prot):
    with ng.Context() as fresh:
        want = edges_of(fresh, prot)
    with ng.Context() as ctx:
        launches = ng.kernel_launches()
        offs = prot["offsets"].astype(np.uint64).copy()
        offs[7] = prot["packed"].size  # past the end
        assert raw_load(ctx, prot["packed"], offs, prot["lens"]) == ng.ERR_ARG
        lens = prot["lens"].copy()
        lens[-1] = 40_000  # the last record would run past the region
        assert raw_load(ctx, prot["packed"], prot["offsets"], lens) == ng.ERR_ARG
        lens = prot["lens"].copy()
        lens[3] = 0x10000  # longer than the format allows
        assert raw_load(ctx, prot["packed"], prot["offsets"], lens) == ng.ERR_ARG
        assert ng.kernel_launches() == launches, "a launch before the host check"
        got = edges_of(ctx, prot)
    assert np.array_equal(got, want)


def test_length_word_not_the_read_length_is_refused(cuda, prot):
    with ng.Context() as fresh:
        want = edges_of(fresh, prot)
    with ng.Context() as ctx:
        packed = prot["packed"].copy()
        i = 11
        o = int(prot["offsets"][i])
        packed[o] = int(prot["lens"][i]) + 4000  # the kernel would read past the record
        assert raw_load(ctx, packed, prot["offsets"], prot["lens"]) == ng.ERR_FORMAT
        got = edges_of(ctx, prot)
    assert np.array_equal(got, want)


def test_run_host_and_streaming_refuse_records_outside(cuda, prot):
    offs = prot["offsets"].astype(np.uint64).copy()
    offs[5] = prot["packed"].size + 100
    packed = np.ascontiguousarray(prot["packed"], np.uint32)
    lens = np.ascontiguousarray(prot["lens"], np.uint32)
    edges = np.zeros(16, ng.EDGE_DTYPE)
    m = C.c_uint64()
    with ng.Context() as ctx:
        rc = ng.lib().ngia_ctx_run_host(ctx._h, packed.ctypes.data, packed.size,
                                        offs.ctypes.data, lens.ctypes.data, lens.size, 50, 64,
                                        edges.ctypes.data, len(edges), C.byref(m), None)
        assert rc == ng.ERR_ARG
    rc = ng.lib().ngia_stream_graph(packed.ctypes.data, packed.size, offs.ctypes.data,
                                    lens.ctypes.data, lens.size, 50, 3, 1 << 20,
                                    edges.ctypes.data, len(edges), C.byref(m), None)
    assert rc == ng.ERR_ARG


def test_lookback_wait_gives_up_and_context_stays_usable(cuda, prot):
    with ng.Context() as fresh:
        want = edges_of(fresh, prot)
    with ng.Context() as ctx:
        ctx.load(prot["packed"], prot["offsets"], prot["lens"])
        ctx.sketch_bucket(64)
        rc = ng.lib().ngia_ctx_test_lookback_timeout(ctx._h, 50, 64, 4096)
        assert rc == ng.ERR_CUDA
        e, _ = ctx.graph(50)
    assert np.array_equal(e, want)


@pytest.fixture(scope="module")
def dna5k(tmp_path_factory, cuda):
    """5,000 DNA sequences: enough records for run_host's pieced upload, which
    takes over once a load has fixed the four-code map."""
    from ngia2_gb300 import synth
    d = tmp_path_factory.mktemp("dna5k")
    synth.dna_families(5_000, 500, 5).write_fasta(d / "in.fa")
    ng.makedb(d / "in.fa", d / "db.packed")
    return ng.read_packed(d / "db.packed")


def run_host(ctx, db, packed=None, identity=95):
    packed = db["packed"] if packed is None else packed
    edges = np.zeros(len(db["lens"]) * 64, ng.EDGE_DTYPE)
    m, st = ctx.run_host(np.ascontiguousarray(packed, np.uint32),
                         np.ascontiguousarray(db["offsets"], np.uint64),
                         np.ascontiguousarray(db["lens"], np.uint32), identity, 64, edges)
    return edges[:m].copy(), st


def test_pieced_upload_refuses_a_wrong_length_word(dna5k):
    """The pieced upload lays out and sketches before it reads its check: a
    record whose length word is not its read length is laid out empty, the
    step is discarded, and the plain load refuses it; the context then builds
    the same graph from the good database, through the pieced upload again."""
    with ng.Context() as ctx:
        want, st0 = run_host(ctx, dna5k)
        bad = dna5k["packed"].copy()
        i = len(dna5k["lens"]) - 3  # a short record: in the first piece uploaded
        bad[int(dna5k["offsets"][i])] = int(dna5k["lens"][i]) + 5000
        with pytest.raises(ng.NgiaError) as err:
            run_host(ctx, dna5k, bad)
        assert err.value.status == ng.ERR_FORMAT
        got, st = run_host(ctx, dna5k)
        assert st["load_pipelined"] == 1
    assert np.array_equal(got, want)


def test_streaming_refuses_a_wrong_length_word(dna5k):
    packed = np.ascontiguousarray(dna5k["packed"], np.uint32).copy()
    offs = np.ascontiguousarray(dna5k["offsets"], np.uint64)
    lens = np.ascontiguousarray(dna5k["lens"], np.uint32)
    packed[int(offs[100])] = int(lens[100]) + 7
    edges = np.zeros(16, ng.EDGE_DTYPE)
    m = C.c_uint64()
    rc = ng.lib().ngia_stream_graph(packed.ctypes.data, packed.size, offs.ctypes.data,
                                    lens.ctypes.data, lens.size, 90, 3, 1 << 20,
                                    edges.ctypes.data, len(edges), C.byref(m), None)
    assert rc == ng.ERR_FORMAT


def test_pieced_upload_refuses_records_outside(dna5k):
    """The pieced upload checks the records on the host while the device
    already sketches them (kernels bounded by the region): an offset past the
    region, or a length beyond the format, is refused after the fact, and the
    context builds the same graph once the good database is loaded again."""
    with ng.Context() as ctx:
        want, _ = run_host(ctx, dna5k)
        offs = dna5k["offsets"].astype(np.uint64).copy()
        offs[7] = dna5k["packed"].size  # past the end
        lens = dna5k["lens"].copy()
        lens[3] = 0x10000  # longer than the format allows
        for bad in (dict(dna5k, offsets=offs), dict(dna5k, lens=lens)):
            with pytest.raises(ng.NgiaError) as err:
                run_host(ctx, bad)
            assert err.value.status == ng.ERR_ARG
            got, st = run_host(ctx, dna5k)
            assert st["load_pipelined"] == 1
            assert np.array_equal(got, want)


def test_hashing_sketch_after_a_pieced_load(dna5k):
    """The pieced upload leaves the residue-code nibbles out (its sketch reads
    the planes); the hashing sketch, which reads them, rebuilds them first."""
    with ng.Context() as ctx:
        want, _ = run_host(ctx, dna5k)
        got, st = run_host(ctx, dna5k)
        assert st["load_pipelined"] == 1 and np.array_equal(got, want)
        ctx.use_sketch_table(False)
        m, _ = ctx.group_align(95, 64)
        assert np.array_equal(ctx.edges(m), want)


def test_server_over_a_pieced_load(dna5k):
    """A server built on a context whose database came through the pieced
    upload (code planes deferred, residue-code nibbles left out) answers
    exactly as one built on the plain load of the same database."""
    p, o, l = dna5k["packed"], dna5k["offsets"], dna5k["lens"]
    sel = np.arange(0, len(l), 50)[:64]  # database records as queries: they assign
    recs = [p[int(o[i]):int(o[i]) + 1 + 4 * ((int(l[i]) + 31) // 32)] for i in sel]
    q_off = np.concatenate([[0], np.cumsum([len(r) for r in recs])[:-1]]).astype(np.uint64)
    q = (np.concatenate(recs).astype(np.uint32), q_off, l[sel].astype(np.uint32))
    results = []
    for pieced in (False, True):
        with ng.Context() as ctx:
            if pieced:
                run_host(ctx, dna5k)
                _, st = run_host(ctx, dna5k)
                assert st["load_pipelined"] == 1
            else:
                ctx.load(p, o, l)
                ctx.sketch_bucket(64)
            cluster = ctx.fast_cluster(95)
            with ng.Server(ctx, cluster, 95, slots=2) as srv:
                res, _ = srv.wait(srv.submit(*q), len(sel))
            results.append((cluster, res))
    assert np.array_equal(results[0][0], results[1][0])
    assert np.array_equal(results[0][1], results[1][1])
    assert (results[1][1] != ng.NEW_CLUSTER).any()
