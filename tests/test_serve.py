"""Serving (rknn_serve_*): continuous batching must not change any result.

Requests from several threads, with mixed k and both modes, are batched by
the server as they arrive and run while other batches are on the GPU; every
result must equal the same query answered alone (rknn_query) and the exact
oracle.  Results are integer id sets: equality is bit-exact."""
import threading

import numpy as np
import pytest

import datagen
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(engine):
    ds = datagen.uniform(20_000, 200_000, seed=31, nq=10, k=5)
    return ds, engine.Index.of(ds), O.Oracle.of(ds)


def test_results_alone_and_in_the_mix(engine, served):
    ds, idx, orc = served
    rng = np.random.default_rng(5)
    n = 600
    qs = rng.integers(0, ds.nf, n)
    ks = np.exp(rng.uniform(0, np.log(48), n)).astype(int) + 1          # k log-uniform in [1, 48]
    modes = np.where(rng.random(n) < 0.5, "fp32", "fp64")
    got = [None] * n
    errors = []
    with engine.Server(idx, slots=3, max_batch=128, scratch_bytes=64 << 20) as srv:
        def client(part):
            try:
                tickets = [(i, srv.submit(qs[i], ks[i], modes[i])) for i in part]
                for i, t in tickets:
                    got[i] = srv.wait(t)
            except Exception as e:      # surfaced below
                errors.append(e)
        parts = [range(j, n, 4) for j in range(4)]
        th = [threading.Thread(target=client, args=(p,)) for p in parts]
        for t in th:
            t.start()
        for t in th:
            t.join()
        st = srv.stats()
    assert not errors, errors
    assert st["completed"] == n and st["failed"] == 0
    assert st["batches"] < n, "requests were never batched together"
    for i in range(n):
        alone = idx.query(int(qs[i]), int(ks[i]), str(modes[i]))
        assert np.array_equal(got[i], alone), (i, int(qs[i]), int(ks[i]), modes[i])
    for i in range(0, n, 15):
        assert got[i].tolist() == orc.query(int(qs[i]), int(ks[i])).tolist(), i


def test_overlapping_batches_and_replay(engine, served):
    ds, idx, orc = served
    rng = np.random.default_rng(9)
    n = 2000
    qs = rng.integers(0, ds.nf, n).astype(np.int32)
    ks = (np.exp(rng.uniform(0, np.log(32), n)).astype(int) + 1).astype(np.int32)
    arrival = np.cumsum(rng.exponential(1.0 / 20_000, n))               # Poisson, 20k requests/s
    with engine.Server(idx, slots=3, max_batch=256) as srv:
        lat, nres = srv.replay(qs, ks, "fp32", arrival)
        st = srv.stats()
    assert st["completed"] == n and st["failed"] == 0
    assert np.all(lat > 0) and st["p99_ms"] >= st["p50_ms"] > 0
    sizes = idx.query_batch(qs[:200], ks[:200], "fp32")
    assert [len(x) for x in sizes] == nres[:200].tolist()


def test_rejects_bad_requests(engine, served):
    ds, idx, _ = served
    with engine.Server(idx, slots=1) as srv:
        for q, k in ((-1, 5), (ds.nf, 5), (0, 0)):
            with pytest.raises(engine.RkNNError) as e:
                srv.submit(q, k)
            assert e.value.status == 1
        t = srv.submit(3, 4, "fp64")
        assert srv.wait(t).tolist() == orc_ids(served, 3, 4)
        with pytest.raises(engine.RkNNError) as e:
            srv.wait(t)                                       # already released
        assert e.value.status == 1


def orc_ids(served, q, k):
    return served[2].query(q, k).tolist()


@pytest.mark.parametrize("kind,status", [("oom", 2), ("launch", 3)])
def test_failed_batches_and_recovery(engine, served, kind, status):
    """A batch whose workspace allocation fails (kind "oom") or whose launch
    fails after its input copy ("launch"), made to fail on the host through
    the server's failure hook (no GPU fault): its requests end with
    RKNN_ERR_OOM / RKNN_ERR_CUDA, every other request of the stream gets the
    oracle's ids, and requests after the failure complete normally."""
    ds, idx, orc = served
    rng = np.random.default_rng(11 if kind == "oom" else 12)
    qs = rng.integers(0, ds.nf, 64)
    ks = rng.integers(1, 20, 64)
    with engine.Server(idx, slots=2, max_batch=16) as srv:
        srv.inject_fault(kind, 1)
        tickets = [srv.submit(int(q), int(k), "fp32" if i % 2 else "fp64") for i, (q, k) in enumerate(zip(qs, ks))]
        failed = 0
        for t, q, k in zip(tickets, qs, ks):
            try:
                got = srv.wait(t)
            except engine.RkNNError as e:
                assert e.status == status, (e.status, str(e))
                failed += 1
                continue
            assert np.array_equal(got, orc.query(int(q), int(k))), (int(q), int(k))
        assert 1 <= failed <= 16
        st = srv.stats()
        assert st["failed"] == failed and st["completed"] == 64 - failed
        # after the failure: the slot allocates afresh and every request completes
        more = [srv.submit(int(q), int(k), "fp32") for q, k in zip(qs[:32], ks[:32])]
        for t, q, k in zip(more, qs[:32], ks[:32]):
            assert np.array_equal(srv.wait(t), orc.query(int(q), int(k)))


def test_request_beyond_the_scratch_budget_is_refused(engine, served):
    """Admission: a request whose own scratch estimate exceeds the server's
    scratch_bytes is refused at submit with RKNN_ERR_CAPACITY (never run over
    budget); requests that fit are served."""
    ds, idx, orc = served
    q = int(ds.queries[0])
    # a batch of one is padded to 32 slots, each with a 32 KB share of the
    # result pool: one request alone needs more than 1 MiB
    with engine.Server(idx, slots=1, max_batch=8, scratch_bytes=1 << 20) as srv:
        with pytest.raises(engine.RkNNError) as e:
            srv.submit(q, 5, "fp32")
        assert e.value.status == 5
    with engine.Server(idx, slots=1, max_batch=8, scratch_bytes=8 << 20) as srv:
        t = srv.submit(q, 5, "fp32")
        assert np.array_equal(srv.wait(t), orc.query(q, 5))
