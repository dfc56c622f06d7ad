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
