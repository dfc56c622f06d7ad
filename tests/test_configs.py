"""The benchmark workloads at full size, checked against the exact oracle on
query subsets (the oracle answers one query in 0.1-1 s at these sizes).
Results are integer id sets: equality is bit-exact."""
import numpy as np
import pytest

import datagen
import oracle as O

pytestmark = pytest.mark.gpu


def test_config3_precision_ties_and_duplicates(engine):
    """200k facilities / 4M users, Gaussian mixture, 1% of users exactly on a
    q-f bisector, 0.1% duplicated coordinates, k=10, 2,000 queries: FP32 and
    FP64 batches agree on every query and equal the oracle on a subset; the
    forced ties reach the exact predicate."""
    ds = datagen.config(3)
    idx = engine.Index.of(ds)
    r32, st32 = idx.query_batch(ds.queries, 10, "fp32", stats=True)
    r64, st64 = idx.query_batch(ds.queries, 10, "fp64", stats=True)
    assert all(np.array_equal(a, b) for a, b in zip(r32, r64))
    assert st32["rechecks"] > 0 and st64["rechecks"] > 0
    o = O.Oracle.of(ds)
    # the tie users' queries first, then spread over the batch
    tie_q = set(int(q) for q in ds.ties[:, 1]) if ds.ties is not None else set()
    picks = [i for i, q in enumerate(ds.queries) if int(q) in tie_q][:15]
    picks += list(range(0, len(ds.queries), 80))
    for i in picks:
        assert np.array_equal(r32[i], o.query(int(ds.queries[i]), 10)), int(ds.queries[i])
    idx.close()


def test_config4_mixed_k_batch(engine):
    """20k facilities / 2M users on a street layout, 16,384 queries with k
    log-uniform in [1,100], one batch (influence zone and slice classes)."""
    ds = datagen.config(4)
    idx = engine.Index.of(ds)
    res, st = idx.query_batch(ds.queries, ds.ks, "fp32", stats=True)
    assert st["overflow"] == 0
    o = O.Oracle.of(ds)
    order = np.argsort(ds.ks)
    picks = list(order[:: len(order) // 30]) + [int(order[-1])]          # every k range, the largest k
    for i in picks:
        assert np.array_equal(res[i], o.query(int(ds.queries[i]), int(ds.ks[i]))), (int(ds.queries[i]), int(ds.ks[i]))
    idx.close()


def test_config5_serving_at_scale(engine):
    """1M facilities / 10M users resident; requests with k log-uniform in
    [1,64] through the serving loop equal the batched answers and the
    oracle."""
    ds = datagen.config(5)
    idx = engine.Index.of(ds)
    rng = np.random.default_rng(4)
    n = 300
    qs = rng.integers(0, ds.nf, n).astype(np.int32)
    ks = np.floor(np.exp(rng.uniform(0, np.log(65), n))).clip(1, 64).astype(np.int32)
    with engine.Server(idx, slots=3, max_batch=64) as srv:
        tickets = [srv.submit(q, k, "fp32" if i % 3 else "fp64") for i, (q, k) in enumerate(zip(qs, ks))]
        got = [srv.wait(t) for t in tickets]
    batch = idx.query_batch(qs, ks, "fp32")
    for i in range(n):
        assert np.array_equal(got[i], batch[i]), i
    o = O.Oracle.of(ds)
    for i in range(0, n, 40):
        assert np.array_equal(got[i], o.query(int(qs[i]), int(ks[i]))), (int(qs[i]), int(ks[i]))
    idx.close()
