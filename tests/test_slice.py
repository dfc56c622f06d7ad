"""Angular-slice filter (large k): results must equal the exact oracle.

The slice filter only bounds the candidate users; the verification decides
exactly, so any filter choice gives the same id sets.  Results are integer
id sets: equality is bit-exact."""
import numpy as np
import pytest

import datagen
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def uni(engine):
    ds = datagen.uniform(20_000, 200_000, seed=51, nq=30, k=1)
    return ds, O.Oracle.of(ds)


def test_slice_filter_matches_oracle(engine, uni):
    ds, o = uni
    idx = engine.Index.of(ds, filter="slice")
    for k in (1, 3, 10, 30, 100):
        got = idx.query_batch(ds.queries, k, "fp32")
        got64 = idx.query_batch(ds.queries[:8], k, "fp64")
        for i, q in enumerate(ds.queries):
            want = o.query(int(q), k)
            assert np.array_equal(got[i], want), (int(q), k)
            if i < 8:
                assert np.array_equal(got64[i], want), (int(q), k, "fp64")
    idx.close()


def test_filters_agree_in_one_batch(engine, uni):
    """A batch of mixed k runs its small-k classes through the influence zone
    and its large-k classes through the slice filter; every answer equals the
    influence-zone-only index's and the oracle's."""
    ds, o = uni
    rng = np.random.default_rng(2)
    qs = rng.integers(0, ds.nf, 200).astype(np.int32)
    ks = rng.integers(1, 80, 200).astype(np.int32)
    auto = engine.Index.of(ds)
    inf = engine.Index.of(ds, filter="inf")
    a = auto.query_batch(qs, ks, "fp32")
    b = inf.query_batch(qs[:40], ks[:40], "fp32")
    for i in range(40):
        assert np.array_equal(a[i], b[i]), (int(qs[i]), int(ks[i]))
    for i in range(0, 200, 7):
        assert np.array_equal(a[i], o.query(int(qs[i]), int(ks[i]))), (int(qs[i]), int(ks[i]))
    auto.close()
    inf.close()


def test_slice_bounds_the_candidates(engine, uni):
    """At k = 100 the influence zone outgrows its shared-memory capacity; the
    slice filter keeps the candidate set within a small multiple of the
    results."""
    ds, o = uni
    idx = engine.Index.of(ds, filter="slice")
    res, st = idx.query_batch(ds.queries, 100, "fp32", stats=True)
    assert st["overflow"] == 0
    assert st["candidates"] < 12 * max(1, st["results"]), st
    idx.close()


def test_slice_on_ties_and_street(engine):
    ds = datagen.gaussmix(20_000, 300_000, seed=8, nq=60, k=10)
    o = O.Oracle.of(ds)
    idx = engine.Index.of(ds, filter="slice")
    got = idx.query_batch(ds.queries, 10, "fp32")
    for i, q in enumerate(ds.queries):
        assert np.array_equal(got[i], o.query(int(q), 10)), int(q)
    st = datagen.street(nu=200_000, nf=2000, seed=9, nq=60)
    os_ = O.Oracle.of(st)
    idx2 = engine.Index.of(st, filter="slice")
    got = idx2.query_batch(st.queries, st.ks, "fp64")
    for q, k, r in zip(st.queries, st.ks, got):
        assert np.array_equal(r, os_.query(int(q), int(k))), (int(q), int(k))
    idx.close()
    idx2.close()


def test_autotune_keeps_results(engine, uni):
    """Tuning rebuilds the grids and reshapes the verification; the answers
    stay the same."""
    ds, o = uni
    idx = engine.Index.of(ds, users_per_thread=2, verify_warps=16)
    rng = np.random.default_rng(7)
    qs = rng.integers(0, ds.nf, 300).astype(np.int32)
    ks = rng.integers(1, 40, 300).astype(np.int32)
    before = idx.query_batch(qs, ks, "fp32")
    r = idx.tune(qs, ks, "fp32")
    assert r["trials"] == 34 and r["best_ms"] <= r["default_ms"]
    assert r["users_per_thread"] in (2, 4, 8) and r["verify_warps"] in (4, 8, 16)
    after = idx.query_batch(qs, ks, "fp32")
    after64 = idx.query_batch(qs[:50], ks[:50], "fp64")
    for i in range(300):
        assert np.array_equal(before[i], after[i]), i
    for i in range(0, 50, 5):
        want = o.query(int(qs[i]), int(ks[i]))
        assert np.array_equal(after[i], want) and np.array_equal(after64[i], want), i
    idx.close()
