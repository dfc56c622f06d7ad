"""rknn_query_noalloc: the allocation-free single query.

Callers that cannot allocate device memory while they query (a plugin whose
host process keeps all device memory for its own allocator, a latency-bound
serving loop that must not stall on cudaMalloc) get one entry point whose per-query scratch sits
in a fixed device array.  Its answers must equal rknn_query's and the exact
oracle's, call after call (the array keeps the previous call's contents, so
consecutive calls check that everything that must start from zero is
cleared).

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

import datagen
import oracle as O

pytestmark = pytest.mark.gpu


def test_noalloc_matches_rknn_query_twice(engine):
    ds = datagen.uniform(5000, 50000, seed=41, nq=12, k=10)
    idx = engine.Index.of(ds)
    o = O.Oracle.of(ds)
    kset = [1, 5, 10, 25, 128]
    for mode in ("fp64", "fp32"):
        for i, q in enumerate(ds.queries):
            k = kset[i % len(kset)]
            want = idx.query(int(q), k, mode)
            first = idx.query_noalloc(int(q), k, mode)
            second = idx.query_noalloc(int(q), k, mode)
            assert np.array_equal(first, want), (q, k, mode)
            assert np.array_equal(second, want), (q, k, mode)
            assert np.array_equal(first, o.query(int(q), k)), (q, k, mode)
    # different queries back to back: no state carried over
    a = idx.query_noalloc(int(ds.queries[0]), 10, "fp32")
    b = idx.query_noalloc(int(ds.queries[1]), 3, "fp32")
    assert np.array_equal(a, idx.query(int(ds.queries[0]), 10, "fp32"))
    assert np.array_equal(b, idx.query(int(ds.queries[1]), 3, "fp32"))
    assert np.array_equal(b, o.query(int(ds.queries[1]), 3))


def test_noalloc_rejects_sizes_beyond_its_limit(engine):
    ds = datagen.uniform(300, 2000, seed=42, nq=2, k=3)
    idx = engine.Index.of(ds)
    with pytest.raises(engine.RkNNError) as e:
        idx.query_noalloc(int(ds.queries[0]), 129)
    assert e.value.status == 5
    with pytest.raises(engine.RkNNError) as e:
        idx.query_noalloc(ds.nf, 3)
    assert e.value.status == 1
    # still usable afterwards
    assert np.array_equal(idx.query_noalloc(int(ds.queries[0]), 3),
                          idx.query(int(ds.queries[0]), 3))


def test_noalloc_rejects_results_beyond_the_fixed_array(engine):
    """One facility and 2.1 million users: every user is in the answer, more
    ids than the fixed array holds (about 2 million).  The call fails with
    RKNN_ERR_CAPACITY instead of writing past its scratch; rknn_query, which
    allocates, returns them all; the next no-alloc call is correct again."""
    rng = np.random.default_rng(43)
    nu = 2_100_000
    ds = datagen.Dataset(np.array([[500.0, 500.0]], np.float32),
                         rng.uniform(0, 1000, (nu, 2)).astype(np.float32),
                         np.zeros(1, np.int32), np.arange(1, nu + 1, dtype=np.int32))
    idx = engine.Index.of(ds)
    with pytest.raises(engine.RkNNError) as e:
        idx.query_noalloc(0, 1)
    assert e.value.status == 5
    full = idx.query(0, 1)
    assert full.shape[0] == nu and np.array_equal(full, ds.uid)
    idx.close()
    small = datagen.uniform(1000, 10000, seed=44, nq=3, k=5)
    idx = engine.Index.of(small)
    o = O.Oracle.of(small)
    for q in small.queries:
        assert np.array_equal(idx.query_noalloc(int(q), 5), o.query(int(q), 5))
    idx.close()
