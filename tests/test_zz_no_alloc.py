"""rknn_query_noalloc: the allocation-free single query.

Callers that cannot allocate device memory while they query (a plugin whose
host process keeps all device memory for its own allocator, a latency-bound
serving loop that must not stall on cudaMalloc) get one entry point whose per-query scratch sits
in a fixed device array.  Its answers must equal rknn_query's, call after
call (the array keeps the previous call's contents, so consecutive calls
check that everything that must start from zero is cleared).

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

import datagen

pytestmark = pytest.mark.gpu


def test_noalloc_matches_rknn_query_twice(engine):
    ds = datagen.uniform(5000, 50000, seed=41, nq=12, k=10)
    idx = engine.Index.of(ds)
    for mode in ("fp64", "fp32"):
        for i, q in enumerate(ds.queries):
            k = [1, 5, 10, 25][i % 4]
            want = idx.query(int(q), k, mode)
            first = idx.query_noalloc(int(q), k, mode)
            second = idx.query_noalloc(int(q), k, mode)
            assert np.array_equal(first, want), (q, k, mode)
            assert np.array_equal(second, want), (q, k, mode)
    # different queries back to back: no state carried over
    a = idx.query_noalloc(int(ds.queries[0]), 10, "fp32")
    b = idx.query_noalloc(int(ds.queries[1]), 3, "fp32")
    assert np.array_equal(a, idx.query(int(ds.queries[0]), 10, "fp32"))
    assert np.array_equal(b, idx.query(int(ds.queries[1]), 3, "fp32"))


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
