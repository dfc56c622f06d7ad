"""The benchmark workloads at full size, every query checked against the
exact oracle's fixtures (tests/golden/oracle_config*.npz: per query the
result size and a digest of the sorted ids, made by
tests/golden/config_fixtures.py from oracle/rknn_oracle.c).  Results are
integer id sets: equality is bit-exact, in both precision modes and on every
path (batched with either filter, one query per launch, the serving loop).

Where this machine's random generator would give other input points than the
fixture's (its data digest differs), the oracle is run here on the same query
list instead; the comparison is the same."""
import os
import sys

import numpy as np
import pytest

import oracle as O

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import config_fixtures as CF  # noqa: E402

pytestmark = pytest.mark.gpu

MODES = ("fp32", "fp64")


def fixture(name):
    ds, qs, ks = CF.spec(name)
    fx = CF.load(name)
    assert np.array_equal(fx["qs"], qs) and np.array_equal(fx["ks"], ks), name
    if CF.data_sha256(ds) != fx["data_sha256"]:
        print(f"{name}: generated points differ from the fixture's; running the oracle here")
        off, ids = O.Oracle.of(ds).query_many(qs, ks)
        fx["count"], fx["digest"] = CF.digests(ids, off)
    return ds, qs, ks, fx


def assert_batch(name, idx, qs, ks, mode, fx):
    ids, off = idx.query_batch_flat(qs, ks, mode)
    bad = CF.check(name, qs, ks, ids, off, fx)
    assert bad.size == 0, (name, mode, bad.size, [(int(qs[i]), int(ks[i])) for i in bad[:8]])


def assert_each(name, results, fx, sel):
    cnt = np.array([r.shape[0] for r in results])
    dig = np.array([CF.ids_digest(r) for r in results], np.uint64)
    bad = np.nonzero((cnt != fx["count"][sel]) | (dig != fx["digest"][sel]))[0]
    assert bad.size == 0, (name, bad.size, bad[:8])


def test_config1_every_query(engine):
    ds, qs, ks, fx = fixture("config1")
    with engine.Index.of(ds) as idx:
        for mode in MODES:
            assert_batch("config1", idx, qs, ks, mode, fx)
            assert_each("config1", [idx.query(int(q), int(k), mode) for q, k in zip(qs, ks)], fx,
                        np.arange(qs.shape[0]))


def test_config2_every_query_every_k(engine):
    """100k / 1M uniform: the 1000 queries at k = 1, 5, 25 and the
    benchmark's 32,000 queries at k = 10, batched (both filters, both modes),
    and the plain form (one FP64 query per launch through the influence
    zone) on the 1000 queries at every k."""
    ds, qs, ks, fx = fixture("config2")
    with engine.Index.of(ds) as idx:
        for mode in MODES:
            assert_batch("config2", idx, qs, ks, mode, fx)
    with engine.Index.of(ds, filter="inf") as idx:
        for mode in MODES:
            assert_batch("config2", idx, qs, ks, mode, fx)
        nq = ds.queries.shape[0]
        # the 1000 queries at k = 1, 5, 25 and (first benchmark set) k = 10
        for base in (0, nq, 2 * nq, 3 * nq):
            sel = np.arange(base, base + nq)
            assert_each("config2", [idx.query(int(qs[i]), int(ks[i]), "fp64") for i in sel], fx, sel)
        sel = np.arange(3 * nq, 4 * nq)
        assert_each("config2", [idx.query(int(qs[i]), int(ks[i]), "fp32") for i in sel], fx, sel)


def test_config3_precision_ties_and_duplicates(engine):
    """200k / 4M Gaussian mixture, 1% of users exactly on a q-f bisector,
    0.1% duplicated coordinates, k=10: all 2,000 queries equal the oracle in
    both modes, and the forced ties reach the exact predicate."""
    ds, qs, ks, fx = fixture("config3")
    with engine.Index.of(ds) as idx:
        for mode in MODES:
            assert_batch("config3", idx, qs, ks, mode, fx)
            st = idx.last_stats()
            assert st["rechecks"] > 0, mode


def test_config4_mixed_k_batch(engine):
    """20k / 2M street layout, 16,384 queries with k log-uniform in [1,100],
    one batch: every query equals the oracle in both modes."""
    ds, qs, ks, fx = fixture("config4")
    with engine.Index.of(ds) as idx:
        for mode in MODES:
            assert_batch("config4", idx, qs, ks, mode, fx)
            assert idx.last_stats()["overflow"] == 0, mode


def test_config5_serving_at_scale(engine):
    """1M / 10M resident; 2,000 requests with k log-uniform in [1,64]
    through the serving loop (each mode alone, then the two mixed) and as
    batches: every result equals the oracle."""
    ds, qs, ks, fx = fixture("config5")
    sel = np.arange(qs.shape[0])
    with engine.Index.of(ds) as idx:
        with engine.Server(idx, slots=3, max_batch=256) as srv:
            for mode in MODES:
                tickets = [srv.submit(int(q), int(k), mode) for q, k in zip(qs, ks)]
                assert_each("config5", [srv.wait(t) for t in tickets], fx, sel)
            tickets = [srv.submit(int(q), int(k), MODES[i % 3 == 0]) for i, (q, k) in enumerate(zip(qs, ks))]
            assert_each("config5", [srv.wait(t) for t in tickets], fx, sel)
        for mode in MODES:
            assert_batch("config5", idx, qs, ks, mode, fx)
