"""Oracle fixtures for every query of the benchmark workloads.

The query lists (which facility, which k) are defined here once and shared
by the fixture generator, the GPU parity tests and the benchmark's
correctness check.  A fixture stores, per query, the result size and a
64-bit digest of the sorted result ids (the first 8 bytes of SHA-256 over
the ids as little-endian int32), computed by the exact CPU oracle
(oracle/rknn_oracle.c, orc_query_many: rknn-naive's predicate,
rknn-naive/rknn.cpp:169-198, with the strict-< tie rule).  Beside them it
stores a SHA-256 of the generated input points, so that a machine whose
random generator would produce other points notices before comparing.

    python tests/golden/config_fixtures.py [names...]     # (re)generate

Sets (workload sizes as the benchmark configurations name them):
  config1   1k facilities / 10k users uniform, its 10 queries at k=5
  config2   100k / 1M uniform: its 1000 queries at k = 1, 5, 25, and the
            benchmark's 32 query sets of 1000 at k=10 (set 0 = the workload's
            own 1000 queries)
  config3   200k / 4M Gaussian mixture with forced ties, 2000 queries, k=10
  config4   20k / 2M street layout, 16384 queries, k log-uniform in [1,100]
  config5   1M / 10M uniform, 2000 requests, k log-uniform in [1,64]
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for sub in ("rt-rknn_gb300", "oracle"):
    p = os.path.join(REPO, sub)
    if p not in sys.path:
        sys.path.insert(0, p)

import datagen  # noqa: E402

NAMES = ("config1", "config2", "config3", "config4", "config5")
BENCH_SETS = 32          # query sets of the benchmark (config 2, k=10)
BENCH_NQ = 1000


def data_sha256(ds) -> str:
    h = hashlib.sha256()
    for a in (ds.fxy, ds.uxy, ds.fid, ds.uid):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def ids_digest(ids) -> int:
    """64-bit digest of a sorted id list."""
    b = np.ascontiguousarray(ids, dtype="<i4").tobytes()
    return int.from_bytes(hashlib.sha256(b).digest()[:8], "little")


def digests(flat_ids, offsets):
    """(counts, digests) of every slot of a flat result list."""
    off = np.asarray(offsets, np.int64)
    ids = np.asarray(flat_ids)
    n = off.shape[0] - 1
    cnt = np.diff(off)
    dig = np.fromiter((ids_digest(ids[off[i]:off[i + 1]]) for i in range(n)), np.uint64, n)
    return cnt, dig


def bench_query_sets(ds, nsets: int = BENCH_SETS, nq: int = BENCH_NQ):
    """The benchmark's query sets on the config-2 workload: set 0 is the
    workload's own queries, the others are seeded draws without
    replacement."""
    rng = np.random.default_rng(17)
    sets = [np.asarray(ds.queries[:nq], np.int32)]
    while len(sets) < nsets:
        sets.append(rng.choice(ds.nf, size=nq, replace=False).astype(np.int32))
    return sets


def bench_set_rows(s: int, nq: int = BENCH_NQ) -> slice:
    """Rows of the config2 fixture that hold benchmark query set s."""
    base = 3 * nq
    return slice(base + s * nq, base + (s + 1) * nq)


def config5_requests(ds, n: int = 2000):
    rng = np.random.default_rng(4)
    qs = rng.integers(0, ds.nf, n).astype(np.int32)
    ks = np.floor(np.exp(rng.uniform(0, np.log(65), n))).clip(1, 64).astype(np.int32)
    return qs, ks


def spec(name: str):
    """(dataset, query facility indices, k per query) of a fixture set."""
    n = int(name[-1])
    ds = datagen.config(n)
    if n == 1:
        return ds, np.asarray(ds.queries, np.int32), np.full(len(ds.queries), 5, np.int32)
    if n == 2:
        qs, ks = [], []
        for k in (1, 5, 25):
            qs.append(np.asarray(ds.queries, np.int32))
            ks.append(np.full(len(ds.queries), k, np.int32))
        for s in bench_query_sets(ds):
            qs.append(s)
            ks.append(np.full(len(s), 10, np.int32))
        return ds, np.concatenate(qs), np.concatenate(ks)
    if n in (3, 4):
        return ds, np.asarray(ds.queries, np.int32), np.asarray(ds.ks, np.int32)
    if n == 5:
        qs, ks = config5_requests(ds)
        return ds, qs, ks
    raise ValueError(name)


def path(name: str) -> str:
    return os.path.join(HERE, f"oracle_{name}.npz")


def load(name: str) -> dict:
    z = np.load(path(name))
    return {"qs": z["qs"], "ks": z["ks"], "count": z["count"], "digest": z["digest"],
            "data_sha256": str(z["data_sha256"])}


def generate(name: str) -> dict:
    import oracle as O
    ds, qs, ks = spec(name)
    t0 = time.time()
    o = O.Oracle.of(ds)
    off, ids = o.query_many(qs, ks)
    cnt, dig = digests(ids, off)
    np.savez_compressed(path(name), qs=qs.astype(np.int32), ks=ks.astype(np.int32),
                        count=cnt.astype(np.int64), digest=dig, data_sha256=np.array(data_sha256(ds)))
    return {"name": name, "queries": int(qs.shape[0]), "ids": int(ids.shape[0]),
            "seconds": round(time.time() - t0, 1)}


def check(name: str, qs, ks, flat_ids, offsets, fx: dict | None = None):
    """Indices of the queries whose results differ from the fixture (qs and
    ks must be the fixture's, in its order)."""
    fx = fx or load(name)
    assert np.array_equal(np.asarray(qs, np.int32), fx["qs"]) and np.array_equal(np.asarray(ks, np.int32), fx["ks"])
    cnt, dig = digests(flat_ids, offsets)
    return np.nonzero((cnt != fx["count"]) | (dig != fx["digest"]))[0]


if __name__ == "__main__":
    for nm in (sys.argv[1:] or NAMES):
        print(generate(nm), flush=True)
