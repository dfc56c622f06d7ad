"""The five benchmark workloads of the engine, one JSON line each.

    python rt-rknn_gb300/workloads.py [--configs 1,2,3,4,5] [--out FILE]

  1  1,000 facilities / 10,000 users uniform, k=5, 10 queries
  2  100,000 / 1,000,000 uniform, k in {1,5,10,25}, 1,000 queries: the plain
     form (one query per launch, FP64 predicates, influence zone) and the
     chosen form (one batch, FP32-filtered predicates, default filter)
  3  200,000 / 4,000,000 Gaussian mixture with 1% bisector ties and 0.1%
     duplicates, k=10, 2,000 queries: FP32 and FP64 batches, recheck fraction,
     FP32 == FP64 on every query
  4  20,000 / 2,000,000 street layout, 16,384 queries with k log-uniform in
     [1,100], one batch
  5  1,000,000 / 10,000,000 uniform resident, Poisson arrivals at 1k-100k
     requests/s with k log-uniform in [1,64] through the serving loop: p50/p99
     latency and throughput for FP32 and FP64

Device times come from the engine's own CUDA events (rknn_query_stats
.device_ms); every batch is run once untimed first.  Parity with the exact
oracle is checked by tests/test_configs.py, not here.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import build  # noqa: E402
import datagen  # noqa: E402
import rknn  # noqa: E402


def _batch(idx, qs, ks, mode, reps=3):
    idx.query_batch_flat(qs, ks, mode)
    ms = []
    st = None
    for _ in range(reps):
        res, st = idx.query_batch(qs, ks, mode, stats=True)
        ms.append(st["device_ms"])
    return float(np.median(ms)), st, res


def config1():
    ds = datagen.config(1)
    with rknn.Index.of(ds) as idx:
        ms, st, _ = _batch(idx, ds.queries, ds.ks, "fp32")
        t = []
        for q in ds.queries:
            t0 = time.perf_counter()
            idx.query(int(q), 5, "fp64")
            t.append(time.perf_counter() - t0)
    return {"config": 1, "fp32_batch_ms": ms, "fp64_single_ms_median": 1e3 * float(np.median(t)),
            "results": st["results"]}


def config2():
    ds = datagen.config(2)
    out = {"config": 2, "k": {}}
    qs = ds.queries.astype(np.int32)
    with rknn.Index.of(ds) as idx, rknn.Index.of(ds, filter="inf") as inf:
        for k in (1, 5, 10, 25):
            ms, st, res = _batch(idx, qs, k, "fp32")
            ms_inf, _, res_inf = _batch(inf, qs, k, "fp32")
            same = all(np.array_equal(a, b) for a, b in zip(res, res_inf))
            lat = []
            for q in qs[:100]:
                t0 = time.perf_counter()
                inf.query(int(q), k, "fp64")
                lat.append(1e3 * (time.perf_counter() - t0))
            lat.sort()
            out["k"][k] = {"fp32_batched_qps": len(qs) / (ms / 1e3), "inf_zone_fp32_batched_qps": len(qs) / (ms_inf / 1e3),
                           "fp64_single_qps": 1e3 / float(np.mean(lat)), "fp64_single_p50_ms": lat[len(lat) // 2],
                           "fp64_single_p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                           "filters_agree": same, "results_per_query": st["results"] / len(qs),
                           "candidates_per_query": st["candidates"] / len(qs)}
    return out


def config3():
    ds = datagen.config(3)
    qs = ds.queries.astype(np.int32)
    with rknn.Index.of(ds) as idx:
        ms32, st32, r32 = _batch(idx, qs, 10, "fp32", reps=2)
        ms64, st64, r64 = _batch(idx, qs, 10, "fp64", reps=2)
    same = sum(np.array_equal(a, b) for a, b in zip(r32, r64))
    return {"config": 3, "fp32_batched_qps": len(qs) / (ms32 / 1e3), "fp64_batched_qps": len(qs) / (ms64 / 1e3),
            "recheck_fraction_fp32": st32["rechecks"] / max(1, st32["fac_checks"]),
            "recheck_fraction_fp64": st64["rechecks"] / max(1, st64["fac_checks"]),
            "rechecks_fp32": st32["rechecks"], "rechecks_fp64": st64["rechecks"],
            "fp32_equals_fp64_queries": int(same), "queries": len(qs), "results": st32["results"]}


def config4():
    """One batch of the 16,384 mixed-k queries, both modes, then the
    autotuner on that batch (FP32): the default and best device times, the
    chosen grid densities, users per lane and warps per block, and both
    modes again with the chosen settings."""
    ds = datagen.config(4)
    qs, ks = ds.queries.astype(np.int32), ds.ks.astype(np.int32)
    out = {"config": 4, "queries": len(qs)}
    with rknn.Index.of(ds) as idx:
        for mode in ("fp32", "fp64"):
            ms, st, _ = _batch(idx, qs, ks, mode, reps=2)
            out[mode] = {"device_ms": ms, "qps": len(qs) / (ms / 1e3), "results": st["results"],
                         "candidates": st["candidates"], "survivors": st["survivors"]}
        out["tune"] = idx.tune(qs, ks, "fp32")
        for mode in ("fp32", "fp64"):
            ms, st, _ = _batch(idx, qs, ks, mode, reps=2)
            out[mode + "_tuned"] = {"device_ms": ms, "qps": len(qs) / (ms / 1e3)}
    return out


def config5():
    ds = datagen.config(5)
    rng = np.random.default_rng(55)
    out = {"config": 5, "rates": {}}
    with rknn.Index.of(ds) as idx, rknn.Server(idx, slots=3, max_batch=4096) as srv:
        for rate in (1_000, 10_000, 50_000, 100_000):
            n = int(min(200_000, max(2_000, rate * 2)))
            qs = rng.integers(0, ds.nf, n).astype(np.int32)
            ks = (np.floor(np.exp(rng.uniform(0, np.log(65), n)))).clip(1, 64).astype(np.int32)
            arr = np.cumsum(rng.exponential(1.0 / rate, n))
            row = {}
            for mode in ("fp32", "fp64"):
                srv.replay(qs[:1000], ks[:1000], mode, arr[:1000])
                srv.stats(reset=True)
                lat, _ = srv.replay(qs, ks, mode, arr)
                st = srv.stats(reset=True)
                row[mode] = {"p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "throughput_qps": st["throughput_qps"],
                             "mean_batch": st["mean_batch"], "requests": n}
            out["rates"][rate] = row
    return out


def order_ab():
    """Batch device time with the work queue ordered by k alone against
    ordered by the candidate estimate within each k class (RKNN_ORDER=est at
    index creation), on workloads 2 (k=10 and mixed k), 3 and 4, FP32 and
    FP64; the result sets must not change."""
    out = {"order_ab": {}}
    rng = np.random.default_rng(8)
    cases = []
    ds2 = datagen.config(2)
    cases.append(("config2_k10", ds2, ds2.queries.astype(np.int32), np.full(len(ds2.queries), 10, np.int32)))
    cases.append(("config2_mixed", ds2, ds2.queries.astype(np.int32),
                  np.floor(np.exp(rng.uniform(0, np.log(65), len(ds2.queries)))).clip(1, 64).astype(np.int32)))
    ds3 = datagen.config(3)
    cases.append(("config3", ds3, ds3.queries.astype(np.int32), ds3.ks.astype(np.int32)))
    ds4 = datagen.config(4)
    cases.append(("config4", ds4, ds4.queries.astype(np.int32), ds4.ks.astype(np.int32)))
    for name, ds, qs, ks in cases:
        row = {}
        res = {}
        for order in ("k", "est"):
            os.environ["RKNN_ORDER"] = order
            with rknn.Index.of(ds) as idx:
                for mode in ("fp32", "fp64"):
                    ms, _, r = _batch(idx, qs, ks, mode, reps=3)
                    row[f"{mode}_{order}_ms"] = ms
                    res[(order, mode)] = r
        os.environ.pop("RKNN_ORDER", None)
        row["same_results"] = all(all(np.array_equal(a, b) for a, b in zip(res[("k", m)], res[("est", m)]))
                                  for m in ("fp32", "fp64"))
        out["order_ab"][name] = row
    return out


def profile_verify(upt: int, warps: int, nq: int = 16384):
    """One batch of nq workload-2 queries at k=10 in FP32 (too many for the
    fused verification: the separate verification kernel runs) with the
    verification's users per lane and warps per block given, run twice (the
    second launch is the one to capture), then its per-kernel device times
    in profiling mode and its statistics."""
    ds = datagen.config(2)
    qs = np.random.default_rng(99).choice(ds.nf, size=nq, replace=False).astype(np.int32)
    with rknn.Index.of(ds, users_per_thread=upt, verify_warps=warps) as idx:
        idx.query_batch_flat(qs, 10, "fp32")
        idx.query_batch_flat(qs, 10, "fp32")
        idx.set_profiling(True)
        ms = []
        for _ in range(3):
            idx.query_batch_flat(qs, 10, "fp32")
            ms.append(idx.kernel_ms())
        st = idx.last_stats()
    kms = {n: float(np.median([m[n] for m in ms])) for n in ms[0]}
    print(json.dumps({"upt": upt, "warps": warps, "queries": nq, "kernel_ms": kms,
                      "plane_evals": st["plane_evals"], "candidates": st["candidates"],
                      "bisectors": st["bisectors"], "survivors": st["survivors"]}), flush=True)


def vertex_test_ab():
    """The influence zone with rknn-inf's vertex test against the
    zone-boundary test (rknn_index_opts.zone_vertex_test): bisectors,
    candidate users and survivors per query, batch device time, and the
    single-query latency, on workload 2 at k = 5, 10, 25; the result sets
    must be the same."""
    ds = datagen.config(2)
    qs = ds.queries.astype(np.int32)
    out = {"vertex_test_ab": {}}
    for k in (5, 10, 25):
        row, res = {}, {}
        for vt in ("reference", "boundary"):
            with rknn.Index.of(ds, filter="inf", zone_vertex_test=vt) as idx:
                ms, st, r = _batch(idx, qs, k, "fp64", reps=2)
                res[vt] = r
                lat = []
                for q in qs[:60]:
                    t0 = time.perf_counter()
                    idx.query(int(q), k, "fp64")
                    lat.append(1e3 * (time.perf_counter() - t0))
                n = len(qs)
                row[vt] = {"bisectors_per_query": st["bisectors"] / n, "candidates_per_query": st["candidates"] / n,
                           "survivors_per_query": st["survivors"] / n, "batch_fp64_ms": ms,
                           "single_p50_ms": float(np.median(lat))}
        row["same_results"] = all(np.array_equal(a, b) for a, b in zip(res["reference"], res["boundary"]))
        out["vertex_test_ab"][k] = row
    return out


def profile_single(k: int, n: int):
    """n single FP64 queries through the influence zone on the config-2
    workload (the plain form; the launch to capture with ncu is the last)."""
    ds = datagen.config(2)
    with rknn.Index.of(ds, filter="inf") as idx:
        for q in ds.queries[:n]:
            print(int(q), len(idx.query(int(q), k, "fp64")))


def explain(c: int):
    """Where one FP32 batch of workload c (2, 3 or 4; its own queries and k)
    spends its time: per-kernel device ms (profiling mode, events between
    the kernels), the filter's phase cycles per query (warp 0 of each
    query: ring walk, of it the facility offers; the slice bound; the
    half-planes and user segments; the fused verification), and the work
    per query."""
    ds = datagen.config(c)
    qs = ds.queries.astype(np.int32)
    ks = ds.ks.astype(np.int32) if c == 4 else np.full(len(qs), 10, np.int32)
    nq = len(qs)
    with rknn.Index.of(ds) as idx:
        for _ in range(2):
            idx.query_batch_flat(qs, ks, "fp32")
        ms, st, _ = _batch(idx, qs, ks, "fp32", reps=3)
        idx.set_profiling(True)
        km = []
        for _ in range(3):
            idx.query_batch(qs, ks, "fp32")
            km.append(idx.kernel_ms())
        idx.set_profiling(False)
    cyc = np.array(st["zone_cycles"], float) / nq
    out = {"config": c, "queries": nq, "device_ms": ms, "qps": nq / (ms / 1e3),
           "kernel_ms": {k: float(np.median([m[k] for m in km])) for k in km[0]},
           "filter_cycles_per_query": {"ring_walk": cyc[0], "of_it_offers": cyc[1], "slice_bound": cyc[2],
                                       "half_planes_and_segments": cyc[7], "fused_verification": cyc[6]},
           "per_query": {k: st[k] / nq for k in ("bisectors", "candidates", "plane_evals", "survivors",
                                                   "fac_checks", "rechecks", "results")},
           "fused_queries": st.get("fused_slots")}
    print(json.dumps(out), flush=True)
    return out


def profile_index(c: int):
    """Only the index build of workload c (the grid build kernels)."""
    ds = datagen.config(c)
    with rknn.Index.of(ds) as idx:
        print(idx.info())


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", default="1,2,3,4,5")
    ap.add_argument("--out", default=None)
    ap.add_argument("--profile-single", nargs=2, type=int, metavar=("K", "N"),
                    help="only N single FP64 influence-zone queries at k=K on workload 2")
    ap.add_argument("--profile-index", type=int, metavar="C", help="only the index build of workload C")
    ap.add_argument("--explain", type=int, metavar="C", help="only the time split of one batch of workload C")
    ap.add_argument("--order-ab", action="store_true", help="only the work-order comparison")
    ap.add_argument("--vertex-test-ab", action="store_true", help="only the zone vertex-test comparison")
    ap.add_argument("--profile-verify", nargs=2, type=int, metavar=("UPT", "WARPS"),
                    help="only a 16384-query workload-2 batch with this verification shape")
    a = ap.parse_args(argv)
    build.build()
    if a.profile_verify:
        profile_verify(*a.profile_verify)
        return 0
    if a.vertex_test_ab:
        print(json.dumps(vertex_test_ab()), flush=True)
        return 0
    if a.order_ab:
        print(json.dumps(order_ab()), flush=True)
        return 0
    if a.explain:
        explain(a.explain)
        return 0
    if a.profile_single:
        profile_single(*a.profile_single)
        return 0
    if a.profile_index:
        profile_index(a.profile_index)
        return 0
    fns = {1: config1, 2: config2, 3: config3, 4: config4, 5: config5}
    fh = open(a.out, "w") if a.out else None
    for c in (int(x) for x in a.configs.split(",")):
        t0 = time.perf_counter()
        r = fns[c]()
        r["wall_s"] = time.perf_counter() - t0
        line = json.dumps(r)
        print(line, flush=True)
        if fh:
            fh.write(line + "\n")
            fh.flush()
    return 0


if __name__ == "__main__":
    sys.exit(main())
