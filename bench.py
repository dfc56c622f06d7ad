"""Benchmark: batched RkNN queries on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the reference's headline configuration): 100,000 facilities and
1,000,000 users, float32 uniform in [0,1000]^2 (seeded synthetic data), k=10.
One step = one batch of 1,000 random facility queries through the engine:
angular-slice filter, which at this batch size also verifies each query's
users itself (fused) -> verification of left-over queries -> exact recount
of the survivors -> finalize, which also writes the result offsets (one
CUDA graph), FP32-filtered predicates with exact fallback.  Step i answers
query set i mod 32 of a seeded pool; every step's results (device-timed and
end-to-end) are checked against the exact oracle's fixture of that pool
(tests/golden/oracle_config2.npz) outside the timed intervals.
Prints one JSON line (rank 0).

  value      queries/s with the facility/user index and the query batch
             resident in HBM, device time from CUDA events on the engine's
             stream, L2 flushed (256 MB write) before every timed step
  e2e        queries/s through rknn_query_batch (the C ABI with host
             buffers; ids land in a page-locked buffer): query ids H2D,
             result offsets and ids D2H, per step, L2 flushed (untimed)
             before every step
  mismatches_vs_oracle  queries of the timed and end-to-end steps whose ids
             differ from the oracle's
  roofline   the dominant kernel (the filter with its fused verification),
             timed live per launch with CUDA events in profiling mode,
             against HBM and against peak instruction issue;
             roofline_other: the verification and recount kernels;
             roofline_saturated: both kernels on the same workload as one
             batch of 16384 queries (GPU full), against peak instruction
             issue (their bound there), HBM and FP32
  fp64_single_query  the plain form: one query per launch, FP64 predicates,
             rknn-inf's influence zone (the drop-in); p50/p99 latency
  serving    open-loop Poisson arrivals through the continuous batcher, on
             this workload and on the resident 1M-facility / 10M-user index
             (k log-uniform in [1,64], 1k-100k requests/s)
  cpu_baseline  the reference's own rknn-inf binary (built from its sources
             into oracle/_ref) on the host's cores, one query per process as
             the binary answers them, over a bounded sample of the same
             workload; without the binary, the C restatement of its query
             path (oracle/inf_port.c)

--impl reference times the reference's own CPU implementation alone (the
rknn-inf binary, one process per host core, each answering one query of the
step; the C restatement where the binary was not built) on the same workload
and prints the same JSON line with "impl": "reference", beside the
reference's other binaries on this host: rknn-naive at 1k/10k, and its two
CUDA binaries, rknn-inf-gpu at this workload and rknn-naive-gpu at 1k/10k.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "rt-rknn_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests", "golden"))

METRIC = "RkNN queries/s (1M users,100k fac,k=10) FP32-filtered vs FP64; p99 ms"
NF, NU, K, NQ = 100_000, 1_000_000, 10, 1000
WORKLOAD = "uniform 100k facilities / 1M users, k=10, 1000 queries per step"

# DRAM bytes (read + write) per launch of the slice filter with the fused
# verification on this workload's 1000-query batch, from one ncu capture of
# that launch (the capture's commit is recorded with its summary)
TRAFFIC = {"fused_slice_kernel": 4883968}
# warp instructions per query of that kernel (two warps a query), same capture
FUSED_INSTR_PER_QUERY = 21.4742e6 / 1000
# warp instructions per unit of work of the two kernels in a batch of SAT_NQ
# queries of this workload, from one ncu capture (smsp__inst_executed.sum of
# the launch over its queries or its half-plane evaluations)
SAT_NQ = 16384
INSTR = {"slice_kernel_per_query": 160.539e6 / 16384, "verify_kernel_per_eval": 95.848e6 / 176643960}


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.p:
            time.sleep(0.25)
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dataset():
    import datagen
    return datagen.config(2)


def query_pool(ds, nq):
    """Step i answers pool[i % len(pool)]; the 1000-query pool is the one the
    oracle fixture covers."""
    import config_fixtures as CF
    if nq == CF.BENCH_NQ:
        return CF.bench_query_sets(ds), True
    rng = np.random.default_rng(17)
    return [rng.choice(ds.nf, size=nq, replace=nq > ds.nf).astype(np.int32) for _ in range(8)], False


class OracleCheck:
    """Counts queries whose ids differ from the oracle fixture's (per query
    size and digest of the sorted ids)."""

    def __init__(self, ds):
        import config_fixtures as CF
        self.CF = CF
        fx = CF.load("config2")
        self.ok = CF.data_sha256(ds) == fx["data_sha256"]
        self.fx = fx
        self.checked = 0
        self.mismatches = 0

    def add(self, set_index, ids, offsets):
        if not self.ok:
            return
        rows = self.CF.bench_set_rows(set_index % self.CF.BENCH_SETS)
        cnt, dig = self.CF.digests(ids, offsets)
        bad = (cnt != self.fx["count"][rows]) | (dig != self.fx["digest"][rows])
        self.checked += int(cnt.shape[0])
        self.mismatches += int(bad.sum())

    def add_one(self, set_index, slot, ids):
        if not self.ok:
            return
        row = self.CF.bench_set_rows(set_index % self.CF.BENCH_SETS).start + slot
        self.checked += 1
        self.mismatches += int(ids.shape[0] != self.fx["count"][row]
                               or self.CF.ids_digest(ids) != int(self.fx["digest"][row]))


class _CudaArray:
    """A device int32 array as __cuda_array_interface__ (read by torch)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<i4", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def device_results_to_host(idx, nq, device):
    """The last device batch's (ids, offsets), copied to the host."""
    import torch
    ids_p, off_p = idx.device_results()          # synchronizes the index's stream
    off = torch.as_tensor(_CudaArray(off_p, nq + 1), device=device).cpu().numpy().astype(np.int64)
    n = int(off[-1])
    ids = torch.as_tensor(_CudaArray(ids_p, max(n, 1)), device=device)[:n].cpu().numpy()
    return ids, off


# ---------------------------------------------------------------- reference
REF_DIR = os.path.join(REPO, "oracle", "_ref")
_NUM = r"([-+0-9.eE]+)"


def ref_binary(name):
    """Path of a reference binary built for this host, or None."""
    p = os.path.join(REF_DIR, name)
    if not (os.path.isfile(p) and os.access(p, os.X_OK)):
        return None
    try:
        subprocess.run([p, "-h"], capture_output=True, timeout=20)
    except (OSError, subprocess.TimeoutExpired):
        return None                               # not runnable here (other architecture)
    return p


def parse_ref(out: str) -> dict:
    r = {}
    for key, pat in (("total_s", r"Total time: " + _NUM), ("build_s", r"R\*-tree is built in " + _NUM),
                     ("search_s", r"completed in " + _NUM), ("filter_s", r"Filtering time: " + _NUM),
                     ("verify_s", r"Verification time(?: \(\w+\))?: " + _NUM), ("found", r"Found (\d+) RkNN")):
        m = re.search(pat, out)
        if m:
            r[key] = float(m.group(1))
    return r


def run_ref_procs(binary, path, qs, k, parallel, extra=()):
    """Runs binary once per query (qs), at most `parallel` processes at a
    time; returns the parsed outputs with each process's wall time."""
    out, pending = [], list(qs)
    running = []
    while pending or running:
        while pending and len(running) < parallel:
            q = pending.pop(0)
            p = subprocess.Popen([binary, "-if", path, "-k", str(k), "-q", str(int(q)), *extra],
                                 stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                                 errors="replace")
            running.append((q, p, time.perf_counter()))
        q, p, t0 = running.pop(0)
        so, se = p.communicate()
        r = parse_ref(so)
        r.update(q=int(q), rc=p.returncode, wall_s=time.perf_counter() - t0)
        if p.returncode != 0 or "total_s" not in r and "search_s" not in r:
            r["error"] = (se or so)[-300:]
        out.append(r)
    return out


def cpu_port_run(ds, nq_sample, nthreads, seed=5):
    """Time the rknn-inf restatement (oracle/inf_port.c) over nq_sample
    queries at k=10 on nthreads host threads.  Returns (q/s, seconds)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    port = O.InfPort(ds.fxy, ds.uxy)
    rng = np.random.default_rng(seed)
    qs = rng.choice(ds.nf, size=nq_sample, replace=nq_sample > ds.nf).astype(np.int64)
    t0 = time.perf_counter()
    cnt = port.query_many(qs, K, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return nq_sample / dt, dt, int(cnt.sum())


def write_workload_text(ds, tmp, name="config2.txt", integer=False):
    import datagen
    p = os.path.join(tmp, name)
    datagen.write_text(p, ds, integer=integer)
    return p


def ref_inf_sample(ds, path, nproc, seed):
    """One bounded sample of the reference's rknn-inf: nproc processes at
    once, one random query each.  Returns the processes' results."""
    rng = np.random.default_rng(seed)
    qs = rng.choice(ds.nf, size=nproc, replace=False)
    res = run_ref_procs(ref_binary("rknn-inf"), path, qs, K, nproc)
    bad = [r for r in res if "error" in r]
    if bad:
        raise RuntimeError(f"rknn-inf failed: {bad[0]['error']}")
    return res


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replicas_throughput(dev_s: float, ws: int, units: int, device: str = "cpu") -> float:
    """Whole-job throughput of ws replicas: the units all ranks processed over
    the slowest rank's time (max over ranks; one all-reduce, no data-path
    collective)."""
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([dev_s], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s = float(t.item())
    return ws * units / dev_s


def reference_suite(ds, tmp, path2, nproc):
    """The reference's other binaries on this host, beside the timed arm:
    rknn-naive at 1k/10k (integer twin: it reads integer coordinates), and
    its CUDA binaries rknn-inf-gpu (this workload) and rknn-naive-gpu
    (1k/10k integer twin; its |U|x|F| matrix does not fit at this workload)."""
    import datagen
    out = {}
    c1 = datagen.uniform(1000, 10000, seed=1, nq=10, k=5, integer=True)
    p1 = write_workload_text(c1, tmp, "config1_int.txt", integer=True)
    nb = ref_binary("rknn-naive")
    if nb:
        res = run_ref_procs(nb, p1, c1.queries, 5, nproc)
        ok = [r["search_s"] for r in res if "search_s" in r]
        out["rknn_naive_1k10k_int_k5"] = {"queries": len(ok), "mean_s_per_query": statistics.mean(ok),
                                         "queries_per_s_1core": 1.0 / statistics.mean(ok),
                                         "processes_at_once": nproc}
    g = ref_binary("rknn-naive-gpu")
    if g:
        res = run_ref_procs(g, p1, c1.queries[:5], 5, 1, extra=("--gpu",))
        ok = [r["search_s"] for r in res if "search_s" in r]
        out["rknn_naive_gpu_1k10k_int_k5"] = {"queries": len(ok), "errors": len(res) - len(ok),
                                             "mean_s_per_query": statistics.mean(ok) if ok else None,
                                             "queries_per_s": 1.0 / statistics.mean(ok) if ok else None}
    g = ref_binary("rknn-inf-gpu")
    if g:
        rng = np.random.default_rng(77)
        res = run_ref_procs(g, path2, rng.choice(ds.nf, 4, replace=False), K, 2)
        ok = [r for r in res if "total_s" in r]
        out["rknn_inf_gpu_100k1M_k10"] = {
            "queries": len(ok), "errors": len(res) - len(ok),
            "mean_total_s": statistics.mean(r["total_s"] for r in ok) if ok else None,
            "mean_verify_s": statistics.mean(r.get("verify_s", 0.0) for r in ok) if ok else None,
            "queries_per_s": 1.0 / statistics.mean(r["total_s"] for r in ok) if ok else None,
            "note": "filter on the CPU, verification of all users on the GPU per query (cudaMalloc, "
                    "copies, one thread per user); Total time as the binary prints it"}
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    ds = dataset()
    nthreads = os.cpu_count() or 1
    tmp = tempfile.mkdtemp(prefix="rknn_ref_")
    try:
        binary = ref_binary("rknn-inf")
        extra = {}
        if binary:
            path = write_workload_text(ds, tmp)
            # warm-up steps (untimed); the first runs one process alone: the
            # uncontended single-core query time and the R*-tree build
            alone = ref_inf_sample(ds, path, 1, seed=99)[0]
            for w in range(1, args.warmup):
                ref_inf_sample(ds, path, nthreads, seed=99 + w)
            per_q, builds, walls = [], [], []
            for s in range(args.steps):
                res = ref_inf_sample(ds, path, nthreads, seed=1000 + s)
                per_q.append([r["total_s"] for r in res])
                builds += [r["build_s"] for r in res]
                walls += [r["wall_s"] for r in res]
            qn = sum(len(x) for x in per_q)
            busy = sum(sum(x) for x in per_q)
            value = nthreads * qn / busy
            ms_step = 1e3 * busy / nthreads / args.steps
            kind = "reference"
            sample = (f"{nthreads} rknn-inf processes per step, one random query each (k=10); value = "
                      f"{nthreads} cores / mean per-query Total time (filter + verification, the "
                      f"binary's own timer; load and R*-tree build excluded, as the binary reports it)")
            extra = {"reference_binary": "rknn-inf (reference sources, g++ -O2)",
                     "single_core_alone": {"total_ms": 1e3 * alone["total_s"],
                                           "queries_per_s": 1.0 / alone["total_s"],
                                           "rtree_build_s": alone.get("build_s"),
                                           "load_s": alone["wall_s"] - alone.get("build_s", 0) - alone["total_s"]},
                     "all_cores": {"processes": nthreads, "mean_total_ms": 1e3 * busy / qn,
                                   "queries_per_s": value,
                                   "rtree_build_s_mean": statistics.mean(builds),
                                   "process_wall_s_mean": statistics.mean(walls)}}
            if not args.no_ref_suite:
                extra["reference_other_binaries"] = reference_suite(ds, tmp, path, nthreads)
        else:
            for _ in range(args.warmup):
                cpu_port_run(ds, NQ, nthreads, seed=99)
            times = []
            for s in range(args.steps):
                _, dt, _ = cpu_port_run(ds, NQ, nthreads, seed=1000 + s)
                times.append(dt)
            busy = sum(times)
            value = NQ * args.steps / busy
            ms_step = 1e3 * busy / args.steps
            kind = "port"
            sample = (f"{NQ} queries per step, C restatement of rknn-inf (R-tree, influence zone + "
                      f"verification) on {nthreads} threads (the reference binary was not built here)")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded uniform float32, the reference's text format values)",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "nf": NF, "nu": NU, "k": K, "queries_per_step": NQ},
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": nthreads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    line.update(extra)
    print(json.dumps(line), flush=True)
    return 0


def serving_config5(rknn, device, modes=("fp32", "fp64")):
    """The serving workload: resident 1M facilities / 10M users, open-loop
    Poisson arrivals at 1k-100k requests/s, k log-uniform in [1,64] (the
    oracle fixture's 2000 requests, cycled); result sizes are checked
    against the fixture."""
    import datagen
    import config_fixtures as CF
    ds5 = datagen.config(5)
    qs, ks = CF.config5_requests(ds5)
    fx = CF.load("config5")
    check = CF.data_sha256(ds5) == fx["data_sha256"]
    out = {"workload": "1M facilities / 10M users resident, Poisson arrivals, k log-uniform in [1,64]"}
    size_mismatches = 0
    with rknn.Index.of(ds5, device=device) as idx5:
        with rknn.Server(idx5, slots=3, max_batch=2048) as srv:
            # warm every slot in both modes at a low and a high rate (workspace
            # sizes and the k-class shapes the open-loop runs will meet)
            for mode in modes:
                for rate in (2e3, 1e5):
                    arrival = np.cumsum(np.random.default_rng(1).exponential(1.0 / rate, 600))
                    srv.replay(qs[:600], ks[:600], mode, arrival)
            srv.stats(reset=True)
            for rate, n in ((1e3, 1000), (1e4, 4000), (5e4, 8000), (1e5, 10000)):
                rng = np.random.default_rng(int(rate))
                arrival = np.cumsum(rng.exponential(1.0 / rate, n))
                sel = np.arange(n) % qs.shape[0]
                for mode in modes:
                    _, nr = srv.replay(qs[sel], ks[sel], mode, arrival)
                    st = srv.stats(reset=True)
                    if check:
                        size_mismatches += int((nr != fx["count"][sel]).sum())
                    out[f"{mode}@{int(rate)}"] = {"offered_qps": rate, "requests": n,
                                                  "throughput_qps": st["throughput_qps"],
                                                  "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                                                  "mean_batch": st["mean_batch"],
                                                  "max_inflight": st["max_inflight"]}
    out["result_size_mismatches_vs_oracle"] = size_mismatches if check else None
    return out


def run_ours(args):
    import torch
    import rknn
    import build
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    build.build()
    ds = dataset()
    # the chosen form: batched, FP32-filtered predicates, default candidate
    # filter (angular slices); the plain form: rknn-inf's influence zone
    cells = {}
    if args.cells:
        f, u = (float(x) for x in args.cells.split(","))
        cells = {"fac_per_cell": f, "usr_per_cell": u}
    idx = rknn.Index.of(ds, device=local, **cells)
    idx_inf = rknn.Index.of(ds, device=local, filter="inf")
    stream = torch.cuda.Stream(device=local)
    idx.set_stream(stream.cuda_stream)
    idx_inf.set_stream(stream.cuda_stream)
    nsteps = args.steps
    pool, checkable = query_pool(ds, NQ)
    qsets = [pool[i % len(pool)] for i in range(nsteps + args.warmup)]
    ks = np.full(NQ, K, np.int32)
    orc = OracleCheck(ds) if checkable else None

    # FP32 and FP64 predicates, both filters, give the same id sets (extra
    # information beside the oracle check; also sizes the pools)
    res = idx.query_batch(qsets[0], ks, "fp32")
    res64 = idx.query_batch(qsets[0], ks, "fp64")
    res64_inf = idx_inf.query_batch(qsets[0][:100], ks[:100], "fp64")
    mism_modes = sum(not np.array_equal(a, b) for a, b in zip(res, res64))
    mism_modes += sum(not np.array_equal(a, b) for a, b in zip(res[:100], res64_inf))

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    d_qs = [torch.from_numpy(q).to(dev) for q in pool]
    d_k = torch.from_numpy(ks).to(dev)

    def step(i, ev=None):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
            if ev:
                ev[0].record(stream)
            idx.query_batch_device(d_qs[i % len(pool)].data_ptr(), d_k.data_ptr(), NQ, K, "fp32")
            if ev:
                ev[1].record(stream)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(nsteps)]
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    got = []
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for i in range(nsteps):
            step(args.warmup + i, evs[i])
            if orc:
                # after the step's closing event: outside its timed interval
                got.append((args.warmup + i, device_results_to_host(idx, NQ, dev)))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if ws > 1:
        torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    value = replicas_throughput(sum(step_ms) / 1e3, ws, NQ * nsteps, dev)
    dev_s = ws * NQ * nsteps / value
    for si, (ids, off) in got:
        orc.add(si % len(pool), ids, off)

    # ---- end to end through the C ABI with host buffers ------------------
    e2e_times, e2e_dev, got_e2e, h2d, d2h = [], [], [], 0, 0
    idx.query_batch_flat(qsets[0], ks, "fp32")                      # sizes the output buffers
    idx.query_batch_flat(qsets[1], ks, "fp32")                      # warm: ids written in place from now on
    for i in range(nsteps):
        si = (args.warmup + i) % len(pool)
        q = pool[si]
        with torch.cuda.stream(stream):
            flush.fill_(float(-i))                                  # L2 flushed between steps, untimed
        stream.synchronize()
        t1 = time.perf_counter()
        ids, offs = idx.query_batch_flat(q, ks, "fp32")
        e2e_times.append(time.perf_counter() - t1)
        e2e_dev.append(idx.last_stats()["device_ms"])               # the engine's events around its launch
        h2d = q.nbytes + ks.nbytes
        d2h = 4 * (NQ + 1) + 4 * int(ids.shape[0])
        if orc:
            # copied out (the buffers are reused) and checked after the loop:
            # hashing a thousand id lists between calls would leave the next
            # call's host code to run cold
            got_e2e.append((si, ids.copy(), offs.copy()))
    e2e = NQ / statistics.mean(e2e_times) * ws
    for si, ids, offs in got_e2e:
        orc.add(si, ids, offs)
    # the same calls back to back, without the flush and its synchronization
    nf_times = []
    for i in range(nsteps):
        q = pool[(args.warmup + i) % len(pool)]
        t1 = time.perf_counter()
        idx.query_batch_flat(q, ks, "fp32")
        nf_times.append(time.perf_counter() - t1)
    e2e_diag = {"call_us_mean": 1e6 * statistics.mean(e2e_times), "call_us_median": 1e6 * statistics.median(e2e_times),
                "call_us_max": 1e6 * max(e2e_times), "device_us_median": 1e3 * statistics.median(e2e_dev),
                "no_flush_call_us_median": 1e6 * statistics.median(nf_times),
                "note": "call = rknn_query_batch through the Python binding with host buffers; device = the "
                        "engine's CUDA events around its launch inside the call"}

    # ---- plain FP64 single-query form (one query per launch, influence zone)
    single = pool[0][:200]
    lat = []
    for q in single[:10]:
        idx_inf.query(int(q), K, "fp64")
    for j, q in enumerate(single):
        t1 = time.perf_counter()
        r1 = idx_inf.query(int(q), K, "fp64")
        lat.append(1e3 * (time.perf_counter() - t1))
        if orc:
            orc.add_one(0, j, r1)
    fp64_single_qps = 1e3 / statistics.mean(lat)
    lat.sort()
    p50 = lat[len(lat) // 2]
    p99 = lat[min(len(lat) - 1, int(0.99 * len(lat)))]
    # batched device time of other modes and filters: one untimed call (its
    # graph is made there), then the mean of `reps` calls, L2 flushed before each
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def dev_qps(ix, mode, reps=3):
        ms = []
        for r in range(reps + 1):
            with torch.cuda.stream(stream):
                flush.fill_(3.0 + r)
                e0.record(stream)
                ix.query_batch_device(d_qs[r % len(d_qs)].data_ptr(), d_k.data_ptr(), NQ, K, mode)
                e1.record(stream)
            torch.cuda.synchronize()
            if r:
                ms.append(e0.elapsed_time(e1))
        return NQ / (statistics.mean(ms) / 1e3)
    fp64_batch_qps = dev_qps(idx, "fp64", reps=5)
    # the influence-zone filter batched in FP32
    inf_batch_qps = dev_qps(idx_inf, "fp32")

    # ---- serving: open-loop Poisson arrivals through the continuous batcher
    srv_rate, srv_n = 100_000.0, 20_000
    srng = np.random.default_rng(23)
    sq = srng.integers(0, ds.nf, srv_n).astype(np.int32)
    arrival = np.cumsum(srng.exponential(1.0 / srv_rate, srv_n))
    serving = {}
    with rknn.Server(idx, slots=3, max_batch=2048) as srv:
        for mode in ("fp32", "fp64"):
            srv.replay(sq[:2000], K, mode, arrival[:2000])            # warm the slots
            srv.stats(reset=True)
            srv.replay(sq, K, mode, arrival)
            st_s = srv.stats(reset=True)
            serving[mode] = {"offered_qps": srv_rate, "throughput_qps": st_s["throughput_qps"],
                             "p50_ms": st_s["p50_ms"], "p99_ms": st_s["p99_ms"],
                             "mean_batch": st_s["mean_batch"], "max_inflight": st_s["max_inflight"]}
    serving5 = None if args.no_serving5 else serving_config5(rknn, local)

    # ---- rooflines (live, profiling mode: per-kernel CUDA events) ----------
    idx.set_profiling(True)
    kms = []
    for i in range(3):
        with torch.cuda.stream(stream):
            flush.fill_(2.0 + i)
        stream.synchronize()
        idx.query_batch(qsets[(args.warmup + i) % len(qsets)], ks, "fp32")
        kms.append(idx.kernel_ms())
    st = idx.last_stats()
    idx.set_profiling(False)
    kavg = {n: statistics.mean(m[n] for m in kms) for n in kms[0]}
    hbm_peak, kind = peaks()
    props = torch.cuda.get_device_properties(local)
    fp32_peak = props.multi_processor_count * 128 * 2 * 2.07e9 / 1e12     # nominal
    # filter kernel (angular slices for this workload): bytes it must move
    # per launch = facilities streamed (8 B), facility cell-range starts read
    # (8 B per ring range), half-planes and their positions written (20 B),
    # one 64 B query descriptor and its user segments (8 B per row) per query.
    # At this batch size it also verifies its own queries (fused): users read
    # (8 B) and result ids written (4 B) on top.
    fused = st.get("fused_slots", 0) > 0
    zms = kavg["zone"]
    zbytes = 8 * st["zone_points"] + 8 * st["zone_cells"] + 20 * st["bisectors"] + 64 * NQ
    if fused:
        zbytes += 8 * st["candidates"] + 4 * st["results"]
    zgbs = zbytes / (zms / 1e3) / 1e9
    clk_ghz = (clk.summary().get("sm_mhz") or 2070.0) / 1e3
    issue_peak = 4 * props.multi_processor_count * clk_ghz * 1e9          # warp instructions / s
    froof = {"bound": "hbm", "achieved": zgbs, "peak": hbm_peak, "unit": "GB/s",
             "frac": zgbs / hbm_peak, "peak_kind": kind,
             "kernel": "slice_kernel2 (filter + fused verification)" if fused else "slice_kernel",
             "launch_ms": zms, "alg_bytes": zbytes,
             "traffic": TRAFFIC.get("fused_slice_kernel") if fused else None,
             "note": ("latency-bound: two warps a query walk the facility rings, then verify the query's "
                      "users against the half-planes in shared memory" if fused else
                      "latency-bound: one warp per query streams facilities ring by ring")}
    if fused:
        zi = FUSED_INSTR_PER_QUERY * NQ
        froof["issue"] = {"warp_instr": zi, "achieved_warp_instr_per_s": zi / (zms / 1e3),
                          "peak_warp_instr_per_s": issue_peak, "frac": zi / (zms / 1e3) / issue_peak,
                          "note": "instructions per query from ncu; peak = 4 per SM per cycle at the sampled clock"}
    # verification kernels: users read (8 B), half-planes staged (16 B each
    # per query), result ids written (4 B), facilities read by the exact
    # recount (8 B); FLOP = 4 per (user, half-plane) evaluation executed.
    # Fused batches leave them only the left-over queries and the listed
    # survivors' exact recount.
    vms = kavg["verify"] + kavg["recount"]
    if fused:
        vbytes = 8 * st["survivors"] + 4 * st["survivors"] + 8 * st["fac_checks"]
        vflops = 0
    else:
        vbytes = 8 * st["candidates"] + 16 * st["bisectors"] + 4 * st["results"] + 8 * st["fac_checks"]
        vflops = 4 * st["plane_evals"]
    vgbs = vbytes / (vms / 1e3) / 1e9
    vtfs = vflops / (vms / 1e3) / 1e12
    vroof = {"bound": "hbm", "achieved": vgbs, "peak": hbm_peak, "unit": "GB/s", "frac": vgbs / hbm_peak,
             "peak_kind": kind, "kernel": "verify_kernel", "kernels": "verify_kernel + recount_kernel",
             "launch_ms": vms,
             "alg_bytes": vbytes, "alg_flop": vflops, "traffic": None,
             "fp32": {"achieved_tflops": vtfs, "frac": vtfs / fp32_peak, "peak": fp32_peak,
                      "peak_kind": "nominal (SMs x 128 FMA x 2.07 GHz)"}}
    # the dominant kernel's roofline leads; the other rides beside it
    roof, other = (froof, vroof) if zms >= vms else (vroof, froof)
    roof = dict(roof, kernel_ms=kavg, share={n: v / sum(kavg.values()) for n, v in kavg.items()},
                fused_queries=int(st.get("fused_slots", 0)))

    # ---- the same workload with the GPU full: one batch of SAT_NQ queries.
    # Both kernels are bound by instruction issue there; their issue roofline
    # is the warp instructions the work needs (per query for the filter, per
    # half-plane evaluation for the verification, from one ncu capture of this
    # batch) at the SMs' peak issue rate (4 warp instructions per cycle per
    # SM at the sampled clock).
    sat = None
    if not args.no_saturation and NQ < SAT_NQ:
        qsat = np.random.default_rng(99 + rank).choice(ds.nf, size=SAT_NQ, replace=False).astype(np.int32)
        idx.query_batch_flat(qsat, K, "fp32")
        idx.set_profiling(True)
        with torch.cuda.stream(stream):
            flush.fill_(7.0)
        stream.synchronize()
        idx.query_batch_flat(qsat, K, "fp32")
        ksat = idx.kernel_ms()
        sst = idx.last_stats()
        idx.set_profiling(False)
        sz = ksat["zone"] / 1e3
        sv = ksat["verify"] / 1e3
        zi = INSTR["slice_kernel_per_query"] * SAT_NQ
        vi = INSTR["verify_kernel_per_eval"] * sst["plane_evals"]
        sat = {"queries": SAT_NQ, "queries_per_s_device": SAT_NQ / (sum(ksat.values()) / 1e3),
               "issue_peak_warp_instr_per_s": issue_peak,
               "slice_kernel": {"launch_ms": ksat["zone"], "warp_instr": zi, "frac_issue": zi / sz / issue_peak,
                                "hbm_frac": (8 * sst["zone_points"] + 8 * sst["zone_cells"] + 20 * sst["bisectors"]
                                             + 64 * SAT_NQ) / sz / (hbm_peak * 1e9)},
               "verify_kernel": {"launch_ms": ksat["verify"], "warp_instr": vi, "frac_issue": vi / sv / issue_peak,
                                 "tflops": 4 * sst["plane_evals"] / sv / 1e12,
                                 "fp32_frac": 4 * sst["plane_evals"] / sv / 1e12 / fp32_peak,
                                 "hbm_frac": (8 * sst["candidates"] + 16 * sst["bisectors"] + 4 * sst["results"])
                                             / sv / (hbm_peak * 1e9)},
               "note": "warp instructions per unit of work from one ncu capture of this batch"}

    # ---- CPU baseline (rank 0, N=1 only) ---------------------------------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        if ref_binary("rknn-inf"):
            tmp = tempfile.mkdtemp(prefix="rknn_ref_")
            try:
                path = write_workload_text(ds, tmp)
                t0 = time.perf_counter()
                res = []
                while time.perf_counter() - t0 < args.cpu_seconds:
                    res += ref_inf_sample(ds, path, nthreads, seed=5000 + len(res))
            finally:
                shutil.rmtree(tmp, ignore_errors=True)
            tot = [r["total_s"] for r in res]
            cpu = {"value": nthreads / statistics.mean(tot), "unit": "queries/s", "cores": nthreads,
                   "kind": "reference",
                   "sample": f"{len(res)} random facility queries at k=10, rknn-inf binary, {nthreads} "
                             f"processes at once, one query each; value = {nthreads} / mean per-query Total "
                             f"time ({1e3 * statistics.mean(tot):.3f} ms; R*-tree build "
                             f"{statistics.mean(r['build_s'] for r in res):.1f} s per process, excluded)"}
        sample = args.cpu_sample
        qps, dt, _ = cpu_port_run(ds, sample, nthreads)
        port = {"value": qps, "unit": "queries/s", "cores": nthreads, "kind": "port",
                "sample": f"{sample} random facility queries at k=10 ({dt:.1f} s on {nthreads} threads), "
                          "rknn-inf restatement: R-tree, influence-zone filter, verification"}
        if cpu:
            cpu["port"] = port
        else:
            cpu = port

    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws,
        "steps": nsteps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / nsteps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform float32 in [0,1000]^2)",
        "config": {"workload": WORKLOAD,
                   "nf": NF, "nu": NU, "k": K, "queries_per_step": NQ, "mode": "fp32 batched",
                   "filter": "angular slices (rknn-slice rule, 32 slices); plain form: influence zone",
                   "l2": "256 MB flush before each timed step", "parallelism": f"replicas x{ws}"},
        "wall_s": wall,
        "e2e": {"value": e2e, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "e2e_diag": e2e_diag,
        "gpu_launches": 5 * nsteps,
        "mismatches_vs_oracle": orc.mismatches if orc and orc.ok else None,
        "checked_vs_oracle": (f"{orc.checked} query results (every timed device step, every end-to-end "
                              f"step, the plain form's queries) against the exact oracle's fixture"
                              if orc and orc.ok else "not checked (no fixture for this batch size)"),
        "fp64_single_query": {"qps": fp64_single_qps, "p50_ms": p50, "p99_ms": p99,
                              "filter": "influence zone (rknn-inf rules)"},
        "fp64_batched_qps": fp64_batch_qps,
        "inf_zone_fp32_batched_qps": inf_batch_qps,
        "serving": dict(serving, workload=f"{srv_n} Poisson requests at {srv_rate:.0f}/s, k={K}"),
        "serving_config5": serving5,
        "speedup_fp32_batched_vs_fp64_single": value / ws / fp64_single_qps,
        "roofline": roof,
        "roofline_other": other,
        "roofline_saturated": sat,
        "stats": {k2: st[k2] for k2 in ("bisectors", "zone_vertices_max", "zone_candidates", "zone_fp64",
                                        "zone_points", "zone_cells",
                                        "candidates", "plane_evals", "survivors", "fac_checks",
                                        "rechecks", "results", "overflow")},
        "recheck_fraction": st["rechecks"] / max(1, st["fac_checks"]),
        "mismatches_fp32_vs_fp64": mism_modes,
        "mismatches_fp32_vs_fp64_checked": f"{NQ} queries FP32 vs FP64 (default filter) + 100 vs FP64 influence zone",
        "clocks": clk.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    global NQ
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=400000, help="queries of the C restatement's timing")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="seconds of reference-binary rounds in the CPU baseline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ref-suite", action="store_true",
                    help="reference arm: skip the reference's other binaries")
    ap.add_argument("--no-serving5", action="store_true", help="skip the 1M/10M serving workload")
    ap.add_argument("--no-saturation", action="store_true", help="skip the 16384-query saturation batch")
    ap.add_argument("--cells", default="", metavar="F,U",
                    help="facilities and users per grid cell of the batch index (default: the index's defaults)")
    ap.add_argument("--queries", type=int, default=NQ,
                    help="queries per step (default 1000, the headline workload; larger batches for profiling)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    NQ = args.queries
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
