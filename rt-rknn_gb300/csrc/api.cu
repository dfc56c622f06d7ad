// C ABI of the engine (include/rknn_gpu.h): index creation, single-query
// and batched queries, device-resident batches, statistics.
//
// One query batch is five kernels on the index's stream, captured once per
// batch shape into a CUDA graph and replayed:
//   zone_kernel      one warp per query (persistent, queries in descending-k
//                    order): influence zone, half-planes, candidate segments
//   plan_kernel      candidate and work-item offsets
//   verify_kernel    persistent warps over 128-user work items: half-plane
//                    filter, exact recount, warp-aggregated result append
//   scan_counts      result offsets
//   finalize_kernel  one block per query: sort its ids into the output
#include "../../include/rknn_gpu.h"
#include "index.cuh"
#include "rknn_common.cuh"
#include "verify.cuh"
#include "zone.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

using namespace rknn;

namespace {

thread_local std::string g_err;

rknn_status fail(rknn_status s, const std::string& msg)
{
    g_err = msg;
    return s;
}

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return fail(e_ == cudaErrorMemoryAllocation ? RKNN_ERR_OOM : RKNN_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

template <typename T>
cudaError_t dalloc(T*& p, size_t n)
{
    p = nullptr;
    return cudaMalloc(&p, sizeof(T) * (n > 0 ? n : 1));
}

ZoneCaps caps_for(int kmax)
{
    ZoneCaps c;
    long long k = std::max(1, kmax);
    c.vc = (int)std::min<long long>(4 * k * k + 96, 1 << 22);
    c.lc = (int)std::min<long long>(6 * k + 40, 1 << 16);
    c.pc = (int)std::min<long long>(256 + 24 * k, 1 << 20);
    c.rm = 64;
    return c;
}

struct GraphKey {
    int nq, mode, vc, lc, pc, rm, use_global;
    long long pool;
    bool operator<(const GraphKey& o) const
    {
        return std::tie(nq, mode, vc, lc, pc, rm, use_global, pool) <
               std::tie(o.nq, o.mode, o.vc, o.lc, o.pc, o.rm, o.use_global, o.pool);
    }
};

struct Workspace {
    int nq_cap = 0, lc = 0, seg_cap = 0;
    int *d_q = nullptr, *d_k = nullptr, *d_order = nullptr;
    QDesc* d_qd = nullptr;
    float4* d_planes = nullptr;
    int* d_bispos = nullptr;
    int2* d_segs = nullptr;
    ZStats* d_zst = nullptr;
    int *d_cand_off = nullptr, *d_chunk_off = nullptr, *d_res_count = nullptr, *d_out_off = nullptr;
    int* d_counters = nullptr;     // [0] zone work, [1] verify work, [4..8] zone fault record
    VStats* d_vstats = nullptr;
    int *d_pool = nullptr, *d_out = nullptr;
    long long pool_cap = 0;
    char* d_zscratch = nullptr;
    size_t zscratch_bytes = 0;
    int *h_q = nullptr, *h_k = nullptr, *h_order = nullptr, *h_off = nullptr;
    int* h_ids = nullptr;
    long long h_ids_cap = 0;
    std::map<GraphKey, cudaGraphExec_t> graphs;
};

}  // namespace

struct rknn_index {
    int device = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    long long nf = 0, nu = 0;
    Grid gf{}, gu{};
    double sx0 = 0, sy0 = 0, sx1 = 0, sy1 = 0;
    float2* d_fxy = nullptr;
    int *d_fidx = nullptr, *d_fpos = nullptr, *d_fstart = nullptr;
    float4* d_fmbr = nullptr;
    float2* d_uxy = nullptr;
    int *d_uid = nullptr, *d_ustart = nullptr;
    std::vector<int> h_fidx;       // cell-sorted position -> facility input index
    int skip_coincident = 1;
    int num_sms = 0;
    size_t smem_optin = 0;
    Workspace ws;
    std::mutex mu;
    rknn_query_stats last{};
    int last_nq = 0, last_mode = 0, last_lc = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int profiling = 0;
    cudaEvent_t kev[6] = {};
};

namespace {

void free_ws(Workspace& w)
{
    for (auto& g : w.graphs) cudaGraphExecDestroy(g.second);
    w.graphs.clear();
    cudaFree(w.d_q); cudaFree(w.d_k); cudaFree(w.d_order);
    cudaFree(w.d_qd); cudaFree(w.d_planes); cudaFree(w.d_bispos); cudaFree(w.d_segs); cudaFree(w.d_zst);
    cudaFree(w.d_cand_off); cudaFree(w.d_chunk_off); cudaFree(w.d_res_count); cudaFree(w.d_out_off);
    cudaFree(w.d_counters); cudaFree(w.d_vstats);
    cudaFree(w.d_pool); cudaFree(w.d_out); cudaFree(w.d_zscratch);
    cudaFreeHost(w.h_q); cudaFreeHost(w.h_k); cudaFreeHost(w.h_order); cudaFreeHost(w.h_off);
    cudaFreeHost(w.h_ids);
    w = Workspace();
}

void drop_graphs(Workspace& w)
{
    for (auto& g : w.graphs) cudaGraphExecDestroy(g.second);
    w.graphs.clear();
}

// Launch geometry of the zone kernel for given caps.  The zone state always
// lives in shared memory (one warp per block); caps_fit() has already sized
// it to fit the per-block limit.
struct ZoneLaunch {
    size_t slice, smem;
    int grid;
};

ZoneLaunch zone_launch(rknn_index* ix, const ZoneCaps& c, int nq)
{
    ZoneLaunch L;
    L.slice = zone_layout(c).bytes;
    L.smem = L.slice * ZONE_WARPS;
    int per_sm = 1;
    if (L.smem > 48 * 1024)
        cudaFuncSetAttribute(zone_kernel_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zone_kernel_smem, 32 * ZONE_WARPS, L.smem);
    if (per_sm < 1) per_sm = 1;
    long long want = (nq + ZONE_WARPS - 1) / ZONE_WARPS;
    L.grid = (int)std::max(1LL, std::min<long long>(want, (long long)per_sm * ix->num_sms));
    return L;
}

// Shrink the vertex and queue capacities until the per-warp state fits the
// shared memory a block may use.  A zone that outgrows them stops early
// (fewer bisectors, a weaker filter); results stay exact.
ZoneCaps caps_fit(rknn_index* ix, ZoneCaps c)
{
    const size_t budget = std::min<size_t>(ix->smem_optin, 200 * 1024) - 1024;
    while (zone_layout(c).bytes * ZONE_WARPS > budget && c.vc > 256) c.vc = c.vc * 7 / 8;
    while (zone_layout(c).bytes * ZONE_WARPS > budget && c.pc > 512) c.pc = c.pc * 7 / 8;
    while (zone_layout(c).bytes * ZONE_WARPS > budget && c.lc > 64) c.lc = c.lc * 7 / 8;
    // vertex counts and indices are stored in 16 bits
    c.vc = std::min(c.vc, 65535);
    c.lc = std::min(c.lc, 65535);
    return c;
}

rknn_status ensure_ws(rknn_index* ix, int nq, const ZoneCaps& caps, long long pool_need)
{
    Workspace& w = ix->ws;
    const int seg_cap = 2 * caps.rm + 2;
    if (nq > w.nq_cap || caps.lc > w.lc || seg_cap > w.seg_cap) {
        int nqc = std::max(nq, w.nq_cap);
        int lc = std::max(caps.lc, w.lc);
        int sc = std::max(seg_cap, w.seg_cap);
        long long pool = w.pool_cap;
        free_ws(w);
        w.pool_cap = pool;
        w.nq_cap = nqc; w.lc = lc; w.seg_cap = sc;
        CK(dalloc(w.d_q, nqc)); CK(dalloc(w.d_k, nqc)); CK(dalloc(w.d_order, nqc));
        CK(dalloc(w.d_qd, nqc));
        CK(dalloc(w.d_planes, (size_t)nqc * lc));
        CK(dalloc(w.d_bispos, (size_t)nqc * lc));
        CK(dalloc(w.d_segs, (size_t)nqc * sc));
        CK(dalloc(w.d_zst, nqc));
        CK(dalloc(w.d_cand_off, nqc + 1)); CK(dalloc(w.d_chunk_off, nqc + 1));
        CK(dalloc(w.d_res_count, nqc)); CK(dalloc(w.d_out_off, nqc + 1));
        CK(dalloc(w.d_counters, 16));
        CK(cudaMemset(w.d_counters, 0, sizeof(int) * 16));
        CK(dalloc(w.d_vstats, 1));
        CK(cudaMallocHost(&w.h_q, sizeof(int) * nqc));
        CK(cudaMallocHost(&w.h_k, sizeof(int) * nqc));
        CK(cudaMallocHost(&w.h_order, sizeof(int) * nqc));
        CK(cudaMallocHost(&w.h_off, sizeof(int) * (nqc + 1)));
        w.pool_cap = 0;
    }
    if (pool_need > w.pool_cap) {
        drop_graphs(w);
        cudaFree(w.d_pool);
        cudaFree(w.d_out);
        w.d_pool = w.d_out = nullptr;
        long long cap = std::max<long long>(pool_need, 1 << 20);
        CK(dalloc(w.d_pool, (size_t)cap));
        CK(dalloc(w.d_out, (size_t)cap));
        w.pool_cap = cap;
    }
    return RKNN_OK;
}

// Launch geometry of one batch; computed (and kernel attributes set) before
// any stream capture.
struct BatchLaunch {
    ZoneLaunch zl;
    size_t vsmem;
    int vgrid;
};

BatchLaunch batch_launch(rknn_index* ix, int nq, int mode, const ZoneCaps& caps)
{
    BatchLaunch b;
    b.zl = zone_launch(ix, caps, nq);
    b.vsmem = (size_t)VERIFY_WARPS * caps.lc * (mode == MODE_FP32 ? 16 : 32);
    if (b.vsmem > 48 * 1024)
        cudaFuncSetAttribute(verify_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b.vsmem);
    int vper = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&vper, verify_kernel, VERIFY_WARPS * 32, b.vsmem);
    if (vper < 1) vper = 1;
    b.vgrid = vper * ix->num_sms;
    cudaFuncSetAttribute(finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(SORT_CAP * sizeof(unsigned)));
    return b;
}

// Enqueue the five kernels (no synchronization, no non-stream CUDA calls:
// this runs under stream capture).
rknn_status enqueue(rknn_index* ix, int nq, int mode, const ZoneCaps& caps, bool use_order,
                    const BatchLaunch& bl, bool events = false)
{
    Workspace& w = ix->ws;
    cudaStream_t st = ix->stream;
    auto mark = [&](int i) { if (events) cudaEventRecord(ix->kev[i], st); };
    const ZoneLaunch& zl = bl.zl;
    CK(cudaMemsetAsync(w.d_counters, 0, sizeof(int) * 4, st));
    CK(cudaMemsetAsync(w.d_res_count, 0, sizeof(int) * nq, st));
    CK(cudaMemsetAsync(w.d_vstats, 0, sizeof(VStats), st));

    ZoneArgs za;
    za.fxy = ix->d_fxy; za.fstart = ix->d_fstart; za.fmbr = ix->d_fmbr; za.fpos = ix->d_fpos;
    za.gf = ix->gf; za.nf = (int)ix->nf;
    za.ustart = ix->d_ustart; za.gu = ix->gu; za.nu = (int)ix->nu;
    za.sx0 = ix->sx0; za.sy0 = ix->sy0; za.sx1 = ix->sx1; za.sy1 = ix->sy1;
    za.q_in = w.d_q; za.k_in = w.d_k; za.order = use_order ? w.d_order : nullptr; za.nq = nq;
    za.work_counter = w.d_counters + 0;
    za.caps = caps;
    za.use_global = 0;
    za.gscratch = nullptr;
    za.skip_coincident = ix->skip_coincident;
    za.rmax = caps.rm;
    za.seg_cap = w.seg_cap;
    za.qd = w.d_qd; za.planes = w.d_planes; za.bis_pos = w.d_bispos; za.segs = w.d_segs; za.zst = w.d_zst;
    za.fault = w.d_counters + 4;
    // planes/bis_pos are strided by the workspace lc
    za.caps.lc = caps.lc;
    mark(0);
    zone_kernel_smem<<<zl.grid, 32 * ZONE_WARPS, zl.smem, st>>>(za);
    CK(cudaGetLastError());
    mark(1);

    plan_kernel<<<1, 1024, 0, st>>>(w.d_qd, nq, w.d_cand_off, w.d_chunk_off, (int)std::min<long long>(w.pool_cap, INT32_MAX));
    CK(cudaGetLastError());
    mark(2);

    VerifyArgs va;
    va.qd = w.d_qd; va.planes = w.d_planes; va.bis_pos = w.d_bispos; va.lc = caps.lc;
    va.segs = w.d_segs; va.seg_cap = w.seg_cap;
    va.chunk_off = w.d_chunk_off; va.cand_off = w.d_cand_off; va.nq = nq;
    va.uxy = ix->d_uxy; va.uid = ix->d_uid; va.fxy = ix->d_fxy; va.fstart = ix->d_fstart; va.gf = ix->gf;
    va.res_count = w.d_res_count; va.res_pool = w.d_pool; va.work_counter = w.d_counters + 1;
    va.vstats = w.d_vstats; va.mode = mode;
    va.nu = (int)ix->nu; va.nf = (int)ix->nf; va.ncf = ix->gf.gx * ix->gf.gy;
    va.pool_cap = w.pool_cap; va.fault = w.d_counters + 10;
    verify_kernel<<<bl.vgrid, VERIFY_WARPS * 32, bl.vsmem, st>>>(va);
    CK(cudaGetLastError());
    mark(3);

    scan_counts_kernel<<<1, 1024, 0, st>>>(w.d_res_count, nq, w.d_out_off);
    CK(cudaGetLastError());
    mark(4);
    finalize_kernel<<<nq, 256, SORT_CAP * sizeof(unsigned), st>>>(w.d_pool, w.d_cand_off, w.d_res_count,
                                                                  w.d_out_off, w.d_out, nq);
    CK(cudaGetLastError());
    mark(5);
    return RKNN_OK;
}

// Launch through a cached graph for this batch shape.
rknn_status launch(rknn_index* ix, int nq, int mode, const ZoneCaps& caps, bool use_order)
{
    Workspace& w = ix->ws;
    const BatchLaunch bl = batch_launch(ix, nq, mode, caps);
    if (ix->profiling) return enqueue(ix, nq, mode, caps, use_order, bl, true);
    const ZoneLaunch& zl = bl.zl;
    GraphKey key{nq, mode, caps.vc, caps.lc, caps.pc, caps.rm, 0, w.pool_cap};
    key.nq = use_order ? nq : -nq;
    auto it = w.graphs.find(key);
    if (it == w.graphs.end()) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(ix->stream, cudaStreamCaptureModeThreadLocal));
        rknn_status s = enqueue(ix, nq, mode, caps, use_order, bl);
        cudaError_t e = cudaStreamEndCapture(ix->stream, &g);
        if (s != RKNN_OK) { if (e == cudaSuccess) cudaGraphDestroy(g); return s; }
        CK(e);
        cudaGraphExec_t ge;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        CK(e);
        it = w.graphs.emplace(key, ge).first;
    }
    CK(cudaGraphLaunch(it->second, ix->stream));
    return RKNN_OK;
}

rknn_status collect_stats(rknn_index* ix, int nq, rknn_query_stats* out)
{
    Workspace& w = ix->ws;
    std::vector<ZStats> z(nq);
    std::vector<QDesc> qd(nq);
    VStats v;
    CK(cudaMemcpyAsync(z.data(), w.d_zst, sizeof(ZStats) * nq, cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaMemcpyAsync(qd.data(), w.d_qd, sizeof(QDesc) * nq, cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaMemcpyAsync(&v, w.d_vstats, sizeof(VStats), cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaStreamSynchronize(ix->stream));
    rknn_query_stats s{};
    s.queries = nq;
    for (int i = 0; i < nq; ++i) {
        s.bisectors += z[i].nb;
        s.zone_vertices_max = std::max<int64_t>(s.zone_vertices_max, z[i].vmax);
        s.zone_candidates += z[i].cand;
        s.zone_fp64 += z[i].cand64;
        if (qd[i].flags & (QF_ZONE_V_OVERFLOW | QF_ZONE_L_OVERFLOW | QF_ZONE_PQ_OVERFLOW)) s.overflow++;
        for (int j = 0; j < 8; ++j) s.zone_cycles[j] += z[i].cyc[j];
        s.zone_points += z[i].pts;
        s.zone_cells += z[i].cells;
    }
    s.results = (int64_t)v.results;
    s.candidates = (int64_t)v.cand;
    s.plane_evals = (int64_t)v.plane_evals;
    s.survivors = (int64_t)v.survivors;
    s.fac_checks = (int64_t)v.fac_checks;
    s.rechecks = (int64_t)v.rechecks;
    s.device_ms = ix->last.device_ms;
    *out = s;
    return RKNN_OK;
}

// Run a batch whose q/k are already in ws.d_q / ws.d_k.  Grows the result
// pool and reruns when a query's candidate region did not fit.
rknn_status run_sync(rknn_index* ix, int nq, int mode, int kmax, bool use_order)
{
    Workspace& w = ix->ws;
    ZoneCaps caps = caps_fit(ix, caps_for(kmax));
    long long need = std::max<long long>(w.pool_cap, (long long)nq * 4096);
    rknn_status s = ensure_ws(ix, nq, caps, need);
    if (s != RKNN_OK) return s;
    for (int attempt = 0; attempt < 3; ++attempt) {
        CK(cudaEventRecord(ix->ev0, ix->stream));
        s = launch(ix, nq, mode, caps, use_order);
        if (s != RKNN_OK) return s;
        CK(cudaEventRecord(ix->ev1, ix->stream));
        int tot[2];
        CK(cudaMemcpyAsync(&tot[0], w.d_cand_off + nq, sizeof(int), cudaMemcpyDeviceToHost, ix->stream));
        CK(cudaMemcpyAsync(w.h_off, w.d_out_off, sizeof(int) * (nq + 1), cudaMemcpyDeviceToHost, ix->stream));
        CK(cudaStreamSynchronize(ix->stream));
        float ms = 0;
        cudaEventElapsedTime(&ms, ix->ev0, ix->ev1);
        ix->last.device_ms = ms;
        long long cand_total = (unsigned)tot[0];
        if (cand_total <= w.pool_cap) return RKNN_OK;
        s = ensure_ws(ix, nq, caps, cand_total + cand_total / 4);
        if (s != RKNN_OK) return s;
    }
    return fail(RKNN_ERR_CAPACITY, "result pool could not be sized");
}

rknn_status check_queries(rknn_index* ix, const int32_t* q, const int32_t* k, int nq, int* kmax)
{
    *kmax = 1;
    for (int i = 0; i < nq; ++i) {
        if (q[i] < 0 || q[i] >= ix->nf)
            return fail(RKNN_ERR_ARG, "query index " + std::to_string(q[i]) + " out of range [0, " +
                                          std::to_string(ix->nf) + ")");
        if (k[i] <= 0) return fail(RKNN_ERR_ARG, "k must be a positive integer");
        *kmax = std::max(*kmax, (int)k[i]);
    }
    return RKNN_OK;
}

}  // namespace

// ============================================================== public API
extern "C" {

const char* rknn_last_error(void) { return g_err.c_str(); }

const char* rknn_version(void) { return "rknn-gb300 0.1 (sm_103a)"; }

void rknn_index_opts_default(rknn_index_opts* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->device = 0;
    o->fac_per_cell = 2.0f;
    o->usr_per_cell = 8.0f;
    o->skip_coincident = 1;
}

rknn_status rknn_index_create(const float* fxy, const int32_t* fid, int64_t nf, const float* uxy,
                              const int32_t* uid, int64_t nu, const rknn_index_opts* opts,
                              rknn_index** out)
{
    g_err.clear();
    if (!out) return fail(RKNN_ERR_ARG, "out is null");
    *out = nullptr;
    if (!fxy || nf < 1) return fail(RKNN_ERR_ARG, "need at least one facility");
    if (nu < 0 || (nu > 0 && (!uxy || !uid))) return fail(RKNN_ERR_ARG, "bad user arrays");
    if (nf >= INT32_MAX / 2 || nu >= INT32_MAX / 2) return fail(RKNN_ERR_ARG, "too many points");
    rknn_index_opts o;
    rknn_index_opts_default(&o);
    if (opts) o = *opts;
    if (!(o.fac_per_cell > 0)) o.fac_per_cell = 2.0f;
    if (!(o.usr_per_cell > 0)) o.usr_per_cell = 8.0f;

    // bounding box of all points (rknn-inf/inf.cpp:181-199)
    double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    for (int64_t i = 0; i < nf; ++i) {
        double x = fxy[2 * i], y = fxy[2 * i + 1];
        if (!std::isfinite(x) || !std::isfinite(y)) return fail(RKNN_ERR_ARG, "non-finite facility coordinate");
        x0 = std::min(x0, x); x1 = std::max(x1, x); y0 = std::min(y0, y); y1 = std::max(y1, y);
    }
    for (int64_t i = 0; i < nu; ++i) {
        double x = uxy[2 * i], y = uxy[2 * i + 1];
        if (!std::isfinite(x) || !std::isfinite(y)) return fail(RKNN_ERR_ARG, "non-finite user coordinate");
        x0 = std::min(x0, x); x1 = std::max(x1, x); y0 = std::min(y0, y); y1 = std::max(y1, y);
    }

    rknn_index* ix = new (std::nothrow) rknn_index();
    if (!ix) return fail(RKNN_ERR_OOM, "host allocation failed");
    auto bail = [&](rknn_status s) { rknn_index_destroy(ix); return s; };
    ix->device = o.device;
    ix->skip_coincident = o.skip_coincident ? 1 : 0;
    ix->nf = nf;
    ix->nu = nu;
    ix->sx0 = x0; ix->sy0 = y0; ix->sx1 = x1; ix->sy1 = y1;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return bail(fail(RKNN_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e)));
    if (o.device < 0 || o.device >= ndev) return bail(fail(RKNN_ERR_ARG, "bad device ordinal"));
#define CKB(call)                                                                            \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return bail(fail(e_ == cudaErrorMemoryAllocation ? RKNN_ERR_OOM : RKNN_ERR_CUDA, \
                             std::string(#call) + ": " + cudaGetErrorString(e_)));           \
    } while (0)
    CKB(cudaSetDevice(o.device));
    CKB(cudaStreamCreateWithFlags(&ix->own_stream, cudaStreamNonBlocking));
    ix->stream = ix->own_stream;
    CKB(cudaEventCreate(&ix->ev0));
    CKB(cudaEventCreate(&ix->ev1));
    CKB(cudaDeviceGetAttribute(&ix->num_sms, cudaDevAttrMultiProcessorCount, o.device));
    int optin = 0;
    CKB(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, o.device));
    ix->smem_optin = (size_t)optin;

    ix->gf = make_grid(x0, y0, x1, y1, nf, o.fac_per_cell, 4096);
    ix->gu = make_grid(x0, y0, x1, y1, nu, o.usr_per_cell, 8192);
    cudaStream_t st = ix->stream;
    float2 *tf = nullptr, *tu = nullptr;
    int* tuid = nullptr;
    CKB(dalloc(tf, nf));
    CKB(cudaMemcpyAsync(tf, fxy, sizeof(float2) * nf, cudaMemcpyHostToDevice, st));
    if (nu > 0) {
        CKB(dalloc(tu, nu));
        CKB(dalloc(tuid, nu));
        CKB(cudaMemcpyAsync(tu, uxy, sizeof(float2) * nu, cudaMemcpyHostToDevice, st));
        CKB(cudaMemcpyAsync(tuid, uid, sizeof(int) * nu, cudaMemcpyHostToDevice, st));
    }
    long long ncf = (long long)ix->gf.gx * ix->gf.gy, ncu = (long long)ix->gu.gx * ix->gu.gy;
    CKB(dalloc(ix->d_fxy, nf));
    CKB(dalloc(ix->d_fidx, nf));
    CKB(dalloc(ix->d_fpos, nf));
    CKB(dalloc(ix->d_fstart, ncf + 1));
    CKB(dalloc(ix->d_fmbr, ncf));
    CKB(dalloc(ix->d_uxy, nu));
    CKB(dalloc(ix->d_uid, nu));
    CKB(dalloc(ix->d_ustart, ncu + 1));
    CKB(grid_sort(tf, nullptr, (int)nf, ix->gf, ix->d_fxy, nullptr, ix->d_fidx, ix->d_fpos, ix->d_fstart, st));
    CKB(cell_mbrs(ix->d_fxy, ix->d_fstart, ix->gf, ix->d_fmbr, st));
    CKB(grid_sort(tu, tuid, (int)nu, ix->gu, ix->d_uxy, ix->d_uid, nullptr, nullptr, ix->d_ustart, st));
    ix->h_fidx.resize(nf);
    CKB(cudaMemcpyAsync(ix->h_fidx.data(), ix->d_fidx, sizeof(int) * nf, cudaMemcpyDeviceToHost, st));
    CKB(cudaStreamSynchronize(st));
    cudaFree(tf);
    cudaFree(tu);
    cudaFree(tuid);
#undef CKB
    *out = ix;
    return RKNN_OK;
}

rknn_status rknn_index_destroy(rknn_index* ix)
{
    if (!ix) return RKNN_OK;
    cudaSetDevice(ix->device);
    if (ix->stream) cudaStreamSynchronize(ix->stream);
    free_ws(ix->ws);
    cudaFree(ix->d_fxy); cudaFree(ix->d_fidx); cudaFree(ix->d_fpos); cudaFree(ix->d_fstart);
    cudaFree(ix->d_fmbr); cudaFree(ix->d_uxy); cudaFree(ix->d_uid); cudaFree(ix->d_ustart);
    if (ix->ev0) cudaEventDestroy(ix->ev0);
    if (ix->ev1) cudaEventDestroy(ix->ev1);
    for (int i = 0; i < 6; ++i) if (ix->kev[i]) cudaEventDestroy(ix->kev[i]);
    if (ix->own_stream) cudaStreamDestroy(ix->own_stream);
    delete ix;
    return RKNN_OK;
}

rknn_status rknn_index_size(const rknn_index* ix, int64_t* nf, int64_t* nu)
{
    if (!ix) return fail(RKNN_ERR_ARG, "index is null");
    if (nf) *nf = ix->nf;
    if (nu) *nu = ix->nu;
    return RKNN_OK;
}

rknn_status rknn_index_get_info(const rknn_index* ix, rknn_index_info* info)
{
    if (!ix || !info) return fail(RKNN_ERR_ARG, "null argument");
    info->nf = ix->nf;
    info->nu = ix->nu;
    info->x0 = ix->sx0; info->y0 = ix->sy0; info->x1 = ix->sx1; info->y1 = ix->sy1;
    info->fgrid_x0 = ix->gf.x0; info->fgrid_y0 = ix->gf.y0; info->fgrid_inv = ix->gf.inv;
    info->fgrid_gx = ix->gf.gx; info->fgrid_gy = ix->gf.gy;
    info->ugrid_x0 = ix->gu.x0; info->ugrid_y0 = ix->gu.y0; info->ugrid_inv = ix->gu.inv;
    info->ugrid_gx = ix->gu.gx; info->ugrid_gy = ix->gu.gy;
    return RKNN_OK;
}

rknn_status rknn_set_profiling(rknn_index* ix, int32_t on)
{
    if (!ix) return fail(RKNN_ERR_ARG, "index is null");
    std::lock_guard<std::mutex> lk(ix->mu);
    if (on && !ix->kev[0])
        for (int i = 0; i < 6; ++i) CK(cudaEventCreate(&ix->kev[i]));
    ix->profiling = on ? 1 : 0;
    return RKNN_OK;
}

rknn_status rknn_last_kernel_ms(rknn_index* ix, double* ms)
{
    if (!ix || !ms) return fail(RKNN_ERR_ARG, "null argument");
    if (!ix->kev[0]) return fail(RKNN_ERR_STATE, "profiling was never enabled");
    CK(cudaEventSynchronize(ix->kev[5]));
    for (int i = 0; i < 5; ++i) {
        float t = 0;
        CK(cudaEventElapsedTime(&t, ix->kev[i], ix->kev[i + 1]));
        ms[i] = t;
    }
    return RKNN_OK;
}

// Zone-kernel fault record of a build with RKNN_CHECKED (all zero otherwise):
// {flag, array id, index, capacity, source line}.  Not part of the public
// header; used by bounds-check runs.
rknn_status rknn_debug_zone_fault(rknn_index* ix, int32_t* out5)
{
    if (!ix || !out5 || !ix->ws.d_counters) return fail(RKNN_ERR_ARG, "no workspace");
    CK(cudaMemcpy(out5, ix->ws.d_counters + 4, sizeof(int) * 5, cudaMemcpyDeviceToHost));
    if (!out5[0]) CK(cudaMemcpy(out5, ix->ws.d_counters + 10, sizeof(int) * 5, cudaMemcpyDeviceToHost));
    return RKNN_OK;
}

rknn_status rknn_set_stream(rknn_index* ix, void* stream)
{
    if (!ix) return fail(RKNN_ERR_ARG, "index is null");
    std::lock_guard<std::mutex> lk(ix->mu);
    cudaStream_t s = stream ? (cudaStream_t)stream : ix->own_stream;
    if (s != ix->stream) {
        drop_graphs(ix->ws);
        ix->stream = s;
    }
    return RKNN_OK;
}

rknn_status rknn_sync(rknn_index* ix)
{
    if (!ix) return fail(RKNN_ERR_ARG, "index is null");
    CK(cudaStreamSynchronize(ix->stream));
    return RKNN_OK;
}

rknn_status rknn_query_batch(rknn_index* ix, const int32_t* q, const int32_t* k, int32_t nq,
                             int32_t mode, int32_t* out_ids, int64_t cap, int64_t* offsets,
                             rknn_query_stats* stats)
{
    g_err.clear();
    if (!ix || !q || !k || nq < 0 || !offsets) return fail(RKNN_ERR_ARG, "null argument");
    if (mode != RKNN_MODE_FP32 && mode != RKNN_MODE_FP64) return fail(RKNN_ERR_ARG, "bad mode");
    if (nq == 0) { offsets[0] = 0; return RKNN_OK; }
    int kmax = 1;
    rknn_status s = check_queries(ix, q, k, nq, &kmax);
    if (s != RKNN_OK) return s;
    std::lock_guard<std::mutex> lk(ix->mu);
    CK(cudaSetDevice(ix->device));
    s = ensure_ws(ix, nq, caps_fit(ix, caps_for(kmax)), ix->ws.pool_cap);
    if (s != RKNN_OK) return s;
    Workspace& w = ix->ws;
    // descending k: the longest zones start first
    bool uniform = true;
    for (int i = 1; i < nq && uniform; ++i) uniform = k[i] == k[0];
    std::memcpy(w.h_q, q, sizeof(int) * nq);
    std::memcpy(w.h_k, k, sizeof(int) * nq);
    if (!uniform) {
        for (int i = 0; i < nq; ++i) w.h_order[i] = i;
        std::stable_sort(w.h_order, w.h_order + nq, [&](int a, int b) { return k[a] > k[b]; });
        CK(cudaMemcpyAsync(w.d_order, w.h_order, sizeof(int) * nq, cudaMemcpyHostToDevice, ix->stream));
    }
    CK(cudaMemcpyAsync(w.d_q, w.h_q, sizeof(int) * nq, cudaMemcpyHostToDevice, ix->stream));
    CK(cudaMemcpyAsync(w.d_k, w.h_k, sizeof(int) * nq, cudaMemcpyHostToDevice, ix->stream));
    s = run_sync(ix, nq, mode, kmax, !uniform);
    if (s != RKNN_OK) return s;
    ix->last_lc = caps_fit(ix, caps_for(kmax)).lc;
    const long long total = w.h_off[nq];
    for (int i = 0; i <= nq; ++i) offsets[i] = w.h_off[i];
    ix->last_nq = nq;
    ix->last_mode = mode;
    if (stats) {
        s = collect_stats(ix, nq, stats);
        if (s != RKNN_OK) return s;
    }
    if (total > cap || (!out_ids && total > 0))
        return fail(RKNN_ERR_CAPACITY, "output buffer holds " + std::to_string(cap) + " ids, " +
                                           std::to_string(total) + " needed");
    if (total > 0) {
        CK(cudaMemcpyAsync(out_ids, w.d_out, sizeof(int) * total, cudaMemcpyDeviceToHost, ix->stream));
        CK(cudaStreamSynchronize(ix->stream));
    }
    return RKNN_OK;
}

rknn_status rknn_query(rknn_index* ix, int32_t q, int32_t k, int32_t mode, int32_t* out_ids,
                       int64_t cap, int64_t* n_out, rknn_query_stats* stats)
{
    if (!n_out) return fail(RKNN_ERR_ARG, "n_out is null");
    int64_t off[2] = {0, 0};
    rknn_status s = rknn_query_batch(ix, &q, &k, 1, mode, out_ids, cap, off, stats);
    *n_out = off[1] - off[0];
    return s;
}

rknn_status rknn_query_batch_device(rknn_index* ix, const int32_t* d_q, const int32_t* d_k, int32_t nq,
                                    int32_t kmax, int32_t mode)
{
    g_err.clear();
    if (!ix || !d_q || !d_k || nq <= 0 || kmax <= 0) return fail(RKNN_ERR_ARG, "bad argument");
    if (mode != RKNN_MODE_FP32 && mode != RKNN_MODE_FP64) return fail(RKNN_ERR_ARG, "bad mode");
    std::lock_guard<std::mutex> lk(ix->mu);
    Workspace& w = ix->ws;
    ZoneCaps caps = caps_fit(ix, caps_for(kmax));
    ix->last_lc = caps.lc;
    rknn_status s = ensure_ws(ix, nq, caps, std::max<long long>(w.pool_cap, (long long)nq * 4096));
    if (s != RKNN_OK) return s;
    CK(cudaMemcpyAsync(w.d_q, d_q, sizeof(int) * nq, cudaMemcpyDeviceToDevice, ix->stream));
    CK(cudaMemcpyAsync(w.d_k, d_k, sizeof(int) * nq, cudaMemcpyDeviceToDevice, ix->stream));
    s = launch(ix, nq, mode, caps, false);
    ix->last_nq = nq;
    ix->last_mode = mode;
    return s;
}

rknn_status rknn_batch_device_results(rknn_index* ix, const int32_t** d_ids, const int32_t** d_offsets)
{
    if (!ix || !d_ids || !d_offsets) return fail(RKNN_ERR_ARG, "null argument");
    *d_ids = ix->ws.d_out;
    *d_offsets = ix->ws.d_out_off;
    return RKNN_OK;
}

rknn_status rknn_last_stats(rknn_index* ix, rknn_query_stats* stats)
{
    if (!ix || !stats) return fail(RKNN_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ix->mu);
    if (ix->last_nq <= 0) return fail(RKNN_ERR_STATE, "no query has run");
    return collect_stats(ix, ix->last_nq, stats);
}

rknn_status rknn_last_zone(rknn_index* ix, int32_t slot, int32_t* bis_fac, int32_t cap, int32_t* n_bis,
                           int32_t* flags)
{
    if (!ix || !n_bis) return fail(RKNN_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ix->mu);
    if (slot < 0 || slot >= ix->last_nq) return fail(RKNN_ERR_ARG, "slot out of range");
    Workspace& w = ix->ws;
    QDesc d;
    CK(cudaMemcpy(&d, w.d_qd + slot, sizeof(QDesc), cudaMemcpyDeviceToHost));
    *n_bis = d.nb;
    if (flags) *flags = d.flags;
    int n = std::min(d.nb, cap);
    if (n > 0 && bis_fac) {
        std::vector<int> pos(n);
        CK(cudaMemcpy(pos.data(), w.d_bispos + (size_t)slot * ix->last_lc, sizeof(int) * n, cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; ++i) bis_fac[i] = ix->h_fidx[pos[i]];
    }
    return RKNN_OK;
}

}  // extern "C"

// ====================================================================
// Allocation-free single query.
//
// Some callers may not allocate device memory at query time: plugins loaded
// into a host process whose device memory all belongs to that host's own
// allocator, or latency-critical serving loops that must not stall on
// cudaMalloc.  For them rknn_query_noalloc answers one query with all of
// its per-query scratch (query descriptor, half-planes, user segments,
// offsets, counters and the result pool) in one file-scope device array of
// fixed size; the kernels are the same ones rknn_query launches.  The index
// itself is built beforehand by rknn_index_create.
namespace {

constexpr size_t NOALLOC_BYTES = 16u << 20;      // 16 MiB per device, held until exit
constexpr int NOALLOC_KMAX = 128;
constexpr int NOALLOC_MAX_DEVICES = 64;

// scratch shared by every call on this device; calls are serialized below
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

struct NoallocLayout {
    int *counters, *q, *k, *cand_off, *chunk_off, *res_count, *out_off, *bispos, *pool, *out;
    QDesc* qd;
    ZStats* zst;
    float4* planes;
    int2* segs;
    VStats* vstats;
    long long pool_cap;
};

inline size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }

NoallocLayout noalloc_layout(unsigned char* base, int lc, int seg_cap)
{
    NoallocLayout L;
    size_t o = 0;
    auto take = [&](size_t bytes) { unsigned char* p = base + o; o = na_align(o + bytes); return p; };
    L.counters = (int*)take(sizeof(int) * 16);
    L.q = (int*)take(sizeof(int));
    L.k = (int*)take(sizeof(int));
    L.cand_off = (int*)take(sizeof(int) * 2);
    L.chunk_off = (int*)take(sizeof(int) * 2);
    L.res_count = (int*)take(sizeof(int));
    L.out_off = (int*)take(sizeof(int) * 2);
    L.qd = (QDesc*)take(sizeof(QDesc));
    L.zst = (ZStats*)take(sizeof(ZStats));
    L.vstats = (VStats*)take(sizeof(VStats));
    L.planes = (float4*)take(sizeof(float4) * lc);
    L.bispos = (int*)take(sizeof(int) * lc);
    L.segs = (int2*)take(sizeof(int2) * seg_cap);
    const size_t rest = NOALLOC_BYTES > o ? NOALLOC_BYTES - o : 0;
    L.pool_cap = (long long)(rest / 2 / sizeof(int)) - 64;
    L.pool = (int*)take(sizeof(int) * (size_t)L.pool_cap);
    L.out = (int*)take(sizeof(int) * (size_t)L.pool_cap);
    return L;
}

}  // namespace

extern "C" rknn_status rknn_query_noalloc(rknn_index* ix, int32_t q, int32_t k, int32_t mode,
                                          int32_t* out_ids, int64_t cap, int64_t* n_out)
{
    g_err.clear();
    if (!ix || !n_out || (cap > 0 && !out_ids)) return fail(RKNN_ERR_ARG, "null argument");
    *n_out = 0;
    if (mode != RKNN_MODE_FP32 && mode != RKNN_MODE_FP64) return fail(RKNN_ERR_ARG, "bad mode");
    if (q < 0 || q >= ix->nf) return fail(RKNN_ERR_ARG, "query index out of range");
    if (k <= 0) return fail(RKNN_ERR_ARG, "k must be a positive integer");
    if (k > NOALLOC_KMAX)
        return fail(RKNN_ERR_CAPACITY, "rknn_query_noalloc supports k <= 128 (fixed scratch); use rknn_query");
    if (ix->device < 0 || ix->device >= NOALLOC_MAX_DEVICES) return fail(RKNN_ERR_ARG, "device ordinal too large");

    std::lock_guard<std::mutex> glk(g_noalloc_mu);
    std::lock_guard<std::mutex> lk(ix->mu);
    CK(cudaSetDevice(ix->device));
    // once per device, with that device current: the array's device address
    if (!g_noalloc_ptr[ix->device]) {
        void* p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[ix->device] = (unsigned char*)p;
    }
    const ZoneCaps caps = caps_fit(ix, caps_for(k));
    const int seg_cap = 2 * caps.rm + 2;
    NoallocLayout L = noalloc_layout(g_noalloc_ptr[ix->device], caps_for(NOALLOC_KMAX).lc, seg_cap);
    cudaStream_t st = ix->stream;

    // inputs and zeroed counters (the array keeps the previous call's contents)
    int qk[2] = {q, k};
    CK(cudaMemcpyAsync(L.q, &qk[0], sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(L.k, &qk[1], sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(L.counters, 0, sizeof(int) * 16, st));
    CK(cudaMemsetAsync(L.res_count, 0, sizeof(int), st));
    CK(cudaMemsetAsync(L.vstats, 0, sizeof(VStats), st));

    ZoneArgs za;
    za.fxy = ix->d_fxy; za.fstart = ix->d_fstart; za.fmbr = ix->d_fmbr; za.fpos = ix->d_fpos;
    za.gf = ix->gf; za.nf = (int)ix->nf;
    za.ustart = ix->d_ustart; za.gu = ix->gu; za.nu = (int)ix->nu;
    za.sx0 = ix->sx0; za.sy0 = ix->sy0; za.sx1 = ix->sx1; za.sy1 = ix->sy1;
    za.q_in = L.q; za.k_in = L.k; za.order = nullptr; za.nq = 1;
    za.work_counter = L.counters + 0;
    za.caps = caps;
    za.use_global = 0;
    za.gscratch = nullptr;
    za.skip_coincident = ix->skip_coincident;
    za.rmax = caps.rm;
    za.seg_cap = seg_cap;
    za.qd = L.qd; za.planes = L.planes; za.bis_pos = L.bispos; za.segs = L.segs; za.zst = L.zst;
    za.fault = L.counters + 4;
    const size_t zsmem = zone_layout(caps).bytes * ZONE_WARPS;
    if (zsmem > 48 * 1024)
        CK(cudaFuncSetAttribute(zone_kernel_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsmem));
    zone_kernel_smem<<<1, 32 * ZONE_WARPS, zsmem, st>>>(za);
    CK(cudaGetLastError());
    plan_kernel<<<1, 1024, 0, st>>>(L.qd, 1, L.cand_off, L.chunk_off, (int)std::min<long long>(L.pool_cap, INT32_MAX));
    CK(cudaGetLastError());

    VerifyArgs va;
    va.qd = L.qd; va.planes = L.planes; va.bis_pos = L.bispos; va.lc = caps.lc;
    va.segs = L.segs; va.seg_cap = seg_cap;
    va.chunk_off = L.chunk_off; va.cand_off = L.cand_off; va.nq = 1;
    va.uxy = ix->d_uxy; va.uid = ix->d_uid; va.fxy = ix->d_fxy; va.fstart = ix->d_fstart; va.gf = ix->gf;
    va.res_count = L.res_count; va.res_pool = L.pool; va.work_counter = L.counters + 1;
    va.vstats = L.vstats; va.mode = mode;
    va.nu = (int)ix->nu; va.nf = (int)ix->nf; va.ncf = ix->gf.gx * ix->gf.gy;
    va.pool_cap = L.pool_cap; va.fault = L.counters + 10;
    const size_t vsmem = (size_t)VERIFY_WARPS * caps.lc * (mode == MODE_FP32 ? 16 : 32);
    if (vsmem > 48 * 1024)
        CK(cudaFuncSetAttribute(verify_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vsmem));
    verify_kernel<<<2 * ix->num_sms, VERIFY_WARPS * 32, vsmem, st>>>(va);
    CK(cudaGetLastError());
    scan_counts_kernel<<<1, 1024, 0, st>>>(L.res_count, 1, L.out_off);
    CK(cudaGetLastError());
    CK(cudaFuncSetAttribute(finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)(SORT_CAP * sizeof(unsigned))));
    finalize_kernel<<<1, 256, SORT_CAP * sizeof(unsigned), st>>>(L.pool, L.cand_off, L.res_count, L.out_off,
                                                                  L.out, 1);
    CK(cudaGetLastError());

    QDesc d;
    int off[2] = {0, 0};
    CK(cudaMemcpyAsync(&d, L.qd, sizeof(QDesc), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(off, L.out_off, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (d.flags & QF_RESULT_OVERFLOW)
        return fail(RKNN_ERR_CAPACITY, "rknn_query_noalloc: the query's candidate users exceed the fixed "
                                       "scratch (about 2M); use rknn_query");
    const int64_t n = off[1];
    *n_out = n;
    if (n > cap) return fail(RKNN_ERR_CAPACITY, "output buffer too small");
    if (n > 0) {
        CK(cudaMemcpyAsync(out_ids, L.out, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return RKNN_OK;
}
