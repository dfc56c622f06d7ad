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
//   finalize_kernel  one warp per query (the block for large sets): sort its
//                    ids into the output
#include "../../include/rknn_gpu.h"
#include "index.cuh"
#include "rknn_common.cuh"
#include "verify.cuh"
#include "zone.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <utility>
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

// Drops the cached device address of the no-alloc scratch array on one
// device (defined with that entry point below).
void noalloc_forget(int device);

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

// A cached graph is keyed by everything its launches depend on: batch size,
// mode, order, result-pool size and the (size, largest k) of each k class.
using GraphKey = std::vector<long long>;

constexpr int NAUX = 3;            // side streams for concurrent k-class zone launches
constexpr int MAX_CLASSES = 16;

// A captured batch: its graph, the executable, and the filter kernels'
// nodes with their arguments, so that the query arrays can be re-pointed per
// call (the caller's device arrays, or the page-locked staging) without
// copies or a new capture.
struct CachedGraph {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaGraphNode_t> fnodes;
    std::vector<cudaKernelNodeParams> fparams;
    std::vector<ZoneArgs> fargs;
    const int *q = nullptr, *k = nullptr, *order = nullptr;   // what the filter nodes read now
};

constexpr int ZB_COUNTERS = 64;     // counter ints at the head of the zeroed block
// most candidates the fused slice filter verifies itself (more go to the
// verification kernel, which spreads a slot over the whole GPU)
constexpr int FUSE_CAND = 4096;
constexpr int ZB_VSTATS_INTS = 32;  // room for the statistics after them
// counter ints: 1 verification work, 2 dropped, 3 listed survivors, 4-8 and
// 10-14 bounds-check records, 16-31 slice filter work per k class, 36
// slots the fused filter left over, 37 its blocks done, 40-41 the 64-bit
// result-region total

struct Workspace {
    bool last_fuse = false;        // the last batch ran the fused verification
    int nq_cap = 0, lc = 0, seg_cap = 0;
    // a batch of nq queries: q at [0, nq), k at [nq, 2 nq), the k order at
    // [2 nq, 3 nq) of one buffer, on the device and in page-locked staging,
    // so that one copy moves them
    int* d_qko = nullptr;
    QDesc* d_qd = nullptr;
    float4* d_planes = nullptr;
    float* d_slice_r = nullptr;    // [slot][32] slice filter bounds
    int* d_bispos = nullptr;
    int2* d_segs = nullptr;
    ZStats* d_zst = nullptr;
    long long* d_cand_off = nullptr;   // result region of each slot (64-bit offsets)
    int* d_reg_len = nullptr;          // and its length
    int* d_deflist = nullptr;          // slots the fused filter leaves to the verification kernel
    int *d_chunk_off = nullptr, *d_res_count = nullptr, *d_out_off = nullptr;
    int rcap = 1 << 18;            // ids a slot's region holds at most (raised when exceeded)
    int* d_counters = nullptr;     // ZB_COUNTERS ints, then the statistics and the result counts:
                                   // [0] zone work, [1] verify work, [2] region exceeded,
                                   // [3] survivors listed, [4..8] zone fault record,
                                   // [10..14] verify fault record, [16..31] zone work per k class
                                   // (the block of the last batch launched: one of d_zb)
    int* d_zb[2] = {nullptr, nullptr};   // two such blocks, used by alternate batches: each
                                         // batch's finalize clears the other for the next one,
                                         // so no batch starts with a memset
    int zb_next = 0;               // the block the next batch uses
    long long zb_ints = 0;         // ints in each block
    VStats* d_vstats = nullptr;
    int *d_pool = nullptr, *d_out = nullptr;
    long long pool_cap = 0;
    int2* d_surv = nullptr;        // survivors of the half-plane filter, for recount_kernel
    long long surv_cap = 0;
    char* d_zscratch = nullptr;
    size_t zscratch_bytes = 0;
    int *h_qko = nullptr, *h_off = nullptr;   // h_off: nq+1 offsets, then the run's flags (OFF_TAIL)
    int *h_qko_dev = nullptr, *h_off_dev = nullptr;   // the same, as device pointers
    int* h_ids = nullptr;
    long long h_ids_cap = 0;
    std::map<GraphKey, CachedGraph> graphs;
    cudaStream_t aux[NAUX] = {};
    cudaEvent_t fork = nullptr, join[NAUX] = {};
    bool inject_oom = false;       // failure test hook: the next ensure_ws fails (host only)
};

}  // namespace

namespace {
struct BatchPlan;
}

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
    std::vector<float> h_fxy;      // facility coordinates in input order
    std::vector<int> h_fstart, h_ustart;   // cell starts of both grids (host copies)
    bool order_est = false;        // host batches: order each k class by candidate estimate
                                   // (RKNN_ORDER=est), else by k alone
    std::vector<int32_t> h_fid;    // facility ids as given (for snapshots)
    // the input points, kept on the device so the grids can be rebuilt
    // with other cell sizes (rknn_index_tune)
    float2 *d_fin = nullptr, *d_uin = nullptr;
    int* d_uidin = nullptr;
    float fac_per_cell = 2.0f, usr_per_cell = 8.0f;
    int vupt = VERIFY_UPT;         // verification: users per lane per work item
    int vwarps = VERIFY_WARPS;     // verification: warps per block
    int skip_coincident = 1;
    int zone_vertex_test = 0;   // see rknn_index_opts.zone_vertex_test
    int filter = RKNN_FILTER_AUTO;
    int slice_min_k = 1;
    int num_sms = 0;
    int recount_grid = 0;       // one wave of recount_kernel blocks
    bool pdl = true;            // programmatic dependent launch between the batch kernels
    // the last uniform-k host batch's plan, reused by the next batch of the
    // same size, mode and k (dropped when the grids or the verification's
    // shape change)
    std::unique_ptr<BatchPlan> plan_cache;
    int plan_nq = 0, plan_mode = -1, plan_k = 0;
    bool fuse = true;           // FP32 slice batches: the filter verifies its own slots
    int zone_cta = ZCTA_THREADS;  // influence-zone batches small enough for a block per query run
                                  // the one-block kernel with this many threads (RKNN_ZONE_CTA:
                                  // 0 = the one-warp kernel, 128 or 256)
                                // (RKNN_FUSE=0 in the environment turns it off)
    // occupancy answers by (kernel, threads, dynamic shared memory): a batch's
    // plan asks the same few questions on every call
    std::mutex occ_mu;
    std::map<std::tuple<const void*, int, size_t>, int> occ;
    size_t smem_optin = 0;
    Workspace ws;
    std::mutex mu;
    rknn_query_stats last{};
    int last_nq = 0, last_mode = 0, last_lc = 0;
    long long last_total = 0;   // ids the previous host batch returned
    int32_t* last_out = nullptr;   // the previous host batch's id buffer and capacity
    long long last_cap = 0;
    int dev_nq = 0, dev_kmax = 0, dev_mode = 0;   // the last device batch (0: none pending a check)
    const int32_t *dev_q = nullptr, *dev_k = nullptr;   // its caller's arrays
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int profiling = 0;
    cudaEvent_t kev[7] = {};
};

namespace {

// Where a batch runs: a workspace, a stream, timing events.  The index has
// one (its own calls); a server owns one per in-flight slot.
// Where a batch reads its queries and leaves its results.  By default the
// workspace's device buffers; the host batch call instead lets the kernels
// read q, k and the order from the page-locked staging buffer and write the
// offsets (and flags) into page-locked host memory, and -- for a page-locked
// id buffer the caller passes again -- the sorted ids straight into it (all
// device-accessible host memory: no copies on the stream).
struct Io {
    const int* q = nullptr;         // the queries' facility indices (null: the workspace's d_qko)
    const int* k = nullptr;         // their k
    const int* order = nullptr;     // slots by descending k (non-uniform batches)
    int* off_host = nullptr;        // offsets and flags, mirrored into host memory
    int* ids = nullptr;             // sorted ids (null: the workspace's d_out)
    long long ids_cap = 0;          // capacity of ids (slots that would pass it are skipped)
};

struct Ctx {
    Workspace& w;
    cudaStream_t st;
    cudaEvent_t ev0, ev1;
    cudaEvent_t* kev;          // per-kernel events (profiling), or null
    double* device_ms;         // where run_sync stores the batch's device time
    Io io{};
};

Ctx main_ctx(rknn_index* ix)
{
    return Ctx{ix->ws, ix->stream, ix->ev0, ix->ev1, ix->profiling ? ix->kev : nullptr, &ix->last.device_ms};
}

void free_ws(Workspace& w)
{
    for (auto& g : w.graphs) {
        cudaGraphExecDestroy(g.second.exec);
        cudaGraphDestroy(g.second.g);
    }
    w.graphs.clear();
    cudaFree(w.d_qko);
    cudaFree(w.d_qd); cudaFree(w.d_planes); cudaFree(w.d_bispos); cudaFree(w.d_segs); cudaFree(w.d_zst);
    cudaFree(w.d_slice_r);
    cudaFree(w.d_cand_off); cudaFree(w.d_reg_len); cudaFree(w.d_deflist); cudaFree(w.d_chunk_off);
    cudaFree(w.d_out_off);
    cudaFree(w.d_zb[0]);        // the counters, statistics and result counts
    cudaFree(w.d_zb[1]);
    w.d_zb[0] = w.d_zb[1] = w.d_counters = nullptr;
    cudaFree(w.d_pool); cudaFree(w.d_out); cudaFree(w.d_zscratch); cudaFree(w.d_surv);
    cudaFreeHost(w.h_qko); cudaFreeHost(w.h_off);
    cudaFreeHost(w.h_ids);
    for (int i = 0; i < NAUX; ++i) {
        if (w.aux[i]) cudaStreamDestroy(w.aux[i]);
        if (w.join[i]) cudaEventDestroy(w.join[i]);
    }
    if (w.fork) cudaEventDestroy(w.fork);
    w = Workspace();
}

void drop_graphs(Workspace& w)
{
    for (auto& g : w.graphs) {
        cudaGraphExecDestroy(g.second.exec);
        cudaGraphDestroy(g.second.g);
    }
    w.graphs.clear();
}

// Launch geometry of the zone kernel for given caps.  The zone state always
// lives in shared memory (one warp per block); caps_fit() has already sized
// it to fit the per-block limit.
struct ZoneLaunch {
    size_t slice, smem;
    int grid;
    int threads = 32 * ZONE_WARPS;   // 64: the slice filter with two warps per query
    bool cta = false;                // zone_kernel_cta, one block of ZCTA_THREADS per query
};

// Resident blocks per SM of kernel fn at this block size and dynamic shared
// memory (at least 1), remembered per index.
int occupancy(rknn_index* ix, const void* fn, int threads, size_t smem)
{
    std::lock_guard<std::mutex> lk(ix->occ_mu);
    const auto key = std::make_tuple(fn, threads, smem);
    auto it = ix->occ.find(key);
    if (it != ix->occ.end()) return it->second;
    int per = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        per = 1;
    }
    per = std::max(per, 1);
    ix->occ.emplace(key, per);
    return per;
}

// The slice filter's kernel for a class whose largest k is kmax.
using ZoneFn = void (*)(ZoneArgs);
ZoneFn slice_fn(int kmax, bool two = false)
{
    if (two)
        return kmax <= 4 ? slice_kernel2_r4 : kmax <= 8 ? slice_kernel2_r8 : kmax <= 10 ? slice_kernel2_r10
             : kmax <= 12 ? slice_kernel2_r12
             : kmax <= 16 ? slice_kernel2_r16 : kmax <= 24 ? slice_kernel2_r24 : slice_kernel2_r32;
    return kmax <= 4 ? slice_kernel_r4 : kmax <= 8 ? slice_kernel_r8 : kmax <= 10 ? slice_kernel_r10
         : kmax <= 12 ? slice_kernel_r12
         : kmax <= 16 ? slice_kernel_r16 : kmax <= 24 ? slice_kernel_r24 : kmax <= 32 ? slice_kernel_r32
         : slice_kernel;
}

// Whether a kernel is one of the filter kernels (the readers of the query
// arrays).
bool is_filter_kernel(const void* f)
{
    for (const void* g : {(const void*)zone_kernel_smem, (const void*)zone_kernel_cta, (const void*)zone_kernel_cta_half,
                          (const void*)slice_kernel,
                          (const void*)slice_kernel_r4,
                          (const void*)slice_kernel_r8, (const void*)slice_kernel_r10, (const void*)slice_kernel_r12, (const void*)slice_kernel_r16,
                          (const void*)slice_kernel_r24, (const void*)slice_kernel_r32, (const void*)slice_kernel2_r4,
                          (const void*)slice_kernel2_r8, (const void*)slice_kernel2_r10, (const void*)slice_kernel2_r12, (const void*)slice_kernel2_r16,
                          (const void*)slice_kernel2_r24, (const void*)slice_kernel2_r32})
        if (f == g) return true;
    return false;
}

// Register-list width of the slice filter for a class's largest k (0: heap).
int slice_kr(int kmax)
{
    return kmax <= 4 ? 4 : kmax <= 8 ? 8 : kmax <= 12 ? 12 : kmax <= 16 ? 16 : kmax <= 24 ? 24 : kmax <= 32 ? 32 : 0;
}

// fuse_sc, fuse_ss > 0: the slice filter keeps that many half-planes and
// segments in shared memory for the fused verification.
ZoneLaunch zone_launch(rknn_index* ix, const ZoneCaps& c, int nq, bool slice = false, int kmax = 0,
                       int fuse_sc = 0, int fuse_ss = 0)
{
    ZoneLaunch L;
    L.slice = slice ? slice_layout(c).bytes : zone_layout(c).bytes;
    L.smem = L.slice * ZONE_WARPS;
    const bool fuse = slice && fuse_sc > 0;
    if (fuse) L.smem = fuse_layout(slice_own_bytes(L.slice, 1, 0), fuse_sc, fuse_ss).bytes;
    const int kr = slice ? slice_kr(kmax) : 0;
    if (kr > 0) {
        // two warps per query (shorter chains) when every query of the class
        // keeps a block resident; one warp each otherwise (more queries in
        // flight)
        size_t smem2 = slice_own_bytes(L.slice, 2, kr);
        if (fuse) smem2 = fuse_layout(smem2, fuse_sc, fuse_ss).bytes;
        const int per2 = occupancy(ix, (const void*)slice_fn(kmax, true), 64, smem2);
        if ((long long)nq <= (long long)per2 * ix->num_sms) {
            L.smem = smem2;
            L.threads = 64;
            L.grid = std::max(1, nq);
            return L;
        }
    }
    // (the one-block kernel tags vertex indices with bit 15 in a 16-bit list)
    if (!slice && ix->zone_cta && c.pc <= ZCTA_PQ_MAX && c.vc < 32768) {
        // the influence zone with a block per query when every query of the
        // class gets one at once: the same search, its steps spread over the
        // block (lower latency per query)
        const int nt = ix->zone_cta;
        const void* fn = nt == ZCTA_THREADS ? (const void*)zone_kernel_cta : (const void*)zone_kernel_cta_half;
        const int per = occupancy(ix, fn, nt, L.slice);
        if ((long long)nq <= (long long)per * ix->num_sms) {
            L.smem = L.slice;
            L.threads = nt;
            L.cta = true;
            L.grid = std::max(1, nq);
            return L;
        }
    }
    const int per_sm = occupancy(ix, (const void*)(slice ? slice_fn(kmax) : zone_kernel_smem), 32 * ZONE_WARPS, L.smem);
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

// Point the workspace's counters, statistics and result counts at zeroed
// block i.
void use_block(Workspace& w, int i)
{
    w.d_counters = w.d_zb[i];
    w.d_vstats = (VStats*)(w.d_counters + ZB_COUNTERS);
    w.d_res_count = w.d_counters + ZB_COUNTERS + ZB_VSTATS_INTS;
}

rknn_status grow_ws(Workspace& w, int nqc, int lc, int sc);

// Sizes a workspace for a batch.  Every failure leaves the workspace either
// as it was or released entirely (all capacities zero), never half grown: a
// failed allocation in the middle of a growth frees everything, so the next
// call allocates afresh instead of finding null arrays behind nonzero
// capacities.
rknn_status ensure_ws(Workspace& w, int nq, const ZoneCaps& caps, long long pool_need)
{
    const int seg_cap = 2 * caps.rm + 2;
    if (w.inject_oom) {
        // failure test hook (rknn_serve_inject_fault): this growth fails as
        // a cudaMalloc would, after the old arrays were released
        w.inject_oom = false;
        free_ws(w);
        return fail(RKNN_ERR_OOM, "workspace growth failed (injected for a failure test)");
    }
    if (nq > w.nq_cap || caps.lc > w.lc || seg_cap > w.seg_cap) {
        const rknn_status s = grow_ws(w, std::max(nq, w.nq_cap), std::max(caps.lc, w.lc), std::max(seg_cap, w.seg_cap));
        if (s != RKNN_OK) {
            free_ws(w);
            return s;
        }
    }
    if (!w.d_surv) {
        const long long cap = std::max<long long>(w.surv_cap, 1 << 22);
        const cudaError_t e = dalloc(w.d_surv, (size_t)cap);
        if (e != cudaSuccess) {
            w.d_surv = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? RKNN_ERR_OOM : RKNN_ERR_CUDA,
                        std::string("survivor list: ") + cudaGetErrorString(e));
        }
        w.surv_cap = cap;
    }
    if (pool_need > w.pool_cap) {
        drop_graphs(w);
        cudaFree(w.d_pool);
        cudaFree(w.d_out);
        w.d_pool = w.d_out = nullptr;
        w.pool_cap = 0;
        long long cap = std::max<long long>(pool_need, 1 << 20);
        cudaError_t e = dalloc(w.d_pool, (size_t)cap);
        if (e == cudaSuccess) e = dalloc(w.d_out, (size_t)cap);
        if (e != cudaSuccess) {
            cudaFree(w.d_pool);
            cudaFree(w.d_out);
            w.d_pool = w.d_out = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? RKNN_ERR_OOM : RKNN_ERR_CUDA,
                        std::string("result pool: ") + cudaGetErrorString(e));
        }
        w.pool_cap = cap;
    }
    return RKNN_OK;
}

// Reallocates the per-slot arrays for nqc slots (the result pool and the
// survivor list are kept out: the caller sizes them).
rknn_status grow_ws(Workspace& w, int nqc, int lc, int sc)
{
    {
        const long long pool = w.pool_cap;
        const int rcap = w.rcap;
        const long long scap = w.surv_cap;
        free_ws(w);
        w.pool_cap = pool;
        w.rcap = rcap;
        w.surv_cap = scap;
        w.nq_cap = nqc; w.lc = lc; w.seg_cap = sc;
        CK(dalloc(w.d_qko, (size_t)3 * nqc));
        CK(dalloc(w.d_qd, nqc));
        CK(dalloc(w.d_planes, (size_t)nqc * lc));
        CK(dalloc(w.d_slice_r, (size_t)nqc * 32));
        CK(dalloc(w.d_bispos, (size_t)nqc * lc));
        CK(dalloc(w.d_segs, (size_t)nqc * sc));
        CK(dalloc(w.d_zst, nqc));
        CK(dalloc(w.d_cand_off, nqc + 1)); CK(dalloc(w.d_reg_len, nqc + 1)); CK(dalloc(w.d_chunk_off, nqc + 1));
        CK(dalloc(w.d_deflist, nqc));
        // counters, statistics and per-slot result counts in one block, two
        // of them for alternate batches, both zero to begin with
        static_assert(sizeof(VStats) <= ZB_VSTATS_INTS * sizeof(int), "VStats outgrew its room");
        w.zb_ints = (long long)ZB_COUNTERS + ZB_VSTATS_INTS + nqc;
        for (int z = 0; z < 2; ++z) {
            CK(dalloc(w.d_zb[z], (size_t)w.zb_ints));
            CK(cudaMemset(w.d_zb[z], 0, sizeof(int) * (size_t)w.zb_ints));
        }
        w.zb_next = 0;
        use_block(w, 0);
        CK(dalloc(w.d_out_off, nqc + 1 + OFF_TAIL));
        for (int i = 0; i < NAUX; ++i) {
            CK(cudaStreamCreateWithFlags(&w.aux[i], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&w.join[i], cudaEventDisableTiming));
        }
        CK(cudaEventCreateWithFlags(&w.fork, cudaEventDisableTiming));
        CK(cudaMallocHost(&w.h_qko, sizeof(int) * 3 * (size_t)nqc));
        CK(cudaMallocHost(&w.h_off, sizeof(int) * (nqc + 1 + OFF_TAIL)));
        CK(cudaHostGetDevicePointer((void**)&w.h_qko_dev, w.h_qko, 0));
        CK(cudaHostGetDevicePointer((void**)&w.h_off_dev, w.h_off, 0));
        w.pool_cap = 0;
    }
    return RKNN_OK;
}

cudaError_t allow_dynamic_smem(const void* fn, int optin)
{
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, fn);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes);
}

// The verification kernel for a users-per-lane setting.
void (*verify_fn(int upt))(VerifyArgs)
{
    return upt == 2 ? verify_kernel_u2 : upt == 8 ? verify_kernel_u8 : verify_kernel;
}

// ceil(log2 k), capped: queries of one class share zone capacities
int k_class(int k)
{
    int c = 0;
    while ((1 << c) < k && c < MAX_CLASSES - 1) ++c;
    return c;
}

// One zone launch per k class, with capacities sized for the class's
// largest k: a batch of mixed k does not give every query the shared-memory
// state (and the low occupancy) of its largest k.
struct ZClass {
    int off, n, kmax;
    bool slice;                 // angular-slice filter instead of the influence zone
    ZoneCaps caps;
    ZoneLaunch zl;
};

// Capacities of the slice filter: a k-entry heap per slice, half-planes of
// the nearest facilities for the verification (no more than it stages, so
// that all of them take part in its exact shortcut).
ZoneCaps slice_caps(int kmax, int lc_cap = 512)
{
    ZoneCaps c;
    c.vc = std::max(1, kmax);
    // half-planes: the first 24 k + 60 facilities streamed (more half-planes
    // reach farther: fewer users left to the exact recount; at k=10 on the
    // uniform workload 0.03 a query instead of 0.53 with 10 k + 60)
    c.lc = (int)std::max<long long>(1, std::min<long long>(24LL * c.vc + 60, lc_cap));
    c.pc = 0;
    c.rm = 64;
    return c;
}

// Which filter a k class uses.
bool use_slice(rknn_index* ix, int kmax)
{
    if (ix->filter == RKNN_FILTER_INF) return false;
    const size_t budget = std::min<size_t>(ix->smem_optin, 200 * 1024) - 1024;
    if (slice_layout(slice_caps(kmax)).bytes > budget) return false;    // k beyond the heaps' room
    return ix->filter == RKNN_FILTER_SLICE || kmax >= ix->slice_min_k;
}

// Launch geometry of one batch, computed before any stream capture.
struct BatchPlan {
    int nq = 0, mode = 0;
    bool use_order = false;
    std::vector<ZClass> cls;
    int pstride = 0;            // half-plane row stride: the largest class lc
    int stage_cap = 0;          // half-planes the verification stages per warp
    int seg_stage = 0;          // user segments it stages per warp
    int vupt = VERIFY_UPT, vwarps = VERIFY_WARPS;
    bool fuse = false;          // the slice filter verifies its own slots (FP32, every class a slice class)
    size_t vsmem = 0;
    int vgrid = 0;
    GraphKey key;
};

// k_sorted: the batch's k in processing order (descending) when use_order,
// else null (every query in one class sized for kmax).
BatchPlan plan_batch(rknn_index* ix, int nq, int mode, bool use_order, const int* k_sorted, int kmax)
{
    BatchPlan b;
    b.nq = nq;
    b.mode = mode;
    b.use_order = use_order;
    if (use_order && k_sorted) {
        for (int i = 0; i < nq;) {
            const int c = k_class(k_sorted[i]);
            int j = i + 1;
            while (j < nq && k_class(k_sorted[j]) == c) ++j;
            int km = 1;
            for (int t = i; t < j; ++t) km = std::max(km, k_sorted[t]);   // the class's largest k
            b.cls.push_back(ZClass{i, j - i, km, false, {}, {}});
            i = j;
        }
    } else {
        b.cls.push_back(ZClass{0, nq, std::max(1, kmax), false, {}, {}});
    }
    b.key = {nq, mode, use_order ? 1 : 0};
    // half-planes the verification can stage per warp (128 KB per block at
    // 32 bytes each: FP64, and the fused filter's pre-duplicated FP32 pairs
    // for the packed FMA; the verification kernel's FP32 staging is compact)
    const int bpp = 32;
    const int stage_max = std::max(1, (128 << 10) / (ix->vwarps * bpp));
    for (auto& c : b.cls) {
        c.slice = use_slice(ix, c.kmax);
        c.caps = c.slice ? slice_caps(c.kmax, std::min(512, stage_max)) : caps_fit(ix, caps_for(c.kmax));
        b.pstride = std::max(b.pstride, c.caps.lc);
        b.key.push_back(c.n);
        b.key.push_back(c.kmax);
        b.key.push_back(c.slice ? 1 : 0);
    }
    // the verification stages each query's half-planes in shared memory, at
    // most 96 KB per block (a longer list is cut: the filter weakens, the
    // exact recount still decides)
    b.vupt = ix->vupt;
    b.vwarps = ix->vwarps;
    // a handful of queries: smaller work items spread each query's users over
    // more warps (a lone FP64 query's evaluations are bound by one warp's
    // FP64 issue rate)
    if (nq <= 16 && b.vupt > 2) b.vupt = 2;
    b.stage_cap = std::max(1, std::min(b.pstride, stage_max));
    int rm = 0;
    for (auto& c : b.cls) rm = std::max(rm, c.caps.rm);
    b.seg_stage = std::min(2 * rm + 2, 512);
    // Fused verification for FP32 batches whose every class runs the slice
    // filter two warps a query (batches that fit resident): there it takes
    // the verification kernel's latency off each query's path.  Larger
    // batches keep the separate verification, whose wider blocks hide the
    // half-plane loop's latency better than one-warp filter blocks.
    b.fuse = ix->fuse && mode == MODE_FP32;
    for (auto& c : b.cls) b.fuse = b.fuse && c.slice;
    if (b.fuse)
        for (auto& c : b.cls) {
            c.zl = zone_launch(ix, c.caps, c.n, c.slice, c.kmax, b.stage_cap, b.seg_stage);
            b.fuse = b.fuse && c.zl.threads == 64;
        }
    if (!b.fuse)
        for (auto& c : b.cls) c.zl = zone_launch(ix, c.caps, c.n, c.slice, c.kmax);
    b.key.push_back(b.fuse ? 1 : 0);
    // (the verification kernel stages FP32 half-planes in 16 bytes)
    const size_t vbpp = mode == MODE_FP32 ? 16 : (size_t)bpp;
    b.vsmem = (size_t)b.vwarps * ((size_t)b.stage_cap * vbpp + (size_t)b.seg_stage * sizeof(int2) + 32 * sizeof(float));
    const int vper = occupancy(ix, (const void*)verify_fn(b.vupt), b.vwarps * 32, b.vsmem);
    b.vgrid = vper * ix->num_sms;
    b.key.push_back(b.vupt);
    b.key.push_back(b.vwarps);
    return b;
}

// Workspace capacities a plan needs (lc = the half-plane stride).
ZoneCaps plan_caps(const BatchPlan& b)
{
    ZoneCaps c = b.cls[0].caps;
    for (auto& z : b.cls) c.rm = std::max(c.rm, z.caps.rm);
    c.lc = b.pstride;
    return c;
}

// Launch with programmatic stream serialization when pdl is set: the kernel
// may start while its predecessor in the stream drains, and waits for it with
// pdl_wait() before reading its outputs.
template <typename... Exp, typename... Act>
cudaError_t launch_k(void (*k)(Exp...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl, Act&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, std::forward<Act>(args)...);
}

// Enqueue the batch's kernels (no synchronization, no non-stream CUDA calls:
// this runs under stream capture).  k classes after the first run on side
// streams, forked from and joined back to the context's stream.
// the 64-bit total of the batch's result regions (zeroed with the counters)
inline long long* region_top(Workspace& w) { return (long long*)(w.d_counters + 40); }

rknn_status enqueue(rknn_index* ix, Ctx& c, const BatchPlan& b, bool events = false, bool chain = false)
{
    Workspace& w = c.w;
    cudaStream_t st = c.st;
    const int nq = b.nq;
    auto mark = [&](int i) { if (events) cudaEventRecord(c.kev[i], st); };
    // the counters, statistics and result counts start zero: the previous
    // batch's finalize cleared this block (or it is new)

    ZoneArgs za;
    za.fxy = ix->d_fxy; za.fstart = ix->d_fstart; za.fmbr = ix->d_fmbr; za.fpos = ix->d_fpos;
    za.gf = ix->gf; za.nf = (int)ix->nf;
    za.ustart = ix->d_ustart; za.uxy = ix->d_uxy; za.uid = ix->d_uid; za.gu = ix->gu; za.nu = (int)ix->nu;
    za.sx0 = ix->sx0; za.sy0 = ix->sy0; za.sx1 = ix->sx1; za.sy1 = ix->sy1;
    const int* qin = c.io.q ? c.io.q : w.d_qko;
    const int* kin = c.io.q ? c.io.k : w.d_qko + nq;
    const int* oin = c.io.q ? c.io.order : w.d_qko + 2 * nq;
    za.q_in = qin; za.k_in = kin;
    za.skip_coincident = ix->skip_coincident;
    za.vertex_test = ix->zone_vertex_test;
    za.seg_cap = w.seg_cap;
    za.qd = w.d_qd; za.planes = w.d_planes; za.bis_pos = w.d_bispos; za.segs = w.d_segs; za.zst = w.d_zst;
    za.slice_r = w.d_slice_r;
    za.pstride = b.pstride;
    VerifyArgs va;
    va.qd = w.d_qd; va.planes = w.d_planes; va.bis_pos = w.d_bispos; va.lc = b.pstride;
    va.slice_r = w.d_slice_r;
    va.stage_cap = b.stage_cap;
    va.segs = w.d_segs; va.seg_cap = w.seg_cap; va.seg_stage = b.seg_stage;
    va.chunk_off = w.d_chunk_off; va.cand_off = w.d_cand_off; va.reg_len = w.d_reg_len; va.nq = nq;
    va.uxy = ix->d_uxy; va.uid = ix->d_uid; va.fxy = ix->d_fxy; va.fstart = ix->d_fstart; va.gf = ix->gf;
    va.res_count = w.d_res_count; va.res_pool = w.d_pool; va.work_counter = w.d_counters + 1;
    va.vstats = w.d_vstats; va.mode = b.mode;
    va.nu = (int)ix->nu; va.nf = (int)ix->nf; va.ncf = ix->gf.gx * ix->gf.gy;
    va.pool_cap = w.pool_cap; va.fault = w.d_counters + 10; va.dropped = w.d_counters + 2;
    va.surv = w.d_surv; va.surv_cap = (int)std::min<long long>(w.surv_cap, INT32_MAX); va.surv_count = w.d_counters + 3;
    va.region_top = region_top(w);
    if (b.fuse) {
        // the verification takes only the slots the filter left over
        va.deflist = w.d_deflist;
        va.ndef = w.d_counters + 36;
    }
    za.fault = w.d_counters + 4;
    if (b.fuse) {
        za.fuse = 1;
        za.fuse_cand = FUSE_CAND;
        za.fuse_sc = b.stage_cap;
        za.fuse_ss = b.seg_stage;
        za.rcap = w.rcap;
        za.cand_off_w = w.d_cand_off;
        za.reg_len_w = w.d_reg_len;
        za.deflist = w.d_deflist;
        za.ndef = w.d_counters + 36;
        za.chunk_off_w = w.d_chunk_off;
        za.vchunk = 32 * b.vupt;
        za.done_total = 0;
        for (const ZClass& z : b.cls) za.done_total += z.zl.grid;
        za.v = va;
        za.v.done = w.d_counters + 37;
    }
    mark(0);
    const int ncls = (int)b.cls.size();
    if (ncls > 1) {
        CK(cudaEventRecord(w.fork, st));
        for (int i = 0; i < NAUX && i < ncls - 1; ++i) CK(cudaStreamWaitEvent(w.aux[i], w.fork, 0));
    }
    for (int i = 0; i < ncls; ++i) {
        const ZClass& z = b.cls[i];
        za.order = b.use_order ? oin + z.off : nullptr;
        za.nq = z.n;
        za.caps = z.caps;
        za.rmax = z.caps.rm;
        za.work_counter = w.d_counters + 16 + i;
        cudaStream_t zs = i == 0 ? st : w.aux[(i - 1) % NAUX];
        if (z.slice) slice_fn(z.kmax, z.zl.threads == 64)<<<z.zl.grid, z.zl.threads, z.zl.smem, zs>>>(za);
        else if (z.zl.cta && z.zl.threads == ZCTA_THREADS) zone_kernel_cta<<<z.zl.grid, ZCTA_THREADS, z.zl.smem, zs>>>(za);
        else if (z.zl.cta) zone_kernel_cta_half<<<z.zl.grid, ZCTA_THREADS / 2, z.zl.smem, zs>>>(za);
        else zone_kernel_smem<<<z.zl.grid, 32 * ZONE_WARPS, z.zl.smem, zs>>>(za);
        CK(cudaGetLastError());
    }
    if (ncls > 1) {
        for (int i = 0; i < NAUX && i < ncls - 1; ++i) {
            CK(cudaEventRecord(w.join[i], w.aux[i]));
            CK(cudaStreamWaitEvent(st, w.join[i], 0));
        }
    }
    mark(1);

    // the kernels after the filter start while their predecessor drains
    // (captured batches only: not between profiling events, nor after a
    // cross-stream join, nor in serving, where blocks waiting early would
    // hold resources that other slots' kernels need)
    const bool pdl = chain && !events && ix->pdl;
    // fused batches: the filter's last block planned the left-over slots,
    // and the verification takes only those
    if (!b.fuse)
        CK(launch_k(plan_kernel, 1, 1024, 0, st, pdl && ncls == 1, w.d_qd, nq, w.d_cand_off, w.d_reg_len,
                    region_top(w), w.d_chunk_off, w.pool_cap, w.rcap, 32 * b.vupt));
    mark(2);
    CK(launch_k(verify_fn(b.vupt), b.vgrid, b.vwarps * 32, b.vsmem, st, pdl && (ncls == 1 || !b.fuse), va));
    mark(3);
    CK(launch_k(recount_kernel, ix->recount_grid, 256, 0, st, pdl, va));
    mark(4);
    // the output offsets: in finalize itself for batches of up to
    // FIN_SCAN_MAX slots, else by the scan kernel
    FinScan fs;
    if (nq <= FIN_SCAN_MAX) {
        fs.on = 1;
        fs.out_off_host = c.io.off_host;
        fs.region_top = region_top(w);
        fs.counters = w.d_counters;
    } else {
        CK(launch_k(scan_counts_kernel, 1, 1024, 0, st, pdl, (const int*)w.d_res_count, (const int*)w.d_reg_len,
                    (const long long*)region_top(w), nq, w.d_out_off, (const int*)w.d_counters, c.io.off_host));
    }
    mark(5);
    int* ids = c.io.ids ? c.io.ids : w.d_out;
    const long long ids_cap = c.io.ids ? c.io.ids_cap : w.pool_cap;
    CK(launch_k(finalize_kernel, (nq + FIN_WARPS - 1) / FIN_WARPS, 32 * FIN_WARPS, 0, st, pdl, w.d_pool,
                (const long long*)w.d_cand_off, (const int*)w.d_reg_len, (const int*)w.d_res_count,
                w.d_out_off, ids, nq, ids_cap, w.d_zb[w.zb_next], w.zb_ints, fs));
    mark(6);
    return RKNN_OK;
}

// Launch a batch: replay the graph cached for its plan (captured on first
// use), or enqueue directly (profiling, or when graph is false).
rknn_status launch(rknn_index* ix, Ctx& c, const BatchPlan& b, bool graph = true)
{
    Workspace& w = c.w;
    w.last_fuse = b.fuse;
    // this batch's zeroed block; its finalize clears the other one
    const int zb = w.zb_next;
    w.zb_next ^= 1;
    use_block(w, zb);
    if (c.kev) return enqueue(ix, c, b, true);
    if (!graph) return enqueue(ix, c, b);
    GraphKey key = b.key;
    key.push_back(zb);
    key.push_back(w.pool_cap);
    key.push_back(w.rcap);
    key.push_back(w.surv_cap);
    key.push_back((long long)(uintptr_t)c.io.off_host);
    key.push_back((long long)(uintptr_t)c.io.ids);
    key.push_back(c.io.ids_cap);
    const int* q = c.io.q ? c.io.q : w.d_qko;
    const int* k = c.io.q ? c.io.k : w.d_qko + b.nq;
    const int* order = c.io.q ? c.io.order : w.d_qko + 2 * b.nq;
    auto it = w.graphs.find(key);
    if (it == w.graphs.end()) {
        CachedGraph cg;
        CK(cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal));
        rknn_status s = enqueue(ix, c, b, false, true);
        cudaError_t e = cudaStreamEndCapture(c.st, &cg.g);
        if (s != RKNN_OK) { if (e == cudaSuccess) cudaGraphDestroy(cg.g); return s; }
        CK(e);
        e = cudaGraphInstantiate(&cg.exec, cg.g, 0);
        if (e != cudaSuccess) { cudaGraphDestroy(cg.g); CK(e); }
        // the filter kernels' nodes: the only ones that read the query arrays
        size_t nn = 0;
        CK(cudaGraphGetNodes(cg.g, nullptr, &nn));
        std::vector<cudaGraphNode_t> nodes(nn);
        CK(cudaGraphGetNodes(cg.g, nodes.data(), &nn));
        for (cudaGraphNode_t nd : nodes) {
            cudaGraphNodeType t;
            CK(cudaGraphNodeGetType(nd, &t));
            if (t != cudaGraphNodeTypeKernel) continue;
            cudaKernelNodeParams kp;
            CK(cudaGraphKernelNodeGetParams(nd, &kp));
            if (!is_filter_kernel(kp.func)) continue;
            cg.fnodes.push_back(nd);
            cg.fparams.push_back(kp);
            cg.fargs.push_back(*(const ZoneArgs*)kp.kernelParams[0]);
        }
        cg.q = q;
        cg.k = k;
        cg.order = order;
        it = w.graphs.emplace(key, std::move(cg)).first;
    }
    CachedGraph& cg = it->second;
    if (cg.q != q || cg.k != k || cg.order != order) {
        for (size_t i = 0; i < cg.fnodes.size(); ++i) {
            ZoneArgs& a = cg.fargs[i];
            a.q_in = q;
            a.k_in = k;
            if (a.order) a.order = order + (a.order - cg.order);
            void* args[1] = {&a};
            cudaKernelNodeParams kp = cg.fparams[i];
            kp.kernelParams = args;
            kp.extra = nullptr;
            CK(cudaGraphExecKernelNodeSetParams(cg.exec, cg.fnodes[i], &kp));
        }
        cg.q = q;
        cg.k = k;
        cg.order = order;
    }
    CK(cudaGraphLaunch(cg.exec, c.st));
    return RKNN_OK;
}

rknn_status collect_stats(Ctx& c, int nq, rknn_query_stats* out)
{
    Workspace& w = c.w;
    std::vector<ZStats> z(nq);
    std::vector<QDesc> qd(nq);
    VStats v;
    CK(cudaMemcpyAsync(z.data(), w.d_zst, sizeof(ZStats) * nq, cudaMemcpyDeviceToHost, c.st));
    CK(cudaMemcpyAsync(qd.data(), w.d_qd, sizeof(QDesc) * nq, cudaMemcpyDeviceToHost, c.st));
    CK(cudaMemcpyAsync(&v, w.d_vstats, sizeof(VStats), cudaMemcpyDeviceToHost, c.st));
    int ndef = 0;
    CK(cudaMemcpyAsync(&ndef, w.d_counters + 36, sizeof(int), cudaMemcpyDeviceToHost, c.st));
    CK(cudaStreamSynchronize(c.st));
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
    s.fused_slots = w.last_fuse ? nq - ndef : 0;
    s.device_ms = *c.device_ms;
    *out = s;
    return RKNN_OK;
}

// Run a batch whose q/k are already in the workspace (d_qko).  Grows the result
// pool and reruns when a query's candidate region did not fit.
// Launch, read the offsets and counters back, and rerun when a region or the
// pool was too small.  spec (page-locked, spec_n ids) takes a speculative copy
// of the first spec_n result ids in the same stream round trip: when the batch
// returned at most spec_n ids the caller needs no second copy.
// The flags scan_counts_kernel leaves after the nq+1 offsets (OFF_TAIL ints):
// the sum of the result regions (two halves), whether a slot had more
// results than its region, and how many survivors were listed.
struct RunTail {
    long long region_total;
    int dropped, survivors;
};

RunTail run_tail(const int* h_off, int nq)
{
    const int* t = h_off + nq + 1;
    RunTail r;
    r.region_total = (long long)(((unsigned long long)(unsigned)t[1] << 32) | (unsigned)t[0]);
    r.dropped = t[2];
    r.survivors = t[3];
    return r;
}

rknn_status run_sync(rknn_index* ix, Ctx& c, const BatchPlan& b, bool graph = true, int* spec = nullptr,
                     long long spec_n = 0)
{
    Workspace& w = c.w;
    const int nq = b.nq;
    const ZoneCaps caps = plan_caps(b);
    long long need = std::max<long long>(w.pool_cap, (long long)nq * 4096);
    rknn_status s = ensure_ws(w, nq, caps, need);
    if (s != RKNN_OK) return s;
    for (int attempt = 0; attempt < 8; ++attempt) {
        CK(cudaEventRecord(c.ev0, c.st));
        s = launch(ix, c, b, graph);
        if (s != RKNN_OK) return s;
        CK(cudaEventRecord(c.ev1, c.st));
        // offsets and the run's flags in one copy (none when the scan wrote
        // them to host memory itself)
        if (c.io.off_host != w.h_off_dev || !c.io.off_host)
            CK(cudaMemcpyAsync(w.h_off, w.d_out_off, sizeof(int) * (nq + 1 + OFF_TAIL), cudaMemcpyDeviceToHost, c.st));
        const long long sn = std::min(spec_n, w.pool_cap);
        if (spec && sn > 0) CK(cudaMemcpyAsync(spec, w.d_out, sizeof(int) * sn, cudaMemcpyDeviceToHost, c.st));
        CK(cudaStreamSynchronize(c.st));
        float ms = 0;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        *c.device_ms = ms;
        const RunTail tail = run_tail(w.h_off, nq);
        const long long region_total = tail.region_total;
        const int dropped = tail.dropped;
        const int flags[2] = {tail.dropped, tail.survivors};
#ifdef RKNN_CHECKED
        {
            // bounds-checked build: a recorded out-of-range access fails the batch
            int rec[16];
            CK(cudaMemcpy(rec, w.d_counters, sizeof(rec), cudaMemcpyDeviceToHost));
            for (int base : {4, 10})
                if (rec[base])
                    return fail(RKNN_ERR_CUDA, "bounds check: array " + std::to_string(rec[base + 1]) + " index " +
                                                       std::to_string(rec[base + 2]) + " of " +
                                                       std::to_string(rec[base + 3]) + " at line " +
                                                       std::to_string(rec[base + 4]));
        }
#endif
        if ((unsigned)flags[1] > (unsigned long long)w.surv_cap) {
            // survivors overflowed the list (they were recounted in-warp):
            // give the next batch room for all of them
            drop_graphs(w);
            cudaFree(w.d_surv);
            w.d_surv = nullptr;
            w.surv_cap = (long long)(unsigned)flags[1] + (long long)(unsigned)flags[1] / 4;
            s = ensure_ws(w, nq, caps, w.pool_cap);
            if (s != RKNN_OK) return s;
        }
        if (region_total > w.pool_cap) {
            // some regions did not fit the pool (those slots were skipped)
            s = ensure_ws(w, nq, caps, region_total + region_total / 4);
            if (s != RKNN_OK) return s;
            continue;
        }
        if (dropped) {
            // a slot had more results than its region: give every slot more room
            w.rcap = (int)std::min<long long>((long long)w.rcap * 8, std::max<long long>(ix->nu, 1));
            continue;
        }
        return RKNN_OK;
    }
    return fail(RKNN_ERR_CAPACITY, "result pool could not be sized");
}

rknn_status check_queries(rknn_index* ix, const int32_t* q, const int32_t* k, int nq, int* kmax,
                          bool* uniform = nullptr)
{
    // one pass of minima and maxima; the error message comes from the
    // second loop only when a query is bad
    int32_t qlo = INT32_MAX, qhi = INT32_MIN, klo = INT32_MAX, khi = INT32_MIN;
    for (int i = 0; i < nq; ++i) {
        qlo = std::min(qlo, q[i]);
        qhi = std::max(qhi, q[i]);
        klo = std::min(klo, k[i]);
        khi = std::max(khi, k[i]);
    }
    if (nq > 0 && qlo >= 0 && (int64_t)qhi < ix->nf && klo > 0) {
        *kmax = std::max(1, (int)khi);
        if (uniform) *uniform = klo == khi;
        return RKNN_OK;
    }
    *kmax = 1;
    if (uniform) *uniform = true;
    for (int i = 0; i < nq; ++i) {
        if (q[i] < 0 || q[i] >= ix->nf)
            return fail(RKNN_ERR_ARG, "query index " + std::to_string(q[i]) + " out of range [0, " +
                                          std::to_string(ix->nf) + ")");
        if (k[i] <= 0) return fail(RKNN_ERR_ARG, "k must be a positive integer");
        *kmax = std::max(*kmax, (int)k[i]);
    }
    return RKNN_OK;
}

// (Re)build the facility and user grids from the device copies of the input
// points: cell ids, stable radix sort, cell starts, per-cell facility boxes.
rknn_status build_grids(rknn_index* ix, float fac_per_cell, float usr_per_cell)
{
    ix->plan_cache.reset();
    cudaStream_t st = ix->stream;
    CK(cudaStreamSynchronize(st));
    cudaFree(ix->d_fxy); cudaFree(ix->d_fidx); cudaFree(ix->d_fpos); cudaFree(ix->d_fstart);
    cudaFree(ix->d_fmbr); cudaFree(ix->d_uxy); cudaFree(ix->d_uid); cudaFree(ix->d_ustart);
    ix->d_fxy = nullptr; ix->d_fidx = ix->d_fpos = ix->d_fstart = nullptr; ix->d_fmbr = nullptr;
    ix->d_uxy = nullptr; ix->d_uid = ix->d_ustart = nullptr;
    drop_graphs(ix->ws);                        // graphs hold the old grids' pointers
    const long long nf = ix->nf, nu = ix->nu;
    ix->fac_per_cell = fac_per_cell;
    ix->usr_per_cell = usr_per_cell;
    ix->gf = make_grid(ix->sx0, ix->sy0, ix->sx1, ix->sy1, nf, fac_per_cell, 4096);
    ix->gu = make_grid(ix->sx0, ix->sy0, ix->sx1, ix->sy1, nu, usr_per_cell, 8192);
    const long long ncf = (long long)ix->gf.gx * ix->gf.gy, ncu = (long long)ix->gu.gx * ix->gu.gy;
    CK(dalloc(ix->d_fxy, nf));
    CK(dalloc(ix->d_fidx, nf));
    CK(dalloc(ix->d_fpos, nf));
    CK(dalloc(ix->d_fstart, ncf + 1));
    CK(dalloc(ix->d_fmbr, ncf));
    CK(dalloc(ix->d_uxy, nu));
    CK(dalloc(ix->d_uid, nu));
    CK(dalloc(ix->d_ustart, ncu + 1));
    CK(grid_sort(ix->d_fin, nullptr, (int)nf, ix->gf, ix->d_fxy, nullptr, ix->d_fidx, ix->d_fpos, ix->d_fstart, st));
    CK(cell_mbrs(ix->d_fxy, ix->d_fstart, ix->gf, ix->d_fmbr, st));
    CK(grid_sort(ix->d_uin, ix->d_uidin, (int)nu, ix->gu, ix->d_uxy, ix->d_uid, nullptr, nullptr, ix->d_ustart, st));
    ix->h_fidx.resize(nf);
    CK(cudaMemcpyAsync(ix->h_fidx.data(), ix->d_fidx, sizeof(int) * nf, cudaMemcpyDeviceToHost, st));
    ix->h_fstart.resize(ncf + 1);
    ix->h_ustart.resize(ncu + 1);
    CK(cudaMemcpyAsync(ix->h_fstart.data(), ix->d_fstart, sizeof(int) * (ncf + 1), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ix->h_ustart.data(), ix->d_ustart, sizeof(int) * (ncu + 1), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return RKNN_OK;
}

// Cheap estimate of a query's candidate users: k times the users per
// facility around q -- the facilities of the 5 x 5 facility cells centred
// on q's cell and the users of the user cells covering the same box, from
// the host copies of both grids' cell starts.  Used only to order work.
double cand_estimate(const rknn_index* ix, int q, int k)
{
    const Grid& g = ix->gf;
    const Grid& u = ix->gu;
    const float x = ix->h_fxy[2 * (size_t)q], y = ix->h_fxy[2 * (size_t)q + 1];
    const int cx = cell_coord(x, g.x0, g.inv, g.gx), cy = cell_coord(y, g.y0, g.inv, g.gy);
    const int x0 = std::max(0, cx - 2), x1 = std::min(g.gx - 1, cx + 2);
    const int y0 = std::max(0, cy - 2), y1 = std::min(g.gy - 1, cy + 2);
    long long nfac = 0;
    for (int r = y0; r <= y1; ++r)
        nfac += ix->h_fstart[(size_t)r * g.gx + x1 + 1] - ix->h_fstart[(size_t)r * g.gx + x0];
    const int ux0 = cell_coord(g.x0 + (float)x0 * g.cs, u.x0, u.inv, u.gx);
    const int ux1 = cell_coord(g.x0 + (float)(x1 + 1) * g.cs, u.x0, u.inv, u.gx);
    const int uy0 = cell_coord(g.y0 + (float)y0 * g.cs, u.y0, u.inv, u.gy);
    const int uy1 = cell_coord(g.y0 + (float)(y1 + 1) * g.cs, u.y0, u.inv, u.gy);
    long long nusr = 0;
    for (int r = uy0; r <= uy1; ++r)
        nusr += ix->h_ustart[(size_t)r * u.gx + ux1 + 1] - ix->h_ustart[(size_t)r * u.gx + ux0];
    return (double)k * (double)nusr / (double)std::max(nfac, 1LL);
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
    if (o.zone_vertex_test != 0 && o.zone_vertex_test != 1) return bail(fail(RKNN_ERR_ARG, "zone_vertex_test must be 0 or 1"));
    ix->zone_vertex_test = o.zone_vertex_test;
    if (o.filter < RKNN_FILTER_AUTO || o.filter > RKNN_FILTER_SLICE) return bail(fail(RKNN_ERR_ARG, "bad filter"));
    ix->filter = o.filter;
    ix->slice_min_k = o.slice_min_k > 0 ? o.slice_min_k : 1;
    if (const char* f = std::getenv("RKNN_FUSE")) ix->fuse = std::strcmp(f, "0") != 0;
    if (const char* f = std::getenv("RKNN_ZONE_CTA")) {
        const int v = std::atoi(f);
        ix->zone_cta = v == 0 ? 0 : v == ZCTA_THREADS / 2 ? ZCTA_THREADS / 2 : ZCTA_THREADS;
    }
    ix->nf = nf;
    ix->nu = nu;
    ix->h_fxy.assign(fxy, fxy + 2 * nf);
    if (const char* f = std::getenv("RKNN_ORDER")) ix->order_est = std::strcmp(f, "est") == 0;
    if (fid) ix->h_fid.assign(fid, fid + nf);
    else {
        ix->h_fid.resize(nf);
        for (int64_t i = 0; i < nf; ++i) ix->h_fid[i] = (int32_t)i;
    }
    ix->sx0 = x0; ix->sy0 = y0; ix->sx1 = x1; ix->sy1 = y1;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return bail(fail(RKNN_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e)));
    if (o.device < 0 || o.device >= ndev) return bail(fail(RKNN_ERR_ARG, "bad device ordinal"));
    noalloc_forget(o.device);
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
    // dynamic shared memory limit of the batch kernels: the device's opt-in
    // maximum less the kernel's static shared memory, set once (each launch
    // asks for what its plan needs)
    CKB(allow_dynamic_smem((const void*)zone_kernel_smem, optin));
    CKB(allow_dynamic_smem((const void*)zone_kernel_cta, optin));
    CKB(allow_dynamic_smem((const void*)zone_kernel_cta_half, optin));
    {
        int per = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, recount_kernel, 256, 0);
        ix->recount_grid = std::max(1, per) * ix->num_sms;
    }
    CKB(allow_dynamic_smem((const void*)slice_kernel, optin));
    for (const void* f : {(const void*)slice_kernel_r4, (const void*)slice_kernel_r8, (const void*)slice_kernel_r10, (const void*)slice_kernel_r12,
                          (const void*)slice_kernel_r16, (const void*)slice_kernel_r24, (const void*)slice_kernel_r32,
                          (const void*)slice_kernel2_r4, (const void*)slice_kernel2_r8, (const void*)slice_kernel2_r10, (const void*)slice_kernel2_r12,
                          (const void*)slice_kernel2_r16, (const void*)slice_kernel2_r24, (const void*)slice_kernel2_r32})
        CKB(allow_dynamic_smem(f, optin));
    CKB(allow_dynamic_smem((const void*)verify_kernel, optin));
    CKB(allow_dynamic_smem((const void*)verify_kernel_u2, optin));
    CKB(allow_dynamic_smem((const void*)verify_kernel_u8, optin));

    if (o.users_per_thread != 0 && o.users_per_thread != 2 && o.users_per_thread != 4 && o.users_per_thread != 8)
        return bail(fail(RKNN_ERR_ARG, "users_per_thread must be 2, 4 or 8"));
    if (o.verify_warps != 0 && o.verify_warps != 4 && o.verify_warps != 8 && o.verify_warps != 16)
        return bail(fail(RKNN_ERR_ARG, "verify_warps must be 4, 8 or 16"));
    if (o.users_per_thread) ix->vupt = o.users_per_thread;
    if (o.verify_warps) ix->vwarps = o.verify_warps;
    cudaStream_t st = ix->stream;
    CKB(dalloc(ix->d_fin, nf));
    CKB(cudaMemcpyAsync(ix->d_fin, fxy, sizeof(float2) * nf, cudaMemcpyHostToDevice, st));
    if (nu > 0) {
        CKB(dalloc(ix->d_uin, nu));
        CKB(dalloc(ix->d_uidin, nu));
        CKB(cudaMemcpyAsync(ix->d_uin, uxy, sizeof(float2) * nu, cudaMemcpyHostToDevice, st));
        CKB(cudaMemcpyAsync(ix->d_uidin, uid, sizeof(int) * nu, cudaMemcpyHostToDevice, st));
    }
    {
        rknn_status bs = build_grids(ix, o.fac_per_cell, o.usr_per_cell);
        if (bs != RKNN_OK) return bail(bs);
    }
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
    cudaFree(ix->d_fin); cudaFree(ix->d_uin); cudaFree(ix->d_uidin);
    if (ix->ev0) cudaEventDestroy(ix->ev0);
    if (ix->ev1) cudaEventDestroy(ix->ev1);
    for (int i = 0; i < 7; ++i) if (ix->kev[i]) cudaEventDestroy(ix->kev[i]);
    if (ix->own_stream) cudaStreamDestroy(ix->own_stream);
    delete ix;
    return RKNN_OK;
}

// ---------------------------------------------------------------- snapshots
namespace {
constexpr char SNAP_MAGIC[8] = {'R', 'K', 'N', 'N', 'S', 'N', 'P', '1'};

// FNV-1a over 64-bit little-endian words (the tail zero-padded), streamed.
struct SnapHash {
    uint64_t h = 1469598103934665603ull;
    unsigned char pend[8];
    int npend = 0;
    void word(uint64_t w)
    {
        h ^= w;
        h *= 1099511628211ull;
    }
    static uint64_t le64(const unsigned char* p)
    {
        uint64_t w = 0;
        for (int i = 7; i >= 0; --i) w = (w << 8) | p[i];
        return w;
    }
    void add(const void* data, size_t n)
    {
        const unsigned char* p = (const unsigned char*)data;
        while (n && npend) {
            pend[npend++] = *p++;
            --n;
            if (npend == 8) { word(le64(pend)); npend = 0; }
        }
        for (; n >= 8; n -= 8, p += 8) word(le64(p));
        while (n--) pend[npend++] = *p++;
    }
    uint64_t done()
    {
        if (npend) {
            while (npend < 8) pend[npend++] = 0;
            word(le64(pend));
            npend = 0;
        }
        return h;
    }
};

// Writes n bytes and adds them to the hash.
bool snap_put(FILE* f, SnapHash& hs, const void* p, size_t n)
{
    hs.add(p, n);
    return n == 0 || std::fwrite(p, 1, n, f) == n;
}

bool snap_get(FILE* f, SnapHash& hs, void* p, size_t n)
{
    if (n && std::fread(p, 1, n, f) != n) return false;
    hs.add(p, n);
    return true;
}
}  // namespace

rknn_status rknn_snapshot_write(const char* path, const float* fxy, const int32_t* fid, int64_t nf,
                                const float* uxy, const int32_t* uid, int64_t nu)
{
    g_err.clear();
    if (!path || !fxy || !fid || nf < 1 || nu < 0 || (nu > 0 && (!uxy || !uid)))
        return fail(RKNN_ERR_ARG, "bad snapshot arguments");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(RKNN_ERR_ARG, std::string("cannot write ") + path);
    SnapHash hs;
    const uint32_t ver[2] = {1, 0};
    const int64_t n[2] = {nf, nu};
    bool ok = snap_put(f, hs, SNAP_MAGIC, 8) && snap_put(f, hs, ver, sizeof(ver)) && snap_put(f, hs, n, sizeof(n)) &&
              snap_put(f, hs, fxy, sizeof(float) * 2 * (size_t)nf) && snap_put(f, hs, fid, sizeof(int32_t) * (size_t)nf) &&
              snap_put(f, hs, uxy, sizeof(float) * 2 * (size_t)nu) && snap_put(f, hs, uid, sizeof(int32_t) * (size_t)nu);
    const uint64_t h = hs.done();
    ok = ok && std::fwrite(&h, 1, sizeof(h), f) == sizeof(h);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(RKNN_ERR_ARG, std::string("write failed: ") + path);
    return RKNN_OK;
}

rknn_status rknn_snapshot_read(const char* path, float** fxy, int32_t** fid, int64_t* nf, float** uxy,
                               int32_t** uid, int64_t* nu)
{
    g_err.clear();
    if (!path || !fxy || !fid || !nf || !uxy || !uid || !nu) return fail(RKNN_ERR_ARG, "null argument");
    *fxy = *uxy = nullptr;
    *fid = *uid = nullptr;
    *nf = *nu = 0;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(RKNN_ERR_ARG, std::string("cannot open ") + path);
    SnapHash hs;
    char magic[8];
    uint32_t ver[2];
    int64_t n[2];
    if (!snap_get(f, hs, magic, 8) || std::memcmp(magic, SNAP_MAGIC, 8) != 0 || !snap_get(f, hs, ver, sizeof(ver)) ||
        ver[0] != 1 || !snap_get(f, hs, n, sizeof(n)) || n[0] < 1 || n[1] < 0 || n[0] >= INT32_MAX / 2 ||
        n[1] >= INT32_MAX / 2) {
        std::fclose(f);
        return fail(RKNN_ERR_ARG, std::string("not an index snapshot: ") + path);
    }
    float* a = (float*)std::malloc(sizeof(float) * 2 * (size_t)n[0]);
    int32_t* b = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)n[0]);
    float* c = (float*)std::malloc(sizeof(float) * 2 * (size_t)std::max<int64_t>(n[1], 1));
    int32_t* d = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(n[1], 1));
    uint64_t h = 0;
    bool ok = a && b && c && d && snap_get(f, hs, a, sizeof(float) * 2 * (size_t)n[0]) &&
              snap_get(f, hs, b, sizeof(int32_t) * (size_t)n[0]) && snap_get(f, hs, c, sizeof(float) * 2 * (size_t)n[1]) &&
              snap_get(f, hs, d, sizeof(int32_t) * (size_t)n[1]);
    const uint64_t want = hs.done();
    ok = ok && std::fread(&h, 1, sizeof(h), f) == sizeof(h) && h == want;
    std::fclose(f);
    if (!ok) {
        std::free(a); std::free(b); std::free(c); std::free(d);
        return fail(RKNN_ERR_ARG, std::string("truncated or corrupt index snapshot: ") + path);
    }
    *fxy = a; *fid = b; *uxy = c; *uid = d;
    *nf = n[0]; *nu = n[1];
    return RKNN_OK;
}

void rknn_snapshot_free(void* p) { std::free(p); }

rknn_status rknn_index_open(const char* path, const rknn_index_opts* opts, rknn_index** out)
{
    float *fxy = nullptr, *uxy = nullptr;
    int32_t *fid = nullptr, *uid = nullptr;
    int64_t nf = 0, nu = 0;
    rknn_status s = rknn_snapshot_read(path, &fxy, &fid, &nf, &uxy, &uid, &nu);
    if (s != RKNN_OK) return s;
    s = rknn_index_create(fxy, fid, nf, uxy, uid, nu, opts, out);
    std::free(fxy); std::free(fid); std::free(uxy); std::free(uid);
    return s;
}

rknn_status rknn_index_save(const rknn_index* ix, const char* path)
{
    g_err.clear();
    if (!ix || !path) return fail(RKNN_ERR_ARG, "null argument");
    std::vector<float> fxy(2 * (size_t)ix->nf), uxy(2 * (size_t)ix->nu);
    std::vector<int32_t> uid((size_t)ix->nu);
    CK(cudaSetDevice(ix->device));
    CK(cudaMemcpy(fxy.data(), ix->d_fin, sizeof(float) * fxy.size(), cudaMemcpyDeviceToHost));
    if (ix->nu > 0) {
        CK(cudaMemcpy(uxy.data(), ix->d_uin, sizeof(float) * uxy.size(), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(uid.data(), ix->d_uidin, sizeof(int32_t) * uid.size(), cudaMemcpyDeviceToHost));
    }
    return rknn_snapshot_write(path, fxy.data(), ix->h_fid.data(), ix->nf, uxy.data(), uid.data(), ix->nu);
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
        for (int i = 0; i < 7; ++i) CK(cudaEventCreate(&ix->kev[i]));
    ix->profiling = on ? 1 : 0;
    return RKNN_OK;
}

rknn_status rknn_last_kernel_ms(rknn_index* ix, double* ms)
{
    if (!ix || !ms) return fail(RKNN_ERR_ARG, "null argument");
    if (!ix->kev[0]) return fail(RKNN_ERR_STATE, "profiling was never enabled");
    CK(cudaEventSynchronize(ix->kev[6]));
    for (int i = 0; i < 6; ++i) {
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

// Per-query zone statistics of the last call (nq records of the kernel's
// ZStats layout: 8 ints, then 8 int64 cycle counters).  Not part of the
// public header; used by profiling runs.
rknn_status rknn_debug_zone_stats(rknn_index* ix, void* out, int32_t nq)
{
    if (!ix || !out || nq < 0 || !ix->ws.d_zst) return fail(RKNN_ERR_ARG, "no workspace");
    std::lock_guard<std::mutex> lk(ix->mu);
    if (nq > ix->last_nq) return fail(RKNN_ERR_ARG, "more records than the last call's queries");
    CK(cudaStreamSynchronize(ix->stream));
    CK(cudaMemcpy(out, ix->ws.d_zst, sizeof(ZStats) * (size_t)nq, cudaMemcpyDeviceToHost));
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
    bool uniform = true;
    rknn_status s = check_queries(ix, q, k, nq, &kmax, &uniform);
    if (s != RKNN_OK) return s;
    std::lock_guard<std::mutex> lk(ix->mu);
    CK(cudaSetDevice(ix->device));
    ix->dev_nq = 0;     // the workspace now holds this batch
    // descending k: the longest zones start first, and each k class gets its
    // own zone launch
    std::vector<int> order, ksorted;
    const bool use_order = !uniform || ix->order_est;
    if (use_order) {
        order.resize(nq);
        for (int i = 0; i < nq; ++i) order[i] = i;
        if (ix->order_est) {
            // each k class in descending candidate estimate (longest first)
            std::vector<double> est(nq);
            for (int i = 0; i < nq; ++i) est[i] = cand_estimate(ix, q[i], k[i]);
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                const int ca = k_class(k[a]), cb = k_class(k[b]);
                return ca != cb ? ca > cb : est[a] > est[b];
            });
        } else {
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return k[a] > k[b]; });
        }
        ksorted.resize(nq);
        for (int i = 0; i < nq; ++i) ksorted[i] = k[order[i]];
    }
    BatchPlan fresh;
    const BatchPlan* bp = nullptr;
    if (!use_order && ix->plan_cache && ix->plan_nq == nq && ix->plan_mode == mode && ix->plan_k == kmax) {
        bp = ix->plan_cache.get();
    } else {
        fresh = plan_batch(ix, nq, mode, use_order, use_order ? ksorted.data() : nullptr, kmax);
        bp = &fresh;
        if (!use_order) {
            ix->plan_cache = std::make_unique<BatchPlan>(fresh);
            ix->plan_nq = nq;
            ix->plan_mode = mode;
            ix->plan_k = kmax;
            bp = ix->plan_cache.get();
        }
    }
    const BatchPlan& b = *bp;
    s = ensure_ws(ix->ws, nq, plan_caps(b), ix->ws.pool_cap);
    if (s != RKNN_OK) return s;
    Workspace& w = ix->ws;
    Ctx c = main_ctx(ix);
    // the kernels read the queries from the page-locked staging buffer and
    // the offsets scan writes into page-locked host memory: no copies
    std::memcpy(w.h_qko, q, sizeof(int) * nq);
    std::memcpy(w.h_qko + nq, k, sizeof(int) * nq);
    if (use_order) std::memcpy(w.h_qko + 2 * nq, order.data(), sizeof(int) * nq);
    c.io.q = w.h_qko_dev;
    c.io.k = w.h_qko_dev + nq;
    c.io.order = w.h_qko_dev + 2 * nq;
    c.io.off_host = w.h_off_dev;
    bool locked = false;
    int* ids_dev = nullptr;
    // asked on every call: a freed page-locked buffer's address may come back
    // as ordinary memory
    if (out_ids && cap > 0) {
        cudaPointerAttributes pa;
        locked = cudaPointerGetAttributes(&pa, out_ids) == cudaSuccess && pa.type == cudaMemoryTypeHost;
        if (locked) ids_dev = (int*)pa.devicePointer;
        cudaGetLastError();
    }
    // A device-accessible page-locked id buffer that the caller passes again
    // (same address and capacity as on the previous call) receives the ids
    // from finalize_kernel itself; the captured graph is kept for it.
    const bool direct = ids_dev && out_ids == ix->last_out && cap == ix->last_cap;
    ix->last_out = out_ids;
    ix->last_cap = cap;
    if (direct) {
        c.io.ids = ids_dev;
        c.io.ids_cap = cap;
    }
    // Otherwise the ids come back with the offsets when the batch returns no
    // more than the previous one plus a margin: page-locked caller buffers
    // take them directly, pageable ones through the workspace's staging.
    long long guess = ix->last_total + ix->last_total / 4 + 4096;
    int* spec = nullptr;
    if (direct) {
        guess = 0;
    } else if (locked) {
        guess = std::min<long long>(guess, cap);
        spec = out_ids;
    } else if (out_ids && cap > 0) {
        guess = std::min<long long>(guess, cap);
        if (guess > w.h_ids_cap) {
            cudaFreeHost(w.h_ids);
            w.h_ids = nullptr;
            w.h_ids_cap = 0;
            const long long hc = std::max<long long>(guess, 1 << 16);
            CK(cudaMallocHost(&w.h_ids, sizeof(int) * hc));
            w.h_ids_cap = hc;
        }
        spec = w.h_ids;
    }
    s = run_sync(ix, c, b, true, spec, spec ? guess : 0);
    if (s != RKNN_OK) return s;
    ix->last_lc = b.pstride;
    const long long total = w.h_off[nq];
    for (int i = 0; i <= nq; ++i) offsets[i] = w.h_off[i];
    ix->last_nq = nq;
    ix->last_mode = mode;
    ix->last_total = total;
    if (stats) {
        s = collect_stats(c, nq, stats);
        if (s != RKNN_OK) return s;
    }
    if (total > cap || (!out_ids && total > 0))
        return fail(RKNN_ERR_CAPACITY, "output buffer holds " + std::to_string(cap) + " ids, " +
                                           std::to_string(total) + " needed");
    if (total > 0 && !direct && total > std::min(guess, w.pool_cap)) {
        // more ids than the speculative copy held: fetch them all
        if (!locked && total > w.h_ids_cap) {
            cudaFreeHost(w.h_ids);
            w.h_ids = nullptr;
            w.h_ids_cap = 0;
            const long long hc = std::max<long long>(total + total / 4, 1 << 16);
            CK(cudaMallocHost(&w.h_ids, sizeof(int) * hc));
            w.h_ids_cap = hc;
        }
        CK(cudaMemcpyAsync(locked ? out_ids : w.h_ids, w.d_out, sizeof(int) * total, cudaMemcpyDeviceToHost,
                           ix->stream));
        CK(cudaStreamSynchronize(ix->stream));
    }
    if (total > 0 && !locked && !direct) std::memcpy(out_ids, w.h_ids, sizeof(int) * total);
    return RKNN_OK;
}

rknn_status rknn_host_alloc(int64_t bytes, void** out)
{
    g_err.clear();
    if (!out || bytes <= 0) return fail(RKNN_ERR_ARG, "bad argument");
    *out = nullptr;
    CK(cudaMallocHost(out, (size_t)bytes));
    return RKNN_OK;
}

rknn_status rknn_host_free(void* p)
{
    g_err.clear();
    if (p) CK(cudaFreeHost(p));
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
    CK(cudaSetDevice(ix->device));
    Workspace& w = ix->ws;
    const BatchPlan b = plan_batch(ix, nq, mode, false, nullptr, kmax);
    ix->last_lc = b.pstride;
    rknn_status s = ensure_ws(w, nq, plan_caps(b), std::max<long long>(w.pool_cap, (long long)nq * 4096));
    if (s != RKNN_OK) return s;
    // the filter kernels read the caller's arrays (kept for a rerun by
    // rknn_batch_device_results)
    Ctx c = main_ctx(ix);
    c.io.q = d_q;
    c.io.k = d_k;
    ix->dev_q = d_q;
    ix->dev_k = d_k;
    s = launch(ix, c, b);
    ix->last_nq = nq;
    ix->last_mode = mode;
    ix->dev_nq = s == RKNN_OK ? nq : 0;
    ix->dev_kmax = kmax;
    ix->dev_mode = mode;
    return s;
}

rknn_status rknn_batch_device_results(rknn_index* ix, const int32_t** d_ids, const int32_t** d_offsets)
{
    g_err.clear();
    if (!ix || !d_ids || !d_offsets) return fail(RKNN_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ix->mu);
    CK(cudaSetDevice(ix->device));
    if (ix->dev_nq > 0) {
        // a slot whose results outgrew its region, or regions that outgrew
        // the pool, left the device batch incomplete: run it again (from the
        // caller's q and k) with room for all of them
        Workspace& w = ix->ws;
        const int nq = ix->dev_nq;
        CK(cudaMemcpyAsync(w.h_off, w.d_out_off, sizeof(int) * (nq + 1 + OFF_TAIL), cudaMemcpyDeviceToHost, ix->stream));
        CK(cudaStreamSynchronize(ix->stream));
        const RunTail tail = run_tail(w.h_off, nq);
        const long long region_total = tail.region_total;
        const int dropped = tail.dropped;
        if (region_total > w.pool_cap || dropped) {
            if (dropped) w.rcap = (int)std::min<long long>((long long)w.rcap * 8, std::max<long long>(ix->nu, 1));
            const BatchPlan b = plan_batch(ix, nq, ix->dev_mode, false, nullptr, ix->dev_kmax);
            Ctx c = main_ctx(ix);
            c.io.q = ix->dev_q;
            c.io.k = ix->dev_k;
            rknn_status s = run_sync(ix, c, b);
            if (s != RKNN_OK) return s;
        }
        ix->dev_nq = 0;
    }
    *d_ids = ix->ws.d_out;
    *d_offsets = ix->ws.d_out_off;
    return RKNN_OK;
}

rknn_status rknn_last_stats(rknn_index* ix, rknn_query_stats* stats)
{
    if (!ix || !stats) return fail(RKNN_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ix->mu);
    if (ix->last_nq <= 0) return fail(RKNN_ERR_STATE, "no query has run");
    Ctx c = main_ctx(ix);
    return collect_stats(c, ix->last_nq, stats);
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
    int *counters, *q, *k, *chunk_off, *res_count, *out_off, *bispos, *pool, *out, *reg_len;
    long long *cand_off, *region_top;
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
    L.cand_off = (long long*)take(sizeof(long long) * 2);
    L.region_top = (long long*)take(sizeof(long long));
    L.reg_len = (int*)take(sizeof(int));
    L.chunk_off = (int*)take(sizeof(int) * 2);
    L.res_count = (int*)take(sizeof(int));
    L.out_off = (int*)take(sizeof(int) * (2 + OFF_TAIL));
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

namespace {
void noalloc_forget(int device)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return;
    std::lock_guard<std::mutex> glk(g_noalloc_mu);
    g_noalloc_ptr[device] = nullptr;
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
    // (host code must not pass the symbol itself).  rknn_index_create drops
    // the cached address of its device, so an index built after a
    // cudaDeviceReset looks it up again in the new context.
    if (!g_noalloc_ptr[ix->device]) {
        void* p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[ix->device] = (unsigned char*)p;
    }
    const ZoneCaps caps = caps_fit(ix, caps_for(k));
    const int seg_cap = 2 * caps.rm + 2;
    NoallocLayout L = noalloc_layout(g_noalloc_ptr[ix->device], caps_for(NOALLOC_KMAX).lc, seg_cap);
    cudaStream_t st = ix->stream;
    // Every return after the first enqueued operation, failures included,
    // leaves the stream idle: the next call (once the lock is released)
    // clears and reuses the same array, which kernels still running from
    // this call would otherwise share.  Declared after the locks, so it runs
    // before they are released.
    struct DrainStream {
        cudaStream_t s;
        ~DrainStream() { (void)cudaStreamSynchronize(s); }
    } drain{st};

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
    za.ustart = ix->d_ustart; za.uxy = ix->d_uxy; za.uid = ix->d_uid; za.gu = ix->gu; za.nu = (int)ix->nu;
    za.sx0 = ix->sx0; za.sy0 = ix->sy0; za.sx1 = ix->sx1; za.sy1 = ix->sy1;
    za.q_in = L.q; za.k_in = L.k; za.order = nullptr; za.nq = 1;
    za.work_counter = L.counters + 0;
    za.caps = caps;
    za.skip_coincident = ix->skip_coincident;
    za.vertex_test = ix->zone_vertex_test;
    za.rmax = caps.rm;
    za.seg_cap = seg_cap;
    za.pstride = caps.lc;
    za.slice_r = nullptr;
    za.qd = L.qd; za.planes = L.planes; za.bis_pos = L.bispos; za.segs = L.segs; za.zst = L.zst;
    za.fault = L.counters + 4;
    // the kernels rknn_query picks for one query: the zone over a block
    // (when its capacities allow it, as in zone_launch) and the verification
    // in items of 64 users, which spread a lone query's FP64 evaluations
    // over more warps
    const size_t zl = zone_layout(caps).bytes;
    const bool cta = ix->zone_cta && caps.pc <= ZCTA_PQ_MAX && caps.vc < 32768;
    if (cta && ix->zone_cta == ZCTA_THREADS) zone_kernel_cta<<<1, ZCTA_THREADS, zl, st>>>(za);
    else if (cta) zone_kernel_cta_half<<<1, ZCTA_THREADS / 2, zl, st>>>(za);
    else zone_kernel_smem<<<1, 32 * ZONE_WARPS, zl * ZONE_WARPS, st>>>(za);
    CK(cudaGetLastError());
    constexpr int NA_UPT = 2;
    plan_kernel<<<1, 1024, 0, st>>>(L.qd, 1, L.cand_off, L.reg_len, L.region_top, L.chunk_off, L.pool_cap,
                                    (int)std::min<long long>(L.pool_cap, INT32_MAX), 32 * NA_UPT);
    CK(cudaGetLastError());

    VerifyArgs va;
    va.qd = L.qd; va.planes = L.planes; va.bis_pos = L.bispos; va.lc = caps.lc;
    va.slice_r = nullptr;
    va.segs = L.segs; va.seg_cap = seg_cap;
    va.chunk_off = L.chunk_off; va.cand_off = L.cand_off; va.reg_len = L.reg_len; va.nq = 1;
    va.uxy = ix->d_uxy; va.uid = ix->d_uid; va.fxy = ix->d_fxy; va.fstart = ix->d_fstart; va.gf = ix->gf;
    va.res_count = L.res_count; va.res_pool = L.pool; va.work_counter = L.counters + 1;
    va.vstats = L.vstats; va.mode = mode;
    va.nu = (int)ix->nu; va.nf = (int)ix->nf; va.ncf = ix->gf.gx * ix->gf.gy;
    va.pool_cap = L.pool_cap; va.fault = L.counters + 10; va.dropped = L.counters + 2;
    va.surv = nullptr; va.surv_cap = 0; va.surv_count = L.counters + 3;
    // at most 512 half-planes staged per warp, as in batches (128 KB of
    // staging per block); fewer staged planes only send more users to the
    // exact count
    va.stage_cap = std::max(1, std::min(caps.lc, (128 << 10) / (VERIFY_WARPS * 32)));
    const size_t vsmem = (size_t)VERIFY_WARPS * ((size_t)va.stage_cap * 32 + 32 * sizeof(float));
    verify_fn(NA_UPT)<<<2 * ix->num_sms, VERIFY_WARPS * 32, vsmem, st>>>(va);
    CK(cudaGetLastError());
    scan_counts_kernel<<<1, 1024, 0, st>>>(L.res_count, L.reg_len, L.region_top, 1, L.out_off, L.counters, nullptr);
    CK(cudaGetLastError());
    finalize_kernel<<<1, 32 * FIN_WARPS, 0, st>>>(L.pool, L.cand_off, L.reg_len, L.res_count, L.out_off, L.out, 1,
                                                  L.pool_cap, nullptr, 0, FinScan{});
    CK(cudaGetLastError());

    QDesc d;
    int off[2] = {0, 0};
    int dropped = 0;
    CK(cudaMemcpyAsync(&d, L.qd, sizeof(QDesc), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(off, L.out_off, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&dropped, L.counters + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
#ifdef RKNN_CHECKED
    int rec[16];
    CK(cudaMemcpyAsync(rec, L.counters, sizeof(rec), cudaMemcpyDeviceToHost, st));
#endif
    CK(cudaStreamSynchronize(st));
#ifdef RKNN_CHECKED
    // bounds-checked build: a recorded out-of-range access fails the call
    // (zone record at counters[4..9), verification record at [10..15))
    for (int base : {4, 10})
        if (rec[base])
            return fail(RKNN_ERR_CUDA, "bounds check: array " + std::to_string(rec[base + 1]) + " index " +
                                           std::to_string(rec[base + 2]) + " of " + std::to_string(rec[base + 3]) +
                                           " at line " + std::to_string(rec[base + 4]));
#endif
    if ((d.flags & QF_RESULT_OVERFLOW) || dropped)
        return fail(RKNN_ERR_CAPACITY, "rknn_query_noalloc: the query's results exceed the fixed "
                                       "scratch (about 2M ids); use rknn_query");
    const int64_t n = off[1];
    *n_out = n;
    if (n > cap) return fail(RKNN_ERR_CAPACITY, "output buffer too small");
    if (n > 0) {
        CK(cudaMemcpyAsync(out_ids, L.out, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return RKNN_OK;
}

// ====================================================================
// Serving: continuous batching over a resident index.
//
// One worker thread per server.  Each slot owns a workspace, a stream and a
// completion event.  The worker retires finished slots (copies their results
// to the waiting requests) and fills free slots with batches formed from the
// queue, so batches launched at different times run on the GPU together.
// Batch sizes are padded to powers of two (padding slots carry an invalid
// query index, which the zone kernel marks and every later kernel skips).
// Batches are launched directly rather than through cached graphs: their
// composition (size per k class) changes from batch to batch.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

namespace {

using Clock = std::chrono::steady_clock;

struct ServeReq {
    int32_t q = 0, k = 1, mode = 0;
    uint64_t ticket = 0;
    Clock::time_point t_sub, t_done;
    std::vector<int32_t> ids;
    rknn_status status = RKNN_OK;
    std::string err;
    bool done = false;
};
using ReqPtr = std::shared_ptr<ServeReq>;

struct Slot {
    Workspace ws;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, done = nullptr;
    double device_ms = 0;
    std::vector<ReqPtr> reqs;        // the batch in flight
    BatchPlan plan;
    bool busy = false;
};

int pad_pow2(int n)
{
    int p = 32;
    while (p < n) p <<= 1;
    return p;
}

// Scratch a batch slot uses per query at a given largest k: half-planes and
// bisector positions, segments, descriptors and offsets, and the result
// pool's starting share (two 4096-entry int arrays).
long long scratch_per_query(rknn_index* ix, int kmax)
{
    const ZoneCaps c = caps_fit(ix, caps_for(kmax));
    return 20LL * c.lc + 8LL * (2 * c.rm + 2) + (long long)sizeof(QDesc) + (long long)sizeof(ZStats) + 32 +
           2LL * 4 * 4096;
}

}  // namespace

struct rknn_server {
    rknn_index* ix = nullptr;
    rknn_serve_opts o{};
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ReqPtr> pending;
    std::unordered_map<uint64_t, ReqPtr> live;
    uint64_t next_ticket = 1;
    bool stopping = false;
    std::thread th;
    // failure test hooks (under mu): the next batches that fail on purpose
    int inject_oom = 0, inject_launch = 0;
    // statistics (under mu)
    int64_t submitted = 0, completed = 0, failed = 0, batches = 0, batched = 0;
    int inflight = 0, max_inflight = 0;
    std::vector<double> lat;
    bool have_first = false;
    Clock::time_point t_first, t_last;
};

namespace {

void finish(rknn_server* sv, const ReqPtr& r, rknn_status st, const std::string& err)
{
    r->status = st;
    r->err = err;
    r->t_done = Clock::now();
    r->done = true;
    if (st == RKNN_OK) {
        sv->completed++;
        sv->lat.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_sub).count());
        sv->t_last = r->t_done;
    } else {
        sv->failed++;
    }
}

// Failure test hooks (rknn_serve_inject_fault): made on the host, no GPU
// fault is involved.
enum { INJECT_NONE = 0, INJECT_OOM = 1, INJECT_LAUNCH = 2 };

// Launch a batch on a free slot (worker thread, mu not held).
rknn_status slot_launch(rknn_server* sv, Slot& sl, int inject)
{
    rknn_index* ix = sv->ix;
    const int nq = (int)sl.reqs.size();
    const int nqp = pad_pow2(nq);
    // descending k: the longest zones start first; each k class gets its own
    // zone launch.  Padding slots (invalid query, k = 1) come last.
    std::vector<int> order(nqp), ksorted(nqp);
    for (int i = 0; i < nqp; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.begin() + nq, [&](int a, int b) { return sl.reqs[a]->k > sl.reqs[b]->k; });
    int kmax = 1;
    for (int i = 0; i < nqp; ++i) {
        ksorted[i] = order[i] < nq ? sl.reqs[order[i]]->k : 1;
        kmax = std::max(kmax, ksorted[i]);
    }
    sl.plan = plan_batch(ix, nqp, sl.reqs[0]->mode, true, ksorted.data(), kmax);
    Workspace& w = sl.ws;
    if (inject == INJECT_OOM) w.inject_oom = true;
    rknn_status s = ensure_ws(w, nqp, plan_caps(sl.plan), std::max<long long>(w.pool_cap, (long long)nqp * 4096));
    if (s != RKNN_OK) return s;
    for (int i = 0; i < nqp; ++i) {
        w.h_qko[i] = i < nq ? sl.reqs[i]->q : -1;
        w.h_qko[nqp + i] = i < nq ? sl.reqs[i]->k : 1;
        w.h_qko[2 * nqp + i] = order[i];
    }
    CK(cudaMemcpyAsync(w.d_qko, w.h_qko, sizeof(int) * 3 * (size_t)nqp, cudaMemcpyHostToDevice, sl.st));
    if (inject == INJECT_LAUNCH)
        return fail(RKNN_ERR_CUDA, "batch launch failed after its input copy (injected for a failure test)");
    Ctx c{w, sl.st, sl.ev0, sl.ev1, nullptr, &sl.device_ms};
    CK(cudaEventRecord(sl.ev0, sl.st));
    s = launch(ix, c, sl.plan, false);
    if (s != RKNN_OK) return s;
    CK(cudaEventRecord(sl.ev1, sl.st));
    CK(cudaMemcpyAsync(w.h_off, w.d_out_off, sizeof(int) * (nqp + 1 + OFF_TAIL), cudaMemcpyDeviceToHost, sl.st));
    CK(cudaEventRecord(sl.done, sl.st));
    return RKNN_OK;
}

// Collect a finished slot's results (worker thread, mu not held).
rknn_status slot_collect(rknn_server* sv, Slot& sl)
{
    Workspace& w = sl.ws;
    const int nq = (int)sl.reqs.size();
    const RunTail tail = run_tail(w.h_off, sl.plan.nq);
    if (tail.region_total > w.pool_cap || tail.dropped != 0) {
        // a result region did not fit the pool, or held too few ids: rerun
        Ctx c{w, sl.st, sl.ev0, sl.ev1, nullptr, &sl.device_ms};
        rknn_status s = run_sync(sv->ix, c, sl.plan, false);
        if (s != RKNN_OK) return s;
    }
    const long long total = w.h_off[nq];
    if (total > w.h_ids_cap) {
        cudaFreeHost(w.h_ids);
        w.h_ids = nullptr;
        w.h_ids_cap = 0;
        long long cap = std::max<long long>(total, 1 << 16);
        CK(cudaMallocHost(&w.h_ids, sizeof(int) * cap));
        w.h_ids_cap = cap;
    }
    if (total > 0) {
        CK(cudaMemcpyAsync(w.h_ids, w.d_out, sizeof(int) * total, cudaMemcpyDeviceToHost, sl.st));
        CK(cudaStreamSynchronize(sl.st));
    }
    for (int i = 0; i < nq; ++i) sl.reqs[i]->ids.assign(w.h_ids + w.h_off[i], w.h_ids + w.h_off[i + 1]);
    return RKNN_OK;
}

void serve_loop(rknn_server* sv)
{
    cudaSetDevice(sv->ix->device);
    const long long budget = sv->o.scratch_bytes;
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        // retire finished batches
        for (auto& sl : sv->slots) {
            if (!sl.busy) continue;
            cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) continue;
            lk.unlock();
            rknn_status s = q == cudaSuccess ? slot_collect(sv, sl) : RKNN_ERR_CUDA;
            std::string err = s == RKNN_OK ? "" : (q == cudaSuccess ? g_err : std::string(cudaGetErrorString(q)));
            lk.lock();
            for (auto& r : sl.reqs) finish(sv, r, s, err);
            sl.reqs.clear();
            sl.busy = false;
            sv->inflight--;
            sv->cv_done.notify_all();
        }
        // fill free slots from the queue
        for (auto& sl : sv->slots) {
            if (sl.busy || sv->pending.empty()) continue;
            const int mode = sv->pending.front()->mode;
            int kmax = 1;
            for (auto it = sv->pending.begin(); it != sv->pending.end() && (int)sl.reqs.size() < sv->o.max_batch;) {
                ReqPtr r = *it;
                if (r->mode != mode) { ++it; continue; }
                const int km = std::max(kmax, (int)r->k);
                // a request's own estimate never exceeds the budget (submit
                // refuses such requests), so the first one always fits
                const long long need = (long long)pad_pow2((int)sl.reqs.size() + 1) * scratch_per_query(sv->ix, km);
                if (!sl.reqs.empty() && need > budget) break;
                sl.reqs.push_back(r);
                kmax = km;
                it = sv->pending.erase(it);
            }
            int inject = INJECT_NONE;
            if (sv->inject_oom > 0) {
                sv->inject_oom--;
                inject = INJECT_OOM;
            } else if (sv->inject_launch > 0) {
                sv->inject_launch--;
                inject = INJECT_LAUNCH;
            }
            lk.unlock();
            rknn_status s = slot_launch(sv, sl, inject);
            std::string err = s == RKNN_OK ? "" : g_err;
            lk.lock();
            sv->batches++;
            sv->batched += (int64_t)sl.reqs.size();
            if (s != RKNN_OK) {
                // the batch's requests fail with the launch's status; the
                // slot stays free and takes the next batch (its workspace,
                // released by a failed growth, is allocated afresh)
                cudaStreamSynchronize(sl.st);
                for (auto& r : sl.reqs) finish(sv, r, s, err);
                sl.reqs.clear();
                sv->cv_done.notify_all();
                continue;
            }
            sl.busy = true;
            sv->inflight++;
            sv->max_inflight = std::max(sv->max_inflight, sv->inflight);
        }
        if (sv->inflight == 0 && sv->pending.empty()) {
            if (sv->stopping) break;
            sv->cv_work.wait(lk);
        } else {
            // batches on the GPU: look again shortly (new arrivals wake us at once)
            sv->cv_work.wait_for(lk, std::chrono::microseconds(20));
        }
    }
}

void destroy_server(rknn_server* sv)
{
    for (auto& sl : sv->slots) {
        if (sl.st) cudaStreamSynchronize(sl.st);
        free_ws(sl.ws);
        if (sl.ev0) cudaEventDestroy(sl.ev0);
        if (sl.ev1) cudaEventDestroy(sl.ev1);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.st) cudaStreamDestroy(sl.st);
    }
    delete sv;
}

}  // namespace

extern "C" {

void rknn_serve_opts_default(rknn_serve_opts* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->slots = 3;
    o->max_batch = 4096;
    o->scratch_bytes = 256LL << 20;
}

rknn_status rknn_serve_start(rknn_index* ix, const rknn_serve_opts* opts, rknn_server** out)
{
    g_err.clear();
    if (!ix || !out) return fail(RKNN_ERR_ARG, "null argument");
    *out = nullptr;
    rknn_serve_opts o;
    rknn_serve_opts_default(&o);
    if (opts) o = *opts;
    if (o.slots < 1 || o.slots > 64) return fail(RKNN_ERR_ARG, "slots must be in [1, 64]");
    if (o.max_batch < 1 || o.max_batch > (1 << 20)) return fail(RKNN_ERR_ARG, "max_batch must be in [1, 2^20]");
    if (o.scratch_bytes <= 0) return fail(RKNN_ERR_ARG, "scratch_bytes must be positive");
    CK(cudaSetDevice(ix->device));
    rknn_server* sv = new (std::nothrow) rknn_server();
    if (!sv) return fail(RKNN_ERR_OOM, "host allocation failed");
    sv->ix = ix;
    sv->o = o;
    sv->slots.resize(o.slots);
    for (auto& sl : sv->slots) {
        cudaError_t e = cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.ev1);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            destroy_server(sv);
            return fail(RKNN_ERR_CUDA, std::string("server setup: ") + cudaGetErrorString(e));
        }
    }
    sv->th = std::thread(serve_loop, sv);
    *out = sv;
    return RKNN_OK;
}

rknn_status rknn_serve_submit(rknn_server* sv, int32_t q, int32_t k, int32_t mode, uint64_t* ticket)
{
    if (!sv || !ticket) return fail(RKNN_ERR_ARG, "null argument");
    if (q < 0 || q >= sv->ix->nf)
        return fail(RKNN_ERR_ARG, "query index " + std::to_string(q) + " out of range [0, " +
                                      std::to_string(sv->ix->nf) + ")");
    if (k <= 0) return fail(RKNN_ERR_ARG, "k must be a positive integer");
    if (mode != RKNN_MODE_FP32 && mode != RKNN_MODE_FP64) return fail(RKNN_ERR_ARG, "bad mode");
    // admission: a request whose scratch estimate alone (as a batch of its
    // own) exceeds the server's budget is refused, so that no batch passes
    // the budget
    const long long need1 = (long long)pad_pow2(1) * scratch_per_query(sv->ix, k);
    if (need1 > sv->o.scratch_bytes)
        return fail(RKNN_ERR_CAPACITY, "request needs about " + std::to_string(need1) +
                                           " bytes of scratch, more than the server's scratch_bytes (" +
                                           std::to_string(sv->o.scratch_bytes) + ")");
    auto r = std::make_shared<ServeReq>();
    r->q = q;
    r->k = k;
    r->mode = mode;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stopping) return fail(RKNN_ERR_STATE, "server is stopping");
        r->ticket = sv->next_ticket++;
        r->t_sub = Clock::now();
        if (!sv->have_first) { sv->have_first = true; sv->t_first = r->t_sub; }
        sv->submitted++;
        sv->pending.push_back(r);
        sv->live.emplace(r->ticket, r);
        *ticket = r->ticket;
    }
    sv->cv_work.notify_one();
    return RKNN_OK;
}

rknn_status rknn_serve_wait(rknn_server* sv, uint64_t ticket, int32_t timeout_ms, int32_t* out_ids,
                            int64_t cap, int64_t* n_out, double* latency_ms)
{
    if (!sv || !n_out) return fail(RKNN_ERR_ARG, "null argument");
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->live.find(ticket);
    if (it == sv->live.end()) return fail(RKNN_ERR_ARG, "unknown ticket " + std::to_string(ticket));
    ReqPtr r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) sv->cv_done.wait(lk, ready);
    else if (!sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return fail(RKNN_ERR_TIMEOUT, "request not finished");
    if (r->status != RKNN_OK) {
        sv->live.erase(ticket);
        return fail(r->status, r->err);
    }
    *n_out = (int64_t)r->ids.size();
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_sub).count();
    if ((int64_t)r->ids.size() > cap || (!out_ids && !r->ids.empty()))
        return fail(RKNN_ERR_CAPACITY, "output buffer holds " + std::to_string(cap) + " ids, " +
                                           std::to_string(r->ids.size()) + " needed");
    if (!r->ids.empty()) std::memcpy(out_ids, r->ids.data(), sizeof(int32_t) * r->ids.size());
    sv->live.erase(ticket);
    return RKNN_OK;
}

rknn_status rknn_serve_replay(rknn_server* sv, int64_t n, const int32_t* q, const int32_t* k,
                              const int32_t* mode, const double* arrival_s, double* latency_ms,
                              int64_t* n_results)
{
    if (!sv || n < 0 || (n > 0 && (!q || !k || !mode || !arrival_s))) return fail(RKNN_ERR_ARG, "null argument");
    std::vector<uint64_t> tickets((size_t)n);
    const Clock::time_point t0 = Clock::now();
    for (int64_t i = 0; i < n; ++i) {
        const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
        while (Clock::now() < due) {
            const auto left = due - Clock::now();
            if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
        }
        rknn_status s = rknn_serve_submit(sv, q[i], k[i], mode[i], &tickets[(size_t)i]);
        if (s != RKNN_OK) return s;
    }
    rknn_status first = RKNN_OK;
    std::string first_err;
    for (int64_t i = 0; i < n; ++i) {
        std::unique_lock<std::mutex> lk(sv->mu);
        auto it = sv->live.find(tickets[(size_t)i]);
        if (it == sv->live.end()) continue;
        ReqPtr r = it->second;
        sv->cv_done.wait(lk, [&] { return r->done; });
        if (latency_ms) latency_ms[i] = std::chrono::duration<double, std::milli>(r->t_done - r->t_sub).count();
        if (n_results) n_results[i] = (int64_t)r->ids.size();
        if (r->status != RKNN_OK && first == RKNN_OK) { first = r->status; first_err = r->err; }
        sv->live.erase(it);
    }
    if (first != RKNN_OK) return fail(first, first_err);
    return RKNN_OK;
}

rknn_status rknn_serve_stats_get(rknn_server* sv, int32_t reset, rknn_serve_stats* st)
{
    if (!sv || !st) return fail(RKNN_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    rknn_serve_stats s{};
    s.submitted = sv->submitted;
    s.completed = sv->completed;
    s.failed = sv->failed;
    s.batches = sv->batches;
    s.mean_batch = sv->batches ? (double)sv->batched / (double)sv->batches : 0.0;
    s.max_inflight = sv->max_inflight;
    if (!sv->lat.empty()) {
        std::vector<double> v = sv->lat;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (double)v.size()))]; };
        s.p50_ms = pct(0.50);
        s.p99_ms = pct(0.99);
        s.max_ms = v.back();
        double sum = 0;
        for (double x : v) sum += x;
        s.mean_ms = sum / (double)v.size();
        const double span = std::chrono::duration<double>(sv->t_last - sv->t_first).count();
        s.throughput_qps = span > 0 ? (double)v.size() / span : 0.0;
    }
    *st = s;
    if (reset) {
        sv->lat.clear();
        sv->submitted = sv->completed = sv->failed = sv->batches = sv->batched = 0;
        sv->max_inflight = sv->inflight;
        sv->have_first = false;
    }
    return RKNN_OK;
}

rknn_status rknn_serve_inject_fault(rknn_server* sv, int32_t kind, int32_t count)
{
    if (!sv || count < 0) return fail(RKNN_ERR_ARG, "bad argument");
    if (kind != INJECT_OOM && kind != INJECT_LAUNCH) return fail(RKNN_ERR_ARG, "unknown fault kind");
    std::lock_guard<std::mutex> lk(sv->mu);
    (kind == INJECT_OOM ? sv->inject_oom : sv->inject_launch) = count;
    return RKNN_OK;
}

rknn_status rknn_serve_stop(rknn_server* sv)
{
    if (!sv) return RKNN_OK;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stopping = true;
    }
    sv->cv_work.notify_all();
    if (sv->th.joinable()) sv->th.join();
    destroy_server(sv);
    return RKNN_OK;
}

}  // extern "C"

// ====================================================================
// Autotuning: grid densities and the verification kernel's shape, timed on
// the caller's sample batch with the engine's own events.
extern "C" rknn_status rknn_index_tune(rknn_index* ix, const int32_t* q, const int32_t* k, int32_t nq,
                                       int32_t mode, rknn_tune_result* result)
{
    g_err.clear();
    if (!ix || !q || !k || nq <= 0 || !result) return fail(RKNN_ERR_ARG, "bad argument");
    if (mode != RKNN_MODE_FP32 && mode != RKNN_MODE_FP64) return fail(RKNN_ERR_ARG, "bad mode");
    int kmax = 1;
    rknn_status s = check_queries(ix, q, k, nq, &kmax);
    if (s != RKNN_OK) return s;
    std::vector<int64_t> off((size_t)nq + 1);
    // device time of the sample batch: best of two runs after one untimed run
    auto time_batch = [&](double& ms) -> rknn_status {
        ms = 1e300;
        for (int r = 0; r < 3; ++r) {
            rknn_query_stats st;
            rknn_status e = rknn_query_batch(ix, q, k, nq, mode, nullptr, 0, off.data(), &st);
            if (e != RKNN_OK && e != RKNN_ERR_CAPACITY) return e;
            if (r > 0) ms = std::min(ms, st.device_ms);
        }
        g_err.clear();
        return RKNN_OK;
    };
    const float fpc0 = ix->fac_per_cell, upc0 = ix->usr_per_cell;
    const int upt0 = ix->vupt, vw0 = ix->vwarps;
    rknn_tune_result r{};
    r.fac_per_cell = fpc0; r.usr_per_cell = upc0; r.users_per_thread = upt0; r.verify_warps = vw0;
    s = time_batch(r.default_ms);
    if (s != RKNN_OK) return s;
    r.best_ms = r.default_ms;
    // stage 1: grid densities (finer ones pay off on clustered data), with
    // the verification shape on entry; stage 2: the verification shape
    const float fpcs[5] = {0.25f, 0.5f, 1.0f, 2.0f, 4.0f}, upcs[5] = {1.0f, 2.0f, 4.0f, 8.0f, 16.0f};
    const int upts[3] = {2, 4, 8}, vws[3] = {4, 8, 16};
    for (float fpc : fpcs)
        for (float upc : upcs) {
            {
                std::lock_guard<std::mutex> lk(ix->mu);
                s = build_grids(ix, fpc, upc);
            }
            if (s != RKNN_OK) return s;
            double ms = 0;
            s = time_batch(ms);
            if (s != RKNN_OK) return s;
            r.trials++;
            if (ms < r.best_ms) {
                r.best_ms = ms;
                r.fac_per_cell = fpc;
                r.usr_per_cell = upc;
            }
        }
    {
        std::lock_guard<std::mutex> lk(ix->mu);
        s = build_grids(ix, r.fac_per_cell, r.usr_per_cell);
    }
    if (s != RKNN_OK) return s;
    for (int upt : upts)
        for (int vw : vws) {
            ix->vupt = upt;
            ix->vwarps = vw;
            ix->plan_cache.reset();
            double ms = 0;
            s = time_batch(ms);
            if (s != RKNN_OK) return s;
            r.trials++;
            if (ms < r.best_ms) {
                r.best_ms = ms;
                r.users_per_thread = upt;
                r.verify_warps = vw;
            }
        }
    {
        std::lock_guard<std::mutex> lk(ix->mu);
        s = build_grids(ix, r.fac_per_cell, r.usr_per_cell);
    }
    if (s != RKNN_OK) return s;
    ix->vupt = r.users_per_thread;
    ix->vwarps = r.verify_warps;
    ix->plan_cache.reset();
    *result = r;
    return RKNN_OK;
}
