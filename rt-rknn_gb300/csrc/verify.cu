// Verification: for every candidate user of a query, count the facilities
// strictly nearer than the query facility q and keep the user when the count
// is below k (rknn-inf-gpu/inf_kernel.cu:41-66 counts bisector violations per
// user; rknn-rt/rt.cu:95-111 counts half-plane hits and stops at k).
//
// Stage 1 (half-plane filter).  A user is tested against the zone's
// bisectors written as exact half-planes relative to q,
//     m_f(u) = a (ux-qx) + b (uy-qy) + c = d2(u,f) - d2(u,q),
// two FMAs per (user, half-plane).  m_f(u) < -bound certifies that f is
// strictly nearer; k certified half-planes reject the user.  The bound
//     8u (2F'(|x'|+|y'|) + F'^2),  F' = max |f - q| over the bisectors,
// exceeds the float (or double) evaluation error of m_f (at most
// 4.01u(|a x'| + |b y'| + |c|)).  Lanes own users (coalesced float2 loads,
// four per lane); the warp leaves the half-plane loop as soon as every lane
// has k certified violations for all its users (__all_sync).
//
// Stage 2 (exact count).  Users that survive stage 1 go to a survivor list,
// and recount_kernel counts each one exactly, a warp (or a group of up to
// eight warps, when warps outnumber survivors) per survivor: the facility
// cells covering the disc of radius d(u,q) around u, row by row (one
// contiguous range of the cell-sorted facility array per row, trimmed to the
// disc's chord), 32 facilities a round, counting d2(u,f) < d2(u,q) and
// stopping at k.  Each comparison is decided in float (or double) with its
// error bound, and the undecided ones by the exact expansion predicate.
// Accepted users are appended to their query's result region.  When the
// survivor list is full, the warp counts its own survivors, one lane per
// facility.  The item code itself lives in verify_item.cuh, shared with the
// slice filter's fused verification.
#include "verify_item.cuh"
#include <climits>

namespace rknn {

using namespace vitem;

template <int UPT, bool BITS = false>
__device__ __forceinline__ void verify_body(const VerifyArgs& A)
{
    extern __shared__ __align__(16) char smem[];
    // every st-th work-item offset, for the item -> slot lookup
    __shared__ int csmp[VERIFY_SAMPLES];
    pdl_wait();
    pdl_trigger();
    // a fused batch with no slot left over: nothing to do here
    if (A.deflist && __ldcg(A.ndef) == 0) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // per warp: stage_cap half-planes (16 bytes each in FP32, compact: the
    // packed pairs are made in registers; 32 in FP64), seg_stage segments,
    // the slot's 32 slice bounds
    const size_t plane_bytes = (size_t)A.stage_cap * (A.mode == MODE_FP32 ? 16 : 32);
    char* sp = smem + w * (plane_bytes + (size_t)A.seg_stage * sizeof(int2) + 32 * sizeof(float));
    int2* ssg = (int2*)(sp + plane_bytes);
    float* sr = (float*)(ssg + A.seg_stage);
    // the listed slots: every slot, or those the fused slice filter left
    const int nl = A.deflist ? __ldcg(A.ndef) : A.nq;
    const int st = max(1, (nl + VERIFY_SAMPLES) / VERIFY_SAMPLES);       // ceil((nl + 1) / samples)
    const int nsmp = nl / st + 1;                                         // samples i * st <= nl
    if (nl > 0)
        for (int i = threadIdx.x; i < nsmp; i += blockDim.x) csmp[i] = A.chunk_off[i * st];
    __syncthreads();
    int cur = -1;
    bool seg_staged = false;
    // per-warp statistics (32-bit here, 64-bit in the totals)
    VCount vc = {};
    const int total = nl > 0 ? A.chunk_off[nl] : 0;
    // Warp gw's first item is item gw; later items come from the counter,
    // numbered after the nwarps taken that way, and only when items
    // outnumber warps.  (Thousands of warps taking even their first item
    // from one counter queue their atomics on one address for many
    // microseconds, and a small batch's few items wait behind them.)
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    int g = blockIdx.x * (blockDim.x >> 5) + w;
    for (bool first = true;; first = false) {
        if (!first) {
            if (total <= nwarps) break;
            int nx = 0;
            if (lane == 0) nx = nwarps + atomicAdd(A.work_counter, 1);
            g = __shfl_sync(FULL, nx, 0);
        }
        if (g >= total) break;
        // list entry e of item g: chunk_off[e] <= g < chunk_off[e+1].  The
        // samples narrow it to [ws, ws + st); there the count of offsets <= g
        // places it (offsets never decrease).
        int lo = 0, hi = nsmp;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (csmp[mid] <= g) lo = mid; else hi = mid;
        }
        int e = lo, c_off = 0;      // c_off = chunk_off[e]
        if (st > 1) {
            const int ws = lo * st, we = min(ws + st, nl);
            if (st <= 31) {
                const int j = ws + lane;
                const int co = j <= we ? A.chunk_off[VX(j, nl + 1, 215)] : INT_MAX;
                e = ws + __popc(__ballot_sync(FULL, co <= g)) - 1;
                c_off = __shfl_sync(FULL, co, e - ws);
            } else {
                int l = ws, h = we;
                while (h - l > 1) {
                    const int mid = (l + h) >> 1;
                    if (A.chunk_off[mid] <= g) l = mid; else h = mid;
                }
                e = l;
                c_off = A.chunk_off[e];
            }
        } else {
            c_off = csmp[e];
        }
        const int s = A.deflist ? A.deflist[VX(e, A.nq, 222)] : e;
        const QDesc d = A.qd[s];
        if (s != cur && A.mode == MODE_FP32) {
            // the slot's half-planes (as many as are staged at most),
            // seg_stage segments and the slice bounds, each lane's loads
            // issued together
            __syncwarp();
            const float4* src = A.planes + (size_t)s * A.lc;
            const int nst = min(d.nb, A.stage_cap);
            for (int m0 = lane; m0 < nst; m0 += 32 * 8) {
                float4 p[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int m = m0 + 32 * j;
                    p[j] = m < nst ? src[m] : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int m = m0 + 32 * j;
                    if (m < nst) ((float4*)sp)[m] = p[j];
                }
            }
            // the slot's segments (nseg ranges and the terminal entry), when
            // they fit; the record has arrived with the half-planes in flight
            const int2* gsg = A.segs + (size_t)s * A.seg_cap;
            const int nss = d.nseg + 1 <= A.seg_stage ? d.nseg + 1 : 0;
            for (int m0 = lane; m0 < nss; m0 += 32 * 8) {
                int2 e[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int m = m0 + 32 * j;
                    e[j] = m < nss ? gsg[m] : make_int2(0, 0);
                }
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (m0 + 32 * j < nss) ssg[m0 + 32 * j] = e[j];
            }
            if (A.slice_r) sr[lane] = A.slice_r[(size_t)s * 32 + lane];
        }
        if (s != cur) {
            if (A.mode == MODE_FP32) {
                seg_staged = d.nseg + 1 <= A.seg_stage;
            } else {
                __syncwarp();
                const int* bp = A.bis_pos + (size_t)s * A.lc;
                for (int m = lane; m < min(d.nb, A.stage_cap); m += 32) {
                    float2 f = A.fxy[VX(bp[m], A.nf, 204)];
                    double dx = (double)f.x - (double)d.qx, dy = (double)f.y - (double)d.qy;
                    double* p = (double*)sp + 4 * m;
                    p[0] = -2.0 * dx;
                    p[1] = -2.0 * dy;
                    p[2] = fma(dx, dx, dy * dy);
                    p[3] = (double)A.planes[(size_t)s * A.lc + m].w;
                }
                // the slot's user segments (nseg ranges and the terminal entry)
                seg_staged = d.nseg + 1 <= A.seg_stage;
                if (seg_staged) {
                    const int2* gsg = A.segs + (size_t)s * A.seg_cap;
                    for (int m = lane; m <= d.nseg; m += 32) ssg[m] = gsg[m];
                }
                if (A.slice_r) sr[lane] = A.slice_r[(size_t)s * 32 + lane];
            }
            cur = s;
            __syncwarp();
        }
        const int v0 = (g - c_off) * (32 * UPT);
        const int2* sg = seg_staged ? ssg : A.segs + (size_t)s * A.seg_cap;
        verify_item<UPT, true, BITS>(A, d, s, v0, sp, sg, sr, min(d.nb, A.stage_cap), -1, -1, vc);
    }
    vc.flush(A.vstats);
}

// The verification kernel with 2, 4 or 8 users per lane per work item
// (32 * UPT users per item); blocks of up to 16 warps.
__global__ void __maxnreg__(80) verify_kernel(VerifyArgs a) { verify_body<4>(a); }
__global__ void __maxnreg__(80) verify_kernel_u2(VerifyArgs a) { verify_body<2, true>(a); }
__global__ void __launch_bounds__(512) verify_kernel_u8(VerifyArgs a) { verify_body<8>(a); }

// One warp per listed survivor.  Lane r computes the facility range of
// disc row r (trimmed to the chord), a warp prefix sum flattens the rows,
// and each round tests 32 facilities (__ballot_sync/__popc), stopping at k:
// the survivor costs a couple of load latencies, not one per facility.
__device__ __forceinline__ void group_barrier(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Exact count of the facilities strictly nearer to u than q, stopping at k,
// by a group of G warps (G = 1, 2, 4, 8; gi this warp's index in it): lane r
// computes the facility range of disc row r (trimmed to the disc's chord), a
// warp prefix sum flattens the rows, and the group's warps take alternate
// rounds of 32 facilities (__ballot_sync/__popc), adding their counts to the
// group's shared counter *sc and stopping once it reaches k.  The count is
// exact below k and at least k otherwise, whatever G.  Groups of more than
// one warp synchronise on named barrier bar (G * 32 threads).
__device__ __forceinline__ int group_exact_count(float ux, float uy, const QDesc& d, const VerifyArgs& A, int G,
                                                 int gi, int bar, int* sc, unsigned long long& fac,
                                                 unsigned long long& rech)
{
    const int lane = threadIdx.x & 31;
    const float qx = d.qx, qy = d.qy;
    const bool f32 = A.mode == MODE_FP32;
    float Dq32 = 0.0f;
    double Dq64 = 0.0;
    float r;
    const float slack = 4.0f * kU32 * (fabsf(ux) + fabsf(uy) + fabsf(qx) + fabsf(qy)) + 1e-30f;
    if (f32) {
        const float dx = ux - qx, dy = uy - qy;
        Dq32 = fmaf(dx, dx, dy * dy);
        r = sqrtf(Dq32) * (1.0f + 4e-6f) + slack;
    } else {
        const double dx = (double)ux - (double)qx, dy = (double)uy - (double)qy;
        Dq64 = fma(dx, dx, dy * dy);
        r = (float)sqrt_rn64(Dq64) * (1.0f + 4e-6f) + slack;
    }
    if (G > 1) {
        if (gi == 0 && lane == 0) *sc = 0;
        group_barrier(bar, G * 32);
    }
    const Grid& g = A.gf;
    const float ym = 1e-5f * g.cs + 8.0f * kU32 * (fabsf(g.y0) + fabsf(uy) + g.cs * (float)g.gy);
    const int cy0 = cell_coord(uy - r, g.y0, g.inv, g.gy), cy1 = cell_coord(uy + r, g.y0, g.inv, g.gy);
    int cnt = 0;
    bool stop = false;
    for (int rb = cy0; rb <= cy1 && !stop; rb += 32) {
        const int cy = rb + lane;
        int f0 = 0, len = 0;
        if (cy <= cy1) {
            const float ylo = g.y0 + (float)cy * g.cs - ym, yhi = g.y0 + (float)(cy + 1) * g.cs + ym;
            const float dyn = fmaxf(fmaxf(ylo - uy, uy - yhi), 0.0f) * (1.0f - 1e-6f);
            const float w = sqrtf(fmaxf(fmaf(r, r, -dyn * dyn), 0.0f)) * (1.0f + 1e-6f) + slack;
            const int cx0 = cell_coord(ux - w, g.x0, g.inv, g.gx), cx1 = cell_coord(ux + w, g.x0, g.inv, g.gx);
            f0 = A.fstart[VX(cy * g.gx + cx0, A.ncf + 1, 211)];
            len = A.fstart[VX(cy * g.gx + cx1 + 1, A.ncf + 1, 212)] - f0;
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        for (int t0 = gi * 32; t0 < total; t0 += G * 32) {
            const int j = t0 + lane;
            int lo = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int probe = __shfl_sync(FULL, incl, lo + step - 1);
                if (probe <= j) lo += step;
            }
            const int rs = __shfl_sync(FULL, f0, lo & 31);
            const int ri = __shfl_sync(FULL, incl, lo & 31);
            const int rl = __shfl_sync(FULL, len, lo & 31);
            const int i = rs + (j - (ri - rl));
            bool c = false;
            if (j < total && i != d.qpos) {
                const float2 f = A.fxy[VX(i, A.nf, 213)];
                c = f32 ? closer_f32(ux, uy, f.x, f.y, qx, qy, Dq32, &rech)
                        : closer_f64(ux, uy, f.x, f.y, qx, qy, Dq64, &rech);
            }
            const int pc = __popc(__ballot_sync(FULL, c));
            fac += (unsigned long long)min(32, total - t0);
            if (G == 1) {
                cnt += pc;
            } else {
                int now = 0;
                if (lane == 0) now = atomicAdd(sc, pc) + pc;
                cnt = __shfl_sync(FULL, now, 0);
            }
            if (cnt >= d.k) { stop = true; break; }
        }
    }
    if (G > 1) {
        group_barrier(bar, G * 32);
        cnt = *(volatile int*)sc;
        group_barrier(bar, G * 32);      // the counter is read before the next survivor resets it
    }
    return cnt;
}

// Exact recount of the listed survivors; accepted users are appended with
// one atomic per survivor.  A survivor gets a group of G warps of one block
// (G a power of two up to the block's warps, as large as the grid's warps
// allow for all survivors at once), which split its rounds of facilities:
// the count's latency, not its work, bounds a small batch.  sc: one shared
// counter per group.
__device__ __forceinline__ void recount_listed(const VerifyArgs& A, VCount& vc, int* sc)
{
    const int lane = threadIdx.x & 31;
    const int n = min(*A.surv_count, A.surv_cap);
    unsigned long long s_fac = 0, s_rech = 0, s_res = 0;
    const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5;
    const int nw = gridDim.x * wpb;
    int G = 1;
    while (2 * G <= wpb && (long long)n * 2 * G <= nw) G *= 2;
    const int gi = w % G, gid = w / G, gpb = wpb / G;
    for (int i = blockIdx.x * gpb + gid; i < n; i += gridDim.x * gpb) {
        const int2 e = A.surv[VX(i, A.surv_cap, 215)];
        if (e.x < 0) continue;           // the group's warps skip it alike
        const int slot = e.x, pos = e.y;
        const QDesc d = A.qd[slot];
        const float2 u = A.uxy[VX(pos, A.nu, 216)];
        const int c = group_exact_count(u.x, u.y, d, A, G, gi, 1 + gid, sc + gid, s_fac, s_rech);
        if (c < d.k && gi == 0 && lane == 0) {
            const int at = atomicAdd(A.res_count + slot, 1);
            const long long r0 = A.cand_off[slot], region = A.reg_len[slot];
            if (at < region) A.res_pool[VX(r0 + at, A.pool_cap, 217)] = A.uid[VX(pos, A.nu, 218)];
            else atomicOr(A.dropped, 1);
            s_res += 1;
        }
    }
    vc.fac += (unsigned)s_fac;
    vc.rech += (unsigned)s_rech;
    vc.res += (unsigned)s_res;
}

__global__ void __launch_bounds__(256) recount_kernel(VerifyArgs A)
{
    pdl_wait();
    pdl_trigger();
    __shared__ int sc[8];
    VCount vc = {};
    recount_listed(A, vc, sc);
    vc.flush(A.vstats);
}

// ---------------------------------------------------------------- scans
// Scans over the batch's slots run in one block of SCAN_THREADS threads, a
// tile of SCAN_TILE slots per round: values are read coalesced into shared
// memory, each thread scans SCAN_PT consecutive slots of the tile, and a
// block scan of the per-thread sums plus the running carry places them.
constexpr int SCAN_THREADS = 1024, SCAN_PT = 4, SCAN_TILE = SCAN_THREADS * SCAN_PT;

// Result region of each slot: min(candidates, rcap) entries, at 64-bit
// offsets; slots whose region does not fit the pool are flagged and skipped
// (the host grows the pool and runs the batch again).  Work items cover
// every candidate of the slots that fit.
__global__ void __launch_bounds__(SCAN_THREADS)
plan_kernel(QDesc* qd, int nq, long long* cand_off, int* reg_len, long long* region_top, int* chunk_off,
            long long pool_cap, int rcap, int chunk)
{
    pdl_wait();
    pdl_trigger();
    __shared__ int sn[SCAN_TILE];
    __shared__ long long tmp64[32];
    __shared__ int tmp[32];
    const int tid = threadIdx.x;
    long long carry64 = 0;
    int carryc = 0;
    for (int base = 0; base < nq; base += SCAN_TILE) {
        for (int j = tid; j < SCAN_TILE; j += SCAN_THREADS) sn[j] = base + j < nq ? qd[base + j].ncand : 0;
        __syncthreads();
        int n[SCAN_PT];
        long long r[SCAN_PT], rs = 0;
#pragma unroll
        for (int t = 0; t < SCAN_PT; ++t) {
            n[t] = sn[tid * SCAN_PT + t];
            r[t] = min(n[t], rcap);
            rs += r[t];
        }
        long long tot64 = 0;
        long long off = carry64 + block_scan_excl<long long>(rs, tmp64, &tot64);
        int cs = 0;
        bool fits[SCAN_PT];
#pragma unroll
        for (int t = 0; t < SCAN_PT; ++t) {
            const int i = base + tid * SCAN_PT + t;
            fits[t] = off + r[t] <= pool_cap;
            if (i < nq) {
                cand_off[i] = off;
                reg_len[i] = (int)r[t];
                if (!fits[t]) qd[i].flags |= QF_RESULT_OVERFLOW;
            }
            off += r[t];
            cs += fits[t] ? (n[t] + chunk - 1) / chunk : 0;
        }
        int ctot = 0;
        int coff = carryc + block_scan_excl<int>(cs, tmp, &ctot);
#pragma unroll
        for (int t = 0; t < SCAN_PT; ++t) {
            const int i = base + tid * SCAN_PT + t;
            if (i < nq) chunk_off[i] = coff;
            coff += fits[t] ? (n[t] + chunk - 1) / chunk : 0;
        }
        carry64 += tot64;
        carryc += ctot;
        __syncthreads();
    }
    if (tid == 0) {
        *region_top = carry64;
        chunk_off[nq] = carryc;
    }
}

// Output offsets of the stored results (a slot stores at most its region).
__global__ void __launch_bounds__(SCAN_THREADS)
scan_counts_kernel(const int* res_count, const int* reg_len, const long long* region_top, int nq, int* out_off,
                   const int* counters, int* out_off_host)
{
    pdl_wait();
    pdl_trigger();
    __shared__ int sn[SCAN_TILE];
    __shared__ int tmp[32];
    const int tid = threadIdx.x;
    int carry = 0;
    for (int base = 0; base < nq; base += SCAN_TILE) {
        for (int j = tid; j < SCAN_TILE; j += SCAN_THREADS) {
            const int i = base + j;
            sn[j] = i < nq ? min(res_count[i], reg_len[i]) : 0;
        }
        __syncthreads();
        int v[SCAN_PT], vs = 0;
#pragma unroll
        for (int t = 0; t < SCAN_PT; ++t) { v[t] = sn[tid * SCAN_PT + t]; vs += v[t]; }
        int tot = 0;
        int off = carry + block_scan_excl<int>(vs, tmp, &tot);
#pragma unroll
        for (int t = 0; t < SCAN_PT; ++t) {
            const int i = base + tid * SCAN_PT + t;
            if (i < nq) {
                out_off[i] = off;
                if (out_off_host) out_off_host[i] = off;
            }
            off += v[t];
        }
        carry += tot;
        __syncthreads();
    }
    if (tid == 0) {
        const unsigned long long rt = (unsigned long long)*region_top;
        const int tail[1 + OFF_TAIL] = {carry, (int)(unsigned)(rt & 0xffffffffu), (int)(unsigned)(rt >> 32),
                                        counters[2], counters[3]};
        for (int j = 0; j <= OFF_TAIL; ++j) {
            out_off[nq + j] = tail[j];
            if (out_off_host) out_off_host[nq + j] = tail[j];
        }
    }
}

// ---------------------------------------------------------------- finalize
namespace {
__device__ __forceinline__ unsigned okey(int v) { return (unsigned)v ^ 0x80000000u; }

// LSD radix sort of one slot's ids by its warp: 8-bit digits over the bits
// in which the keys differ (key - min), stable passes of 32 keys at a time
// in order, ping-ponging between the slot's pool region (scratch by now)
// and its output range; bins: the warp's 256 shared counters.  Work linear
// in n (about three passes for ids below 2^24), where a bitonic network
// pads to a power of two and takes log^2 steps.
__device__ void warp_radix_slot(unsigned* src, unsigned* dst, int n, int lane, unsigned* bins)
{
    unsigned mn = 0xffffffffu, mx = 0u;
    for (int i = lane; i < n; i += 32) {
        const unsigned k = okey((int)src[i]);
        src[i] = k;
        mn = min(mn, k);
        mx = max(mx, k);
    }
    mn = __reduce_min_sync(FULL, mn);
    mx = __reduce_max_sync(FULL, mx);
    const unsigned span = mx - mn;
    const int passes = span ? (32 - __clz((int)span) + 7) / 8 : 0;
    unsigned* a = src;
    unsigned* b = dst;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        for (int j = lane; j < 256; j += 32) bins[j] = 0u;
        __syncwarp();
        for (int i = lane; i < n; i += 32) atomicAdd(&bins[((a[i] - mn) >> shift) & 255u], 1u);
        __syncwarp();
        // exclusive scan of the bins: lane l owns bins 8l .. 8l + 7
        unsigned v[8], sum = 0u;
#pragma unroll
        for (int j = 0; j < 8; ++j) { v[j] = bins[8 * lane + j]; sum += v[j]; }
        unsigned incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        unsigned run = incl - sum;
#pragma unroll
        for (int j = 0; j < 8; ++j) { bins[8 * lane + j] = run; run += v[j]; }
        __syncwarp();
        for (int i0 = 0; i0 < n; i0 += 32) {
            const int i = i0 + lane;
            const bool ok = i < n;
            const unsigned key = ok ? a[i] : 0u;
            const unsigned d = ok ? ((key - mn) >> shift) & 255u : 256u + (unsigned)lane;   // idle lanes: own groups
            const unsigned mm = __match_any_sync(FULL, d);
            const unsigned base = ok ? bins[d] : 0u;
            __syncwarp();
            if (ok) {
                b[base + __popc(mm & ((1u << lane) - 1))] = key;
                if ((mm >> lane) == 1u) bins[d] = base + __popc(mm);   // the group's last lane moves the bin on
            }
            __syncwarp();
        }
        unsigned* t = a;
        a = b;
        b = t;
    }
    for (int i = lane; i < n; i += 32) dst[i] = a[i] ^ 0x80000000u;   // a is src or dst, element for element
}
}  // namespace

namespace {
// Ascending bitonic sort of 32*E keys held by one warp in registers, key
// t*32 + lane in x[t] (coalesced loads and stores).  Pairs 32 or more apart
// sit in one lane's registers; nearer pairs are exchanged by shuffles.
template <int E>
__device__ __forceinline__ void warp_sort_regs(unsigned (&x)[E], int lane)
{
#pragma unroll
    for (int kk = 2; kk <= 32 * E; kk <<= 1) {
#pragma unroll
        for (int j = kk >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int tj = j >> 5;
#pragma unroll
                for (int t = 0; t < E; ++t) {
                    if ((t & tj) == 0) {
                        const bool up = (((t << 5) | lane) & kk) == 0;
                        const unsigned a = x[t], b = x[t | tj];
                        x[t] = up ? min(a, b) : max(a, b);
                        x[t | tj] = up ? max(a, b) : min(a, b);
                    }
                }
            } else {
                const bool lower = (lane & j) == 0;
#pragma unroll
                for (int t = 0; t < E; ++t) {
                    const unsigned o = __shfl_xor_sync(FULL, x[t], j);
                    const bool up = (((t << 5) | lane) & kk) == 0;
                    x[t] = (lower == up) ? min(x[t], o) : max(x[t], o);
                }
            }
        }
    }
}

template <int E>
__device__ __forceinline__ void warp_sort_slot(const unsigned* src, unsigned* dst, int n, int lane)
{
    unsigned x[E];
#pragma unroll
    for (int t = 0; t < E; ++t) {
        const int i = (t << 5) | lane;
        x[t] = i < n ? okey((int)src[i]) : 0xffffffffu;
    }
    warp_sort_regs<E>(x, lane);
#pragma unroll
    for (int t = 0; t < E; ++t) {
        const int i = (t << 5) | lane;
        if (i < n) dst[i] = x[t] ^ 0x80000000u;
    }
}
}  // namespace

// One warp per slot sorts the slot's stored ids into its output range: up to
// 32 ids by rank counting in registers, up to FIN_WCAP by a bitonic network
// in registers, larger sets by a radix sort through the slot's pool region.
__global__ void __launch_bounds__(32 * FIN_WARPS, 1)
finalize_kernel(int* res_pool, const long long* cand_off, const int* reg_len, const int* res_count,
                int* out_off, int* out, int nq, long long out_cap, int* zero, long long zero_n, FinScan S)
{
    // the next batch's counters (no kernel of this batch uses them), while
    // the predecessor drains
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < zero_n;
         i += (long long)gridDim.x * blockDim.x)
        zero[i] = 0;
    pdl_wait();
    __shared__ unsigned bins[FIN_WARPS][256];
    __shared__ int s_part[FIN_WARPS];
    __shared__ int s_off[FIN_WARPS];      // this block's slots' output offsets
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int first = blockIdx.x * FIN_WARPS;
    if (S.on) {
        // stored ids of the slots before this block's (four loads in flight
        // per thread)
        int part = 0;
        for (int i0 = tid; i0 < first; i0 += 4 * (int)blockDim.x) {
            int v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int i = i0 + j * (int)blockDim.x;
                v[j] = i < first ? min(res_count[i], reg_len[i]) : 0;
            }
            part += v[0] + v[1] + v[2] + v[3];
        }
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(FULL, part, o);
        if (lane == 0) s_part[w] = part;
        __syncthreads();
        if (w == 0) {
            int base = lane < FIN_WARPS ? s_part[lane] : 0;
            for (int o = 16; o > 0; o >>= 1) base += __shfl_xor_sync(FULL, base, o);
            const int sj = first + lane;
            const int nj = (lane < FIN_WARPS && sj < nq) ? min(res_count[sj], reg_len[sj]) : 0;
            int incl = nj;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += y;
            }
            const int excl = base + incl - nj;
            if (lane < FIN_WARPS) s_off[lane] = excl;
            if (lane < FIN_WARPS && sj < nq) {
                out_off[sj] = excl;
                if (S.out_off_host) S.out_off_host[sj] = excl;
            }
            const int total = base + __shfl_sync(FULL, incl, 31);
            if (blockIdx.x == gridDim.x - 1 && lane <= OFF_TAIL) {
                // the total and the run's flags (as scan_counts_kernel)
                const unsigned long long rt = (unsigned long long)*S.region_top;
                const int tail[1 + OFF_TAIL] = {total, (int)(unsigned)(rt & 0xffffffffu), (int)(unsigned)(rt >> 32),
                                                S.counters[2], S.counters[3]};
                out_off[nq + lane] = tail[lane];
                if (S.out_off_host) S.out_off_host[nq + lane] = tail[lane];
            }
        }
    }
    __syncthreads();
    const int s = first + w;
    if (s < nq) {
        const int n = min(res_count[s], reg_len[s]);
        const int os = S.on ? s_off[w] : out_off[s];
        unsigned* src = (unsigned*)(res_pool + cand_off[s]);
        unsigned* dst = (unsigned*)(out + os);
        if ((long long)os + n > out_cap) {
            // past the output's capacity: left out (the batch fails on the host)
        } else if (n <= 32) {
            // stable rank: smaller keys, and equal keys in lower lanes
            const unsigned key = lane < n ? okey((int)src[lane]) : 0xffffffffu;
            int rank = 0;
            for (int j = 0; j < 32; ++j) {
                const unsigned o = __shfl_sync(FULL, key, j);
                rank += (o < key) || (o == key && j < lane);
            }
            if (lane < n) dst[rank] = key ^ 0x80000000u;
        } else if (n <= 64) {
            warp_sort_slot<2>(src, dst, n, lane);
        } else if (n <= 128) {
            warp_sort_slot<4>(src, dst, n, lane);
        } else if (n <= 256) {
            warp_sort_slot<8>(src, dst, n, lane);
        } else if (n <= FIN_WCAP) {
            warp_sort_slot<16>(src, dst, n, lane);
        } else {
            warp_radix_slot(src, dst, n, lane, bins[w]);
        }
    }
}

}  // namespace rknn
