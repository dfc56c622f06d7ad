// One work item of the verification: 32 * UPT consecutive candidate users of
// one slot against its staged half-planes (stage 1), then the users' fate
// (stage 2): accepted users are appended to the slot's result region,
// survivors listed for the exact recount (or counted in-warp when the list
// is full).  Shared by the verification kernel and the slice filter, which
// verifies its own slot's users when their count is small.
#pragma once
#include "verify.cuh"
#include <climits>

namespace rknn {
namespace vitem {

constexpr unsigned FULL = 0xffffffffu;

#ifdef RKNN_CHECKED
__device__ __forceinline__ long long vck(const VerifyArgs& A, long long i, long long n, int id, int line)
{
    if (i < 0 || i >= n) {
        if (A.fault && atomicCAS(A.fault, 0, 1) == 0) {
            A.fault[1] = id; A.fault[2] = (int)i; A.fault[3] = (int)n; A.fault[4] = line;
        }
        return 0;
    }
    return i;
}
#define VX(i, n, id) vck(A, (i), (n), (id), __LINE__)
#else
#define VX(i, n, id) (i)
#endif

template <typename T>
__device__ __forceinline__ int exact_count(float ux, float uy, const QDesc& d, const VerifyArgs& A,
                                           unsigned long long& fac, unsigned long long& rech)
{
    const int lane = threadIdx.x & 31;
    float qx = d.qx, qy = d.qy;
    T Dq;
    float r;
    const float slack = 4.0f * kU32 * (fabsf(ux) + fabsf(uy) + fabsf(qx) + fabsf(qy)) + 1e-30f;
    if (sizeof(T) == 4) {
        float dx = ux - qx, dy = uy - qy;
        float D = fmaf(dx, dx, dy * dy);
        Dq = (T)D;
        r = sqrtf(D) * (1.0f + 4e-6f) + slack;
    } else {
        double dx = (double)ux - (double)qx, dy = (double)uy - (double)qy;
        double D = fma(dx, dx, dy * dy);
        Dq = (T)D;
        r = (float)sqrt_rn64(D) * (1.0f + 4e-6f) + slack;
    }
    const Grid& g = A.gf;
    int cx0 = cell_coord(ux - r, g.x0, g.inv, g.gx), cx1 = cell_coord(ux + r, g.x0, g.inv, g.gx);
    int cy0 = cell_coord(uy - r, g.y0, g.inv, g.gy), cy1 = cell_coord(uy + r, g.y0, g.inv, g.gy);
    int cnt = 0;
    for (int cy = cy0; cy <= cy1; ++cy) {
        const int f0 = A.fstart[VX(cy * g.gx + cx0, A.ncf + 1, 201)], f1 = A.fstart[VX(cy * g.gx + cx1 + 1, A.ncf + 1, 202)];
        for (int b = f0; b < f1; b += 32) {
            int i = b + lane;
            bool c = false;
            if (i < f1 && i != d.qpos) {
                float2 f = A.fxy[VX(i, A.nf, 203)];
                if (sizeof(T) == 4) c = closer_f32(ux, uy, f.x, f.y, qx, qy, (float)Dq, &rech);
                else c = closer_f64(ux, uy, f.x, f.y, qx, qy, (double)Dq, &rech);
            }
            cnt += __popc(__ballot_sync(FULL, c));
            fac += (unsigned long long)min(32, f1 - b);
            if (cnt >= d.k) return cnt;
        }
    }
    return cnt;
}

// Stage 1 over the first nb staged half-planes: cnt = certified
// violations (the loop leaves once every lane's users reached k), und =
// half-planes the bound could not decide.
template <typename T, int UPT, bool COMPACT, bool BITS = false>
__device__ __forceinline__ void filter_users(const QDesc& d, int nb, const char* sp, const int* pos,
                                             const float2* u, const bool* valid, int* cnt, int* und,
                                             unsigned& evals, float rho2)
{
    T x[UPT], y[UPT], bu[UPT];
    // und[t] on return: the half-planes alone do not decide user t, because
    // one was too close to call or the user lies beyond rho/2 of q (then a
    // facility strictly nearer to it need not be a half-plane; rho2 is
    // (rho/2)^2 scaled by 4, or 0 when not every half-plane was staged).
    // lim: above 4|u - q|^2 with margin.  The fourth component w of half-plane
    // m bounds |f - q|^2 from below for it and every later one; once w > lim,
    // none of them lies within 2|u - q| of q, so none is strictly nearer to u
    // than q and the user's remaining half-planes are skipped.  (Half-planes
    // whose w is 0 never cut a user short.)
    float lim[UPT];
    int nvalid = 0;
#pragma unroll
    for (int t = 0; t < UPT; ++t) {
        cnt[t] = valid[t] ? 0 : INT_MAX / 2;
        und[t] = 0;
        nvalid += valid[t];
        const float fx = u[t].x - d.qx, fy = u[t].y - d.qy;
        lim[t] = 4.0f * fmaf(fx, fx, fy * fy) * (1.0f + 1e-4f) + 1e-30f;
        if (sizeof(T) == 4) {
            x[t] = fx; y[t] = fy;
            bu[t] = fmaf(d.k2f, fabsf(fx) + fabsf(fy), d.kf2);
        } else {
            double xx = (double)u[t].x - (double)d.qx, yy = (double)u[t].y - (double)d.qy;
            x[t] = (T)xx; y[t] = (T)yy;
            bu[t] = (T)fma(d.k2f64, fabs(xx) + fabs(yy), d.kf264);
        }
    }
    const int k = d.k;
    int m = 0;
    if constexpr (sizeof(T) == 4) {
        // FP32: users in pairs through the packed FMA (each half rounds as
        // fmaf); half-plane m is staged as (a, a, b, b), (c, c, w, w), or,
        // COMPACT, as (a, b, c, w), the pairs made in registers (half the
        // shared memory: twice the warps per SM where the staging bounds it).  With
        // r = fl(mv + bu): mv < -bu exactly when r is negative (a nonzero
        // exact sum of two floats never rounds to zero, and bu > 0 rules out
        // -0), and |mv| <= bu implies 0 <= r <= 2bu (rounding is monotone):
        // the smallest non-negative r, taken as the least unsigned bit
        // pattern (negative floats have the sign bit set), at most 2bu
        // (rounded up) flags a half-plane too close to call.  That test may
        // also flag a few decided ones; such users are only recounted.
        constexpr int H2 = UPT / 2;
        float2 X[H2], Y[H2], B[H2];
        unsigned rmin[UPT];
#pragma unroll
        for (int h = 0; h < H2; ++h) {
            X[h] = make_float2((float)x[2 * h], (float)x[2 * h + 1]);
            Y[h] = make_float2((float)y[2 * h], (float)y[2 * h + 1]);
            B[h] = make_float2((float)bu[2 * h], (float)bu[2 * h + 1]);
        }
#pragma unroll
        for (int t = 0; t < UPT; ++t) rmin[t] = 0xffffffffu;
        const float4* sp4 = (const float4*)sp;
        auto plane = [&](const float4 ab, const float4 cw) {
            const float2 a2 = make_float2(ab.x, ab.y), b2 = make_float2(ab.z, ab.w), c2 = make_float2(cw.x, cw.y);
#pragma unroll
            for (int h = 0; h < H2; ++h) {
                const float2 mv = __ffma2_rn(a2, X[h], __ffma2_rn(b2, Y[h], c2));
                const float2 r = __fadd2_rn(mv, B[h]);
                const unsigned rx = __float_as_uint(r.x), ry = __float_as_uint(r.y);
                cnt[2 * h] += (int)(rx >> 31);
                cnt[2 * h + 1] += (int)(ry >> 31);
                rmin[2 * h] = min(rmin[2 * h], rx);
                rmin[2 * h + 1] = min(rmin[2 * h + 1], ry);
            }
        };
        // two half-planes a trip (the second one's loads overlap the first
        // one's arithmetic); the early exit is tested after every eighth
        bool stopped = false;
        auto load = [&](int i, float4& ab, float4& cw) {
            if constexpr (COMPACT) {
                const float4 p = sp4[i];
                ab = make_float4(p.x, p.x, p.y, p.y);
                cw = make_float4(p.z, p.z, p.w, p.w);
            } else {
                ab = sp4[2 * i];
                cw = sp4[2 * i + 1];
            }
        };
        for (; m + 2 <= nb; m += 2) {
            float4 ab0, cw0, ab1, cw1;
            load(m, ab0, cw0);
            load(m + 1, ab1, cw1);
            plane(ab0, cw0);
            plane(ab1, cw1);
            if ((m & 7) == 6) {
                bool done = true;
#pragma unroll
                for (int t = 0; t < UPT; ++t) done &= cnt[t] >= k || cw1.z > lim[t];
                if (__all_sync(FULL, done)) { m += 2; stopped = true; break; }
            }
        }
        if (!stopped && m < nb) {
            float4 ab, cw;
            load(m, ab, cw);
            plane(ab, cw);
            ++m;
        }
#pragma unroll
        for (int t = 0; t < UPT; ++t)
            und[t] = rmin[t] <= __float_as_uint(__fmul_ru((float)bu[t], 2.0f * (1.0f + 0x1p-20f))) || lim[t] > rho2;
        evals += (unsigned)(m * nvalid);
        return;
    }
    // FP64 with BITS: the compares of each evaluation on the bits (integer
    // pipes).  A warp's FP64 instruction holds its sub-partition's FP64 pipe
    // for about 64 cycles on GB300, so a lone query's evaluations, two FMAs
    // and three compares each, are bound by that pipe; in large batches the
    // extra registers cost more than the compares (the kernels with four
    // and eight users a lane spill).  mv is finite (finite half-planes and
    // users) and bu >= kf264 > 0, so mv < -bu is order_key(mv) < ~bits(bu),
    // and -bu <= mv <= bu is |mv| <= bu on the magnitude bits.
    for (; m < nb; ++m) {
        T a, b, c;
        float wm;
        if (sizeof(T) == 4) {
            float4 p = ((const float4*)sp)[m];
            a = (T)p.x; b = (T)p.y; c = (T)p.z;
            wm = p.w;
        } else {
            const double* p = (const double*)sp + 4 * m;
            a = (T)p[0]; b = (T)p[1]; c = (T)p[2];
            wm = (float)p[3];       // a float to begin with
        }
#pragma unroll
        for (int t = 0; t < UPT; ++t) {
            T mv = fma(a, x[t], fma(b, y[t], c));
            if constexpr (BITS && sizeof(T) == 8) {
                const long long bb = __double_as_longlong((double)bu[t]);
                cnt[t] += order_key((double)mv) < ~bb;
                und[t] += (__double_as_longlong((double)mv) & 0x7fffffffffffffffll) <= bb;
            } else {
                cnt[t] += (mv < -bu[t]);
                und[t] += (mv <= bu[t]) & (mv >= -bu[t]);
            }
        }
        if ((m & 7) == 7) {
            bool done = true;
#pragma unroll
            for (int t = 0; t < UPT; ++t) done &= cnt[t] >= k || wm > lim[t];
            if (__all_sync(FULL, done)) { ++m; break; }
        }
    }
#pragma unroll
    for (int t = 0; t < UPT; ++t) und[t] |= lim[t] > rho2;
    evals += (unsigned)(m * nvalid);
}

// Exclusive block-wide prefix sum; *total receives the block's sum.
template <typename T>
__device__ T block_scan_excl(T v, T* tmp, T* total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T x = v;
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) tmp[w] = x;
    __syncthreads();
    if (w == 0) {
        T t = lane < (int)(blockDim.x >> 5) ? tmp[lane] : (T)0;
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(FULL, t, o);
            if (lane >= o) t += y;
        }
        tmp[lane] = t;
    }
    __syncthreads();
    *total = tmp[(blockDim.x >> 5) - 1];
    const T excl = x - v + (w > 0 ? tmp[w - 1] : (T)0);
    __syncthreads();
    return excl;
}

// One block: work-item offsets (items of chunk users) of the listed slots
// deflist[0 .. n) into chunk_off[0 .. n].
__device__ __forceinline__ void plan_deferred_block(const VerifyArgs& A, int n, int chunk, int* chunk_off, int* tmp)
{
    const int tid = threadIdx.x;
    int carry = 0;
    for (int base = 0; base < n; base += (int)blockDim.x) {
        const int i = base + tid;
        const int c = i < n ? (__ldcg(&A.qd[__ldcg(A.deflist + i)].ncand) + chunk - 1) / chunk : 0;
        int tot = 0;
        const int off = carry + block_scan_excl<int>(c, tmp, &tot);
        if (i < n) chunk_off[i] = off;
        carry += tot;
    }
    if (tid == 0) chunk_off[n] = carry;
}

// Whether this block is the last of total blocks (counted on *done) to get
// here; every thread of the block calls it.  flag: a shared int.  The
// finished blocks' writes are visible to the last one.
__device__ __forceinline__ bool last_block(int* done, int total, int* flag)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        *flag = atomicAdd(done, 1) == total - 1;
    }
    __syncthreads();
    const bool last = *flag != 0;
    if (last) __threadfence();
    return last;
}

// Per-warp statistics of the verification (32-bit here, 64-bit in the
// totals), one atomic per counter per warp at the end.
struct VCount {
    unsigned cand, evals, surv, fac, rech, res;
    __device__ __forceinline__ void flush(VStats* v)
    {
        const unsigned FULLM = 0xffffffffu;
        for (int o = 16; o > 0; o >>= 1) {
            cand += __shfl_xor_sync(FULLM, cand, o);
            evals += __shfl_xor_sync(FULLM, evals, o);
            rech += __shfl_xor_sync(FULLM, rech, o);
        }
        if ((threadIdx.x & 31) == 0 && v && (cand | evals | surv | fac | rech | res)) {
            atomicAdd(&v->cand, (unsigned long long)cand);
            atomicAdd(&v->plane_evals, (unsigned long long)evals);
            atomicAdd(&v->survivors, (unsigned long long)surv);
            atomicAdd(&v->fac_checks, (unsigned long long)fac);
            atomicAdd(&v->rechecks, (unsigned long long)rech);
            atomicAdd(&v->results, (unsigned long long)res);
        }
    }
};

// Item of slot s starting at candidate v0.  sp: the slot's first nbs
// half-planes staged (FP32: 32 bytes each as (a, a, b, b), (c, c, w, w);
// FP64: four doubles), sg: its segments (shared or global memory), sr: its
// 32 slice bounds.  r0_in/region_in: the slot's result region, or -1 to read
// it from cand_off/reg_len.
template <int UPT, bool COMPACT = false, bool BITS = false>
__device__ __forceinline__ void verify_item(const VerifyArgs& A, const QDesc& d, int s, int v0, const char* sp,
                                            const int2* sg, const float* sr, int nbs, long long r0_in,
                                            long long region_in, VCount& vc)
{
    const int lane = threadIdx.x & 31;
    // user v's segment: the largest i < nseg with sg[i].y <= v (sg[0].y
    // is 0), by bisection with one trip count for all lanes, the UPT
    // searches interleaved.  [b, b + n) holds the answer throughout.
    int b[UPT];
#pragma unroll
    for (int t = 0; t < UPT; ++t) b[t] = 0;
    for (int n = d.nseg; n > 1;) {
        const int half = n >> 1;
#pragma unroll
        for (int t = 0; t < UPT; ++t)
            if (sg[b[t] + half].y <= v0 + t * 32 + lane) b[t] += half;
        n -= half;
    }
    int pos[UPT];
    float2 u[UPT];
    bool valid[UPT];
#pragma unroll
    for (int t = 0; t < UPT; ++t) {
        const int v = v0 + t * 32 + lane;
        valid[t] = v < d.ncand;
        pos[t] = 0;
        u[t] = make_float2(0.f, 0.f);
        if (valid[t]) {
            const int2 e = sg[b[t]];
            pos[t] = e.x + (v - e.y);
            u[t] = A.uxy[VX(pos[t], A.nu, 205)];
        }
        vc.cand += valid[t];
    }
    // the ids and the slot's result region are read after the
    // half-planes: bring their lines in now
#pragma unroll
    for (int t = 0; t < UPT; ++t)
        if (valid[t]) prefetch_l1(A.uid + pos[t]);
    if (lane == 0 && region_in < 0) {
        prefetch_l1(A.cand_off + s);
        prefetch_l1(A.reg_len + s);
    }
    // a user beyond its slice's bound R(P) has k facilities strictly nearer
    // than q (the slice filter's rule): drop it before the half-planes.
    // Slices were widened by 2^-14 rad, far beyond slice_of's 1e-7 rad
    // edge uncertainty, so the computed slice's bound holds for the user.
    if (d.flags & QF_SLICE_R) {
        const float* Rq = sr;
#pragma unroll
        for (int t = 0; t < UPT; ++t) {
            if (!valid[t]) continue;
            const float dx = u[t].x - d.qx, dy = u[t].y - d.qy;
            const float Rs = Rq[slice_of(dx, dy)];
            if (fmaf(dx, dx, dy * dy) * (1.0f - 1e-6f) > Rs * Rs) valid[t] = false;
        }
    }
    int cnt[UPT], und[UPT];
    // A user within rho/2 of q is decided by the half-planes alone: every
    // facility strictly nearer to it than q lies within 2|u-q| <= rho of
    // q, so it is a half-plane.  With no undecided half-plane the
    // certified count is the exact count.  (All half-planes must be
    // staged for this.)
    const float rho2 = (nbs == d.nb) ? d.rho * d.rho * (1.0f - 1e-5f) : 0.0f;
    if (A.mode == MODE_FP32) filter_users<float, UPT, COMPACT>(d, nbs, sp, pos, u, valid, cnt, und, vc.evals, rho2);
    else filter_users<double, UPT, false, BITS>(d, nbs, sp, pos, u, valid, cnt, und, vc.evals, rho2);
    bool direct[UPT];
#pragma unroll
    for (int t = 0; t < UPT; ++t) direct[t] = valid[t] && cnt[t] < d.k && und[t] == 0;

    // stage 2: survivors go to the list for recount_kernel (when it is
    // full, the warp counts them itself, one user at a time); directly
    // accepted users are appended to the slot's results.  The accepted
    // users' ids, the slot's region and both reservations are requested
    // before any of them is waited for.
    unsigned sm[UPT], am[UPT];
    int ns = 0, tot = 0;
    int idv[UPT];
#pragma unroll
    for (int t = 0; t < UPT; ++t) {
        idv[t] = direct[t] ? A.uid[VX(pos[t], A.nu, 207)] : 0;
        sm[t] = __ballot_sync(FULL, valid[t] && cnt[t] < d.k && !direct[t]);
        am[t] = __ballot_sync(FULL, direct[t]);
        ns += __popc(sm[t]);
        tot += __popc(am[t]);
    }
    const long long r0 = region_in < 0 ? A.cand_off[s] : r0_in;
    const long long region = region_in < 0 ? (long long)A.reg_len[s] : region_in;
    const bool try_list = ns && A.surv_cap > 0;
    int sbase = 0, rbase = 0;
    if (lane == 0) {
        if (try_list) sbase = atomicAdd(A.surv_count, ns);
        if (tot) rbase = atomicAdd(A.res_count + s, tot);
    }
    sbase = __shfl_sync(FULL, sbase, 0);
    rbase = __shfl_sync(FULL, rbase, 0);
    vc.surv += (lane == 0) ? ns : 0;
    bool listed = false;
    if (try_list) {
        if ((long long)sbase + ns <= A.surv_cap) {
            int o = 0;
#pragma unroll
            for (int t = 0; t < UPT; ++t) {
                if (sm[t] & (1u << lane))
                    A.surv[VX((long long)sbase + o + __popc(sm[t] & ((1u << lane) - 1)), A.surv_cap, 214)] = make_int2(s, pos[t]);
                o += __popc(sm[t]);
            }
            listed = true;
        } else {
            // the reservation straddles the end: mark its listed part empty
            for (int i = sbase + lane; i < A.surv_cap && i < sbase + ns; i += 32) A.surv[i] = make_int2(-1, 0);
        }
    }
    // the slot's region holds min(candidates, rcap) ids; results beyond
    // it are counted, not stored, and the host reruns
    if (tot) {
        if (lane == 0 && rbase + tot > region) atomicOr(A.dropped, 1);
        int o = 0;
#pragma unroll
        for (int t = 0; t < UPT; ++t) {
            const long long at = (long long)rbase + o + __popc(am[t] & ((1u << lane) - 1));
            if (direct[t] && at < region) A.res_pool[VX(r0 + at, A.pool_cap, 206)] = idv[t];
            o += __popc(am[t]);
        }
        vc.res += (lane == 0) ? tot : 0;
    }
    if (!listed && ns) {
        // survivors the list could not take: counted here, appended with
        // one more reservation
        bool acc[UPT];
#pragma unroll
        for (int t = 0; t < UPT; ++t) {
            acc[t] = false;
            unsigned m = sm[t];
            while (m) {
                int l = __ffs(m) - 1;
                m &= m - 1;
                const float2 ul = A.uxy[VX(__shfl_sync(FULL, pos[t], l), A.nu, 219)];
                unsigned long long fac = 0, rech = 0;
                int c = (A.mode == MODE_FP32) ? exact_count<float>(ul.x, ul.y, d, A, fac, rech)
                                              : exact_count<double>(ul.x, ul.y, d, A, fac, rech);
                vc.fac += (unsigned)fac;
                vc.rech += (unsigned)rech;
                if (lane == l) acc[t] = c < d.k;
            }
        }
        unsigned bm[UPT];
        int tot2 = 0;
#pragma unroll
        for (int t = 0; t < UPT; ++t) { bm[t] = __ballot_sync(FULL, acc[t]); tot2 += __popc(bm[t]); }
        if (tot2) {
            int base = 0;
            if (lane == 0) base = atomicAdd(A.res_count + s, tot2);
            base = __shfl_sync(FULL, base, 0);
            if (lane == 0 && base + tot2 > region) atomicOr(A.dropped, 1);
            int o = 0;
#pragma unroll
            for (int t = 0; t < UPT; ++t) {
                const long long at = (long long)base + o + __popc(bm[t] & ((1u << lane) - 1));
                if (acc[t] && at < region) A.res_pool[VX(r0 + at, A.pool_cap, 220)] = A.uid[VX(pos[t], A.nu, 221)];
                o += __popc(bm[t]);
            }
            vc.res += (lane == 0) ? tot2 : 0;
        }
    }
}

}  // namespace vitem
}  // namespace rknn
