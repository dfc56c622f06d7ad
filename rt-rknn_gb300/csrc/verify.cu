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
// and recount_kernel counts each one exactly, one thread per survivor (many
// independent chains of facility loads in flight): the facility cells
// covering the disc of radius d(u,q) around u, row by row (one contiguous
// range of the cell-sorted facility array per row, trimmed to the disc's
// chord), counting d2(u,f) < d2(u,q) and stopping at k.  Each comparison is
// decided in float (or double) with its error bound, and the undecided ones
// by the exact expansion predicate.  Accepted users are appended with
// warp-aggregated atomics (lanes grouped by query with __match_any_sync).
// When the survivor list is full, the warp recounts its own survivors, the
// whole warp scanning one survivor's rows at a time with
// __ballot_sync/__popc.
#include "verify.cuh"
#include <climits>

namespace rknn {

namespace {
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
        r = (float)sqrt(D) * (1.0f + 4e-6f) + slack;
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
template <typename T, int UPT>
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
        // fmaf); half-plane m is staged as (a, a, b, b), (c, c, w, w).  With
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
        for (; m < nb; ++m) {
            const float4 ab = sp4[2 * m], cw = sp4[2 * m + 1];
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
            if ((m & 7) == 7) {
                bool done = true;
#pragma unroll
                for (int t = 0; t < UPT; ++t) done &= cnt[t] >= k || cw.z > lim[t];
                if (__all_sync(FULL, done)) { ++m; break; }
            }
        }
#pragma unroll
        for (int t = 0; t < UPT; ++t)
            und[t] = rmin[t] <= __float_as_uint(__fmul_ru((float)bu[t], 2.0f * (1.0f + 0x1p-20f))) || lim[t] > rho2;
        evals += (unsigned)(m * nvalid);
        return;
    }
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
            cnt[t] += (mv < -bu[t]);
            und[t] += (mv <= bu[t]) & (mv >= -bu[t]);
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

}  // namespace

template <int UPT>
__device__ __forceinline__ void verify_body(const VerifyArgs& A)
{
    extern __shared__ __align__(16) char smem[];
    // every st-th work-item offset, for the item -> slot lookup
    __shared__ int csmp[VERIFY_SAMPLES];
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // per warp: stage_cap half-planes (32 bytes each), seg_stage segments,
    // the slot's 32 slice bounds
    const size_t plane_bytes = (size_t)A.stage_cap * 32;
    char* sp = smem + w * (plane_bytes + (size_t)A.seg_stage * sizeof(int2) + 32 * sizeof(float));
    int2* ssg = (int2*)(sp + plane_bytes);
    float* sr = (float*)(ssg + A.seg_stage);
    const int st = max(1, (A.nq + VERIFY_SAMPLES) / VERIFY_SAMPLES);     // ceil((nq + 1) / samples)
    const int nsmp = A.nq / st + 1;                                       // samples i * st <= nq
    for (int i = threadIdx.x; i < nsmp; i += blockDim.x) csmp[i] = A.chunk_off[i * st];
    __syncthreads();
    int cur = -1;
    bool seg_staged = false;
    // per-warp statistics (32-bit here, 64-bit in the totals)
    unsigned s_cand = 0, s_evals = 0, s_surv = 0, s_fac = 0, s_rech = 0, s_res = 0;
    const int total = A.chunk_off[A.nq];
    for (;;) {
        int g = 0;
        if (lane == 0) g = atomicAdd(A.work_counter, 1);
        g = __shfl_sync(FULL, g, 0);
        if (g >= total) break;
        // slot s of item g: chunk_off[s] <= g < chunk_off[s+1].  The samples
        // narrow it to [ws, ws + st); there the count of offsets <= g places
        // it (offsets never decrease).
        int lo = 0, hi = nsmp;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (csmp[mid] <= g) lo = mid; else hi = mid;
        }
        int s = lo;
        if (st > 1) {
            const int ws = lo * st, we = min(ws + st, A.nq);
            if (st <= 31) {
                const int j = ws + lane;
                const bool le = j <= we && A.chunk_off[VX(j, A.nq + 1, 215)] <= g;
                s = ws + __popc(__ballot_sync(FULL, le)) - 1;
            } else {
                int l = ws, h = we;
                while (h - l > 1) {
                    const int mid = (l + h) >> 1;
                    if (A.chunk_off[mid] <= g) l = mid; else h = mid;
                }
                s = l;
            }
        }
        if (s != cur && A.mode == MODE_FP32) {
            // staged before the slot record arrives (the loads do not wait on
            // it): stage_cap half-planes, seg_stage segments and the slice
            // bounds, whatever the slot uses of them
            __syncwarp();
            const float4* src = A.planes + (size_t)s * A.lc;
            for (int m = lane; m < A.stage_cap; m += 32) {
                const float4 p = src[m];
                ((float4*)sp)[2 * m] = make_float4(p.x, p.x, p.y, p.y);
                ((float4*)sp)[2 * m + 1] = make_float4(p.z, p.z, p.w, p.w);
            }
            const int2* gsg = A.segs + (size_t)s * A.seg_cap;
            for (int m = lane; m < A.seg_stage; m += 32) ssg[m] = gsg[m];
            if (A.slice_r) sr[lane] = A.slice_r[(size_t)s * 32 + lane];
        }
        const QDesc d = A.qd[s];
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
        const int v0 = (g - A.chunk_off[s]) * (32 * UPT);
        const int2* sg = seg_staged ? ssg : A.segs + (size_t)s * A.seg_cap;
        // segment holding v0: largest i < nseg with sg[i].y <= v0
        int i0 = 0;
        {
            int l = 0, h = d.nseg;
            while (h - l > 1) {
                int mid = (l + h) >> 1;
                if (sg[mid].y <= v0) l = mid; else h = mid;
            }
            i0 = l;
        }
        int pos[UPT];
        float2 u[UPT];
        bool valid[UPT];
        int si = i0;
#pragma unroll
        for (int t = 0; t < UPT; ++t) {
            int v = v0 + t * 32 + lane;
            valid[t] = v < d.ncand;
            pos[t] = 0;
            u[t] = make_float2(0.f, 0.f);
            if (valid[t]) {
                while (si + 1 < d.nseg && sg[si + 1].y <= v) ++si;
                pos[t] = sg[si].x + (v - sg[si].y);
                u[t] = A.uxy[VX(pos[t], A.nu, 205)];
            }
            s_cand += valid[t];
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
        const int nbs = min(d.nb, A.stage_cap);
        // A user within rho/2 of q is decided by the half-planes alone: every
        // facility strictly nearer to it than q lies within 2|u-q| <= rho of
        // q, so it is a half-plane.  With no undecided half-plane the
        // certified count is the exact count.  (All half-planes must be
        // staged for this.)
        const float rho2 = (nbs == d.nb) ? d.rho * d.rho * (1.0f - 1e-5f) : 0.0f;
        if (A.mode == MODE_FP32) filter_users<float, UPT>(d, nbs, sp, pos, u, valid, cnt, und, s_evals, rho2);
        else filter_users<double, UPT>(d, nbs, sp, pos, u, valid, cnt, und, s_evals, rho2);
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
        const long long r0 = A.cand_off[s], region = A.cand_off[s + 1] - r0;
        const bool try_list = ns && A.surv_cap > 0;
        int sbase = 0, rbase = 0;
        if (lane == 0) {
            if (try_list) sbase = atomicAdd(A.surv_count, ns);
            if (tot) rbase = atomicAdd(A.res_count + s, tot);
        }
        sbase = __shfl_sync(FULL, sbase, 0);
        rbase = __shfl_sync(FULL, rbase, 0);
        s_surv += (lane == 0) ? ns : 0;
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
            s_res += (lane == 0) ? tot : 0;
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
                    s_fac += (unsigned)fac;
                    s_rech += (unsigned)rech;
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
                s_res += (lane == 0) ? tot2 : 0;
            }
        }
    }
    // statistics: per-lane partials, one atomic per counter per warp
    for (int o = 16; o > 0; o >>= 1) {
        s_cand += __shfl_xor_sync(FULL, s_cand, o);
        s_evals += __shfl_xor_sync(FULL, s_evals, o);
        s_rech += __shfl_xor_sync(FULL, s_rech, o);
    }
    if (lane == 0 && A.vstats) {
        atomicAdd(&A.vstats->cand, (unsigned long long)s_cand);
        atomicAdd(&A.vstats->plane_evals, (unsigned long long)s_evals);
        atomicAdd(&A.vstats->survivors, (unsigned long long)s_surv);
        atomicAdd(&A.vstats->fac_checks, (unsigned long long)s_fac);
        atomicAdd(&A.vstats->rechecks, (unsigned long long)s_rech);
        atomicAdd(&A.vstats->results, (unsigned long long)s_res);
    }
}

// The verification kernel with 2, 4 or 8 users per lane per work item
// (32 * UPT users per item); blocks of up to 16 warps.
__global__ void __maxnreg__(80) verify_kernel(VerifyArgs a) { verify_body<4>(a); }
__global__ void __maxnreg__(80) verify_kernel_u2(VerifyArgs a) { verify_body<2>(a); }
__global__ void __launch_bounds__(512) verify_kernel_u8(VerifyArgs a) { verify_body<8>(a); }

// One warp per listed survivor.  Lane r computes the facility range of
// disc row r (trimmed to the chord), a warp prefix sum flattens the rows,
// and each round tests 32 facilities (__ballot_sync/__popc), stopping at k:
// the survivor costs a couple of load latencies, not one per facility.
__device__ __forceinline__ int warp_exact_count(float ux, float uy, const QDesc& d, const VerifyArgs& A,
                                                unsigned long long& fac, unsigned long long& rech)
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
        r = (float)sqrt(Dq64) * (1.0f + 4e-6f) + slack;
    }
    const Grid& g = A.gf;
    const float ym = 1e-5f * g.cs + 8.0f * kU32 * (fabsf(g.y0) + fabsf(uy) + g.cs * (float)g.gy);
    const int cy0 = cell_coord(uy - r, g.y0, g.inv, g.gy), cy1 = cell_coord(uy + r, g.y0, g.inv, g.gy);
    int cnt = 0;
    for (int rb = cy0; rb <= cy1; rb += 32) {
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
        for (int t0 = 0; t0 < total; t0 += 32) {
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
            cnt += __popc(__ballot_sync(FULL, c));
            fac += (unsigned long long)min(32, total - t0);
            if (cnt >= d.k) return cnt;
        }
    }
    return cnt;
}

// Exact recount of the listed survivors, one warp each; accepted users are
// appended with one atomic per survivor.
__global__ void __launch_bounds__(256) recount_kernel(VerifyArgs A)
{
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const int n = min(*A.surv_count, A.surv_cap);
    unsigned long long s_fac = 0, s_rech = 0, s_res = 0;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += nw) {
        const int2 e = A.surv[VX(i, A.surv_cap, 215)];
        if (e.x < 0) continue;
        const int slot = e.x, pos = e.y;
        const QDesc d = A.qd[slot];
        const float2 u = A.uxy[VX(pos, A.nu, 216)];
        const int c = warp_exact_count(u.x, u.y, d, A, s_fac, s_rech);
        if (c < d.k && lane == 0) {
            const int at = atomicAdd(A.res_count + slot, 1);
            const long long r0 = A.cand_off[slot], region = A.cand_off[slot + 1] - r0;
            if (at < region) A.res_pool[VX(r0 + at, A.pool_cap, 217)] = A.uid[VX(pos, A.nu, 218)];
            else atomicOr(A.dropped, 1);
            s_res += 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) s_rech += __shfl_xor_sync(FULL, s_rech, o);
    if (lane == 0 && A.vstats && (s_fac | s_res | s_rech)) {
        atomicAdd(&A.vstats->fac_checks, s_fac);
        atomicAdd(&A.vstats->rechecks, s_rech);
        atomicAdd(&A.vstats->results, s_res);
    }
}

// ---------------------------------------------------------------- scans
namespace {
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
}  // namespace

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
plan_kernel(QDesc* qd, int nq, long long* cand_off, int* chunk_off, long long pool_cap, int rcap, int chunk)
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
        cand_off[nq] = carry64;
        chunk_off[nq] = carryc;
    }
}

// Output offsets of the stored results (a slot stores at most its region).
__global__ void __launch_bounds__(SCAN_THREADS)
scan_counts_kernel(const int* res_count, const long long* cand_off, int nq, int* out_off, const int* counters,
                   int* out_off_host)
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
            sn[j] = i < nq ? (int)min((long long)res_count[i], cand_off[i + 1] - cand_off[i]) : 0;
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
        const unsigned long long rt = (unsigned long long)cand_off[nq];
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

// stable LSD radix pass of one block over global memory (256 threads)
__device__ void block_radix_pass(const unsigned* in, unsigned* out, int n, int shift,
                                 unsigned* hist, unsigned (*wc)[256])
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    hist[tid] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += 256) atomicAdd(&hist[(in[i] >> shift) & 255], 1u);
    __syncthreads();
    // exclusive scan of the 256 bins (thread tid owns bin tid)
    unsigned v = hist[tid], x = v;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    __shared__ unsigned wsum[8];
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    unsigned add = 0;
    for (int j = 0; j < w; ++j) add += wsum[j];
    __syncthreads();
    hist[tid] = x - v + add;     // running base of digit tid
    __syncthreads();
    for (int t0 = 0; t0 < n; t0 += 256) {
        int i = t0 + tid;
        bool ok = i < n;
        unsigned key = ok ? in[i] : 0u;
        unsigned dg = ok ? (key >> shift) & 255 : 256u;
        unsigned mm = __match_any_sync(FULL, dg);
        int rank = __popc(mm & ((1u << lane) - 1));
        for (int j = 0; j < 8; ++j) wc[w][lane * 8 + j] = 0;
        __syncwarp();
        if (ok && rank == 0) wc[w][dg] = __popc(mm);
        __syncthreads();
        {   // per digit: prefix over warps
            unsigned acc = hist[tid];
            for (int j = 0; j < 8; ++j) { unsigned c = wc[j][tid]; wc[j][tid] = acc; acc += c; }
            hist[tid] = acc;
        }
        __syncthreads();
        if (ok) out[wc[w][dg] + rank] = key;
        __syncthreads();
    }
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
// in registers.  Larger sets are sorted by the whole block afterwards: in
// shared memory up to FIN_BCAP ids, by four stable radix passes through the
// pool region above that.
__global__ void __launch_bounds__(32 * FIN_WARPS, 1)
finalize_kernel(int* res_pool, const long long* cand_off, const int* res_count, const int* out_off,
                int* out, int nq, long long out_cap)
{
    pdl_wait();
    __shared__ unsigned skeys[FIN_BCAP];
    __shared__ int big[FIN_WARPS];
    __shared__ int nbig;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) nbig = 0;
    __syncthreads();
    const int s = blockIdx.x * FIN_WARPS + w;
    if (s < nq) {
        const int n = (int)min((long long)res_count[s], cand_off[s + 1] - cand_off[s]);
        const unsigned* src = (const unsigned*)(res_pool + cand_off[s]);
        unsigned* dst = (unsigned*)(out + out_off[s]);
        if ((long long)out_off[s] + n > out_cap) {
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
        } else if (lane == 0) {
            big[atomicAdd(&nbig, 1)] = s;
        }
    }
    __syncthreads();
    const int nb = nbig;
    __shared__ unsigned hist[256];
    __shared__ unsigned wc[8][256];
    for (int bi = 0; bi < nb; ++bi) {
        const int t = big[bi];
        const int n = (int)min((long long)res_count[t], cand_off[t + 1] - cand_off[t]);
        unsigned* src = (unsigned*)(res_pool + cand_off[t]);
        unsigned* dst = (unsigned*)(out + out_off[t]);
        if (n <= FIN_BCAP) {
            int P = 1;
            while (P < n) P <<= 1;
            for (int i = tid; i < P; i += blockDim.x) skeys[i] = i < n ? okey((int)src[i]) : 0xffffffffu;
            __syncthreads();
            for (int kk = 2; kk <= P; kk <<= 1) {
                for (int j = kk >> 1; j > 0; j >>= 1) {
                    for (int i = tid; i < P; i += blockDim.x) {
                        const int ixj = i ^ j;
                        if (ixj > i) {
                            const unsigned x = skeys[i], y = skeys[ixj];
                            if ((x > y) == ((i & kk) == 0)) { skeys[i] = y; skeys[ixj] = x; }
                        }
                    }
                    __syncthreads();
                }
            }
            for (int i = tid; i < n; i += blockDim.x) dst[i] = skeys[i] ^ 0x80000000u;
        } else {
            for (int i = tid; i < n; i += blockDim.x) src[i] = okey((int)src[i]);
            __syncthreads();
            block_radix_pass(src, dst, n, 0, hist, wc);
            __syncthreads();
            block_radix_pass(dst, src, n, 8, hist, wc);
            __syncthreads();
            block_radix_pass(src, dst, n, 16, hist, wc);
            __syncthreads();
            block_radix_pass(dst, src, n, 24, hist, wc);
            __syncthreads();
            for (int i = tid; i < n; i += blockDim.x) dst[i] = src[i] ^ 0x80000000u;
        }
        __syncthreads();
    }
}

}  // namespace rknn
