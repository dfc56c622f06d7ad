// Influence-zone kernel: one warp per query.
//
// Follows the influence-zone filter of rknn-inf (rknn-inf/inf.cpp:201-585)
// over the engine's uniform facility grid instead of an R*-tree:
//   * best-first search from the query facility q; grid cells play the role
//     of R*-tree leaf nodes (their MBR is the tight box of their facilities)
//     and are pushed lazily, ring by ring, before any entry whose key could
//     follow them;
//   * the same three pruning rules for points and cells (inf.cpp:262-354,
//     460-552): > 2 x furthest zone vertex -> prune; < 2 x nearest bisector ->
//     keep; otherwise the vertex test over vertices with count k-1 and the
//     eight extreme boundary vertices;
//   * an accepted facility adds its perpendicular bisector (inf.h:150-192),
//     bumps the counts of the vertices on its invalid side, adds its
//     intersections with the space boundary and with every earlier bisector
//     (deduplicated at 1e-9, inf.cpp:366-428), and drops vertices whose count
//     reaches k.
// Every decision is taken on the double-precision values the reference
// computes (no contraction: this file is built with -fmad=false).  A
// float32 evaluation with a proven error bound settles each decision first;
// only the undecided ones run in FP64.  Bisector-bisector intersections whose
// float32 interval is certified to lie on the invalid side of at least k
// bisectors are discarded before the FP64 division: the reference creates and
// then erases them in the same step.
//
// Epilogue: the bisectors become exact half-planes relative to q for the
// verification kernel, and a ring scan over the user grid keeps every cell
// that is not certified to lie on the strict far side of >= k bisectors.  The
// region with fewer than k violated half-planes is star-shaped around q (each
// half-plane's invalid side is convex and excludes q), so a full ring of
// pruned cells closes it; users outside the kept cells cannot be results.
#include "rknn_common.cuh"
#include "zone.cuh"
#include <cfloat>

namespace rknn {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr double EPS = 1e-9;           // inf.cpp:270,375,408; inf.h:324

// flags of a vertex
constexpr uint8_t VB_BND = 1, VB_ON = 2;
// flags of a line
constexpr uint8_t LB_VERT = 1, LB_VALID = 2;

struct Line64 {
    double a, b;        // y = a x + b, or x = b when vertical
    int vert, valid;
};

struct WarpScalars {
    int nV, nL, nP, nC;
    int nCons;
    int flags;
    int stop;
    int pad;
    double far_;        // furthest vertex distance (FP64, as the reference)
    double nearb;       // nearest bisector distance
    double maxd2;
};

__device__ __forceinline__ double dsq(double a) { return __dmul_rn(a, a); }

// Point::distance_to (rknn-inf/RStarTree2D.cpp:4-6), squared
__device__ __forceinline__ double d2_64(double ax, double ay, double bx, double by)
{
    double dx = __dsub_rn(ax, bx), dy = __dsub_rn(ay, by);
    return __dadd_rn(dsq(dx), dsq(dy));
}

// min_distance_to_rect (rknn-inf/inf.h:265-272), squared
__device__ __forceinline__ double rect_d2_64(double px, double py, float4 r)
{
    double dx = 0, dy = 0;
    if (px < (double)r.x) dx = __dsub_rn((double)r.x, px);
    else if (px > (double)r.z) dx = __dsub_rn(px, (double)r.z);
    if (py < (double)r.y) dy = __dsub_rn((double)r.y, py);
    else if (py > (double)r.w) dy = __dsub_rn(py, (double)r.w);
    return __dadd_rn(dsq(dx), dsq(dy));
}

__device__ __forceinline__ float rect_dx32(float v, float lo, float hi)
{
    return v < lo ? lo - v : (v > hi ? v - hi : 0.0f);
}

// perpendicular_bisector (rknn-inf/inf.h:150-192), query first
__device__ Line64 make_bisector(double qx, double qy, double px, double py)
{
    Line64 l;
    double mx = __ddiv_rn(__dadd_rn(qx, px), 2.0), my = __ddiv_rn(__dadd_rn(qy, py), 2.0);
    l.a = 0; l.b = 0; l.vert = 0;
    if (qx == px) {
        l.a = 0; l.b = my;
    } else if (qy == py) {
        l.vert = 1; l.b = mx;
    } else {
        double s = __ddiv_rn(__dsub_rn(py, qy), __dsub_rn(px, qx));
        double ps = __ddiv_rn(-1.0, s);
        double yi = __dsub_rn(my, __dmul_rn(ps, mx));
        if (isinf(ps)) { l.vert = 1; l.b = yi; }
        else { l.a = ps; l.b = yi; }
    }
    if (l.vert) l.valid = (qx >= l.b) ? 1 : 0;
    else l.valid = (qy >= __dadd_rn(__dmul_rn(l.a, qx), l.b)) ? 1 : 0;
    return l;
}

// Line::is_on_valid_side (rknn-inf/inf.h:77-93) in FP64
__device__ __forceinline__ bool valid64(double a, double b, int vert, int valid,
                                        double x, double y)
{
    if (vert) return valid ? (x >= b) : (x <= b);
    double t = __dadd_rn(__dmul_rn(a, x), b);
    return valid ? (y >= t) : (y <= t);
}

// find_line_intersection (rknn-inf/inf.h:303-333) in FP64
__device__ __forceinline__ bool intersect64(double a1, double b1, int v1,
                                            double a2, double b2, int v2,
                                            double& x, double& y)
{
    if (v1 && v2) return false;
    if (v1) { x = b1; y = __dadd_rn(__dmul_rn(a2, b1), b2); return true; }
    if (v2) { x = b2; y = __dadd_rn(__dmul_rn(a1, b2), b1); return true; }
    if (fabs(__dsub_rn(a1, a2)) < EPS) return false;
    x = __ddiv_rn(__dsub_rn(b2, b1), __dsub_rn(a1, a2));
    y = __dadd_rn(__dmul_rn(a1, x), b1);
    return true;
}

// min_distance_to_line (rknn-inf/inf.h:275-287)
__device__ double line_dist64(double px, double py, double a, double b, int vert)
{
    if (vert) return fabs(__dsub_rn(px, b));
    double num = fabs(__dadd_rn(__dsub_rn(__dmul_rn(a, px), py), b));
    double den = __dsqrt_rn(__dadd_rn(__dmul_rn(a, a), 1.0));
    return __ddiv_rn(num, den);
}

struct Slice {
    double *vx, *vy, *vd2;
    float *vx32, *vy32;
    int *vcnt;
    uint8_t *vfl;
    int *cons;
    double *la, *lb;
    float *la32, *lb32, *lb3;
    uint8_t *lfl;
    int *lpos;
    uint64_t *pqk;
    uint32_t *pqc;
    double *cx, *cy;
    float *cx32, *cy32;
    int *ccnt;
    uint8_t *cfl;
    uint64_t *tk;
    uint32_t *tc;
    uint32_t *bitmap;
    WarpScalars *sc;
};

__device__ Slice carve(char* base, const ZoneCaps& c)
{
    ZoneLayout L = zone_layout(c);
    Slice s;
    s.vx = (double*)(base + L.vx);
    s.vy = (double*)(base + L.vy);
    s.vd2 = (double*)(base + L.vd2);
    s.vx32 = (float*)(base + L.vx32);
    s.vy32 = (float*)(base + L.vy32);
    s.vcnt = (int*)(base + L.vcnt);
    s.vfl = (uint8_t*)(base + L.vfl);
    s.cons = (int*)(base + L.cons);
    s.la = (double*)(base + L.la);
    s.lb = (double*)(base + L.lb);
    s.la32 = (float*)(base + L.la32);
    s.lb32 = (float*)(base + L.lb32);
    s.lb3 = (float*)(base + L.lb3);
    s.lfl = (uint8_t*)(base + L.lfl);
    s.lpos = (int*)(base + L.lpos);
    s.pqk = (uint64_t*)(base + L.pqk);
    s.pqc = (uint32_t*)(base + L.pqc);
    s.cx = (double*)(base + L.cx);
    s.cy = (double*)(base + L.cy);
    s.cx32 = (float*)(base + L.cx32);
    s.cy32 = (float*)(base + L.cy32);
    s.ccnt = (int*)(base + L.ccnt);
    s.cfl = (uint8_t*)(base + L.cfl);
    s.tk = (uint64_t*)(base + L.tk);
    s.tc = (uint32_t*)(base + L.tc);
    s.bitmap = (uint32_t*)(base + L.vx);   // reused after the zone is built
    s.sc = (WarpScalars*)(base + L.sc);
    return s;
}

// ---- priority queue (lane 0 only) ------------------------------------------
// Keys are squared distances (non-negative doubles), stored as their bit
// patterns: for non-negative doubles the integer order is the numeric order,
// so the heap needs no floating-point comparison.
__device__ __forceinline__ bool pq_less(uint64_t k1, uint32_t c1, uint64_t k2, uint32_t c2)
{
    return k1 < k2 || (k1 == k2 && c1 < c2);
}

__device__ bool pq_push(uint64_t* K, uint32_t* C, int& n, int cap, uint64_t key, uint32_t code)
{
    if (n >= cap) return false;
    int i = n++;
    while (i > 0) {
        int p = (i - 1) >> 1;
        if (!pq_less(key, code, K[p], C[p])) break;
        K[i] = K[p];
        C[i] = C[p];
        i = p;
    }
    K[i] = key;
    C[i] = code;
    return true;
}

__device__ void pq_pop(uint64_t* K, uint32_t* C, int& n)
{
    uint64_t lk = K[n - 1];
    uint32_t lc = C[n - 1];
    --n;
    int i = 0;
    for (;;) {
        int l = 2 * i + 1;
        if (l >= n) break;
        int c = (l + 1 < n && pq_less(K[l + 1], C[l + 1], K[l], C[l])) ? l + 1 : l;
        if (!pq_less(K[c], C[c], lk, lc)) break;
        K[i] = K[c];
        C[i] = C[c];
        i = c;
    }
    if (n > 0) { K[i] = lk; C[i] = lc; }
}

constexpr uint32_t KIND_POINT = 0x80000000u;

// ---- warp helpers -------------------------------------------------------------
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ int warp_sum(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// Decision of the vertex test for one vertex, float32 first.  Returns 1 if
// dist64(p, v) < dist64(q, v) as the reference computes it.
//   D  = squared distance from the facility (or rectangle) to the vertex
//   d2v = vertex's squared distance to q (FP64, the reference's dq squared)
__device__ __forceinline__ bool closer_than_q(float dxp, float dyp, float E, double d2v,
                                              double dx64, double dy64)
{
    float D = fmaf(dxp, dxp, dyp * dyp);
    float ep = E + kU32 * (fabsf(dxp) + fabsf(dyp));
    float err = fmaf(2.0f * (fabsf(dxp) + fabsf(dyp)) + 2.0f * ep, ep, 4.0f * kU32 * D) + 1e-30f;
    float V = (float)d2v;
    float vlo = V * (1.0f - 4.0f * kU32), vhi = V * (1.0f + 4.0f * kU32);
    if (D + err < vlo) return true;
    if (D - err > vhi) return false;
    double dp = __dsqrt_rn(__dadd_rn(dsq(dx64), dsq(dy64)));
    return dp < __dsqrt_rn(d2v);
}

}  // namespace

// ============================================================================
__global__ void __launch_bounds__(ZONE_WARPS * 32)
zone_kernel(ZoneArgs A)
{
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const ZoneLayout LY = zone_layout(A.caps);
    char* base = A.use_global
        ? A.gscratch + (size_t)(blockIdx.x * ZONE_WARPS + wib) * LY.bytes
        : smem + (size_t)wib * LY.bytes;
    Slice S = carve(base, A.caps);
    const int VC = A.caps.vc, LC = A.caps.lc, PC = A.caps.pc;
    const double sx0 = A.sx0, sy0 = A.sy0, sx1 = A.sx1, sy1 = A.sy1;
    // largest rounding error of a vertex coordinate stored as float
    const float E = kU32 * (float)fmax(fmax(fabs(sx0), fabs(sx1)), fmax(fabs(sy0), fabs(sy1))) * 1.01f + 1e-37f;
    const float fsx0 = __double2float_rd(sx0), fsy0 = __double2float_rd(sy0);
    const float fsx1 = __double2float_ru(sx1), fsy1 = __double2float_ru(sy1);
    const double slack = 1e-5 * ((double)A.gf.cs + fmax(fmax(fabs(sx0), fabs(sx1)), fmax(fabs(sy0), fabs(sy1))));

    for (;;) {
        int slot = 0;
        if (lane == 0) slot = atomicAdd(A.work_counter, 1);
        slot = __shfl_sync(FULL, slot, 0);
        if (slot >= A.nq) break;
        const int s = A.order ? A.order[slot] : slot;
        const int qin = A.q_in[s];
        const int k = A.k_in[s];
        QDesc* qd = A.qd + s;
        ZStats zs = {};
        int qflags = 0;
        if (qin < 0 || qin >= A.nf || k <= 0) {
            if (lane == 0) {
                QDesc d = {};
                d.qpos = -1;
                d.k = k;
                d.flags = QF_BAD_QUERY;
                *qd = d;
                A.zst[s] = zs;
                A.segs[(size_t)s * A.seg_cap] = make_int2(0, 0);
            }
            continue;
        }
        const int qpos = A.fpos[qin];
        const float2 qf = A.fxy[qpos];
        const double qx = qf.x, qy = qf.y;
        WarpScalars* sc = S.sc;

        // ---- init: four space corners (inf.cpp:211-226) -------------------
        if (lane < 4) {
            double x = (lane & 1) ? sx1 : sx0;
            double y = (lane & 2) ? sy1 : sy0;
            S.vx[lane] = x;
            S.vy[lane] = y;
            S.vx32[lane] = (float)x;
            S.vy32[lane] = (float)y;
            S.vd2[lane] = d2_64(x, y, qx, qy);
            S.vcnt[lane] = 0;
            S.vfl[lane] = VB_BND;
        }
        if (lane == 0) {
            sc->nV = 4; sc->nL = 0; sc->nP = 0; sc->flags = 0; sc->stop = 0;
            sc->nCons = -1;
            sc->nearb = DBL_MAX;
        }
        __syncwarp();
        {
            double m = lane < 4 ? S.vd2[lane] : 0.0;
            m = warp_max(m);
            if (lane == 0) sc->far_ = __dsqrt_rn(m);
        }
        __syncwarp();

        const int qcx = cell_coord(qf.x, A.gf.x0, A.gf.inv, A.gf.gx);
        const int qcy = cell_coord(qf.y, A.gf.y0, A.gf.inv, A.gf.gy);
        const int rmaxf = max(max(qcx, A.gf.gx - 1 - qcx), max(qcy, A.gf.gy - 1 - qcy));
        int ring = 0;        // next facility ring to expand

        // ---- best-first search --------------------------------------------
        for (;;) {
            // make the top poppable: expand rings whose cells could precede it
            for (;;) {
                int nP = sc->nP;
                double far2 = 2.0 * sc->far_;
                bool can_expand = ring <= rmaxf;
                double Lr = ring == 0 ? 0.0 : (double)(ring - 1) * (double)A.gf.cs - slack;
                if (Lr < 0) Lr = 0;
                if (can_expand && Lr > far2 * (1.0 + 1e-9) + slack) can_expand = false;
                if (!can_expand) break;
                if (nP > 0 && __longlong_as_double((long long)S.pqk[0]) < Lr * Lr) break;
                // expand ring `ring`: 8*ring cells (1 for ring 0)
                int ncell = ring == 0 ? 1 : 8 * ring;
                for (int t0 = 0; t0 < ncell; t0 += 32) {
                    int t = t0 + lane;
                    int cxx = 0, cyy = 0;
                    bool ok = t < ncell;
                    if (ok) {
                        if (ring == 0) { cxx = qcx; cyy = qcy; }
                        else {
                            int side = 2 * ring + 1;
                            if (t < side) { cxx = qcx - ring + t; cyy = qcy - ring; }
                            else if (t < 2 * side) { cxx = qcx - ring + (t - side); cyy = qcy + ring; }
                            else if (t < 2 * side + (2 * ring - 1)) { cxx = qcx - ring; cyy = qcy - ring + 1 + (t - 2 * side); }
                            else { cxx = qcx + ring; cyy = qcy - ring + 1 + (t - 2 * side - (2 * ring - 1)); }
                        }
                        ok = cxx >= 0 && cxx < A.gf.gx && cyy >= 0 && cyy < A.gf.gy;
                    }
                    int cid = 0;
                    if (ok) {
                        cid = cyy * A.gf.gx + cxx;
                        ok = A.fstart[cid + 1] > A.fstart[cid];
                    }
                    double key = ok ? rect_d2_64(qx, qy, A.fmbr[cid]) : 0.0;
                    unsigned m = __ballot_sync(FULL, ok);
                    int rank = __popc(m & ((1u << lane) - 1));
                    if (ok) { S.tk[rank] = (uint64_t)__double_as_longlong(key); S.tc[rank] = (uint32_t)cid; }
                    __syncwarp();
                    if (lane == 0) {
                        int n = sc->nP;
                        for (int i = 0; i < __popc(m); ++i)
                            if (!pq_push(S.pqk, S.pqc, n, PC, S.tk[i], S.tc[i])) { sc->flags |= QF_ZONE_PQ_OVERFLOW; break; }
                        sc->nP = n;
                    }
                    __syncwarp();
                }
                ring++;
                if (sc->flags) break;
            }
            if (sc->flags || sc->nP == 0) break;
            uint64_t keybits = 0;
            uint32_t code = 0;
            if (lane == 0) {
                keybits = S.pqk[0];
                code = S.pqc[0];
                int n = sc->nP;
                pq_pop(S.pqk, S.pqc, n);
                sc->nP = n;
            }
            keybits = __shfl_sync(FULL, keybits, 0);
            code = __shfl_sync(FULL, code, 0);
            const double key = __longlong_as_double((long long)keybits);
            __syncwarp();

            const bool is_point = (code & KIND_POINT) != 0;
            const int id = (int)(code & ~KIND_POINT);
            double px = 0, py = 0;
            float4 mbr = make_float4(0, 0, 0, 0);
            if (is_point) {
                if (id == qpos) continue;
                float2 pf = A.fxy[id];
                px = pf.x; py = pf.y;
                if (A.skip_coincident && pf.x == qf.x && pf.y == qf.y) continue;
                zs.pts++;
            } else {
                mbr = A.fmbr[id];
                zs.cells++;
            }
            // rules 1 and 2 (inf.cpp:262-267, 460-465): key is the squared distance
            const double dq = __dsqrt_rn(key);
            bool prune;
            if (dq > 2.0 * sc->far_) prune = true;
            else if (dq < 2.0 * sc->nearb) prune = false;
            else {
                // ---- vertex test (inf.cpp:268-353, 466-551) -------------
                if (sc->nCons < 0) {
                    // extreme boundary vertices with count < k
                    // e[0..7]: left min/max y, right min/max y, bottom min/max x, top min/max x
                    int nV = sc->nV;
                    int best[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) best[j] = -1;
                    for (int i = lane; i < nV; i += 32) {
                        if (!((S.vfl[i] & VB_BND) && S.vcnt[i] < k)) continue;
                        double x = S.vx[i], y = S.vy[i];
                        bool onL = fabs(__dsub_rn(x, sx0)) < EPS, onR = fabs(__dsub_rn(x, sx1)) < EPS;
                        bool onB = fabs(__dsub_rn(y, sy0)) < EPS, onT = fabs(__dsub_rn(y, sy1)) < EPS;
                        if (onL) {
                            if (best[0] < 0 || y < S.vy[best[0]]) best[0] = i;
                            if (best[1] < 0 || y > S.vy[best[1]]) best[1] = i;
                        }
                        if (onR) {
                            if (best[2] < 0 || y < S.vy[best[2]]) best[2] = i;
                            if (best[3] < 0 || y > S.vy[best[3]]) best[3] = i;
                        }
                        if (onB) {
                            if (best[4] < 0 || x < S.vx[best[4]]) best[4] = i;
                            if (best[5] < 0 || x > S.vx[best[5]]) best[5] = i;
                        }
                        if (onT) {
                            if (best[6] < 0 || x < S.vx[best[6]]) best[6] = i;
                            if (best[7] < 0 || x > S.vx[best[7]]) best[7] = i;
                        }
                    }
                    // reduce: strict improvement, earliest index on ties
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        int b = best[j];
                        for (int o = 16; o > 0; o >>= 1) {
                            int ob = __shfl_xor_sync(FULL, b, o);
                            if (ob < 0) continue;
                            if (b < 0) { b = ob; continue; }
                            double vb = (j < 4) ? S.vy[b] : S.vx[b];
                            double vo = (j < 4) ? S.vy[ob] : S.vx[ob];
                            bool wantMin = (j & 1) == 0;
                            bool better = wantMin ? (vo < vb) : (vo > vb);
                            if (better || (vo == vb && ob < b)) b = ob;
                        }
                        best[j] = b;
                    }
                    // considered list
                    int nC = 0;
                    for (int i0 = 0; i0 < nV; i0 += 32) {
                        int i = i0 + lane;
                        bool c = false;
                        if (i < nV) {
                            int cnt = S.vcnt[i];
                            if (cnt == k - 1) c = true;
                            else if ((S.vfl[i] & VB_BND) && cnt < k) {
                                double x = S.vx[i], y = S.vy[i];
#pragma unroll
                                for (int j = 0; j < 8; ++j) {
                                    int b = best[j];
                                    if (b >= 0 && fabs(__dsub_rn(x, S.vx[b])) < EPS &&
                                        fabs(__dsub_rn(y, S.vy[b])) < EPS) c = true;
                                }
                            }
                        }
                        unsigned m = __ballot_sync(FULL, c);
                        if (c) S.cons[nC + __popc(m & ((1u << lane) - 1))] = i;
                        nC += __popc(m);
                    }
                    if (lane == 0) sc->nCons = nC;
                    __syncwarp();
                }
                const int nC = sc->nCons;
                bool hit = false;
                const float px32 = (float)px, py32 = (float)py;
                for (int t = lane; t < nC && !hit; t += 32) {
                    int i = S.cons[t];
                    double d2v = S.vd2[i];
                    if (is_point) {
                        float dxp = px32 - S.vx32[i], dyp = py32 - S.vy32[i];
                        hit = closer_than_q(dxp, dyp, E, d2v, __dsub_rn(px, S.vx[i]), __dsub_rn(py, S.vy[i]));
                    } else {
                        float dxp = rect_dx32(S.vx32[i], mbr.x, mbr.z);
                        float dyp = rect_dx32(S.vy32[i], mbr.y, mbr.w);
                        double vx = S.vx[i], vy = S.vy[i];
                        double dx64 = 0, dy64 = 0;
                        if (vx < (double)mbr.x) dx64 = __dsub_rn((double)mbr.x, vx);
                        else if (vx > (double)mbr.z) dx64 = __dsub_rn(vx, (double)mbr.z);
                        if (vy < (double)mbr.y) dy64 = __dsub_rn((double)mbr.y, vy);
                        else if (vy > (double)mbr.w) dy64 = __dsub_rn(vy, (double)mbr.w);
                        hit = closer_than_q(dxp, dyp, E, d2v, dx64, dy64);
                    }
                }
                prune = !__any_sync(FULL, hit);
            }
            if (prune) continue;

            if (!is_point) {
                // push the cell's facilities (inf.cpp:556-565)
                const int p0 = A.fstart[id], p1 = A.fstart[id + 1];
                for (int t0 = p0; t0 < p1; t0 += 32) {
                    int t = t0 + lane;
                    bool ok = t < p1;
                    if (ok) {
                        float2 pf = A.fxy[t];
                        S.tk[lane] = (uint64_t)__double_as_longlong(d2_64(qx, qy, (double)pf.x, (double)pf.y));
                        S.tc[lane] = KIND_POINT | (uint32_t)t;
                    }
                    __syncwarp();
                    if (lane == 0) {
                        int n = sc->nP;
                        int cnt = min(32, p1 - t0);
                        for (int i = 0; i < cnt; ++i)
                            if (!pq_push(S.pqk, S.pqc, n, PC, S.tk[i], S.tc[i])) { sc->flags |= QF_ZONE_PQ_OVERFLOW; break; }
                        sc->nP = n;
                    }
                    __syncwarp();
                }
                if (sc->flags) break;
                continue;
            }

            // ================= accept facility `id`: add its bisector ======
            const int nL = sc->nL;
            if (nL >= LC) { if (lane == 0) sc->flags |= QF_ZONE_L_OVERFLOW; __syncwarp(); break; }
            Line64 nb;
            if (lane == 0) nb = make_bisector(qx, qy, px, py);
            nb.a = __shfl_sync(FULL, nb.a, 0);
            nb.b = __shfl_sync(FULL, nb.b, 0);
            nb.vert = __shfl_sync(FULL, nb.vert, 0);
            nb.valid = __shfl_sync(FULL, nb.valid, 0);
            const float na32 = (float)nb.a, nb32 = (float)nb.b;
            const float nab = fabsf(na32);
            zs.nb++;

            // (1) count pass over the existing vertices (inf.cpp:359-364)
            const int nV0 = sc->nV;
            for (int i = lane; i < nV0; i += 32) {
                float x32 = S.vx32[i], y32 = S.vy32[i];
                float r32, err;
                if (nb.vert) {
                    r32 = x32 - nb32;
                    err = 3.0f * kU32 * (fabsf(x32) + fabsf(nb32)) + 1e-37f;
                } else {
                    float t = nab * fabsf(x32);
                    r32 = y32 - fmaf(na32, x32, nb32);
                    err = 5.0f * kU32 * (fabsf(y32) + t + fabsf(nb32)) + 1e-37f;
                }
                bool valid;
                if (r32 > err) valid = nb.valid == 1;
                else if (r32 < -err) valid = nb.valid == 0;
                else valid = valid64(nb.a, nb.b, nb.vert, nb.valid, S.vx[i], S.vy[i]);
                // near the new line: may coincide (within 1e-9) with one of its intersections
                float tol = (1.0f + nab) * 1.2e-9f + err;
                uint8_t fl = S.vfl[i] & ~VB_ON;
                if (fabsf(r32) <= tol || !(fabsf(r32) < FLT_MAX)) fl |= VB_ON;
                S.vfl[i] = fl;
                if (!valid) S.vcnt[i] += 1;
            }
            __syncwarp();

            // (2) candidate intersections: boundary edges (bottom, top, left,
            //     right; inf.h:340-374) then every earlier bisector in order
            const int C = 4 + nL;
            for (int c = lane; c < C; c += 32) {
                double x = 0, y = 0;
                bool ok = false;
                uint8_t cf = 0;
                if (c < 4) {
                    double ea = 0, eb = (c == 0) ? sy0 : (c == 1) ? sy1 : (c == 2) ? sx0 : sx1;
                    int ev = c >= 2;
                    if (intersect64(nb.a, nb.b, nb.vert, ea, eb, ev, x, y)) {
                        ok = (c < 2) ? (x >= sx0 && x <= sx1) : (y >= sy0 && y <= sy1);
                    }
                    cf = VB_BND;
                    zs.cand += ok;
                } else {
                    const int j = c - 4;
                    const double ea = S.la[j], eb = S.lb[j];
                    const int ev = S.lfl[j] & LB_VERT;
                    bool need64 = true;
                    if (!nb.vert && !ev) {
                        // float interval of the intersection (directed rounding)
                        float a1l = __double2float_rd(nb.a), a1h = __double2float_ru(nb.a);
                        float b1l = __double2float_rd(nb.b), b1h = __double2float_ru(nb.b);
                        float a2l = __double2float_rd(ea), a2h = __double2float_ru(ea);
                        float b2l = __double2float_rd(eb), b2h = __double2float_ru(eb);
                        float dl = __fsub_rd(a1l, a2h), dh = __fsub_ru(a1h, a2l);
                        float nl = __fsub_rd(b2l, b1h), nh = __fsub_ru(b2h, b1l);
                        if ((dl > 4e-9f || dh < -4e-9f) && fabsf(nl) < FLT_MAX && fabsf(nh) < FLT_MAX &&
                            fabsf(dl) < FLT_MAX && fabsf(dh) < FLT_MAX) {
                            float q1 = __fdiv_rd(nl, dl), q2 = __fdiv_rd(nl, dh), q3 = __fdiv_rd(nh, dl), q4 = __fdiv_rd(nh, dh);
                            float r1 = __fdiv_ru(nl, dl), r2 = __fdiv_ru(nl, dh), r3 = __fdiv_ru(nh, dl), r4 = __fdiv_ru(nh, dh);
                            float xl = fminf(fminf(q1, q2), fminf(q3, q4));
                            float xh = fmaxf(fmaxf(r1, r2), fmaxf(r3, r4));
                            // y = a1 x + b1 over the box
                            float m1 = __fmul_rd(a1l, xl), m2 = __fmul_rd(a1l, xh), m3 = __fmul_rd(a1h, xl), m4 = __fmul_rd(a1h, xh);
                            float n1 = __fmul_ru(a1l, xl), n2 = __fmul_ru(a1l, xh), n3 = __fmul_ru(a1h, xl), n4 = __fmul_ru(a1h, xh);
                            float yl = __fadd_rd(fminf(fminf(m1, m2), fminf(m3, m4)), b1l);
                            float yh = __fadd_ru(fmaxf(fmaxf(n1, n2), fmaxf(n3, n4)), b1h);
                            // pad for the FP64 rounding of the reference's evaluation
                            float px_ = 1e-12f * fmaxf(fabsf(xl), fabsf(xh)) + 1e-37f;
                            float py_ = 1e-12f * (fmaxf(fabsf(yl), fabsf(yh)) + fabsf(a1h) * fmaxf(fabsf(xl), fabsf(xh)) + fabsf(b1h)) + 1e-37f;
                            xl = __fsub_rd(xl, px_); xh = __fadd_ru(xh, px_);
                            yl = __fsub_rd(yl, py_); yh = __fadd_ru(yh, py_);
                            if (xl <= xh && yl <= yh && fabsf(xl) < FLT_MAX && fabsf(xh) < FLT_MAX &&
                                fabsf(yl) < FLT_MAX && fabsf(yh) < FLT_MAX) {
                                if (xh < fsx0 || xl > fsx1 || yh < fsy0 || yl > fsy1) need64 = false;  // outside
                                else {
                                    // certified violations of earlier bisectors
                                    float xc = 0.5f * xl + 0.5f * xh, yc = 0.5f * yl + 0.5f * yh;
                                    float rx = (0.5f * xh - 0.5f * xl) * (1.0f + 4.0f * kU32) + fabsf(xc) * 2.0f * kU32 + 1e-37f;
                                    float ry = (0.5f * yh - 0.5f * yl) * (1.0f + 4.0f * kU32) + fabsf(yc) * 2.0f * kU32 + 1e-37f;
                                    float K1 = rx * (1.0f + kU32) + 3.01f * kU32 * fabsf(xc);
                                    float K0 = ry + 3.01f * kU32 * fabsf(yc) + 1e-37f;
                                    int cert = 0;
                                    for (int m = 0; m < nL && cert < k; ++m) {
                                        uint8_t lf = S.lfl[m];
                                        float a = S.la32[m], b = S.lb32[m];
                                        float sgn, err;
                                        if (lf & LB_VERT) {
                                            sgn = xc - b;
                                            err = K1 + 3.01f * kU32 * fabsf(b);
                                        } else {
                                            sgn = yc - fmaf(a, xc, b);
                                            err = fmaf(fabsf(a), K1, K0 + S.lb3[m]);
                                        }
                                        bool inval = (lf & LB_VALID) ? (sgn < -err) : (sgn > err);
                                        cert += inval;
                                    }
                                    if (cert >= k) need64 = false;
                                }
                            }
                        }
                    }
                    if (need64) {
                        zs.cand64++;
                        if (intersect64(nb.a, nb.b, nb.vert, ea, eb, ev, x, y))
                            ok = x >= sx0 && x <= sx1 && y >= sy0 && y <= sy1;
                    }
                    zs.cand++;
                }
                S.cx[c] = x;
                S.cy[c] = y;
                S.cx32[c] = (float)x;
                S.cy32[c] = (float)y;
                S.cfl[c] = ok ? (uint8_t)(cf | 0x80) : (uint8_t)0;
            }
            __syncwarp();

            // (3) deduplicate (|dx| < 1e-9 and |dy| < 1e-9) against existing
            //     vertices near the new line and against earlier candidates
            {
                // online vertices
                int nOn = 0;
                for (int i0 = 0; i0 < nV0; i0 += 32) {
                    int i = i0 + lane;
                    bool on = i < nV0 && (S.vfl[i] & VB_ON);
                    unsigned m = __ballot_sync(FULL, on);
                    if (on) S.cons[nOn + __popc(m & ((1u << lane) - 1))] = i;   // cons reused as scratch
                    nOn += __popc(m);
                }
                __syncwarp();
                if (lane == 0) sc->nCons = -1;   // considered list must be rebuilt
                bool anyclose = false;
                for (int c = lane; c < C; c += 32) {
                    if (!(S.cfl[c] & 0x80)) continue;
                    double x = S.cx[c], y = S.cy[c];
                    bool dup = false;
                    for (int t = 0; t < nOn && !dup; ++t) {
                        int i = S.cons[t];
                        if (fabs(__dsub_rn(S.vx[i], x)) < EPS && fabs(__dsub_rn(S.vy[i], y)) < EPS) dup = true;
                    }
                    if (dup) S.cfl[c] &= 0x7f;
                    else {
                        // any earlier valid candidate within float reach?
                        // doubles within 1e-9 give floats within 1e-9 + u(|x1|+|x2|)
                        float x32 = S.cx32[c], y32 = S.cy32[c];
                        float tx = 3.0f * kU32 * fabsf(x32) + 2e-9f, ty = 3.0f * kU32 * fabsf(y32) + 2e-9f;
                        for (int c2 = 0; c2 < c; ++c2) {
                            if (!(S.cfl[c2] & 0x80)) continue;
                            if (fabsf(S.cx32[c2] - x32) <= tx && fabsf(S.cy32[c2] - y32) <= ty) { anyclose = true; break; }
                        }
                    }
                }
                __syncwarp();
                if (__any_sync(FULL, anyclose) && lane == 0) {
                    // exact sequential resolution, in candidate order
                    for (int c = 0; c < C; ++c) {
                        if (!(S.cfl[c] & 0x80)) continue;
                        for (int c2 = 0; c2 < c; ++c2) {
                            if (!(S.cfl[c2] & 0x80)) continue;
                            if (fabs(__dsub_rn(S.cx[c2], S.cx[c])) < EPS &&
                                fabs(__dsub_rn(S.cy[c2], S.cy[c])) < EPS) { S.cfl[c] &= 0x7f; break; }
                        }
                    }
                }
                __syncwarp();
            }

            // (4) counts of the surviving candidates over earlier bisectors
            for (int c = lane; c < C; c += 32) {
                int cnt = k;
                if (S.cfl[c] & 0x80) {
                    double x = S.cx[c], y = S.cy[c];
                    float xc = S.cx32[c], yc = S.cy32[c];
                    float K1 = kU32 * fabsf(xc) * (1.0f + kU32) + 3.01f * kU32 * fabsf(xc);
                    float K0 = kU32 * fabsf(yc) + 3.01f * kU32 * fabsf(yc) + 1e-37f;
                    cnt = 0;
                    for (int m = 0; m < nL; ++m) {
                        uint8_t lf = S.lfl[m];
                        float a = S.la32[m], b = S.lb32[m];
                        float sgn, err;
                        if (lf & LB_VERT) {
                            sgn = xc - b;
                            err = K1 + 3.01f * kU32 * fabsf(b);
                        } else {
                            sgn = yc - fmaf(a, xc, b);
                            err = fmaf(fabsf(a), K1, K0 + S.lb3[m]);
                        }
                        bool inval;
                        if (sgn > err) inval = !(lf & LB_VALID);
                        else if (sgn < -err) inval = (lf & LB_VALID) != 0;
                        else inval = !valid64(S.la[m], S.lb[m], lf & LB_VERT, (lf & LB_VALID) ? 1 : 0, x, y);
                        cnt += inval;
                    }
                }
                S.ccnt[c] = cnt;
            }
            __syncwarp();

            // (5) erase old vertices with count >= k (order kept), then append
            //     the new vertices with count < k in candidate order
            int w = 0;
            for (int i0 = 0; i0 < nV0; i0 += 32) {
                int i = i0 + lane;
                bool keep = i < nV0 && S.vcnt[i] < k;
                double x = 0, y = 0, d2 = 0;
                float x32 = 0, y32 = 0;
                int cnt = 0;
                uint8_t fl = 0;
                if (keep) {
                    x = S.vx[i]; y = S.vy[i]; d2 = S.vd2[i];
                    x32 = S.vx32[i]; y32 = S.vy32[i]; cnt = S.vcnt[i]; fl = S.vfl[i] & ~VB_ON;
                }
                unsigned m = __ballot_sync(FULL, keep);
                __syncwarp();
                if (keep) {
                    int o = w + __popc(m & ((1u << lane) - 1));
                    S.vx[o] = x; S.vy[o] = y; S.vd2[o] = d2;
                    S.vx32[o] = x32; S.vy32[o] = y32; S.vcnt[o] = cnt; S.vfl[o] = fl;
                }
                w += __popc(m);
                __syncwarp();
            }
            int nnew = 0;
            for (int c0 = 0; c0 < C; c0 += 32) {
                int c = c0 + lane;
                bool keep = c < C && (S.cfl[c] & 0x80) && S.ccnt[c] < k;
                unsigned m = __ballot_sync(FULL, keep);
                int o = w + nnew + __popc(m & ((1u << lane) - 1));
                if (keep && o < VC) {
                    double x = S.cx[c], y = S.cy[c];
                    S.vx[o] = x; S.vy[o] = y;
                    S.vx32[o] = S.cx32[c]; S.vy32[o] = S.cy32[c];
                    S.vd2[o] = d2_64(x, y, qx, qy);
                    S.vcnt[o] = S.ccnt[c];
                    S.vfl[o] = S.cfl[c] & VB_BND;
                }
                nnew += __popc(m);
            }
            zs.kept += nnew;
            int nV = w + nnew;
            bool vover = nV > VC;
            if (vover) nV = VC;

            // (6) nearest bisector distance, store the line (inf.cpp:430-434)
            if (lane == 0) {
                double dl = line_dist64(qx, qy, nb.a, nb.b, nb.vert);
                if (dl < sc->nearb) sc->nearb = dl;
                S.la[nL] = nb.a;
                S.lb[nL] = nb.b;
                S.lfl[nL] = (uint8_t)((nb.vert ? LB_VERT : 0) | (nb.valid ? LB_VALID : 0));
                S.la32[nL] = na32;
                S.lb32[nL] = nb32;
                S.lb3[nL] = 3.01f * kU32 * fabsf(nb32) + 1e-37f;
                S.lpos[nL] = id;
                sc->nL = nL + 1;
                sc->nV = nV;
                if (vover) sc->flags |= QF_ZONE_V_OVERFLOW;
            }
            if (nV > zs.vmax) zs.vmax = nV;
            __syncwarp();
            // (7) furthest remaining vertex (inf.cpp:445-451)
            {
                double m = 0.0;
                for (int i = lane; i < nV; i += 32) m = fmax(m, S.vd2[i]);
                m = warp_max(m);
                if (lane == 0) sc->far_ = __dsqrt_rn(m);
            }
            __syncwarp();
            if (sc->flags) break;
        }
        qflags |= sc->flags;
        const int nL = sc->nL;
        zs.nb = nL;
        zs.cand = warp_sum(zs.cand);
        zs.cand64 = warp_sum(zs.cand64);

        // ---- epilogue 1: exact half-planes relative to q -------------------
        // m(u) = a (ux - qx) + b (uy - qy) + c = d2(u,f) - d2(u,q);  f strictly
        // nearer than q  <=>  m < 0.
        float4* planes = A.planes + (size_t)s * LC;
        double cmax = 0.0;
        float4* splanes = (float4*)S.cx;      // staging copy for the cell scan
        for (int m = lane; m < nL; m += 32) {
            int pos = S.lpos[m];
            float2 f = A.fxy[pos];
            double dx = (double)f.x - qx, dy = (double)f.y - qy;
            double c = dx * dx + dy * dy;
            float4 p = make_float4((float)(-2.0 * dx), (float)(-2.0 * dy), (float)c, 0.0f);
            planes[m] = p;
            splanes[m] = p;
            A.bis_pos[(size_t)s * LC + m] = pos;
            cmax = fmax(cmax, c);
        }
        cmax = warp_max(cmax);
        const double Fp = sqrt(cmax) * (1.0 + 1e-6) + 1e-30;
        // per-user bound 8u (2F'(|x'|+|y'|) + F'^2)
        const float k2f = (float)(8.0 * (double)kU32 * 2.0 * Fp * (1.0 + 1e-6));
        const float kf2 = (float)(8.0 * (double)kU32 * Fp * Fp * (1.0 + 1e-6)) + 1e-30f;
        const double k2f64 = 8.0 * kU64 * 2.0 * Fp * (1.0 + 1e-6);
        const double kf264 = 8.0 * kU64 * Fp * Fp * (1.0 + 1e-6) + 1e-300;
        __syncwarp();

        // ---- epilogue 2: ring scan over user cells ------------------------
        const Grid gu = A.gu;
        const int ucx = cell_coord(qf.x, gu.x0, gu.inv, gu.gx);
        const int ucy = cell_coord(qf.y, gu.y0, gu.inv, gu.gy);
        const int RM = A.rmax;
        const int W = 2 * RM + 1;
        const int nwords = (W * W + 31) / 32;
        for (int i = lane; i < nwords; i += 32) S.bitmap[i] = 0u;
        __syncwarp();
        const float delta = 8.0f * kU32 * (fabsf(gu.x0) + fabsf(gu.y0) + gu.cs * (float)max(gu.gx, gu.gy) + fabsf(qf.x) + fabsf(qf.y) + gu.cs) + 1e-30f;
        const int rmaxu = max(max(ucx, gu.gx - 1 - ucx), max(ucy, gu.gy - 1 - ucy));
        bool all_users = nL == 0 && A.nu > 0;
        int rend = -1;
        if (!all_users && A.nu > 0) {
            for (int r = 0;; ++r) {
                if (r > rmaxu) { rend = r - 1; break; }
                if (r > RM) { all_users = true; break; }
                int ncell = r == 0 ? 1 : 8 * r;
                bool anykeep = false;
                for (int t0 = 0; t0 < ncell; t0 += 32) {
                    int t = t0 + lane;
                    int dx = 0, dy = 0;
                    bool ok = t < ncell;
                    if (ok && r > 0) {
                        int side = 2 * r + 1;
                        if (t < side) { dx = -r + t; dy = -r; }
                        else if (t < 2 * side) { dx = -r + (t - side); dy = r; }
                        else if (t < 2 * side + (2 * r - 1)) { dx = -r; dy = -r + 1 + (t - 2 * side); }
                        else { dx = r; dy = -r + 1 + (t - 2 * side - (2 * r - 1)); }
                    }
                    int cxx = ucx + dx, cyy = ucy + dy;
                    ok = ok && cxx >= 0 && cxx < gu.gx && cyy >= 0 && cyy < gu.gy;
                    bool keep = false;
                    if (ok) {
                        float X0 = (gu.x0 + (float)cxx * gu.cs) - qf.x - delta;
                        float X1 = (gu.x0 + (float)(cxx + 1) * gu.cs) - qf.x + delta;
                        float Y0 = (gu.y0 + (float)cyy * gu.cs) - qf.y - delta;
                        float Y1 = (gu.y0 + (float)(cyy + 1) * gu.cs) - qf.y + delta;
                        int viol = 0;
                        for (int m = 0; m < nL && viol < k; ++m) {
                            float4 p = splanes[m];
                            float X = p.x > 0.0f ? X1 : X0;
                            float Y = p.y > 0.0f ? Y1 : Y0;
                            float mx = fmaf(p.x, X, fmaf(p.y, Y, p.z));
                            float bd = 8.0f * kU32 * fmaf(fabsf(p.x), fabsf(X), fmaf(fabsf(p.y), fabsf(Y), fabsf(p.z))) + 1e-30f;
                            viol += (mx < -bd);
                        }
                        keep = viol < k;
                    }
                    if (keep) {
                        int bit = (dy + RM) * W + (dx + RM);
                        atomicOr(&S.bitmap[bit >> 5], 1u << (bit & 31));
                    }
                    anykeep |= keep;
                }
                anykeep = __any_sync(FULL, anykeep);
                if (!anykeep && r >= 1) { rend = r - 1; break; }
                rend = r;
            }
            zs.rings = rend + 1;
        }
        __syncwarp();

        // ---- segments: one user range per row ------------------------------
        int2* seg = A.segs + (size_t)s * A.seg_cap;
        int nseg = 0, ncand = 0;
        if (all_users) {
            seg[0] = make_int2(0, 0);
            seg[1] = make_int2(0, A.nu);
            nseg = 1;
            ncand = A.nu;
            qflags |= QF_ALL_USERS;
        } else {
            int y0 = max(0, ucy - rend), y1 = min(gu.gy - 1, ucy + rend);
            int xl0 = max(0, ucx - rend), xl1 = min(gu.gx - 1, ucx + rend);
            for (int r0 = y0; r0 <= y1; r0 += 32) {
                int row = r0 + lane;
                int st = 0, len = 0;
                if (row <= y1) {
                    int dy = row - ucy;
                    int xmin = INT_MAX, xmax = -1;
                    for (int cxx = xl0; cxx <= xl1; ++cxx) {
                        int bit = (dy + RM) * W + (cxx - ucx + RM);
                        if (S.bitmap[bit >> 5] & (1u << (bit & 31))) {
                            xmin = min(xmin, cxx);
                            xmax = cxx;
                        }
                    }
                    if (xmax >= 0) {
                        st = A.ustart[row * gu.gx + xmin];
                        len = A.ustart[row * gu.gx + xmax + 1] - st;
                    }
                }
                bool has = len > 0;
                unsigned m = __ballot_sync(FULL, has);
                int pre = __popc(m & ((1u << lane) - 1));
                // prefix of lengths within the warp
                int incl = has ? len : 0;
                for (int o = 1; o < 32; o <<= 1) {
                    int v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += v;
                }
                int excl = incl - (has ? len : 0);
                if (has) seg[nseg + pre] = make_int2(st, ncand + excl);
                nseg += __popc(m);
                ncand += __shfl_sync(FULL, incl, 31);
            }
            if (lane == 0) seg[nseg] = make_int2(0, ncand);
        }

        if (lane == 0) {
            QDesc d;
            d.qx = qf.x;
            d.qy = qf.y;
            d.qpos = qpos;
            d.k = k;
            d.nb = nL;
            d.nseg = nseg;
            d.k2f = k2f;
            d.kf2 = kf2;
            d.k2f64 = k2f64;
            d.kf264 = kf264;
            d.ncand = ncand;
            d.flags = qflags;
            *qd = d;
            A.zst[s] = zs;
        }
        __syncwarp();
    }
}

}  // namespace rknn
