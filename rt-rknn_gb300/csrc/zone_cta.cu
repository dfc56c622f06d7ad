// Influence-zone kernel, one block per query.
//
// The same search as the one-warp kernel (zone.cu): rknn-inf's influence-zone
// filter (rknn-inf/inf.cpp:201-585) over the uniform facility grid, with the
// same entries taken in the same order, the same three pruning rules, the
// same bisectors, vertices and counts, and every decision on the FP64 values
// the reference computes (this file is built with -fmad=false).  What
// changes is how each step runs:
//   * the priority queue is a sorted array in shared memory: a batch of new
//     entries (one ring's cells, one cell's facilities) is merged into it by
//     every thread at once (each entry's new place is its rank among the old
//     entries plus its rank within the batch), and the queue's head is read
//     by every thread, so a pop needs no broadcast.  Entries are ordered by
//     (squared distance, code) as in the heap of zone.cu; codes are unique,
//     so the pop sequence is the heap's;
//   * the loops over vertices and candidates run over the block's threads
//     (ordered compactions keep the reference's vertex order);
//   * a candidate intersection's certified pre-discard and its count over the
//     earlier bisectors are split over a group of ZG threads, each taking
//     every ZG-th bisector, and summed within the group;
//   * an FP64 instruction holds its warp about 64 cycles on GB300 however
//     few lanes run it (a division about 670), so FP64 values the whole
//     block needs are made once, by one lane: the new bisector by the last
//     warp while the others run the vertex count and candidate passes on a
//     float estimate of it with proven error bounds, the nearest distance
//     and rule 2's bounds by one lane during the FP64 intersections; rule 1
//     and the ring gate use bounds from the farthest squared distance's bits;
//     conversions and comparisons of doubles run on their bits.
// It serves batches in which every query can have a block of its own (the
// plain single-query form first of all); larger batches run the one-warp
// kernel, which keeps more queries in flight per SM.
#include "zone_geom.cuh"

namespace rknn {

namespace {

constexpr int ZMAXT = ZCTA_THREADS;      // the largest block size (shared arrays)
constexpr int ZMAXW = ZMAXT / 32;

struct ZcShared {
    uint64_t tk[ZMAXT];   // a batch of new queue entries: keys
    uint32_t tc[ZMAXT];   //   and codes
    // Per-warp partials of the block reductions, two copies used by
    // alternate calls (the phase bit every thread flips at each call): a
    // copy is written again only after a later call's barrier, which every
    // thread passes after reading it, so one barrier per call suffices.
    int wc[2][2][ZMAXW];  // per-warp counts (ordered compactions)
    double rd[2][ZMAXW];
    long long rl[2][ZMAXW];
    float rf[2][ZMAXW];
    int ri[2][2][ZMAXW];
    long long ek[ZMAXW][8];   // extreme boundary points: per-warp best keys
    int ei[ZMAXW][8];         //   and list positions
    double bd[4];         // values one thread computed for all
    uint64_t bk[2];
    struct {              // the bisector of the facility taken
        double a, b;
        int vert, valid;
        float f[2];       // a, b rounded to nearest
    } sb;
    int bi[16];
    unsigned long long fmax[2];   // (7)'s maximum, by accept parity
};

// Ordered ranks of two predicates over the block (thread order is item
// order): the number of threads before this one with each predicate set,
// and the totals.  One barrier (the per-warp counts alternate between two
// copies, see ZcShared).
template <int ZW>
__device__ __forceinline__ void block_rank2(bool p, bool q, ZcShared& sh, unsigned& ph, int& rp, int& rq, int& tp,
                                            int& tq)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = ph & 1;
    ph ^= 1;
    const unsigned mp = __ballot_sync(FULL, p), mq = __ballot_sync(FULL, q);
    if (lane == 0) {
        sh.wc[b][0][w] = __popc(mp);
        sh.wc[b][1][w] = __popc(mq);
    }
    __syncthreads();
    int bp = 0, bq = 0;
    tp = 0;
    tq = 0;
#pragma unroll
    for (int j = 0; j < ZW; ++j) {
        const int cp = sh.wc[b][0][j], cq = sh.wc[b][1][j];
        if (j < w) { bp += cp; bq += cq; }
        tp += cp;
        tq += cq;
    }
    const unsigned below = (1u << lane) - 1;
    rp = bp + __popc(mp & below);
    rq = bq + __popc(mq & below);
}

template <int ZW>
__device__ __forceinline__ int block_rank(bool p, ZcShared& sh, unsigned& ph, int& tot)
{
    int rp, rq, tq;
    block_rank2<ZW>(p, false, sh, ph, rp, rq, tot, tq);
    return rp;
}

// Exclusive ordered sums of two ints over the block, with totals.
template <int ZW>
__device__ __forceinline__ void block_scan2(int a, int b, ZcShared& sh, unsigned& ph, int& ea, int& eb, int& ta,
                                            int& tb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int bf = ph & 1;
    ph ^= 1;
    int xa = a, xb = b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ya = __shfl_up_sync(FULL, xa, o), yb = __shfl_up_sync(FULL, xb, o);
        if (lane >= o) { xa += ya; xb += yb; }
    }
    if (lane == 31) {
        sh.ri[bf][0][w] = xa;
        sh.ri[bf][1][w] = xb;
    }
    __syncthreads();
    int ba = 0, bb = 0;
    ta = 0;
    tb = 0;
#pragma unroll
    for (int j = 0; j < ZW; ++j) {
        const int ca = sh.ri[bf][0][j], cb = sh.ri[bf][1][j];
        if (j < w) { ba += ca; bb += cb; }
        ta += ca;
        tb += cb;
    }
    ea = ba + xa - a;
    eb = bb + xb - b;
}

template <int ZW>
__device__ __forceinline__ double block_max_d(double v, ZcShared& sh, unsigned& ph)
{
    const int b = ph & 1;
    ph ^= 1;
    v = warp_max(v);
    if ((threadIdx.x & 31) == 0) sh.rd[b][threadIdx.x >> 5] = v;
    __syncthreads();
    double r = sh.rd[b][0];
#pragma unroll
    for (int j = 1; j < ZW; ++j) r = fmax(r, sh.rd[b][j]);
    return r;
}

template <int ZW>
__device__ __forceinline__ int block_sum_i(int v, ZcShared& sh, unsigned& ph)
{
    const int b = ph & 1;
    ph ^= 1;
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh.ri[b][0][threadIdx.x >> 5] = v;
    __syncthreads();
    int r = 0;
#pragma unroll
    for (int j = 0; j < ZW; ++j) r += sh.ri[b][0][j];
    return r;
}

// Sum over the ZG threads of a candidate group (aligned within the warp).
template <int ZG>
__device__ __forceinline__ int group_sum(int v)
{
#pragma unroll
    for (int o = ZG / 2; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o, ZG);
    return v;
}

// Merges the batch sh.tk/tc[0 .. m) into the sorted queue [h, h + n) of
// (K, C); the merged queue starts at 0 afterwards (h = 0).  Entries beyond
// cap are not taken (the batch's later ones first; *over is set).  Every
// thread calls it; it begins and ends at a barrier.
template <int ZT>
__device__ __forceinline__ void pq_merge(uint64_t* K, uint32_t* C, int& h, int& n, int m, int cap, bool& over,
                                         const ZcShared& sh)
{
    constexpr int PQ_PT = ZCTA_PQ_MAX / ZT;   // queue entries a thread holds while merging
    const int tid = threadIdx.x;
    if (n + m > cap) {
        over = true;
        m = cap - n;
    }
    if (m <= 0) return;
    __syncthreads();                       // the batch is complete
    // old entries: read, and moved past the new entries smaller than them
    uint64_t ok[PQ_PT];
    uint32_t oc[PQ_PT];
    int opos[PQ_PT];
#pragma unroll
    for (int t = 0; t < PQ_PT; ++t) {
        const int j = tid + t * ZT;
        opos[t] = -1;
        if (j < n) {
            ok[t] = K[h + j];
            oc[t] = C[h + j];
            int r = 0;
            for (int e = 0; e < m; ++e) r += pq_less(sh.tk[e], sh.tc[e], ok[t], oc[t]);
            opos[t] = j + r;
        }
    }
    // new entries: rank among the old ones (bisection) plus among the batch
    uint64_t nk = 0;
    uint32_t nc = 0;
    int npos = -1;
    if (tid < m) {
        nk = sh.tk[tid];
        nc = sh.tc[tid];
        int lo = 0, len = n;                  // first old entry not less than the new one
        while (len > 0) {
            const int half = len >> 1;
            if (pq_less(K[h + lo + half], C[h + lo + half], nk, nc)) { lo += half + 1; len -= half + 1; }
            else len = half;
        }
        int r = 0;
        for (int e = 0; e < m; ++e) r += pq_less(sh.tk[e], sh.tc[e], nk, nc);
        npos = lo + r;
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < PQ_PT; ++t)
        if (opos[t] >= 0) { K[opos[t]] = ok[t]; C[opos[t]] = oc[t]; }
    if (npos >= 0) { K[npos] = nk; C[npos] = nc; }
    h = 0;
    n += m;
    __syncthreads();
}

}  // namespace

// Extreme boundary points (inf.cpp:283-321): over the boundary list in
// vertex order, extreme j (left min/max y, right min/max y, bottom min/max x,
// top min/max x) is the first strict minimum / maximum among the entries on
// its edge -- the smallest key (largest for a maximum), the earliest entry
// among equal keys.  Each thread keeps its best of the entries it reads, then
// a block reduction by (key, position).  ext[j] = vertex index or -1.
// Run by all warps but the last (which makes the facility's bisector
// meanwhile), synchronised by named barrier 1 over those warps only.
template <int ZT>
__device__ __forceinline__ void extreme_points(const Slice& S, int nV, uint32_t ku, ZcShared& sh, int (&ext)[8])
{
    constexpr int ZW = ZT / 32 - 1;       // the warps taking part
    constexpr int NT = ZW * 32;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    long long bk[8];
    int bp[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) { bk[j] = 0; bp[j] = INT_MAX; }
    // the list of boundary vertices below count k, in vertex order: the
    // vertex index serves as the list position
    for (int t = tid; t < nV; t += NT) {
        const float vw = IX(S.v4, t).w;
        const uint32_t fl = vfl_of(vw);
        if (!(fl & VB_BND) || vcnt_of(vw) >= ku) continue;
        const double2 p = IX(S.vd, t);
        const long long kx = order_key(p.x), ky = order_key(p.y);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t ebit = j < 2 ? VB_EL : j < 4 ? VB_ER : j < 6 ? VB_EB : VB_ET;
            if (!(fl & ebit)) continue;
            const long long kk = j < 4 ? ky : kx;
            // entries come in increasing t: a later one wins only if strictly better
            if (bp[j] == INT_MAX || ((j & 1) == 0 ? kk < bk[j] : kk > bk[j])) { bk[j] = kk; bp[j] = t; }
        }
    }
    // Reduce by (key, position) with 32-bit warp minima: a key becomes an
    // unsigned word pair ordered like it (the sign bit flipped; all bits
    // flipped for a maximum, so that the best is always the least), and the
    // least pair, then the least position among its holders, wins.
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const bool has = bp[j] != INT_MAX;
        unsigned long long u = (unsigned long long)bk[j] ^ 0x8000000000000000ull;
        if (j & 1) u = ~u;
        const unsigned hi = has ? (unsigned)(u >> 32) : 0xffffffffu;
        const unsigned lo = has ? (unsigned)u : 0xffffffffu;
        const unsigned mhi = __reduce_min_sync(FULL, hi);
        const bool c1 = hi == mhi;
        const unsigned mlo = __reduce_min_sync(FULL, c1 ? lo : 0xffffffffu);
        const bool c2 = c1 && lo == mlo;
        const unsigned mpos = __reduce_min_sync(FULL, c2 ? (unsigned)bp[j] : 0xffffffffu);
        if (lane == 0) {
            sh.ek[w][j] = (long long)(((unsigned long long)mhi << 32) | mlo);
            sh.ei[w][j] = mpos == 0xffffffffu ? INT_MAX : (int)mpos;
        }
    }
    asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
    if (tid < 8) {
        const int j = tid;
        unsigned long long k0 = (unsigned long long)sh.ek[0][j];
        int p0 = sh.ei[0][j];
#pragma unroll
        for (int u = 1; u < ZW; ++u) {
            const unsigned long long ok = (unsigned long long)sh.ek[u][j];
            const int op = sh.ei[u][j];
            if (op != INT_MAX && (p0 == INT_MAX || ok < k0 || (ok == k0 && op < p0))) {
                k0 = ok;
                p0 = op;
            }
        }
        sh.bi[4 + j] = p0 == INT_MAX ? -1 : p0;
    }
    asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
#pragma unroll
    for (int j = 0; j < 8; ++j) ext[j] = sh.bi[4 + j];
}

// A float estimate of the bisector make_bisector gives, in its branches,
// with bounds on its error against the FP64 coefficients: |a - a32| <= da,
// |b - b32| <= db (vertical: x = b).  The FP64 line divides twice, each
// with one rounding of 2^-53, on differences and midpoints rounded once; the
// estimate divides once, -dx/dy, with about three float roundings of 2^-24
// (relative error below 2^-22.4), and b = my - a mx adds the error of a
// times |mx| and the roundings of my and of the product: da = 2^-20 |a32| and
// db = 2^-19 (|my| + |a mx|) hold with room.  valid is the side of q
// (q >= a qx + b, or qx >= b when vertical), decided only when the estimate
// leaves no doubt; ok = false when it does not (or the slope overflows),
// and every float test against the estimate then stands aside.
struct Line32 {
    float a, b, da, db;
    int vert, valid;
    bool ok;
};
__device__ __forceinline__ Line32 approx_bisector(float qx, float qy, float px, float py)
{
    Line32 l;
    l.a = 0.0f; l.b = 0.0f; l.da = 0.0f; l.db = 0.0f; l.vert = 0; l.valid = 0; l.ok = true;
    if (qx == px) {                       // y = (qy + py) / 2
        l.b = 0.5f * (qy + py);
        l.db = 0x1p-22f * fabsf(l.b) + 1e-37f;
    } else if (qy == py) {                // x = (qx + px) / 2
        l.vert = 1;
        l.b = 0.5f * (qx + px);
        l.db = 0x1p-22f * fabsf(l.b) + 1e-37f;
    } else {
        const float dx = px - qx, dy = py - qy;
        l.a = __fdiv_rn(-dx, dy);
        const float mx = 0.5f * (qx + px), my = 0.5f * (qy + py);
        const float am = l.a * mx;
        l.b = my - am;
        l.da = 0x1p-20f * fabsf(l.a) + 1e-37f;
        l.db = 0x1p-19f * (fabsf(my) + fabsf(am)) + 1e-37f;
        if (!(fabsf(l.a) < 0x1p100f) || !(fabsf(am) < 0x1p100f)) l.ok = false;
    }
    float r, e;
    if (l.vert) {
        r = qx - l.b;
        e = l.db + 0x1p-22f * (fabsf(qx) + fabsf(l.b)) + 1e-37f;
    } else {
        const float t = fmaf(l.a, qx, l.b);
        r = qy - t;
        e = l.da * fabsf(qx) + l.db + 0x1p-22f * (fabsf(qy) + fabsf(l.a * qx) + fabsf(l.b)) + 1e-37f;
    }
    if (r > e) l.valid = 1;
    else if (r < -e) l.valid = 0;
    else l.ok = false;
    return l;
}

// The bisector of q and the facility at (fx, fy), with its float forms, for
// every thread of the block to read after a barrier.
__device__ __forceinline__ void make_slot(ZcShared& sh, float fx, float fy, double qx, double qy)
{
    const Line64 l = make_bisector(qx, qy, f2d_bits(fx), f2d_bits(fy));
    sh.sb.a = l.a;
    sh.sb.b = l.b;
    sh.sb.vert = l.vert;
    sh.sb.valid = l.valid;
    sh.sb.f[0] = d2f_bits<0>(l.a);
    sh.sb.f[1] = d2f_bits<0>(l.b);
}

template <int ZT>
__device__ __forceinline__ void zone_cta_body(const ZoneArgs& A)
{
    constexpr int ZW = ZT / 32;          // warps
    constexpr int ZG = ZT / 32;          // threads per candidate in the candidate passes
    constexpr int ZGN = ZT / ZG;         // candidates per pass (32)
    pdl_trigger();
    extern __shared__ __align__(16) char smem[];
    __shared__ ZcShared sh;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int gi = tid / ZG, gl = tid % ZG;
    unsigned ph = 0;                     // the block reductions' phase bit (same in every thread)
#ifdef RKNN_CHECKED
    if (tid == 0 && blockIdx.x == 0) g_fault = A.fault;
    __syncthreads();
    if (!g_fault) g_fault = A.fault;
#endif
    Slice S = carve(smem, A.caps);
    const int VC = A.caps.vc, LC = A.caps.lc, PC = min(A.caps.pc, ZCTA_PQ_MAX);
    const long long NCF = (long long)A.gf.gx * A.gf.gy, NCU = (long long)A.gu.gx * A.gu.gy;
    (void)NCF; (void)NCU;
    const double sx0 = A.sx0, sy0 = A.sy0, sx1 = A.sx1, sy1 = A.sy1;
    const float E = kU32 * (float)fmax(fmax(fabs(sx0), fabs(sx1)), fmax(fabs(sy0), fabs(sy1))) * 1.01f + 1e-37f;
    const float fsx0 = __double2float_rd(sx0), fsy0 = __double2float_rd(sy0);
    const float fsx1 = __double2float_ru(sx1), fsy1 = __double2float_ru(sy1);
    const double slack = 1e-5 * ((double)A.gf.cs + fmax(fmax(fabs(sx0), fabs(sx1)), fmax(fabs(sy0), fabs(sy1))));
    const float slack_ru = __double2float_ru(slack);
    const long long kx0 = order_key(sx0), kx1 = order_key(sx1), ky0 = order_key(sy0), ky1 = order_key(sy1);
    const float tolE = (1e-9f + 2.0f * E) * (1.0f + 0x1p-20f);

    for (;;) {
        __syncthreads();
        if (tid == 0) sh.bi[0] = atomicAdd(A.work_counter, 1);
        __syncthreads();
        const int slot = sh.bi[0];
        if (slot >= A.nq) break;
        const int s = A.order ? A.order[slot] : slot;
        const int qin = A.q_in[s];
        const int k = A.k_in[s];
        QDesc* qd = A.qd + s;
        ZStats zs = {};
        int qflags = 0;
        if (qin < 0 || qin >= A.nf || k <= 0) {
            if (tid == 0) {
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
        const int qpos = A.fpos[GX(qin, A.nf, 105)];
        const float2 qf = A.fxy[GX(qpos, A.nf, 101)];
        const double qx = qf.x, qy = qf.y;
        const uint32_t ku = (uint32_t)k;
        // block-uniform state (identical in every thread)
        int nV = 4, nL = 0, nP = 0, hP = 0, nCons = -1, flags = 0;
        double nearb = DBL_MAX;
        float nearf = INFINITY;              // nearb rounded up (thread ZT - 32 keeps it)
        int cand_local = 0, cand64_local = 0;   // per-thread statistics

        // ---- init: four space corners (inf.cpp:211-226) -------------------
        double d2c = 0.0;
        if (tid < 4) {
            const double x = (tid & 1) ? sx1 : sx0;
            const double y = (tid & 2) ? sy1 : sy0;
            d2c = d2_64(x, y, qx, qy);
            IX(S.vd, tid) = make_double2(x, y);
            IX(S.v4, tid) = make_float4((float)x, (float)y, (float)d2c,
                                        vpack(0, VB_BND | edge_bits(x, y, sx0, sy0, sx1, sy1)));
        }
        // the farthest vertex's squared distance (bits), and what rule 1
        // and the ring gate derive from it without its square root
        if (tid == 0) {
            // the first addition's list counters and (7)'s maximum (later
            // ones are cleared by the addition before them)
            sh.bi[3] = 0;
            sh.bi[12] = 0;
            sh.fmax[0] = 0;
        }
        long long far2 = __double_as_longlong(block_max_d<ZW>(d2c, sh, ph));
        Cut K1 = far_cut(far2);
        float ring_T = ring_limit32(far2, slack_ru);
        Cut K2 = sqrt_cut(2.0 * DBL_MAX, true);

        long long tph = clock64();
#define PHASE(i) do { long long t_ = clock64(); zs.cyc[i] += t_ - tph; tph = t_; } while (0)
        const int qcx = cell_coord(qf.x, A.gf.x0, A.gf.inv, A.gf.gx);
        const int qcy = cell_coord(qf.y, A.gf.y0, A.gf.inv, A.gf.gy);
        const int rmaxf = max(max(qcx, A.gf.gx - 1 - qcx), max(qcy, A.gf.gy - 1 - qcy));
        int ring = 0;
        bool ring_open;
        uint64_t ring_key;
        ring_gate32(ring, rmaxf, A.gf.cs, slack_ru, ring_T, ring_open, ring_key);

        // ---- best-first search --------------------------------------------
        for (;;) {
            // make the top poppable: expand rings whose cells could precede it
            for (;;) {
                if (!ring_open) break;
                if (nP > 0 && IX(S.pqk, hP) < ring_key) break;
                const int ncell = ring == 0 ? 1 : 8 * ring;
                for (int t0 = 0; t0 < ncell; t0 += ZT) {
                    const int t = t0 + tid;
                    int cxx = 0, cyy = 0;
                    bool ok = t < ncell;
                    if (ok) {
                        if (ring == 0) { cxx = qcx; cyy = qcy; }
                        else {
                            const int side = 2 * ring + 1;
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
                        ok = A.fstart[GX(cid + 1, NCF + 1, 102)] > A.fstart[GX(cid, NCF + 1, 102)];
                    }
                    const double key = ok ? rect_d2_64(qx, qy, A.fmbr[GX(cid, NCF, 103)]) : 0.0;
                    int m;
                    const int r = block_rank<ZW>(ok, sh, ph, m);
                    if (ok) { sh.tk[r] = (uint64_t)__double_as_longlong(key); sh.tc[r] = (uint32_t)cid; }
                    bool over = false;
                    pq_merge<ZT>(S.pqk.p, S.pqc.p, hP, nP, m, PC, over, sh);
                    if (over) { flags |= QF_ZONE_PQ_OVERFLOW; break; }
                }
                ring++;
                ring_gate32(ring, rmaxf, A.gf.cs, slack_ru, ring_T, ring_open, ring_key);
                if (flags) break;
            }
            PHASE(0);
            if (flags || nP == 0) break;
            // pop: every thread reads the head (nothing writes the queue
            // until the next merge, which starts at a barrier)
            const uint64_t keybits = IX(S.pqk, hP);
            const uint32_t code = IX(S.pqc, hP);
            hP++;
            nP--;
            const double key = __longlong_as_double((long long)keybits);

            const bool is_point = (code & KIND_POINT) != 0;
            const int id = (int)(code & ~KIND_POINT);
            float2 pf = make_float2(0, 0);
            float4 mbr = make_float4(0, 0, 0, 0);
            if (is_point) {
                if (id == qpos) continue;
                pf = A.fxy[GX(id, A.nf, 101)];
                if (A.skip_coincident && pf.x == qf.x && pf.y == qf.y) continue;
                zs.pts++;
            } else {
                mbr = A.fmbr[GX(id, NCF, 103)];
                zs.cells++;
            }
            bool prune;
            PHASE(1);
            // rule 1: prunes this entry and every later one (the zone is final)
            bool r1;
            if (keybits >= K1.hi) r1 = true;
            else if (keybits <= K1.lo) r1 = false;
            else r1 = sqrt_rn64(key) > 2.0 * sqrt_rn64(__longlong_as_double(far2));
            if (r1) break;
            // rule 2: keep when nearer than twice the nearest bisector
            bool r2;
            if (keybits >= K2.hi) r2 = false;
            else if (keybits <= K2.lo) r2 = true;
            else r2 = sqrt_rn64(key) < 2.0 * nearb;
            if (r2) prune = false;
            else {
                // ---- vertex test (inf.cpp:268-353, 466-551) -------------
                if (nCons < 0) {
                    // Mark the vertices the test considers (VB_CONS): count
                    // k-1, and the space-boundary vertices below count k that
                    // lie within EPS of an extreme point (inf.cpp:283-346); or,
                    // with the zone-boundary test, every space-boundary vertex
                    // below count k.  The marks hold until the zone changes.
                    // The vertex update marks them itself except when
                    // rknn-inf's extreme points are needed (some
                    // space-boundary vertex below count k) and at the start.
                    int ext[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) ext[j] = -1;
                    if (!A.vertex_test && tid < ZT - 32) extreme_points<ZT>(S, nV, ku, sh, ext);
                    float ex[8], ey[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        ex[j] = 0.0f; ey[j] = 0.0f;
                        if (ext[j] >= 0) {
                            const float4 e = IX(S.v4, ext[j]);
                            ex[j] = e.x; ey[j] = e.y;
                        }
                    }
                    for (int i = tid; i < nV && tid < ZT - 32; i += ZT - 32) {
                        const float4 v = IX(S.v4, i);
                        const uint32_t cnt = vcnt_of(v.w), fl = vfl_of(v.w);
                        const bool bnd = (fl & VB_BND) && cnt < ku;
                        bool c = cnt == ku - 1 || (A.vertex_test && bnd);
                        if (!c && bnd && !A.vertex_test) {
#pragma unroll
                            for (int j = 0; j < 8; ++j) {
                                if (c || ext[j] < 0 || fabsf(v.x - ex[j]) > tolE || fabsf(v.y - ey[j]) > tolE) continue;
                                const double2 a = IX(S.vd, i), b = IX(S.vd, ext[j]);
                                if (within_eps(a.x, b.x) && within_eps(a.y, b.y)) c = true;
                            }
                        }
                        const uint32_t nfl = c ? (fl | VB_CONS) : (fl & ~VB_CONS);
                        if (nfl != fl) IX(S.v4, i).w = vpack(cnt, nfl);
                    }
                    nCons = 1;          // marks valid
                    // (the test below reads only the marks this thread wrote)
                }
                bool hit = false;
                for (int i = tid; i < nV && !hit && tid < ZT - 32; i += ZT - 32) {
                    const float4 v = IX(S.v4, i);
                    if (!(vfl_of(v.w) & VB_CONS)) continue;
                    int r;
                    if (is_point) r = closer32(pf.x - v.x, pf.y - v.y, E, v.z);
                    else r = closer32(rect_dx32(v.x, mbr.x, mbr.z), rect_dx32(v.y, mbr.y, mbr.w), E, v.z);
                    if (r < 0) {
                        const double2 p = IX(S.vd, i);
                        double dx64 = 0, dy64 = 0;
                        if (is_point) {
                            dx64 = __dsub_rn(f2d(pf.x), p.x);
                            dy64 = __dsub_rn(f2d(pf.y), p.y);
                        } else {
                            const double x0 = f2d(mbr.x), y0 = f2d(mbr.y), x1 = f2d(mbr.z), y1 = f2d(mbr.w);
                            if (p.x < x0) dx64 = __dsub_rn(x0, p.x);
                            else if (p.x > x1) dx64 = __dsub_rn(p.x, x1);
                            if (p.y < y0) dy64 = __dsub_rn(y0, p.y);
                            else if (p.y > y1) dy64 = __dsub_rn(p.y, y1);
                        }
                        r = closer64(dx64, dy64, p.x, p.y, qx, qy);
                    }
                    hit = r != 0;
                }
                prune = !__syncthreads_or(hit);
                PHASE(2);
            }
            if (prune) continue;

            if (!is_point) {
                // push the cell's facilities (inf.cpp:556-565)
                const int p0 = A.fstart[GX(id, NCF + 1, 102)], p1 = A.fstart[GX(id + 1, NCF + 1, 102)];
                for (int t0 = p0; t0 < p1; t0 += ZT) {
                    const int t = t0 + tid;
                    if (t < p1) {
                        const float2 pf = A.fxy[GX(t, A.nf, 101)];
                        sh.tk[tid] = (uint64_t)__double_as_longlong(d2_64(qx, qy, f2d_bits(pf.x), f2d_bits(pf.y)));
                        sh.tc[tid] = KIND_POINT | (uint32_t)t;
                    }
                    bool over = false;
                    pq_merge<ZT>(S.pqk.p, S.pqc.p, hP, nP, min(ZT, p1 - t0), PC, over, sh);
                    if (over) { flags |= QF_ZONE_PQ_OVERFLOW; break; }
                }
                if (flags) break;
                continue;
            }

            // ================= accept facility `id`: add its bisector ======
            if (nL >= LC) { flags |= QF_ZONE_L_OVERFLOW; break; }
            // The exact FP64 bisector (two dependent divisions, about 1.5 k
            // cycles) is made by one lane of the last warp, which takes no
            // part in (1) and (2): those run on a float estimate with error
            // bounds and leave what it cannot settle to (2b), after the
            // barrier that makes the exact line visible.
            if (tid == ZT - 32) make_slot(sh, pf.x, pf.y, qx, qy);
            const Line32 la = approx_bisector(qf.x, qf.y, pf.x, pf.y);
            const bool lok = la.ok;
            const float na32 = la.a, nb32 = la.b;
            const float nab = fabsf(na32);
            const bool vw = tid < ZT - 32;       // this thread's warp works in (1) and (2)
            zs.nb++;
            // (1) count pass over the existing vertices (inf.cpp:359-364);
            //     it lists the vertices near the new line for (3) and needs
            //     no barrier before (2), which reads no vertex
            const int nV0 = nV;
            float m32 = 0.0f;
            // The other warps take vertices [0, n0) in turn; the last warp,
            // once the bisector is made (about two passes' time), takes the
            // last n7 of a large set.
            const int npass = (nV0 + ZT - 1) / ZT;
            const int n7 = min(nV0, 32 * max(0, npass - 2));
            const int n0 = nV0 - n7;
            for (int i = vw ? tid : n0 + lane; i < (vw ? n0 : nV0); i += vw ? ZT - 32 : 32) {
                const float4 v = IX(S.v4, i);
                float r32, err;
                if (la.vert) {
                    r32 = v.x - nb32;
                    err = 3.0f * kU32 * (fabsf(v.x) + fabsf(nb32)) + la.db + 1e-37f;
                } else {
                    const float t = nab * fabsf(v.x);
                    r32 = v.y - fmaf(na32, v.x, nb32);
                    err = 5.0f * kU32 * (fabsf(v.y) + t + fabsf(nb32)) + la.da * fabsf(v.x) * (1.0f + 0x1p-20f) +
                          la.db + 1e-37f;
                }
                // 1: the valid side, 0: the invalid one, -1: left to (2b)
                int dec = -1;
                if (lok) {
                    if (r32 > err) dec = la.valid == 1;
                    else if (r32 < -err) dec = la.valid == 0;
                }
                const float tol = (1.0f + nab) * 1.2e-9f + err;
                uint32_t fl = vfl_of(v.w) & ~VB_ON;
                const uint32_t nc = vcnt_of(v.w) + (dec == 0 ? 1u : 0u);
                if (dec < 0 || fabsf(r32) <= tol || !(fabsf(r32) < FLT_MAX)) {
                    fl |= VB_ON;
                    // (3)'s list, in any order; bit 15: the count is (2b)'s
                    IX(S.cons, atomicAdd(&sh.bi[3], 1)) = (uint16_t)(i | (dec < 0 ? 0x8000 : 0));
                }
                IX(S.v4, i).w = vpack(nc, fl);
                if (dec >= 0 && nc < ku) m32 = fmaxf(m32, v.z);
            }
            // the float maximum of the squared distances of the vertices that
            // stay, as per-warp partials read after the next barrier
            const int bm32 = ph & 1;
            ph ^= 1;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m32 = fmaxf(m32, __shfl_xor_sync(FULL, m32, o));
            if (lane == 0) sh.rf[bm32][tid >> 5] = m32;

            PHASE(3);
            // (2) candidate intersections, boundary edges then every earlier
            //     bisector in order: a group of ZG threads per candidate
            //     drops, in float, those certainly outside the space or
            //     certainly beyond k earlier bisectors, and lists the others
            const int C = 4 + nL;
            // intervals holding the FP64 coefficients (unbounded without an estimate)
            const float a1l = lok ? __fsub_rd(la.a, la.da) : -INFINITY, a1h = lok ? __fadd_ru(la.a, la.da) : INFINITY;
            const float b1l = lok ? __fsub_rd(la.b, la.db) : -INFINITY, b1h = lok ? __fadd_ru(la.b, la.db) : INFINITY;
            constexpr int ZGW = (ZT - 32) / ZG;  // candidates per pass (groups of the working warps)
            // (every lane of a warp runs each pass, so that the group sums
            // see the whole warp; a group past C computes nothing)
            for (int c0 = 0; c0 < C && vw; c0 += ZGW) {
                const int c = c0 + gi;
                const bool active = c < C;
                bool need64 = true;           // bisector candidates: intersect in FP64
                bool do_cert = false;         // the group counts certified violations
                float xc = 0, yc = 0, KX = 0, KY = 0;
                const int j = c - 4;
                int ev = 0;
                if (active && c >= 4) {
                    const float4 e4 = IX(S.l4, j);
                    ev = (__float_as_uint(e4.w) & LB_VERT) ? 1 : 0;
                    if (!la.vert && !ev) {
                        // float interval of the intersection (directed rounding)
                        const float a2l = lo32(e4.x), a2h = hi32(e4.x);
                        const float b2l = lo32(e4.y), b2h = hi32(e4.y);
                        const float dl = __fsub_rd(a1l, a2h), dh = __fsub_ru(a1h, a2l);
                        const float nl = __fsub_rd(b2l, b1h), nh = __fsub_ru(b2h, b1l);
                        if ((dl > 4e-9f || dh < -4e-9f) && fabsf(nl) < FLT_MAX && fabsf(nh) < FLT_MAX &&
                            fabsf(dl) < FLT_MAX && fabsf(dh) < FLT_MAX) {
                            float xl, xh;
                            if (dl > 0.0f) {
                                xl = __fdiv_rd(nl, nl >= 0.0f ? dh : dl);
                                xh = __fdiv_ru(nh, nh >= 0.0f ? dl : dh);
                            } else {
                                const float pl = -dh, ph = -dl;
                                xl = -__fdiv_ru(nh, nh >= 0.0f ? pl : ph);
                                xh = -__fdiv_rd(nl, nl >= 0.0f ? ph : pl);
                            }
                            const float m1 = __fmul_rd(a1l, xl), m2 = __fmul_rd(a1l, xh), m3 = __fmul_rd(a1h, xl), m4 = __fmul_rd(a1h, xh);
                            const float n1 = __fmul_ru(a1l, xl), n2 = __fmul_ru(a1l, xh), n3 = __fmul_ru(a1h, xl), n4 = __fmul_ru(a1h, xh);
                            float yl = __fadd_rd(fminf(fminf(m1, m2), fminf(m3, m4)), b1l);
                            float yh = __fadd_ru(fmaxf(fmaxf(n1, n2), fmaxf(n3, n4)), b1h);
                            // pad for the FP64 rounding of the reference's evaluation
                            const float px_ = 1e-12f * fmaxf(fabsf(xl), fabsf(xh)) + 1e-37f;
                            const float py_ = 1e-12f * (fmaxf(fabsf(yl), fabsf(yh)) + fabsf(a1h) * fmaxf(fabsf(xl), fabsf(xh)) + fabsf(b1h)) + 1e-37f;
                            xl = __fsub_rd(xl, px_); xh = __fadd_ru(xh, px_);
                            yl = __fsub_rd(yl, py_); yh = __fadd_ru(yh, py_);
                            if (xl <= xh && yl <= yh && fabsf(xl) < FLT_MAX && fabsf(xh) < FLT_MAX &&
                                fabsf(yl) < FLT_MAX && fabsf(yh) < FLT_MAX) {
                                if (xh < fsx0 || xl > fsx1 || yh < fsy0 || yl > fsy1) need64 = false;  // outside
                                else {
                                    xc = 0.5f * xl + 0.5f * xh;
                                    yc = 0.5f * yl + 0.5f * yh;
                                    const float rx = (0.5f * xh - 0.5f * xl) * (1.0f + 4.0f * kU32) + fabsf(xc) * 2.0f * kU32 + 1e-37f;
                                    const float ry = (0.5f * yh - 0.5f * yl) * (1.0f + 4.0f * kU32) + fabsf(yc) * 2.0f * kU32 + 1e-37f;
                                    KX = rx * (1.0f + kU32) + 3.01f * kU32 * fabsf(xc);
                                    KY = ry + 3.01f * kU32 * fabsf(yc) + 1e-37f;
                                    do_cert = true;
                                }
                            }
                        }
                    }
                }
                // certified violations of earlier bisectors, the group's
                // threads taking every ZG-th one
                int cert = 0;
                if (do_cert)
                    for (int m = gl; m < nL; m += ZG) cert += inval32(IX(S.l4, m), xc, yc, KX, KY);
                cert = group_sum<ZG>(cert);
                if (do_cert && cert >= k) need64 = false;
                // the candidates that need their FP64 intersection go to a
                // list (in any order) for (2b)
                if (active && gl == 0 && c >= 4) {
                    cand_local++;
                    if (need64) {
                        cand64_local++;
                        IX(S.ccnt, atomicAdd(&sh.bi[12], 1)) = c;   // ccnt is free until (4)
                    } else {
                        IX(S.cfl, c) = 0;
                    }
                }
            }
            __syncthreads();            // (1) and (2) are complete, the exact bisector visible
            m32 = sh.rf[bm32][0];
#pragma unroll
            for (int j = 1; j < ZW; ++j) m32 = fmaxf(m32, sh.rf[bm32][j]);
            Line64 nb;
            nb.a = sh.sb.a;
            nb.b = sh.sb.b;
            nb.vert = sh.sb.vert;
            nb.valid = sh.sb.valid;

            PHASE(4);
            // (2b) the intersections in FP64, a thread each: the listed
            //     bisectors' (packed from warp 0 on), with the exact side of
            //     the generating bisector (0x40: on the invalid side), which
            //     (4) counts, and the four boundary edges' (bottom, top,
            //     left, right; inf.h:340-374) on lanes of the next-to-last
            //     warp; then (3), deduplication (|dx| < 1e-9 and |dy| <
            //     1e-9) against the existing vertices near the new line,
            //     listed by (1).  An FP64 instruction takes its warp about 64
            //     cycles however few lanes run it, and the warps of one SM
            //     sub-partition share its FP64 pipe: compares and float
            //     conversions are done on the bits instead.
            {
                const int nX = sh.bi[12], nOn = sh.bi[3];
                // the candidate's float coordinates, its deduplication and
                // its records
                auto finish = [&](int c, double x, double y, bool ok, uint8_t cf) {
                    const float2 c32 = make_float2(d2f_bits<0>(x), d2f_bits<0>(y));
                    if (ok) {
                        for (int u = 0; u < nOn; ++u) {
                            const int i = IX(S.cons, u) & 0x7fff;
                            const float4 v = IX(S.v4, i);
                            if (fabsf(v.x - c32.x) > tolE || fabsf(v.y - c32.y) > tolE) continue;
                            const double2 p = IX(S.vd, i);
                            if (within_eps(p.x, x) && within_eps(p.y, y)) { ok = false; break; }
                        }
                    }
                    IX(S.cd, c) = make_double2(x, y);
                    IX(S.c2, c) = c32;
                    IX(S.cfl, c) = ok ? (uint8_t)(cf | 0x80) : (uint8_t)0;
                };
                // the vertices (1) left undecided: their side of the new line in
                // FP64, and, if they stay, their exact squared distance for (7)
                // (they are outside the float maximum)
                for (int u = tid; u < nOn; u += ZT) {
                    const int e = IX(S.cons, u);
                    if (!(e & 0x8000)) continue;
                    const int i = e & 0x7fff;
                    const double2 p = IX(S.vd, i);
                    const uint32_t vw4 = __float_as_uint(IX(S.v4, i).w);
                    uint32_t nc = vcnt_of(__uint_as_float(vw4));
                    if (!valid64(nb.a, nb.b, nb.vert, nb.valid, p.x, p.y)) {
                        ++nc;
                        IX(S.v4, i).w = vpack(nc, vfl_of(__uint_as_float(vw4)));
                    }
                    if (nc < ku) atomicMax(&sh.fmax[nL & 1], (unsigned long long)__double_as_longlong(d2_64(p.x, p.y, qx, qy)));
                }
                const int c4 = tid - (ZT - 64);
                if (c4 >= 0 && c4 < 4) {
                    const double eb = (c4 == 0) ? sy0 : (c4 == 1) ? sy1 : (c4 == 2) ? sx0 : sx1;
                    double x = 0, y = 0;
                    bool ok = false;
                    if (intersect64(nb.a, nb.b, nb.vert, 0.0, eb, c4 >= 2, x, y))
                        ok = (c4 < 2) ? (order_key(x) >= kx0 && order_key(x) <= kx1)
                                      : (order_key(y) >= ky0 && order_key(y) <= ky1);
                    cand_local += ok;
                    finish(c4, x, y, ok, VB_BND);
                }
                for (int t = tid; t < nX; t += ZT) {
                    const int c = IX(S.ccnt, t);
                    const int j = c - 4;
                    const double2 e = IX(S.ld, j);
                    const uint32_t lf = __float_as_uint(IX(S.l4, j).w);
                    const int ev = (lf & LB_VERT) ? 1 : 0;
                    double x = 0, y = 0;
                    bool ok = false;
                    uint8_t cf = 0;
                    if (intersect64(nb.a, nb.b, nb.vert, e.x, e.y, ev, x, y)) {
                        const long long xk = order_key(x), yk = order_key(y);
                        ok = xk >= kx0 && xk <= kx1 && yk >= ky0 && yk <= ky1;
                        if (ok && !valid64k(e.x, e.y, ev, (lf & LB_VALID) ? 1 : 0, x, y)) cf = 0x40;
                    }
                    finish(c, x, y, ok, cf);
                }
                // the nearest bisector distance (inf.cpp:430-434), rule 2's
                // bounds for it and the new line's records, by one thread of
                // the last warp (idle here): nothing reads them before (6),
                // and nothing before it reads line nL
                if (tid == ZT - 32) {
                    // the exact coefficients rounded to float
                    const float ea32 = sh.sb.f[0], eb32 = sh.sb.f[1];
                    double dl = nearb;
                    bool need = true;
                    if (nearb < DBL_MAX) {
                        float est, err;
                        if (nb.vert) {
                            est = fabsf(qf.x - eb32);
                            err = 4.0f * kU32 * (fabsf(qf.x) + fabsf(eb32)) + 1e-30f;
                        } else {
                            const float den = sqrtf(fmaf(ea32, ea32, 1.0f));
                            est = fabsf(fmaf(ea32, qf.x, eb32 - qf.y)) / den;
                            err = 8.0f * kU32 * ((fabsf(ea32 * qf.x) + fabsf(qf.y) + fabsf(eb32)) / den + est) + 1e-30f;
                        }
                        // certainly farther than nearb (<= nearf): skip; NaN keeps need
                        if (__fsub_rd(est, err) > nearf) need = false;
                    }
                    if (need) {
                        const double d = line_dist64(qx, qy, nb.a, nb.b, nb.vert);
                        if (d < nearb) dl = d;
                    }
                    sh.bd[2] = dl;
                    Cut k2 = K2;
                    if (dl != nearb) {
                        k2 = near_cut(dl);
                        nearf = d2f_bits<1>(dl);
                    }
                    sh.bk[0] = k2.lo;
                    sh.bk[1] = k2.hi;
                    const uint32_t lf = (nb.vert ? LB_VERT : 0) | (nb.valid ? LB_VALID : 0);
                    IX(S.ld, nL) = make_double2(nb.a, nb.b);
                    IX(S.l4, nL) = make_float4(ea32, eb32, 3.01f * kU32 * fabsf(eb32) + 1e-37f, __uint_as_float(lf));
                    IX(S.lpos, nL) = id;
                }
                __syncthreads();
            }

            PHASE(5);
            // (4) counts of the live candidates over earlier bisectors, a
            //     group per candidate: certain violations in float, the
            //     undecided ones in FP64.  Most slots died in (2) or (2b), so
            //     the live ones are listed first (in slot order, ZT slots at
            //     a time) and the groups take the list.
            bool anyclose = false;
            for (int s0 = 0; s0 < C; s0 += ZT) {
                const int cs = s0 + tid;
                const bool lv = cs < C && (IX(S.cfl, cs) & 0x80) != 0;
                int nlv;
                const int r = block_rank<ZW>(lv, sh, ph, nlv);   // every read of the last list precedes it
                if (lv) sh.tc[r] = (uint32_t)cs;
                __syncthreads();
                for (int u0 = 0; u0 < nlv; u0 += ZGN) {
                    const int u = u0 + gi;
                    const bool live = u < nlv;
                    const int c = live ? (int)sh.tc[u] : 0;
                    int cnt = 0, undec = 0;
                    double2 p = make_double2(0, 0);
                    float2 c32 = make_float2(0, 0);
                    float KX = 0, KY = 0;
                    const int gen = c - 4;
                    if (live) {
                        p = IX(S.cd, c);
                        c32 = IX(S.c2, c);
                        KX = kU32 * fabsf(c32.x) * (1.0f + kU32) + 3.01f * kU32 * fabsf(c32.x);
                        KY = kU32 * fabsf(c32.y) + 3.01f * kU32 * fabsf(c32.y) + 1e-37f;
                        // the generating bisector passes through the candidate: its
                        // exact side, from (2b)
                        if (gen >= 0 && gl == 0) cnt += (IX(S.cfl, c) & 0x40) ? 1 : 0;
#pragma unroll 4
                        for (int m = gl; m < nL; m += ZG) {
                            const int sm = (m == gen) ? -1 : side32(IX(S.l4, m), c32.x, c32.y, KX, KY);
                            cnt += sm > 0;
                            undec += sm == 0;
                        }
                    }
                    cnt = group_sum<ZG>(cnt);
                    undec = group_sum<ZG>(undec);
                    // the bisectors the float test left undecided, in FP64
                    // (rare: skipped by warps without any)
                    const bool need = live && cnt < k && undec > 0;
                    if (__any_sync(FULL, need)) {
                        int extra = 0;
                        if (need) {
                            for (int m = gl; m < nL; m += ZG) {
                                if (m == gen) continue;
                                const float4 q = IX(S.l4, m);
                                if (side32(q, c32.x, c32.y, KX, KY) != 0) continue;
                                const double2 g = IX(S.ld, m);
                                const uint32_t lf = __float_as_uint(q.w);
                                extra += !valid64(g.x, g.y, lf & LB_VERT, (lf & LB_VALID) ? 1 : 0, p.x, p.y);
                            }
                        }
                        cnt += group_sum<ZG>(extra);
                    }
                    // (only live slots' counts are read)
                    if (live && gl == 0) IX(S.ccnt, c) = cnt;
                    // (4b), float prefilter: is a kept candidate within 1e-9 of
                    // an earlier live one (the reference keeps the first)?
                    // Doubles within 1e-9 give floats within 1e-9 + u(|x1|+|x2|).
                    if (live && cnt < k) {
                        const float tx = 3.0f * kU32 * fabsf(c32.x) + 2e-9f, ty = 3.0f * kU32 * fabsf(c32.y) + 2e-9f;
                        for (int u2 = gl; u2 < u && !anyclose; u2 += ZG) {
                            const float2 o = IX(S.c2, (int)sh.tc[u2]);
                            if (fabsf(o.x - c32.x) <= tx && fabsf(o.y - c32.y) <= ty) anyclose = true;
                        }
                        for (int c2 = gl; c2 < s0 && !anyclose; c2 += ZG) {   // earlier chunks' slots
                            if (!(IX(S.cfl, c2) & 0x80)) continue;
                            const float2 o = IX(S.c2, c2);
                            if (fabsf(o.x - c32.x) <= tx && fabsf(o.y - c32.y) <= ty) anyclose = true;
                        }
                    }
                }
            }
            // every count is written, and any close pair known, past this barrier
            {
                if (__syncthreads_or(anyclose)) {
                    if (tid == 0) {
                        for (int c = 0; c < C; ++c) {
                            if (!(IX(S.cfl, c) & 0x80)) continue;
                            const double2 p = IX(S.cd, c);
                            for (int c2 = 0; c2 < c; ++c2) {
                                if (!(IX(S.cfl, c2) & 0x80)) continue;
                                const double2 o = IX(S.cd, c2);
                                if (within_eps(o.x, p.x) && within_eps(o.y, p.y)) { IX(S.cfl, c) &= 0x7f; break; }
                            }
                        }
                    }
                    __syncthreads();
                }
            }

            // (5) erase old vertices with count >= k (order kept), then append
            //     the new vertices with count < k in candidate order.  The
            //     same reductions give (7) the largest squared distance to q
            //     of the vertices that stay (the FP64 value of the old ones
            //     whose float value is the float maximum found by (1), and
            //     of every new one), and each vertex written gets its
            //     vertex-test mark.  When every candidate fits one chunk, the
            //     ranks of the new vertices come from the first erase
            //     chunk's reduction.
            const bool one = C <= ZT;
            const bool nkeep = one && tid < C && (IX(S.cfl, tid) & 0x80) && IX(S.ccnt, tid) < k;
            long long mx = 0;               // this thread's candidates for (7), as bits
            bool hbl = false;               // a space-boundary vertex stays (below count k)
            int w = 0, nr = 0, nnew = 0;
            for (int i0 = 0; i0 < max(nV0, 1); i0 += ZT) {
                const int i = i0 + tid;
                bool keep = false;
                float4 v = make_float4(0, 0, 0, 0);
                double2 p = make_double2(0, 0);
                if (i < nV0) {
                    v = IX(S.v4, i);
                    keep = vcnt_of(v.w) < ku;
                    if (keep) p = IX(S.vd, i);
                }
                int r, tot, rq, tq;
                block_rank2<ZW>(keep, i0 == 0 && nkeep, sh, ph, r, rq, tot, tq);   // every read above precedes its barriers
                if (i0 == 0) { nr = rq; nnew = tq; }
                if (keep) {
                    if (v.z == m32) mx = max(mx, __double_as_longlong(d2_64(p.x, p.y, qx, qy)));
                    const int o = w + r;
                    const uint32_t cnt = vcnt_of(v.w), fl = vfl_of(v.w);
                    const bool bnd = (fl & VB_BND) != 0;
                    const bool cons = cnt == ku - 1 || (A.vertex_test && bnd);
                    hbl |= bnd;
                    v.w = vpack(cnt, (fl & ~(VB_ON | VB_CONS)) | (cons ? VB_CONS : 0u));
                    IX(S.vd, o) = p;
                    IX(S.v4, o) = v;
                }
                w += tot;
            }
            if (one) {
                const int o = w + nr;
                if (nkeep) {
                    const double2 np = IX(S.cd, tid);
                    const double nd2 = d2_64(np.x, np.y, qx, qy);
                    mx = max(mx, __double_as_longlong(nd2));
                    if (o < VC) {
                        const int c = tid;
                        const float2 c32 = IX(S.c2, c);
                        const uint32_t cnt = (uint32_t)IX(S.ccnt, c);
                        const bool bnd = (IX(S.cfl, c) & VB_BND) != 0;
                        const bool cons = cnt == ku - 1 || (A.vertex_test && bnd);
                        hbl |= bnd;
                        IX(S.vd, o) = np;
                        uint32_t fl = cons ? VB_CONS : 0u;
                        if (bnd) fl |= VB_BND | edge_bits(np.x, np.y, sx0, sy0, sx1, sy1);   // read for boundary vertices only
                        IX(S.v4, o) = make_float4(c32.x, c32.y, d2f_bits<0>(nd2), vpack(cnt, fl));
                    }
                }
            } else {
                nnew = 0;
                for (int c0 = 0; c0 < C; c0 += ZT) {
                    const int c = c0 + tid;
                    const bool keep = c < C && (IX(S.cfl, c) & 0x80) && IX(S.ccnt, c) < k;
                    int tot;
                    const int r = block_rank<ZW>(keep, sh, ph, tot);
                    const int o = w + nnew + r;
                    if (keep && o < VC) {
                        const double2 p = IX(S.cd, c);
                        const float2 c32 = IX(S.c2, c);
                        const double d2 = d2_64(p.x, p.y, qx, qy);
                        const uint32_t cnt = (uint32_t)IX(S.ccnt, c);
                        const bool bnd = (IX(S.cfl, c) & VB_BND) != 0;
                        const bool cons = cnt == ku - 1 || (A.vertex_test && bnd);
                        hbl |= bnd;
                        mx = max(mx, __double_as_longlong(d2));
                        IX(S.vd, o) = p;
                        uint32_t fl = cons ? VB_CONS : 0u;
                        if (bnd) fl |= VB_BND | edge_bits(p.x, p.y, sx0, sy0, sx1, sy1);
                        IX(S.v4, o) = make_float4(c32.x, c32.y, d2f_bits<0>(d2), vpack(cnt, fl));
                    }
                    nnew += tot;
                }
            }
            // (7)'s maximum over the block, folded into the barrier below
            if (mx != 0) atomicMax(&sh.fmax[nL & 1], (unsigned long long)mx);
            if (tid == 0) {
                // the next addition's list counters and maximum (every read of
                // them in this one lies before the barrier below)
                sh.bi[3] = 0;
                sh.bi[12] = 0;
                sh.fmax[(nL + 1) & 1] = 0;
            }
            zs.kept += nnew;
            nV = w + nnew;
            const bool vover = nV > VC;
            if (vover) nV = VC;
            // the vertex set is complete past this barrier; rknn-inf's
            // extreme points must be found again when a space-boundary vertex
            // stays, else the marks written here are the test's
            if (__syncthreads_or(hbl) && !A.vertex_test) nCons = -1;
            else nCons = 1;
            const long long mxb = (long long)sh.fmax[nL & 1];   // cleared again by the next addition

            // (6) nearest bisector distance and rule 2's bounds (computed by
            //     one thread while the count pass ran; every barrier since
            //     makes them visible)
            nearb = sh.bd[2];
            K2.lo = sh.bk[0];
            K2.hi = sh.bk[1];
            nL += 1;
            if (vover) flags |= QF_ZONE_V_OVERFLOW;
            if (nV > zs.vmax) zs.vmax = nV;
            // (7) furthest remaining vertex (inf.cpp:445-451), from (5)
            if (mxb != far2) {
                far2 = mxb;
                K1 = far_cut(far2);
                ring_T = ring_limit32(far2, slack_ru);
                ring_gate32(ring, rmaxf, A.gf.cs, slack_ru, ring_T, ring_open, ring_key);
            }
            PHASE(6);
            if (flags) break;
        }
        __syncthreads();
        qflags |= flags;
        zs.nb = nL;
        zs.cand = block_sum_i<ZW>(cand_local, sh, ph);
        zs.cand64 = block_sum_i<ZW>(cand64_local, sh, ph);

        // ---- epilogue 1: exact half-planes relative to q -------------------
        float4* planes = A.planes + (size_t)s * A.pstride;
        double cmax = 0.0;
        for (int m = tid; m < nL; m += ZT) {
            const int pos = IX(S.lpos, m);
            const float2 f = A.fxy[GX(pos, A.nf, 101)];
            const double dx = (double)f.x - qx, dy = (double)f.y - qy;
            const double c = dx * dx + dy * dy;
            const float4 p = make_float4((float)(-2.0 * dx), (float)(-2.0 * dy), (float)c, 0.0f);
            planes[GX(m, A.pstride, 106)] = p;
            IX(S.splanes, m) = p;
            A.bis_pos[(size_t)s * A.pstride + GX(m, A.pstride, 107)] = pos;
            cmax = fmax(cmax, c);
        }
        cmax = block_max_d<ZW>(cmax, sh, ph);
        const double Fp = sqrt(cmax) * (1.0 + 1e-6) + 1e-30;
        const float k2f = (float)(8.0 * (double)kU32 * 2.0 * Fp * (1.0 + 1e-6));
        const float kf2 = (float)(8.0 * (double)kU32 * Fp * Fp * (1.0 + 1e-6)) + 1e-30f;
        const double k2f64 = 8.0 * kU64 * 2.0 * Fp * (1.0 + 1e-6);
        const double kf264 = 8.0 * kU64 * Fp * Fp * (1.0 + 1e-6) + 1e-300;

        // ---- epilogue 2: ring scan over user cells ------------------------
        const Grid gu = A.gu;
        const int ucx = cell_coord(qf.x, gu.x0, gu.inv, gu.gx);
        const int ucy = cell_coord(qf.y, gu.y0, gu.inv, gu.gy);
        const int RM = A.rmax;
        const int W = 2 * RM + 1;
        const int nwords = (W * W + 31) / 32;
        for (int i = tid; i < nwords; i += ZT) IX(S.bitmap, i) = 0u;
        __syncthreads();
        const float delta = 8.0f * kU32 * (fabsf(gu.x0) + fabsf(gu.y0) + gu.cs * (float)max(gu.gx, gu.gy) + fabsf(qf.x) + fabsf(qf.y) + gu.cs) + 1e-30f;
        const int rmaxu = max(max(ucx, gu.gx - 1 - ucx), max(ucy, gu.gy - 1 - ucy));
        bool all_users = nL == 0 && A.nu > 0;
        int rend = -1;
        if (!all_users && A.nu > 0) {
            for (int r = 0;; ++r) {
                if (r > rmaxu) { rend = r - 1; break; }
                if (r > RM) { all_users = true; break; }
                const int ncell = r == 0 ? 1 : 8 * r;
                bool anykeep = false;
                // a group of ZG threads per cell, the half-planes split over
                // it (a ring has few cells; one thread each would walk every
                // half-plane in turn)
                for (int t0 = 0; t0 < ncell; t0 += ZGN) {
                    const int t = t0 + gi;
                    int dx = 0, dy = 0;
                    bool ok = t < ncell;
                    if (ok && r > 0) {
                        const int side = 2 * r + 1;
                        if (t < side) { dx = -r + t; dy = -r; }
                        else if (t < 2 * side) { dx = -r + (t - side); dy = r; }
                        else if (t < 2 * side + (2 * r - 1)) { dx = -r; dy = -r + 1 + (t - 2 * side); }
                        else { dx = r; dy = -r + 1 + (t - 2 * side - (2 * r - 1)); }
                    }
                    const int cxx = ucx + dx, cyy = ucy + dy;
                    ok = ok && cxx >= 0 && cxx < gu.gx && cyy >= 0 && cyy < gu.gy;
                    int viol = 0;
                    if (ok) {
                        const float X0 = (gu.x0 + (float)cxx * gu.cs) - qf.x - delta;
                        const float X1 = (gu.x0 + (float)(cxx + 1) * gu.cs) - qf.x + delta;
                        const float Y0 = (gu.y0 + (float)cyy * gu.cs) - qf.y - delta;
                        const float Y1 = (gu.y0 + (float)(cyy + 1) * gu.cs) - qf.y + delta;
                        for (int m = gl; m < nL && viol < k; m += ZG) {
                            const float4 p = IX(S.splanes, m);
                            const float X = p.x > 0.0f ? X1 : X0;
                            const float Y = p.y > 0.0f ? Y1 : Y0;
                            const float mx = fmaf(p.x, X, fmaf(p.y, Y, p.z));
                            const float bd = 8.0f * kU32 * fmaf(fabsf(p.x), fabsf(X), fmaf(fabsf(p.y), fabsf(Y), fabsf(p.z))) + 1e-30f;
                            viol += (mx < -bd);
                        }
                    }
                    // (every lane of a warp takes part in the group sums)
                    viol = group_sum<ZG>(viol);
                    const bool keep = ok && viol < k;
                    if (keep && gl == 0) {
                        const int bit = (dy + RM) * W + (dx + RM);
                        atomicOr(&IX(S.bitmap, bit >> 5), 1u << (bit & 31));
                    }
                    anykeep |= keep;
                }
                anykeep = __syncthreads_or(anykeep);
                if (!anykeep && r >= 1) { rend = r - 1; break; }
                rend = r;
            }
            zs.rings = rend + 1;
        }
        __syncthreads();

        // ---- segments: one user range per row ------------------------------
        int2* seg = A.segs + (size_t)s * A.seg_cap;
        int nseg = 0, ncand = 0;
        if (all_users) {
            if (tid == 0) {
                seg[0] = make_int2(0, 0);
                seg[1] = make_int2(0, A.nu);
            }
            nseg = 1;
            ncand = A.nu;
            qflags |= QF_ALL_USERS;
        } else {
            const int y0 = max(0, ucy - rend), y1 = min(gu.gy - 1, ucy + rend);
            const int xl0 = max(0, ucx - rend), xl1 = min(gu.gx - 1, ucx + rend);
            for (int r0 = y0; r0 <= y1; r0 += ZT) {
                const int row = r0 + tid;
                int st = 0, len = 0;
                if (row <= y1) {
                    const int dy = row - ucy;
                    int xmin = INT_MAX, xmax = -1;
                    for (int cxx = xl0; cxx <= xl1; ++cxx) {
                        const int bit = (dy + RM) * W + (cxx - ucx + RM);
                        if (IX(S.bitmap, bit >> 5) & (1u << (bit & 31))) {
                            xmin = min(xmin, cxx);
                            xmax = cxx;
                        }
                    }
                    if (xmax >= 0) {
                        st = A.ustart[GX(row * gu.gx + xmin, NCU + 1, 104)];
                        len = A.ustart[GX(row * gu.gx + xmax + 1, NCU + 1, 104)] - st;
                    }
                }
                const bool has = len > 0;
                int pre, excl, tot_has, tot_len;
                block_scan2<ZW>(has ? 1 : 0, has ? len : 0, sh, ph, pre, excl, tot_has, tot_len);
                if (has) seg[GX(nseg + pre, A.seg_cap, 108)] = make_int2(st, ncand + excl);
                nseg += tot_has;
                ncand += tot_len;
            }
            if (tid == 0) seg[GX(nseg, A.seg_cap, 109)] = make_int2(0, ncand);
        }

        PHASE(7);
#undef PHASE
        if (tid == 0) {
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
            d.rho = 0.0f;
            d.pad = 0;
            *qd = d;
            A.zst[s] = zs;
        }
    }
}

__global__ void __launch_bounds__(ZCTA_THREADS, 1) zone_kernel_cta(ZoneArgs a) { zone_cta_body<ZCTA_THREADS>(a); }
__global__ void __launch_bounds__(ZCTA_THREADS / 2, 1) zone_kernel_cta_half(ZoneArgs a)
{
    zone_cta_body<ZCTA_THREADS / 2>(a);
}

}  // namespace rknn
