// Angular-slice filter: one warp per query, for large k.
//
// The influence zone of rknn-inf keeps every arrangement vertex below level
// k (about 3.4 k^2 of them), which outgrows shared memory beyond k ~ 35.
// This kernel restates the SLICE filter of rknn-slice (rknn-slice/slice.h:
// 306-367 pruneSpace, 465-551 isCompletelyPruned, 574-586 the user test)
// with state linear in k:
//   * the plane around q is cut into 32 equal angular slices, one per lane
//     (the reference uses 12);
//   * a facility f bounds slice P by its upper arc |f-q| / (2 cos a), a the
//     largest angle between f-q and a direction of P (infinite when a >= 90
//     degrees): every point of P farther than that from q is strictly nearer
//     to f than to q.  With unit directions e1, e2 at the slice's edges the
//     arc is |f-q|^2 / (2 min((f-q).e1, (f-q).e2));
//   * each lane keeps the k smallest arcs of its slice in a max-heap; the
//     k-th smallest, R(P), bounds the results: a user of P farther than R(P)
//     from q has k facilities strictly nearer than q;
//   * facilities stream in ring by ring from q's cell; a facility at
//     distance d has arcs >= d/2, so the stream stops once half a ring's
//     lower distance bound exceeds every slice's min(R(P), C(P)), C(P) the
//     farthest point of the data's bounding box inside P (no user lies
//     beyond it, so a smaller arc there changes nothing).
// Rounding: slices are widened by 2^-14 rad on each side, arcs are computed
// in float and rounded up by explicit error bounds, and R is inflated before
// the user test, so the kept region contains every result.  The verification
// kernel decides exactly; this filter only bounds its work.
//
// Outputs are those of the zone kernel: half-planes of the nearest
// facilities (the first caps.lc streamed) for the verification's filter, and
// the user-cell segments of the kept region (a ring scan over user cells; the
// region {u : |u-q| <= R(slice of u)} is star-shaped around q, so a full ring
// of pruned cells closes it).
#include "rknn_common.cuh"
#include "zone.cuh"
#include "verify_item.cuh"
#include <cfloat>

namespace rknn {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NS = 32;                                  // slices: one per lane
constexpr float SLICE_W = 6.28318530717958647692f / NS;
constexpr float WIDEN = 6.103515625e-05f;               // 2^-14 rad

#ifdef RKNN_CHECKED
__device__ int* s_fault;
__device__ __forceinline__ long long sck(long long i, long long n, int id, int line)
{
    if (i < 0 || i >= n) {
        if (s_fault && atomicCAS(s_fault, 0, 1) == 0) {
            s_fault[1] = id; s_fault[2] = (int)i; s_fault[3] = (int)n; s_fault[4] = line;
        }
        return 0;
    }
    return i;
}
#define SX(i, n, id) sck((i), (n), (id), __LINE__)
#else
#define SX(i, n, id) (i)
#endif

// Upper arc of slice (e1, e2) for facility offset (vx, vy), rounded up.
__device__ __forceinline__ float upper_arc(float vx, float vy, float e1x, float e1y, float e2x, float e2y)
{
    const float d1 = fmaf(vx, e1x, vy * e1y), d2 = fmaf(vx, e2x, vy * e2y);
    const float l1 = fabsf(vx) + fabsf(vy);
    const float dmin = fminf(d1, d2) - 8.0f * kU32 * l1 - 1e-37f;
    if (!(dmin > 0.0f)) return INFINITY;
    const float num = fmaf(vx, vx, vy * vy) * (1.0f + 8.0f * kU32);
    const float den = 2.0f * dmin;
    // __fdividef is within 2 ulp for denominators in [2^-126, 2^126]: a
    // 2^-20 relative inflation covers it; outside that range divide exactly
    if (den > 0x1p-126f && den < 0x1p126f) return __fdividef(num, den) * (1.0f + 0x1p-20f);
    return __fdiv_ru(num, den) * (1.0f + 4.0f * kU32);
}

// upper_arc without branches: +inf when min((f-q).e1, (f-q).e2), less its
// rounding allowance, lies outside [2^-100, 2^100] -- an infinite arc only
// loosens the slice's bound, which stays valid, and there the arc is
// astronomically large anyway (or |f-q|^2 has overflowed).  Inside, the
// quotient by __fdividef (within 2 ulp for such divisors) is inflated past
// its error, as in upper_arc.
__device__ __forceinline__ float upper_arc_fast(float vx, float vy, float e1x, float e1y, float e2x, float e2y)
{
    const float d1 = fmaf(vx, e1x, vy * e1y), d2 = fmaf(vx, e2x, vy * e2y);
    const float l1 = fabsf(vx) + fabsf(vy);
    const float dmin = fminf(d1, d2) - 8.0f * kU32 * l1 - 1e-37f;
    const float num = fmaf(vx, vx, vy * vy);
    // num (1 + 8u) / (2 dmin), the quotient rounded up by 2^-20
    constexpr float C = 0.5f * (1.0f + 8.0f * kU32) * (1.0f + 0x1p-20f) * (1.0f + 4.0f * kU32);
    return (dmin > 0x1p-100f && dmin < 0x1p100f) ? __fdividef(num, dmin) * C : INFINITY;
}

// Distance from q along unit direction (ex, ey) to the box's boundary,
// rounded up (q lies inside the box).
__device__ __forceinline__ float exit_dist(float qx, float qy, float ex, float ey,
                                           float x0, float y0, float x1, float y1)
{
    float t = INFINITY;
    if (ex > 0.0f) t = fminf(t, __fdiv_ru(__fsub_ru(x1, qx), ex));
    else if (ex < 0.0f) t = fminf(t, __fdiv_ru(__fsub_rd(x0, qx), ex));
    if (ey > 0.0f) t = fminf(t, __fdiv_ru(__fsub_ru(y1, qy), ey));
    else if (ey < 0.0f) t = fminf(t, __fdiv_ru(__fsub_rd(y0, qy), ey));
    return t;
}

// Largest of Rs over the slices that the box [X0, X1] x [Y0, Y1] (relative to
// q) meets, or +inf when the box contains q or spans half the circle or
// more.  A box that does not contain q subtends less than 180 degrees, and
// the directions it covers lie between those of its corners: taking the
// corners' slices as offsets from one corner's (mod 32, in [-16, 16)) gives
// the range.  Near a slice edge slice_of may name the neighbour; the box's
// points in that direction are then inside the named slice's widened cone,
// whose bound holds for them.
__device__ __forceinline__ float box_bound(float X0, float X1, float Y0, float Y1, const float* Rs)
{
    if (X0 <= 0.0f && X1 >= 0.0f && Y0 <= 0.0f && Y1 >= 0.0f) return INFINITY;
    const int c0 = slice_of(X0, Y0);
    const int d1 = ((slice_of(X1, Y0) - c0 + 48) & 31) - 16;
    const int d2 = ((slice_of(X0, Y1) - c0 + 48) & 31) - 16;
    const int d3 = ((slice_of(X1, Y1) - c0 + 48) & 31) - 16;
    const int lo = min(0, min(d1, min(d2, d3))), hi = max(0, max(d1, max(d2, d3)));
    if (hi - lo >= 15 || lo == -16) return INFINITY;
    float r = 0.0f;
    for (int sl = c0 + lo; sl <= c0 + hi; ++sl) r = fmaxf(r, Rs[sl & 31]);
    return r;
}

// Cell ri of the square ring at Chebyshev distance ring around (qcx, qcy):
// bottom row, top row, then the left and right columns without corners.
__device__ __forceinline__ void ring_cell(int ring, int ri, int qcx, int qcy, int& cxx, int& cyy)
{
    cxx = qcx;
    cyy = qcy;
    if (ring > 0) {
        const int side = 2 * ring + 1;
        if (ri < side) { cxx = qcx - ring + ri; cyy = qcy - ring; }
        else if (ri < 2 * side) { cxx = qcx - ring + (ri - side); cyy = qcy + ring; }
        else if (ri < 2 * side + (2 * ring - 1)) { cxx = qcx - ring; cyy = qcy - ring + 1 + (ri - 2 * side); }
        else { cxx = qcx + ring; cyy = qcy - ring + 1 + (ri - 2 * side - (2 * ring - 1)); }
    }
}

// Max-heap of one slice, interleaved across lanes: entry i of lane l at
// H[i * 32 + l] (all lanes touching the same level hit distinct banks).
__device__ __forceinline__ void heap_insert(float* H, int lane, int& n, int cap, float v)
{
    if (n < cap) {
        int i = n++;
        while (i > 0) {
            const int p = (i - 1) >> 1;
            const float pv = H[SX(p * 32 + lane, 32LL * cap, 301)];
            if (!(pv < v)) break;
            H[SX(i * 32 + lane, 32LL * cap, 302)] = pv;
            i = p;
        }
        H[SX(i * 32 + lane, 32LL * cap, 303)] = v;
        return;
    }
    if (!(v < H[lane])) return;
    int i = 0;
    for (;;) {
        const int l = 2 * i + 1;
        if (l >= n) break;
        int c = l;
        float cv = H[SX(l * 32 + lane, 32LL * cap, 304)];
        if (l + 1 < n) {
            const float rv = H[SX((l + 1) * 32 + lane, 32LL * cap, 305)];
            if (rv > cv) { c = l + 1; cv = rv; }
        }
        if (!(cv > v)) break;
        H[SX(i * 32 + lane, 32LL * cap, 306)] = cv;
        i = c;
    }
    H[SX(i * 32 + lane, 32LL * cap, 307)] = v;
}

// The k smallest arcs of one slice as an ascending list of KR registers
// (k <= KR): the first KR - k entries hold -inf and never move, the last k
// the k smallest arcs so far (+inf while unfilled), so the k-th smallest is
// always L[KR-1].  Inserting v and dropping the largest is branch-free:
// entry i becomes min(old[i], max(old[i-1], v)).
template <int KR>
__device__ __forceinline__ void list_insert(float (&L)[KR], float v)
{
#pragma unroll
    for (int i = KR - 1; i > 0; --i) L[i] = fminf(L[i], fmaxf(L[i - 1], v));
    L[0] = fminf(L[0], v);
}

constexpr int FUSE_UPT = 4;     // users per lane per item of the fused verification

// Fused verification, thread 0: claim slot s's result region (min(ncand,
// rcap) ids at the pool's running top) and decide where the slot is
// verified: by this block (here), or by the verification kernel (listed).
// A region past the pool's end is flagged and not verified; the host grows
// the pool and runs the batch again.  The record and the region go to
// shared memory for the block.
__device__ __forceinline__ void fuse_claim(const ZoneArgs& A, int s, QDesc& d, char* smem, const FuseLayout& FL,
                                           bool may_here)
{
    const int rl = min(d.ncand, A.rcap);
    const long long r0 = (long long)atomicAdd((unsigned long long*)A.v.region_top, (unsigned long long)rl);
    const bool fits = r0 + rl <= A.v.pool_cap;
    A.cand_off_w[s] = r0;
    A.reg_len_w[s] = rl;
    if (!fits) d.flags |= QF_RESULT_OVERFLOW;
    const bool verify = fits && d.ncand > 0 && !(d.flags & QF_BAD_QUERY);
    const bool here = verify && may_here && d.ncand <= A.fuse_cand;
    if (verify && !here) A.deflist[atomicAdd(A.ndef, 1)] = s;
    *(QDesc*)(smem + FL.d) = d;
    *(long long*)(smem + FL.r0) = r0;
    *(int*)(smem + FL.rlen) = rl;
    *(int*)(smem + FL.here) = here ? 1 : 0;
}

// Fused verification, every warp of the block: the slot's candidates in
// items of 32 * FUSE_UPT users, the block's warps taking alternate items,
// against the half-planes and segments the filter left in shared memory.
template <int NWQ>
__device__ __forceinline__ void fuse_verify(const ZoneArgs& A, int s, const char* smem, const FuseLayout& FL,
                                            const float* Rs, vitem::VCount& vc)
{
    if (!*(const int*)(smem + FL.here)) return;
    const QDesc d = *(const QDesc*)(smem + FL.d);
    const long long r0 = *(const long long*)(smem + FL.r0);
    const int rl = *(const int*)(smem + FL.rlen);
    const int2* sg = d.nseg + 1 <= A.fuse_ss ? (const int2*)(smem + FL.segs) : A.segs + (size_t)s * A.seg_cap;
    const int nbs = min(d.nb, A.fuse_sc);
    const int wq = NWQ == 2 ? (int)(threadIdx.x >> 5) : 0;
    constexpr int CH = 32 * FUSE_UPT;
    for (int v0 = wq * CH; v0 < d.ncand; v0 += NWQ * CH)
        vitem::verify_item<FUSE_UPT>(A.v, d, s, v0, smem + FL.planes, sg, Rs, nbs, r0, rl, vc);
}

}  // namespace

// KR > 0: the slice bounds live in a register list (k <= KR); KR == 0: in a
// shared-memory max-heap per lane (any k up to the class's capacity).
// NWQ = 2 (register lists only): two warps per query.  Both step through the
// same rings with the same stop decisions; each takes alternate cells of a
// ring (loads, tests and offers their facilities to its own lists) and
// appends their half-planes to one list through a shared count.  At every
// ring top the two warps' lists meet in shared memory: the k-th smallest arc
// of their union is the slice's bound (the k smallest of all offered
// facilities are among the two lists' k smallest), computed identically in
// both warps, and the stream's budget is read from a shared count between
// the same barriers.  At the end warp 0 writes the half-planes while warp 1
// scans the user cells.
template <int KR, int NWQ>
__device__ __forceinline__ void slice_body(const ZoneArgs& A)
{
    static_assert(NWQ == 1 || KR > 0, "two warps per query need register lists");
    pdl_trigger();
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31;
    const int wq = NWQ == 2 ? (int)(threadIdx.x >> 5) : 0;   // warp within the query's block
#ifdef RKNN_CHECKED
    if (threadIdx.x == 0 && blockIdx.x == 0) s_fault = A.fault;
    __syncthreads();
    if (!s_fault) s_fault = A.fault;
#endif
    const SliceLayout LY = slice_layout(A.caps);
    char* wsm = smem + (size_t)wq * LY.bytes;           // this warp's region
    float* H = (float*)(wsm + LY.heap);
    float* Rs = (float*)(wsm + LY.R);
    int* lpos = (int*)(wsm + LY.lpos);
    uint32_t* bitmap = (uint32_t*)(wsm + LY.bitmap);
    // NWQ = 2: both warps' lists ([warp][entry][lane]) and a few ints passed
    // between the warps
    float* xl = (float*)(smem + (size_t)NWQ * LY.bytes);
    int* xs = (int*)(xl + (NWQ == 2 ? 2 * KR * 32 : 0));
    // fused verification: the slot's record, region, half-planes and
    // segments after the filter's own shared memory
    const FuseLayout FL = fuse_layout(slice_own_bytes(LY.bytes, NWQ, KR), A.fuse_sc, A.fuse_ss);
    float4* fzp = (float4*)(smem + FL.planes);
    int2* fzs = (int2*)(smem + FL.segs);
    vitem::VCount vc = {};
    // the host fuses only batches that run two warps a query; the one-warp
    // variants keep their registers for more queries in flight
    const bool FUSED = NWQ == 2 && A.fuse;
    const int KC = A.caps.vc, LC = A.caps.lc;
    const long long NCF = (long long)A.gf.gx * A.gf.gy, NCU = (long long)A.gu.gx * A.gu.gy;
    (void)NCF; (void)NCU;
    // this lane's slice, widened: directions from a0 to b0
    float e1x, e1y, e2x, e2y;
    sincosf((float)lane * SLICE_W - WIDEN, &e1y, &e1x);
    sincosf((float)(lane + 1) * SLICE_W + WIDEN, &e2y, &e2x);
    // the data box, rounded outward
    const float bx0 = __double2float_rd(A.sx0), by0 = __double2float_rd(A.sy0);
    const float bx1 = __double2float_ru(A.sx1), by1 = __double2float_ru(A.sy1);
    // rounding slack of the ring distances: 1e-5 (cs + max |box|), rounded up
    const float slack_f = __fmul_ru(1.0001e-5f, __fadd_ru(A.gf.cs,
        fmaxf(fmaxf(fabsf(bx0), fabsf(bx1)), fmaxf(fabsf(by0), fabsf(by1)))));

    for (;;) {
        int slot = 0;
        if constexpr (NWQ == 2) {
            __syncthreads();            // the previous query is done with the shared ints
            if (threadIdx.x == 0) {
                xs[0] = atomicAdd(A.work_counter, 1);
                xs[6] = 0;              // half-planes taken (both warps)
                xs[7] = 0;              // facilities offered (both warps)
            }
            __syncthreads();
            slot = xs[0];
        } else {
            if (lane == 0) slot = atomicAdd(A.work_counter, 1);
            slot = __shfl_sync(FULL, slot, 0);
        }
        if (slot >= A.nq) break;
        const int s = A.order ? A.order[slot] : slot;
        const int qin = A.q_in[s];
        const int k = A.k_in[s];
        QDesc* qd = A.qd + s;
        ZStats zs = {};
        if (qin < 0 || qin >= A.nf || k <= 0) {
            if (threadIdx.x == 0) {
                QDesc d = {};
                d.qpos = -1;
                d.k = k;
                d.flags = QF_BAD_QUERY;
                if (FUSED) fuse_claim(A, s, d, smem, FL, false);
                *qd = d;
                A.zst[s] = zs;
                A.segs[(size_t)s * A.seg_cap] = make_int2(0, 0);
            }
            continue;
        }
        const int qpos = A.fpos[SX(qin, A.nf, 310)];
        const float2 qf = A.fxy[SX(qpos, A.nf, 311)];
        if (k > KC || (KR > 0 && k > KR)) {
            // k beyond the slice bounds' capacity (a device batch whose kmax
            // understates a k): every user is a candidate and the
            // verification counts exactly
            if (threadIdx.x == 0) {
                QDesc d = {};
                d.qx = qf.x;
                d.qy = qf.y;
                d.qpos = qpos;
                d.k = k;
                d.nseg = 1;
                d.kf2 = 1e-30f;
                d.kf264 = 1e-300;
                d.ncand = A.nu;
                d.flags = QF_ALL_USERS;
                if (FUSED) fuse_claim(A, s, d, smem, FL, false);
                *qd = d;
                A.zst[s] = zs;
                int2* seg = A.segs + (size_t)s * A.seg_cap;
                seg[0] = make_int2(0, 0);
                seg[1] = make_int2(0, A.nu);
            }
            continue;
        }
        long long tph = clock64();

        // C(P): farthest point of the box inside this slice, a vertex of the
        // slice's cone clipped to the box (an edge ray's exit or a box corner
        // inside the cone), rounded up
        float clip;
        {
            clip = fmaxf(exit_dist(qf.x, qf.y, e1x, e1y, bx0, by0, bx1, by1),
                         exit_dist(qf.x, qf.y, e2x, e2y, bx0, by0, bx1, by1));
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {
                const float dx = ((c4 & 1) ? bx1 : bx0) - qf.x, dy = ((c4 & 2) ? by1 : by0) - qf.y;
                // inside the cone (or near its edges: then the corner only raises the bound)
                const float c1 = e1x * dy - e1y * dx, c2 = dx * e2y - dy * e2x;
                const float tol = 1e-5f * (fabsf(dx) + fabsf(dy));
                if (c1 >= -tol && c2 >= -tol) clip = fmaxf(clip, sqrtf(fmaf(dx, dx, dy * dy)));
            }
            clip = clip * (1.0f + 1e-5f) + 1e-30f;
        }

        // ---- stream facilities ring by ring -------------------------------
        int n = 0;              // this slice's heap size (KR == 0)
        float RL[KR > 0 ? KR : 1];   // this slice's k smallest arcs (KR > 0)
#pragma unroll
        for (int i = 0; i < (KR > 0 ? KR : 1); ++i) RL[i] = i < KR - k ? -INFINITY : INFINITY;
        // the slice's current bound R: its k-th smallest arc (infinite below k)
#define SLICE_KTH() (KR > 0 ? RL[(KR > 0 ? KR : 1) - 1] : ((n < k) ? INFINITY : H[lane]))
        // the slice's bound over both warps' lists (NWQ = 2): the k-th smallest
        // of their union, min over i of max(a_{i-1}, b_{k-1-i}) for the
        // ascending real entries a, b (the last k of each list)
        // (NWQ = 2: between its barriers it also reads the facilities both
        // warps offered so far, for the budget test: a count both warps see
        // alike)
        int pts_all = 0;
        auto union_kth = [&]() -> float {
            if constexpr (NWQ == 2) {
                float* mine = xl + (size_t)wq * KR * 32 + lane;
#pragma unroll
                for (int i = 0; i < KR; ++i) mine[i * 32] = RL[(KR > 0 ? i : 0)];
                __syncthreads();
                pts_all = xs[7];
                const float* a = xl + lane;
                const float* b = xl + KR * 32 + lane;
                float best = INFINITY;
                for (int i = 0; i <= k; ++i) {
                    const float x = i > 0 ? a[(KR - k + i - 1) * 32] : -INFINITY;
                    const float y = i < k ? b[(KR - 1 - i) * 32] : -INFINITY;
                    best = fminf(best, fmaxf(x, y));
                }
                __syncthreads();
                return best;
            } else {
                return SLICE_KTH();
            }
        };
        int nL = 0;             // half-planes kept (warp-uniform)
        int rho_ring = -1;      // first ring with a streamed facility left out of the half-planes
        const int fbudget = max(8192, 128 * k);
        // cell boxes widened for the rounding of the cell function
        const float cmargin = 1e-5f * A.gf.cs + 8.0f * kU32 * (fabsf(A.gf.x0) + fabsf(A.gf.y0) + fabsf(qf.x) + fabsf(qf.y) +
                                                               A.gf.cs * (float)max(A.gf.gx, A.gf.gy));
        const int qcx = cell_coord(qf.x, A.gf.x0, A.gf.inv, A.gf.gx);
        const int qcy = cell_coord(qf.y, A.gf.y0, A.gf.inv, A.gf.gy);
        const int rmaxf = max(max(qcx, A.gf.gx - 1 - qcx), max(qcy, A.gf.gy - 1 - qcy));
        const int gx = A.gf.gx, gy = A.gf.gy;
        // NWQ = 2: the warps take alternate cells of each ring (warp 0 ring
        // 0's), and append their half-planes to warp 0's list through a
        // shared count
        int* lpos0 = (int*)(smem + LY.lpos);
        // Rings of up to 32 cells have their cell ranges loaded one ring
        // ahead (lane = range index), so that the load latency overlaps the
        // previous ring's work; ring 0's before the loop.
        int pf_fs = 0, pf_fe = 0;
        if (lane == 0) {
            const long long cid = (long long)qcy * gx + qcx;
            pf_fs = A.fstart[SX(cid, NCF + 1, 330)];
            pf_fe = A.fstart[SX(cid + 1, NCF + 1, 331)];
        }
        int ring = 0;
        for (; ring <= rmaxf; ++ring) {
            long long tp = clock64();
            const int cur_fs = pf_fs, cur_fe = pf_fe;
            {
                const int nr1 = 8 * (ring + 1);
                pf_fs = pf_fe = 0;
                if (nr1 <= 32 && ring + 1 <= rmaxf && lane < nr1) {
                    int cxx, cyy;
                    ring_cell(ring + 1, lane, qcx, qcy, cxx, cyy);
                    if (cxx >= 0 && cxx < gx && cyy >= 0 && cyy < gy) {
                        const long long cid = (long long)cyy * gx + cxx;
                        pf_fs = A.fstart[SX(cid, NCF + 1, 332)];
                        pf_fe = A.fstart[SX(cid + 1, NCF + 1, 333)];
                    }
                }
            }
            // stop when no facility at or beyond this ring can change a
            // slice's effective bound min(R, C)
            const float Rl = fminf(union_kth(), clip);
            __syncwarp();
            float Rmax = Rl;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) Rmax = fmaxf(Rmax, __shfl_xor_sync(FULL, Rmax, o));
            if (ring > 0 && Rmax < INFINITY) {
                // in float, rounded toward stopping later
                const float Lr = __fsub_rd(__fmul_rd((float)(ring - 1), A.gf.cs), slack_f);
                if (Lr > 0.0f && 0.5f * Lr > __fmul_ru(Rmax, 1.0f + 1e-6f)) break;
            }
            // Every heap top is an upper bound at any time, so the stream may
            // stop early; past a budget the remaining (sparse-direction)
            // slices keep their bounds and the kept region grows instead.
            if ((NWQ == 2 ? pts_all : zs.pts) >= fbudget) break;
            // Window maxima of the bounds for the ring: a facility helps only
            // slices within 8 of its own, so a cell whose facilities are all
            // farther than twice the largest bound of the slices within 8 of
            // those the cell spans can enter no heap: its facilities become
            // half-planes without being loaded or offered (plane-only).  (Rs
            // serves as scratch until the stream ends.)
            {
                float Rw = Rl;
#pragma unroll
                for (int dd = 1; dd <= 8; ++dd)
                    Rw = fmaxf(Rw, fmaxf(__shfl_sync(FULL, Rl, (lane + dd) & 31), __shfl_sync(FULL, Rl, (lane - dd) & 31)));
                Rs[lane] = Rw;
                __syncwarp();
            }
            zs.cyc[3] += clock64() - tp;
            tp = clock64();
            // the ring's cells (8 ring of them, 1 for ring 0), one range each
            const int nrange = ring == 0 ? 1 : 8 * ring;
            for (int r0 = 0; r0 < nrange; r0 += 32) {
                const int ri = r0 + lane;
                int fs = 0, fe = 0;
                bool po = false;        // plane-only: the cell's facilities can enter no heap
                if (ri < nrange && (NWQ == 1 || (ri & 1) == wq)) {
                    int cxx, cyy;
                    ring_cell(ring, ri, qcx, qcy, cxx, cyy);
                    if (cxx >= 0 && cxx < gx && cyy >= 0 && cyy < gy) {
                        const long long cid = (long long)cyy * gx + cxx;
                        if (nrange <= 32) {
                            fs = cur_fs;
                            fe = cur_fe;
                        } else {
                            fs = A.fstart[SX(cid, NCF + 1, 312)];
                            fe = A.fstart[SX(cid + 1, NCF + 1, 313)];
                        }
                        if (ring > 0 && fe > fs) {
                            // the cell's box widened for the cell function's rounding
                            const float X0 = A.gf.x0 + (float)cxx * A.gf.cs - cmargin, X1 = A.gf.x0 + (float)(cxx + 1) * A.gf.cs + cmargin;
                            const float Y0 = A.gf.y0 + (float)cyy * A.gf.cs - cmargin, Y1 = A.gf.y0 + (float)(cyy + 1) * A.gf.cs + cmargin;
                            const float ddx = fmaxf(fmaxf(X0 - qf.x, qf.x - X1), 0.0f), ddy = fmaxf(fmaxf(Y0 - qf.y, qf.y - Y1), 0.0f);
                            const float Lc2 = fmaf(ddx, ddx, ddy * ddy) * (1.0f - 4e-6f);     // |box - q|^2, rounded down
                            const float Rc = box_bound(X0 - qf.x, X1 - qf.x, Y0 - qf.y, Y1 - qf.y, Rs);
                            if (Rc < INFINITY && 0.25f * Lc2 > Rc * Rc * (1.0f + 4e-6f)) po = true;
                        }
                    }
                }
                // the next ring's facility lines, while this ring is streamed
                if (r0 == 0 && pf_fe > pf_fs) {
                    prefetch_l1(A.fxy + pf_fs);
                    prefetch_l1(A.fxy + (pf_fe - 1));
                }
                zs.cyc[4] += clock64() - tp;
                tp = clock64();
                // flatten the ranges: inclusive prefix of their lengths
                const int len = fe - fs;
                int incl = len;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += v;
                }
                const int total = __shfl_sync(FULL, incl, 31);
                for (int t0 = 0; t0 < total; t0 += 32) {
                    const int j = t0 + lane;
                    // range holding item j: first lane with incl > j
                    int lo = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const int probe = __shfl_sync(FULL, incl, lo + step - 1);
                        if (probe <= j) lo += step;
                    }
                    const int rs = __shfl_sync(FULL, fs, lo);
                    const int rincl = __shfl_sync(FULL, incl, lo);
                    const int rlen = __shfl_sync(FULL, len, lo);
                    const bool rpo = __shfl_sync(FULL, (int)po, lo) != 0;
                    const int fidx = rs + (j - (rincl - rlen));
                    bool ok = j < total && fidx != qpos;
                    float vx = 0.0f, vy = 0.0f;
                    if (ok && !rpo) {
                        const float2 f = A.fxy[SX(fidx, A.nf, 314)];
                        vx = f.x - qf.x;
                        vy = f.y - qf.y;
                        // a facility at q's position is never strictly nearer
                        // (float differences are zero only for equal floats;
                        // such a facility lies in q's cell, never plane-only)
                        ok = vx != 0.0f || vy != 0.0f;
                    }
                    // half-planes: the first LC facilities of the rings, in
                    // ring order, those of plane-only cells included (so that
                    // rho is limited only by the rings, below)
                    const unsigned pm = __ballot_sync(FULL, ok);
                    int at0 = nL;       // this batch's first half-plane slot
                    if constexpr (NWQ == 2) {
                        int a = 0;
                        if (lane == 0 && pm) a = atomicAdd(xs + 6, __popc(pm));
                        at0 = __shfl_sync(FULL, a, 0);
                    }
                    if (ok) {
                        const int at = at0 + __popc(pm & ((1u << lane) - 1));
                        if (at < LC) lpos0[SX(at, LC, 315)] = fidx;
                    }
                    if (at0 + __popc(pm) > LC && rho_ring < 0) rho_ring = ring;
                    if constexpr (NWQ == 1) nL = min(LC, nL + __popc(pm));
                    const unsigned om = __ballot_sync(FULL, ok && !rpo);      // offered to the bounds
                    zs.pts += __popc(om);
                    if constexpr (NWQ == 2)
                        if (lane == 0 && om) atomicAdd(xs + 7, __popc(om));
                    // A facility has finite arcs only for slices within 90 degrees
                    // of its direction (the 8 slices on either side of its own,
                    // counting the widening) and every arc is at least half its
                    // distance: when that exceeds the largest bound R among
                    // them it can enter no heap.  Bounds only shrink, so the
                    // window maxima taken before the batch are conservative.
                    unsigned m = om;
                    {
                        const int sj = ok ? slice_of(vx, vy) : 0;
                        float Rwj;
                        if constexpr (NWQ == 2) {
                            // the ring top's window maxima of min(R, C) over both
                            // warps' lists (arcs beyond C change no effective bound)
                            Rwj = Rs[sj];
                        } else {
                            const float Rl = SLICE_KTH();
                            float Rw = Rl;
#pragma unroll
                            for (int dd = 1; dd <= 8; ++dd)
                                Rw = fmaxf(Rw, fmaxf(__shfl_sync(FULL, Rl, (lane + dd) & 31),
                                                     __shfl_sync(FULL, Rl, (lane - dd) & 31)));
                            Rwj = __shfl_sync(FULL, Rw, sj);
                        }
                        const bool useful = ok && !rpo && !(0.25f * fmaf(vx, vx, vy * vy) * (1.0f - 4.0f * kU32) >= Rwj * Rwj);
                        m = __ballot_sync(FULL, useful);
                    }
                    // every lane offers every useful facility to its slice
                    zs.cand += __popc(m);
                    const long long t_offer = clock64();
                    if constexpr (KR > 0) {
                        // two facilities per step: their arcs are independent
                        while (m) {
                            const int s1 = __ffs(m) - 1;
                            m &= m - 1;
                            const bool two = m != 0;
                            const int s2 = two ? __ffs(m) - 1 : s1;
                            m &= m - 1;
                            const float ax = __shfl_sync(FULL, vx, s1), ay = __shfl_sync(FULL, vy, s1);
                            const float bx = __shfl_sync(FULL, vx, s2), by = __shfl_sync(FULL, vy, s2);
                            const float u1 = upper_arc_fast(ax, ay, e1x, e1y, e2x, e2y);
                            const float u2 = two ? upper_arc_fast(bx, by, e1x, e1y, e2x, e2y) : INFINITY;
                            if (__any_sync(FULL, fminf(u1, u2) < RL[(KR > 0 ? KR : 1) - 1])) {
                                list_insert<KR>(RL, u1);
                                list_insert<KR>(RL, u2);
                            }
                        }
                    } else {
                        while (m) {
                            const int src = __ffs(m) - 1;
                            m &= m - 1;
                            const float ux = __shfl_sync(FULL, vx, src), uy = __shfl_sync(FULL, vy, src);
                            const float u = upper_arc(ux, uy, e1x, e1y, e2x, e2y);
                            if (n < k || u < H[lane]) heap_insert(H, lane, n, k, u);
                        }
                    }
                    zs.cyc[1] += clock64() - t_offer;
                }
                zs.cyc[5] += clock64() - tp;
                tp = clock64();
            }
            zs.cells += nrange;
        }
        zs.rings = ring;
        // NWQ = 2: each warp's first ring with a facility left out of the
        // half-planes, read by both after the barriers of the bound below
        if constexpr (NWQ == 2)
            if (lane == 0) xs[12 + wq] = rho_ring < 0 ? INT_MAX : rho_ring;
        __syncwarp();
        // R(P): k-th smallest arc, rounded up for the user test, and clipped
        // to the box (no user lies farther)
        {
            const float R = union_kth();
            Rs[lane] = fminf(R < INFINITY ? R * (1.0f + 1e-5f) + 1e-30f : INFINITY, clip);
            if (wq == 0) A.slice_r[(size_t)s * 32 + lane] = Rs[lane];
        }
        __syncwarp();
        if constexpr (NWQ == 2) {
            const int rr = min(xs[12], xs[13]);
            rho_ring = rr == INT_MAX ? -1 : rr;
            nL = min(LC, xs[6]);
            zs.pts = xs[7];
        }
        // rho: every facility outside the half-planes lies in ring rho_ring or
        // beyond, at least (rho_ring - 1) cs from q (less the rounding slack)
        float rho;
        {
            if (rho_ring < 0) rho_ring = ring;          // every streamed facility is a half-plane
            if (rho_ring > rmaxf) rho = INFINITY;
            else {
                const float Lr = __fsub_rd(__fmul_rd((float)(rho_ring - 1), A.gf.cs), slack_f);
                rho = Lr > 0.0f ? Lr : 0.0f;
            }
        }
        zs.cyc[0] += clock64() - tph;
        tph = clock64();

        // ---- half-planes relative to q (as the zone kernel's epilogue) -----
        // In float: a = -2 fl(fx - qx) and b likewise equal the rounded exact
        // values (a float difference is correctly rounded); c = |f - q|^2
        // carries about 5u relative error instead of u.  The verification's
        // bound 8u (2F'(|x'|+|y'|) + F'^2) exceeds the evaluation error with
        // it, about 3u|a x'| + 3u|b y'| + 7u|c|, since |a|, |b| <= 2F' and
        // |c| <= F'^2 (F' from the largest c below, rounded up).
        float k2f = 0.0f, kf2 = 0.0f;
        double k2f64 = 0.0, kf264 = 0.0;
        if (NWQ == 1 || wq == 0) {
        float4* planes = A.planes + (size_t)s * A.pstride;
        float cmax = 0.0f;
        for (int m = lane; m < nL; m += 32) {
            const int pos = lpos[SX(m, LC, 316)];
            const float2 f = A.fxy[SX(pos, A.nf, 317)];
            const float dx = f.x - qf.x, dy = f.y - qf.y;
            const float c = fmaf(dx, dx, dy * dy);
            planes[SX(m, A.pstride, 318)] = make_float4(-2.0f * dx, -2.0f * dy, c, 0.0f);
            if (FUSED && m < A.fuse_sc) {
                fzp[2 * m] = make_float4(-2.0f * dx, -2.0f * dx, -2.0f * dy, -2.0f * dy);
                fzp[2 * m + 1] = make_float4(c, c, 0.0f, 0.0f);
            }
            A.bis_pos[(size_t)s * A.pstride + SX(m, A.pstride, 319)] = pos;
            cmax = fmaxf(cmax, c);
            // the slot is free now: |f - q|^2 rounded well down
            lpos[SX(m, LC, 316)] = __float_as_int(__fmul_rd(c, 1.0f - 1e-6f));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cmax = fmaxf(cmax, __shfl_xor_sync(FULL, cmax, o));
        __syncwarp();
        // Fourth component of half-plane m: the least |f - q|^2 (rounded
        // down) over half-planes m, m+1, ...  Only a facility within 2|u - q|
        // of q can be strictly nearer to u than q, so the verification may
        // stop a user's half-planes once this exceeds 4|u - q|^2.
        {
            float carry = INFINITY;
            for (int t0 = ((nL - 1) >> 5) << 5; t0 >= 0; t0 -= 32) {
                const int m = t0 + lane;
                float v = m < nL ? __int_as_float(lpos[SX(m, LC, 316)]) : INFINITY;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const float h = __shfl_down_sync(FULL, v, o);
                    if (lane + o < 32) v = fminf(v, h);
                }
                v = fminf(v, carry);
                if (m < nL) planes[SX(m, A.pstride, 318)].w = v;
                if (FUSED && m < nL && m < A.fuse_sc) ((float2*)(fzp + 2 * m + 1))[1] = make_float2(v, v);
                carry = __shfl_sync(FULL, v, 0);
            }
        }
        // in float, rounded up (the constants carry a 2e-6 margin over their
        // own rounding); an overflow to +inf only makes every test undecided
        const float Fp = __fadd_ru(__fmul_ru(__fsqrt_ru(__fmul_ru(cmax, 1.0f + 1e-5f)), 1.0f + 1e-6f), 1e-30f);
        const float Fp2 = __fmul_ru(Fp, Fp);
        k2f = __fmul_ru(Fp, 16.0f * kU32 * (1.0f + 2e-6f));
        kf2 = __fadd_ru(__fmul_ru(Fp2, 8.0f * kU32 * (1.0f + 2e-6f)), 1e-30f);
        k2f64 = (double)__fmul_ru(Fp, 16.0f * (float)kU64 * (1.0f + 2e-6f));
        kf264 = (double)__fmul_ru(Fp2, 8.0f * (float)kU64 * (1.0f + 2e-6f)) + 1e-300;
        }   // half-planes

        zs.cyc[7] += clock64() - tph;
        tph = clock64();

        int nseg = 0, ncand = 0;
        int qflags = QF_SLICE_R;
        if (NWQ == 1 || wq == 1) {
        // ---- ring scan over user cells --------------------------------------
        const Grid gu = A.gu;
        const int ucx = cell_coord(qf.x, gu.x0, gu.inv, gu.gx);
        const int ucy = cell_coord(qf.y, gu.y0, gu.inv, gu.gy);
        const int RM = A.rmax;
        const int W = 2 * RM + 1;
        const int nwords = (W * W + 31) / 32;
        for (int i = lane; i < nwords; i += 32) bitmap[SX(i, nwords, 320)] = 0u;
        __syncwarp();
        const float delta = 8.0f * kU32 * (fabsf(gu.x0) + fabsf(gu.y0) + gu.cs * (float)max(gu.gx, gu.gy) + fabsf(qf.x) + fabsf(qf.y) + gu.cs) + 1e-30f;
        const int rmaxu = max(max(ucx, gu.gx - 1 - ucx), max(ucy, gu.gy - 1 - ucy));
        bool all_users = false;
        int rend = -1;
        if (A.nu > 0) {
            for (int r = 0;; ++r) {
                if (r > rmaxu) { rend = r - 1; break; }
                if (r > RM) { all_users = true; break; }
                const int ncell = r == 0 ? 1 : 8 * r;
                bool anykeep = false;
                for (int t0 = 0; t0 < ncell; t0 += 32) {
                    const int t = t0 + lane;
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
                    bool keep = false;
                    if (ok) {
                        const float X0 = (gu.x0 + (float)cxx * gu.cs) - qf.x - delta;
                        const float X1 = (gu.x0 + (float)(cxx + 1) * gu.cs) - qf.x + delta;
                        const float Y0 = (gu.y0 + (float)cyy * gu.cs) - qf.y - delta;
                        const float Y1 = (gu.y0 + (float)(cyy + 1) * gu.cs) - qf.y + delta;
                        if (X0 <= 0.0f && X1 >= 0.0f && Y0 <= 0.0f && Y1 >= 0.0f) keep = true;
                        else {
                            // nearest point of the cell against the largest
                            // bound of the slices the cell spans
                            const float ddx = fmaxf(fmaxf(X0, -X1), 0.0f), ddy = fmaxf(fmaxf(Y0, -Y1), 0.0f);
                            const float dmin2 = fmaf(ddx, ddx, ddy * ddy) * (1.0f - 4.0f * kU32);
                            const float Rmax = box_bound(X0, X1, Y0, Y1, Rs);
                            keep = !(dmin2 > Rmax * Rmax);
                        }
                    }
                    if (keep) {
                        const int bit = (dy + RM) * W + (dx + RM);
                        atomicOr(&bitmap[SX(bit >> 5, nwords, 321)], 1u << (bit & 31));
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
        zs.cyc[2] += clock64() - tph;
        tph = clock64();

        // ---- segments: one user range per row ------------------------------
        int2* seg = A.segs + (size_t)s * A.seg_cap;
        // segment i, also kept in shared memory for the fused verification
        auto put_seg = [&](int i, int2 v) {
            seg[i] = v;
            if (FUSED && i < A.fuse_ss) fzs[i] = v;
        };
        if (all_users) {
            put_seg(0, make_int2(0, 0));
            put_seg(1, make_int2(0, A.nu));
            nseg = 1;
            ncand = A.nu;
            qflags |= QF_ALL_USERS;
        } else if (rend >= 0) {
            const int y0 = max(0, ucy - rend), y1 = min(gu.gy - 1, ucy + rend);
            const int xl0 = max(0, ucx - rend), xl1 = min(gu.gx - 1, ucx + rend);
            for (int r0 = y0; r0 <= y1; r0 += 32) {
                const int row = r0 + lane;
                int st = 0, len = 0;
                if (row <= y1) {
                    const int dy = row - ucy;
                    int xmin = INT_MAX, xmax = -1;
                    for (int cxx = xl0; cxx <= xl1; ++cxx) {
                        const int bit = (dy + RM) * W + (cxx - ucx + RM);
                        if (bitmap[SX(bit >> 5, nwords, 322)] & (1u << (bit & 31))) {
                            xmin = min(xmin, cxx);
                            xmax = cxx;
                        }
                    }
                    if (xmax >= 0) {
                        st = A.ustart[SX((long long)row * gu.gx + xmin, NCU + 1, 323)];
                        len = A.ustart[SX((long long)row * gu.gx + xmax + 1, NCU + 1, 324)] - st;
                    }
                }
                const bool has = len > 0;
                const unsigned m = __ballot_sync(FULL, has);
                const int pre = __popc(m & ((1u << lane) - 1));
                int incl = has ? len : 0;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += v;
                }
                const int excl = incl - (has ? len : 0);
                if (has) {
                    put_seg(SX(nseg + pre, A.seg_cap, 325), make_int2(st, ncand + excl));
                    // the verification reads these users next: start their
                    // coordinates and ids on the way to L2 (at most 64 KB a row)
                    const size_t n = (size_t)min(len, 8192);
                    prefetch_l2_span(A.uxy, sizeof(float2) * (size_t)A.nu, sizeof(float2) * (size_t)st, sizeof(float2) * n);
                    prefetch_l2_span(A.uid, sizeof(int) * (size_t)A.nu, sizeof(int) * (size_t)st, sizeof(int) * n);
                }
                nseg += __popc(m);
                ncand += __shfl_sync(FULL, incl, 31);
            }
            if (lane == 0) put_seg(SX(nseg, A.seg_cap, 326), make_int2(0, ncand));
        } else if (lane == 0) {
            put_seg(0, make_int2(0, 0));
        }
        }   // ring scan and segments
        zs.cyc[7] += clock64() - tph;
        zs.nb = nL;
        if constexpr (NWQ == 2) {
            // warp 1's results to warp 0, which writes the descriptor
            if (threadIdx.x == 32) {
                xs[1] = nseg; xs[2] = ncand; xs[3] = qflags; xs[4] = zs.rings; xs[5] = zs.cand;
                ((long long*)(xs + 8))[0] = zs.cyc[2];
                ((long long*)(xs + 8))[1] = zs.cyc[1];
            }
            __syncthreads();
            if (wq == 0) {
                nseg = xs[1]; ncand = xs[2]; qflags = xs[3]; zs.rings = xs[4]; zs.cand += xs[5];
                zs.cyc[2] = ((long long*)(xs + 8))[0];
                zs.cyc[1] += ((long long*)(xs + 8))[1];
            }
        }
        if (threadIdx.x == 0) {
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
            d.rho = rho;
            d.pad = 0;
            if (FUSED) fuse_claim(A, s, d, smem, FL, true);
            *qd = d;
            if (!FUSED) A.zst[s] = zs;
        }
        if (FUSED) {
            if constexpr (NWQ == 2) __syncthreads(); else __syncwarp();
            tph = clock64();
            fuse_verify<NWQ>(A, s, smem, FL, Rs, vc);
            zs.cyc[6] += clock64() - tph;
            if (threadIdx.x == 0) A.zst[s] = zs;
        }
        __syncwarp();
    }
    if (FUSED) {
        vc.flush(A.v.vstats);
        // the batch's last filter block: the work items of the slots left
        // over (the lists' room and a shared int serve as scratch)
        if (vitem::last_block(A.v.done, A.done_total, xs + 15)) {
            const int n = __ldcg(A.ndef);
            if (n > 0) vitem::plan_deferred_block(A.v, n, A.vchunk, A.chunk_off_w, (int*)xl);
        }
    }
}

#undef SLICE_KTH

__global__ void __launch_bounds__(32, 1) slice_kernel(ZoneArgs A) { slice_body<0, 1>(A); }
__global__ void __launch_bounds__(32, 1) slice_kernel_r4(ZoneArgs A) { slice_body<4, 1>(A); }
__global__ void __launch_bounds__(32, 1) slice_kernel_r8(ZoneArgs A) { slice_body<8, 1>(A); }
__global__ void __launch_bounds__(32, 1) slice_kernel_r10(ZoneArgs A) { slice_body<10, 1>(A); }
__global__ void __launch_bounds__(32, 1) slice_kernel_r12(ZoneArgs A) { slice_body<12, 1>(A); }
__global__ void __launch_bounds__(32, 1) slice_kernel_r16(ZoneArgs A) { slice_body<16, 1>(A); }
__global__ void __launch_bounds__(32, 1) slice_kernel_r24(ZoneArgs A) { slice_body<24, 1>(A); }
__global__ void __launch_bounds__(32, 1) slice_kernel_r32(ZoneArgs A) { slice_body<32, 1>(A); }
__global__ void __launch_bounds__(64, 7) slice_kernel2_r4(ZoneArgs A) { slice_body<4, 2>(A); }
__global__ void __launch_bounds__(64, 7) slice_kernel2_r8(ZoneArgs A) { slice_body<8, 2>(A); }
__global__ void __launch_bounds__(64, 7) slice_kernel2_r10(ZoneArgs A) { slice_body<10, 2>(A); }
__global__ void __launch_bounds__(64, 7) slice_kernel2_r12(ZoneArgs A) { slice_body<12, 2>(A); }
__global__ void __launch_bounds__(64, 7) slice_kernel2_r16(ZoneArgs A) { slice_body<16, 2>(A); }
__global__ void __launch_bounds__(64, 7) slice_kernel2_r24(ZoneArgs A) { slice_body<24, 2>(A); }
__global__ void __launch_bounds__(64, 7) slice_kernel2_r32(ZoneArgs A) { slice_body<32, 2>(A); }

}  // namespace rknn
