// Influence-zone geometry and state helpers shared by the one-warp zone
// kernel (zone.cu) and the one-block zone kernel (zone_cta.cu): the
// reference's line, bisector, intersection and distance functions in FP64
// (rknn-inf/inf.h), their float pre-filters with proven error bounds, the
// priority-queue primitives and the per-query state layout in shared
// memory.  Both translation units are compiled with -fmad=false, so every
// FP64 operation here rounds as the reference's x86-64 build does.
#pragma once
#include "rknn_common.cuh"
#include "zone.cuh"
#include <cfloat>

namespace rknn {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr double EPS = 1e-9;           // inf.cpp:270,375,408; inf.h:324

// flags of a vertex: created on the space boundary, near the newest line,
// and within EPS of the left / right / bottom / top edge (decided once in
// FP64 when the vertex is created; inf.cpp:283-321 tests the same per lookup)
constexpr uint32_t VB_BND = 1, VB_ON = 2, VB_EL = 4, VB_ER = 8, VB_EB = 16, VB_ET = 32;
// the one-block kernel's mark of a vertex the vertex test considers (valid
// while the zone is unchanged since it was set)
constexpr uint32_t VB_CONS = 64;
// flags of a line
constexpr uint32_t LB_VERT = 1, LB_VALID = 2;

struct Line64 {
    double a, b;        // y = a x + b, or x = b when vertical
    int vert, valid;
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

// |a - b| < EPS with the difference rounded in FP64 and the comparison on
// its bits (the magnitude's bits order as its value; a NaN compares false).
__device__ __forceinline__ bool within_eps(double a, double b)
{
    return (__double_as_longlong(__dsub_rn(a, b)) & 0x7fffffffffffffffll) < 0x3e112e0be826d695ll;   // bits of 1e-9
}

__device__ __forceinline__ float rect_dx32(float v, float lo, float hi)
{
    return v < lo ? lo - v : (v > hi ? v - hi : 0.0f);
}

// Exact halving: the exponent lowered by one where the result is normal (the
// product by 0.5 otherwise), which rounds as the reference's division by 2.
__device__ __forceinline__ double half64(double d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    if (e > 1u && e < 0x7ffu) return __longlong_as_double((long long)(b - (1ull << 52)));
    return __dmul_rn(d, 0.5);
}

// perpendicular_bisector (rknn-inf/inf.h:150-192), query first.  Equality
// and order tests run on the bits (order_key; coordinates are never NaN):
// each FP64 instruction costs its warp about 64 cycles on GB300, a compare
// as much as a product.
__device__ Line64 make_bisector(double qx, double qy, double px, double py)
{
    Line64 l;
    const double mx = half64(__dadd_rn(qx, px)), my = half64(__dadd_rn(qy, py));
    l.a = 0; l.b = 0; l.vert = 0;
    if (order_key(qx) == order_key(px)) {
        l.a = 0; l.b = my;
    } else if (order_key(qy) == order_key(py)) {
        l.vert = 1; l.b = mx;
    } else {
        double s = div_rn64(__dsub_rn(py, qy), __dsub_rn(px, qx));
        double ps = div_rn64(-1.0, s);
        double yi = __dsub_rn(my, __dmul_rn(ps, mx));
        if ((__double_as_longlong(ps) & 0x7fffffffffffffffll) == 0x7ff0000000000000ll) { l.vert = 1; l.b = yi; }
        else { l.a = ps; l.b = yi; }
    }
    // (a NaN b, from an infinite slope times a zero midpoint, compares false)
    const bool nan_b = (__double_as_longlong(l.b) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
    if (l.vert) l.valid = (!nan_b && order_key(qx) >= order_key(l.b)) ? 1 : 0;
    else l.valid = (order_key(qy) >= order_key(__dadd_rn(__dmul_rn(l.a, qx), l.b))) ? 1 : 0;
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

// valid64 with the final comparison on order keys instead of the FP64 pipe
// (for points that are not NaN: the same result).
__device__ __forceinline__ bool valid64k(double a, double b, int vert, int valid, double x, double y)
{
    const long long u = order_key(vert ? x : y);
    const long long t = order_key(vert ? b : __dadd_rn(__dmul_rn(a, x), b));
    return valid ? (u >= t) : (u <= t);
}

// find_line_intersection (rknn-inf/inf.h:303-333) in FP64
__device__ __forceinline__ bool intersect64(double a1, double b1, int v1,
                                            double a2, double b2, int v2,
                                            double& x, double& y)
{
    if (v1 && v2) return false;
    if (v1) { x = b1; y = __dadd_rn(__dmul_rn(a2, b1), b2); return true; }
    if (v2) { x = b2; y = __dadd_rn(__dmul_rn(a1, b2), b1); return true; }
    if (within_eps(a1, a2)) return false;
    x = div_rn64(__dsub_rn(b2, b1), __dsub_rn(a1, a2));
    y = __dadd_rn(__dmul_rn(a1, x), b1);
    return true;
}

// min_distance_to_line (rknn-inf/inf.h:275-287)
__device__ double line_dist64(double px, double py, double a, double b, int vert)
{
    if (vert) return fabs(__dsub_rn(px, b));
    double num = fabs(__dadd_rn(__dsub_rn(__dmul_rn(a, px), py), b));
    double den = sqrt_rn64(__dadd_rn(__dmul_rn(a, a), 1.0));
    return div_rn64(num, den);
}

// Per-warp state array.  With RKNN_CHECKED every index is checked against
// the capacity; the first violation is recorded (array id, index, capacity,
// source line) and the access goes to a spare element instead.
#ifdef RKNN_CHECKED
__device__ int* g_fault;
template <typename T>
struct Arr {
    T* p;
    int cap, id;
    T* dummy;
    __device__ T& at(long long i, int line) const
    {
        if (i < 0 || i >= cap) {
            if (g_fault && atomicCAS(g_fault, 0, 1) == 0) {
                g_fault[1] = id; g_fault[2] = (int)i; g_fault[3] = cap; g_fault[4] = line;
            }
            return *dummy;
        }
        return p[i];
    }
};
#define IX(a, i) (a).at((i), __LINE__)
// index i into a global array of n elements: checked, clamped to 0 if bad
__device__ __forceinline__ long long gck(long long i, long long n, int id, int line)
{
    if (i < 0 || i >= n) {
        if (g_fault && atomicCAS(g_fault, 0, 1) == 0) {
            g_fault[1] = id; g_fault[2] = (int)i; g_fault[3] = (int)n; g_fault[4] = line;
        }
        return 0;
    }
    return i;
}
#define GX(i, n, id) gck((i), (n), (id), __LINE__)
#else
#define GX(i, n, id) (i)
template <typename T>
struct Arr {
    T* p;
    __device__ __forceinline__ T& at(long long i, int) const { return p[i]; }
};
#define IX(a, i) (a).p[(i)]
#endif

// ---- priority queue (lane 0 only) ------------------------------------------
// Keys are squared distances (non-negative doubles), stored as their bit
// patterns: for non-negative doubles the integer order is the numeric order,
// so the heap needs no floating-point comparison.
__device__ __forceinline__ bool pq_less(uint64_t k1, uint32_t c1, uint64_t k2, uint32_t c2)
{
    return k1 < k2 || (k1 == k2 && c1 < c2);
}

__device__ __forceinline__ bool pq_push(uint64_t* K, uint32_t* C, int& n, int cap, uint64_t key, uint32_t code)
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

__device__ __forceinline__ void pq_pop(uint64_t* K, uint32_t* C, int& n)
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

// Vertex test for one vertex in float32: 1 if the facility (or rectangle)
// is certainly nearer to the vertex than q is, 0 if certainly not, -1 if the
// float evaluation cannot decide (the caller then decides in FP64).
//   dxp, dyp = float offsets from the facility (rectangle) to the vertex
//   E = bound on a vertex coordinate's float rounding error
//   V = the vertex's squared distance to q, rounded to float
__device__ __forceinline__ int closer32(float dxp, float dyp, float E, float V)
{
    float D = fmaf(dxp, dxp, dyp * dyp);
    float ep = E + kU32 * (fabsf(dxp) + fabsf(dyp));
    float err = fmaf(2.0f * (fabsf(dxp) + fabsf(dyp)) + 2.0f * ep, ep, 4.0f * kU32 * D) + 1e-30f;
    float vlo = V * (1.0f - 4.0f * kU32), vhi = V * (1.0f + 4.0f * kU32);
    if (D + err < vlo) return 1;
    if (D - err > vhi) return 0;
    return -1;
}

// The reference's comparison dist(p, v) < dist(q, v) in FP64, with (dx, dy)
// the offset from p (or the rectangle) to v.
__device__ __forceinline__ bool closer64(double dx, double dy, double vx, double vy, double qx, double qy)
{
    return sqrt_rn64(__dadd_rn(dsq(dx), dsq(dy))) < sqrt_rn64(d2_64(vx, vy, qx, qy));
}

// Edge flags of a vertex (within EPS of each side of the space, in FP64).
__device__ __forceinline__ uint8_t edge_bits(double x, double y, double sx0, double sy0,
                                             double sx1, double sy1)
{
    uint8_t f = 0;
    if (within_eps(x, sx0)) f |= VB_EL;
    if (within_eps(x, sx1)) f |= VB_ER;
    if (within_eps(y, sy0)) f |= VB_EB;
    if (within_eps(y, sy1)) f |= VB_ET;
    return f;
}

constexpr uint64_t INF_BITS = 0x7ff0000000000000ull;

// Rules 1 and 2 compare sqrt_rn(key) with a threshold T (2 x furthest
// vertex, 2 x nearest bisector).  Keys are non-negative doubles, so their bit
// patterns order like their values, and two integer bounds settle almost
// every key:
//   key >= hi  =>  sqrt(key) >= T (1 + 2^-51) > next(T)  =>  sqrt_rn(key) > T
//   key <= lo  =>  sqrt(key) <= T (1 - 2^-50) < prev(T)  =>  sqrt_rn(key) < T
// with lo, hi = T*T (1 -/+ 2^-48), each product rounded.  Keys in between
// (within about 2^-48 of T*T) take the square root.
struct Cut {
    uint64_t lo, hi;
};
constexpr uint64_t NEVER = INF_BITS + 1;       // no finite key reaches it

// Callers test hi first, then lo.  For T = 0 the two rules need different
// bounds: rule 1 (sqrt_rn(key) > 0) holds for every key but 0; rule 2
// (sqrt_rn(key) < 0) never holds.
__device__ __forceinline__ Cut sqrt_cut(double T, bool rule2)
{
    Cut c;
    if (!(T <= DBL_MAX)) { c.lo = INF_BITS; c.hi = NEVER; return c; }   // T = +inf
    if (T == 0.0) { c.lo = 0; c.hi = rule2 ? 0 : 1; return c; }
    if (T < 0x1p-900) { c.lo = 0; c.hi = NEVER; return c; }             // no margins near subnormals
    const double t2 = __dmul_rn(T, T);
    c.lo = (uint64_t)__double_as_longlong(__dmul_rn(t2, 1.0 - 0x1p-48));
    c.hi = (uint64_t)__double_as_longlong(__dmul_rn(t2, 1.0 + 0x1p-48));
    return c;
}

// Rule 1's bounds from the farthest vertex's squared distance d2 (as bits),
// without its square root: T = 2 sqrt_rn(d2), and T*T lies within about
// 2^-51 of 4 d2, whose bits are d2's with the exponent raised by two.  Keys
// 64 units in the last place or more above 4 d2 are at least 2^-47 above it,
// so sqrt(key) exceeds T by more than 2^-49 and sqrt_rn(key) > T; keys 64 or
// more below are below T likewise.  Outside [2^-1000, 2^1000] every key takes
// the square root.
__device__ __forceinline__ Cut far_cut(long long d2bits)
{
    Cut c;
    const uint64_t b = (uint64_t)d2bits;
    if (b < (uint64_t)(1023 - 1000) << 52 || b > (uint64_t)(1023 + 1000) << 52) { c.lo = 0; c.hi = NEVER; return c; }
    const uint64_t b4 = b + (2ull << 52);
    c.lo = b4 - 64;
    c.hi = b4 + 64;
    return c;
}

// Rule 2's bounds for the nearest bisector distance dl (T = 2 dl), with the
// margin of far_cut: 4 dl^2 rounded, and 64 units in the last place either
// side.  T = 0: rule 2 (sqrt_rn(key) < 0) never holds; outside [2^-500,
// 2^500] every key takes the square root.
__device__ __forceinline__ Cut near_cut(double dl)
{
    Cut c;
    const uint64_t b = (uint64_t)__double_as_longlong(dl);
    if (b == 0) { c.lo = 0; c.hi = 0; return c; }
    if (b < (uint64_t)(1023 - 500) << 52 || b > (uint64_t)(1023 + 500) << 52) { c.lo = 0; c.hi = NEVER; return c; }
    const double T = __dmul_rn(dl, 2.0);
    const uint64_t t2 = (uint64_t)__double_as_longlong(__dmul_rn(T, T));
    c.lo = t2 - 64;
    c.hi = t2 + 64;
    return c;
}

// FP32 form of ring_gate (below), conservative: Lr rounded down and the
// threshold T >= 2 far (1 + 1e-9) + slack rounded up, so a ring opens no
// later than the FP64 gate opens it (an earlier expansion only puts cells in
// the queue sooner; the order of the entries taken is the same).
__device__ __forceinline__ float ring_limit32(long long far2bits, float slack_ru)
{
    const float f = __fmul_ru(__fsqrt_ru(d2f_bits<1>(__longlong_as_double(far2bits))), 1.0f + 0x1p-22f);
    return __fadd_ru(__fmul_ru(2.0f * (1.0f + 0x1p-22f), f), slack_ru);
}
__device__ __forceinline__ void ring_gate32(int ring, int rmaxf, float cs, float slack_ru, float T_ru, bool& open,
                                            uint64_t& key)
{
    float Lr = ring == 0 ? 0.0f : __fsub_rd(__fmul_rd((float)(ring - 1), cs), slack_ru);
    if (!(Lr > 0.0f)) Lr = 0.0f;
    open = ring <= rmaxf && !(Lr > T_ru);
    key = (uint64_t)__double_as_longlong((double)__fmul_rd(Lr, Lr));
}

// Whether facility ring `ring` (cells at Chebyshev distance `ring` from q's
// cell) may still hold entries that rule 1 keeps, and the squared lower
// bound of its cells' distances to q, as key bits.
__device__ __forceinline__ void ring_gate(int ring, int rmaxf, double cs, double slack, double far_,
                                          bool& open, uint64_t& key)
{
    double Lr = ring == 0 ? 0.0 : (double)(ring - 1) * cs - slack;
    if (!(Lr > 0.0)) Lr = 0.0;
    open = ring <= rmaxf && !(Lr > 2.0 * far_ * (1.0 + 1e-9) + slack);
    key = (uint64_t)__double_as_longlong(Lr * Lr);
}

// Float bounds of the double that rounded (to nearest) to v.
__device__ __forceinline__ float lo32(float v) { return __fsub_rd(v, __fmaf_ru(fabsf(v), 0x1p-23f, 0x1p-126f)); }
__device__ __forceinline__ float hi32(float v) { return __fadd_ru(v, __fmaf_ru(fabsf(v), 0x1p-23f, 0x1p-126f)); }

struct Slice {
    Arr<double2> vd;         // vertex coordinates
    Arr<float4> v4;          // x, y, d2 to q (float), count | flags << 16
    Arr<uint16_t> cons;      // considered vertices of the vertex test
    Arr<uint16_t> blist;     // boundary vertices with count < k (aliases cd)
    Arr<double2> ld;         // bisectors (FP64)
    Arr<float4> l4;          // bisectors (float): a, b, 3.01u|b| + tiny, flags
    Arr<int> lpos;           // facility position of each bisector
    Arr<uint64_t> pqk;
    Arr<uint32_t> pqc;
    Arr<double2> cd;         // candidate intersections (FP64)
    Arr<float2> c2;          // the same rounded to float
    Arr<int> ccnt;
    Arr<uint8_t> cfl;
    Arr<uint64_t> tk;
    Arr<uint32_t> tc;
    Arr<uint32_t> bitmap;    // user-cell ring bitmap (aliases vd once the zone is built)
    Arr<float4> splanes;     // half-planes for the ring scan (aliases cd)
};

__device__ Slice carve(char* base, const ZoneCaps& c)
{
    ZoneLayout L = zone_layout(c);
    Slice s;
    const int VC = c.vc, LC = c.lc, PC = c.pc, CC = c.lc + 4;
    const int W = 2 * c.rm + 1;
#ifdef RKNN_CHECKED
#define CARVE(f, T, off, n, i) s.f = Arr<T>{(T*)(base + L.off), (int)(n), i, (T*)(base + L.sc)}
#else
#define CARVE(f, T, off, n, i) s.f = Arr<T>{(T*)(base + L.off)}
#endif
    CARVE(vd, double2, vd, VC, 1); CARVE(v4, float4, v4, VC, 2); CARVE(cons, uint16_t, cons, VC, 3);
    CARVE(blist, uint16_t, cd, 8 * CC, 4);
    CARVE(ld, double2, ld, LC, 5); CARVE(l4, float4, l4, LC, 6); CARVE(lpos, int, lpos, LC, 7);
    CARVE(pqk, uint64_t, pqk, PC, 8); CARVE(pqc, uint32_t, pqc, PC, 9);
    CARVE(cd, double2, cd, CC, 10); CARVE(c2, float2, c2, CC, 11); CARVE(ccnt, int, ccnt, CC, 12);
    CARVE(cfl, uint8_t, cfl, CC, 13);
    CARVE(tk, uint64_t, tk, 32, 14); CARVE(tc, uint32_t, tc, 32, 15);
    CARVE(bitmap, uint32_t, vd, (W * W + 31) / 32, 16);
    CARVE(splanes, float4, cd, LC, 17);
#undef CARVE
    (void)VC; (void)LC; (void)PC; (void)CC; (void)W;
    return s;
}

// v4.w holds a vertex's count (bits 0-15) and flags (bits 16-23)
__device__ __forceinline__ float vpack(uint32_t cnt, uint32_t fl) { return __uint_as_float(cnt | (fl << 16)); }
__device__ __forceinline__ uint32_t vcnt_of(float w) { return __float_as_uint(w) & 0xffffu; }
__device__ __forceinline__ uint32_t vfl_of(float w) { return __float_as_uint(w) >> 16; }

// Float side test of a point (x, y) against a bisector record L: 1 if it
// lies certainly on the invalid side, -1 if certainly on the valid side, 0
// if the float evaluation cannot decide.  K1, K0 bound the error that the
// point's float coordinates (or interval) contribute; vertical bisectors
// have a = 0 and compare x with b.
__device__ __forceinline__ int side32(const float4& L, float x, float y, float K1, float K0)
{
    const uint32_t lf = __float_as_uint(L.w);
    const bool vert = (lf & LB_VERT) != 0;
    const float sgn = (vert ? x : y) - fmaf(L.x, x, L.y);
    const float err = fmaf(fabsf(L.x), K1, (vert ? K1 : K0) + L.z);
    const bool valid_above = (lf & LB_VALID) != 0;
    if (sgn > err) return valid_above ? -1 : 1;
    if (sgn < -err) return valid_above ? 1 : -1;
    return 0;
}

// Certainly-invalid test only (for the certified pre-discard).
__device__ __forceinline__ int inval32(const float4& L, float x, float y, float K1, float K0)
{
    const uint32_t lf = __float_as_uint(L.w);
    const bool vert = (lf & LB_VERT) != 0;
    const float sgn = (vert ? x : y) - fmaf(L.x, x, L.y);
    const float err = fmaf(fabsf(L.x), K1, (vert ? K1 : K0) + L.z);
    return (lf & LB_VALID) ? (sgn < -err) : (sgn > err);
}

}  // namespace

}  // namespace rknn
