// Shared definitions of the GB300 RkNN engine: grid descriptors, per-query
// descriptors and the exact sign predicate for squared-distance comparisons.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rknn {

constexpr float kU32 = 5.9604644775390625e-08f;      // 2^-24, float unit roundoff
constexpr double kU64 = 1.1102230246251565e-16;      // 2^-53, double unit roundoff

// Uniform grid over the data's bounding box.  A coordinate v falls in cell
// floor((v - o) * inv) (float arithmetic, clamped), which is monotone in v:
// every range test below can use the same function on its end points.
struct Grid {
    float x0, y0;      // origin (bounding-box minimum)
    float inv;         // 1 / cell width
    float cs;          // cell width
    int gx, gy;        // cells per axis
};

// Bring the line holding p into this SM's L1 (no register, no wait).
__device__ __forceinline__ void prefetch_l1(const void* p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// Hint: bring bytes [off, off + bytes) of the array at base (base_bytes
// long) into L2, one bulk prefetch.  The span is widened to 16-byte
// boundaries and clipped to the array's 16-byte-aligned interior, as the
// instruction requires; it does not wait and writes nothing.
__device__ __forceinline__ void prefetch_l2_span(const void* base, size_t base_bytes, size_t off, size_t bytes)
{
    const unsigned long long b = (unsigned long long)base;
    const unsigned long long lo = (b + 15) & ~15ull, hi = (b + base_bytes) & ~15ull;
    const unsigned long long a0 = max((b + off) & ~15ull, lo);
    const unsigned long long a1 = min((b + off + bytes + 15) & ~15ull, hi);
    if (a1 > a0)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a0), "r"((unsigned)(a1 - a0)) : "memory");
}

// Correctly rounded FP64 square root and quotient (the results of
// __dsqrt_rn and __ddiv_rn) as PTX statements.  The compiler may execute a
// square-root or division intrinsic that a branch guards on both sides of the
// branch (it has no side effects), paying for its long FP64 sequence on the
// common path; it does not execute an asm statement speculatively.
__device__ __forceinline__ double sqrt_rn64(double x)
{
    double r;
    asm("sqrt.rn.f64 %0, %1;" : "=d"(r) : "d"(x));
    return r;
}
__device__ __forceinline__ double div_rn64(double a, double b)
{
    double r;
    asm("div.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}

// Exact widening of a float, as a PTX statement for the same reason: a
// conversion to or from double takes an FP64 pipe slot per lane, and the
// compiler would hoist a plain one out of a rarely taken branch.
__device__ __forceinline__ double f2d(float x)
{
    double r;
    asm("cvt.f64.f32 %0, %1;" : "=d"(r) : "f"(x));
    return r;
}

// Float rounding of a double by integer operations: a conversion
// instruction between float and double takes an FP64 pipe slot, as long as
// an FP64 add.  MODE 0 rounds to nearest (ties to even), -1 toward -inf, +1
// toward +inf; results that are not normal floats (zero, subnormal,
// overflow) come from the conversion instruction.
template <int MODE>
__device__ __forceinline__ float d2f_bits(double d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e <= 0 || e >= 255) {
        float r;
        if (MODE == 0) asm("cvt.rn.f32.f64 %0, %1;" : "=f"(r) : "d"(d));
        else if (MODE < 0) asm("cvt.rm.f32.f64 %0, %1;" : "=f"(r) : "d"(d));
        else asm("cvt.rp.f32.f64 %0, %1;" : "=f"(r) : "d"(d));
        return r;
    }
    const unsigned sign = hi & 0x80000000u;
    // the exponent and the top 23 of the 52 fraction bits; the 29 dropped
    unsigned r = ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    if (MODE == 0) {
        if (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) r += 1u;   // a carry raises the exponent
    } else if (MODE < 0) {
        if (sign && rest) r += 1u;
    } else {
        if (!sign && rest) r += 1u;
    }
    return __uint_as_float(sign | r);
}

// Exact widening of a float by integer operations (zero, subnormals, inf and
// nan take the conversion instruction).
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0u || e == 255u) return f2d(f);
    const unsigned hi = (u & 0x80000000u) | ((e + 1023u - 127u) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}

// Integer key with the numeric order of a double (-0 counts as +0; a NaN
// orders above +inf or below -inf by its sign bit), for comparisons without
// the FP64 pipe.
__device__ __forceinline__ long long order_key(double d)
{
    long long b = __double_as_longlong(d);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start while its predecessor in the stream still runs:
// pdl_wait() blocks until that grid has completed and its memory operations
// are visible (a no-op for an ordinary launch), and pdl_trigger() lets the
// successor launch once every block of this grid has issued it.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Angular slice (of 32 around the origin, slice i spanning [i, i+1) * 11.25
// degrees counter-clockwise from +x) of direction (vx, vy): the octant from
// signs and |vx| <= |vy|, then the quarter of the octant from the ratio
// min/max against tan(11.25), tan(22.5), tan(33.75) degrees.  The products
// carry float rounding only, so the index is exact except within about
// 1e-7 rad of a slice edge, where it may name the neighbour.  (0, 0) gives 0.
__host__ __device__ __forceinline__ int slice_of(float vx, float vy)
{
    const float ax = fabsf(vx), ay = fabsf(vy);
    const float mn = fminf(ax, ay), mx = fmaxf(ax, ay);
    const int sub = (mn > 0.198912367f * mx) + (mn > 0.414213562f * mx) + (mn > 0.668178638f * mx);
    int s = ay <= ax ? sub : 7 - sub;       // slice of the first-quadrant reflection
    if (vx < 0.0f) s = vy >= 0.0f ? 15 - s : 16 + s;
    else if (vy < 0.0f) s = 31 - s;
    return s;
}

__host__ __device__ __forceinline__ int cell_coord(float v, float o, float inv, int g)
{
    float t = floorf((v - o) * inv);
    if (!(t >= 0.0f)) return 0;           // also catches NaN
    if (t > (float)(g - 1)) return g - 1;
    return (int)t;
}

// Per-query descriptor written by the zone kernel and read by verification.
struct QDesc {
    float qx, qy;      // query facility coordinates
    int qpos;          // its position in the cell-sorted facility array
    int k;
    int nb;            // bisector half-planes stored
    int nseg;          // user segments stored
    float k2f, kf2;    // per-user FP32 bound: 8u(2F'(|x'|+|y'|) + F'^2) = k2f*(|x'|+|y'|) + kf2
    double k2f64, kf264;
    int ncand;         // users in all segments
    int flags;         // RKNN_QF_* bits
    float rho;         // every facility nearer to q than rho is one of the half-planes
                       // (0 when unknown): a user with 2|u-q| <= rho is decided by them
    int pad;
};

// QDesc.flags
constexpr int QF_ZONE_V_OVERFLOW = 1;    // vertex capacity reached: zone stopped early
constexpr int QF_ZONE_L_OVERFLOW = 2;    // bisector capacity reached
constexpr int QF_ZONE_PQ_OVERFLOW = 4;   // priority queue full
constexpr int QF_ALL_USERS = 8;          // cell scan gave up: every user is a candidate
constexpr int QF_SLICE_R = 64;           // slice bounds of the query are in slice_r (32 floats)
constexpr int QF_RESULT_OVERFLOW = 16;   // result pool too small
constexpr int QF_BAD_QUERY = 32;         // q or k out of range

// Zone statistics per query (all counters, for logs and tests).
struct ZStats {
    int nb;            // bisectors created
    int vmax;          // largest vertex set
    int pts;           // facilities tested
    int cells;         // facility cells tested
    int cand;          // candidate vertices considered
    int cand64;        // candidates whose intersection was computed in FP64
    int kept;          // candidates kept as vertices
    int rings;         // user-cell rings scanned
    long long cyc[8];  // SM cycles per phase: 0 ring expansion, 1 pop + rules,
                       // 2 vertex test, 3 count pass, 4 candidates, 5 dedup,
                       // 6 counts/erase/append, 7 epilogue
};

// Verification statistics, accumulated over a batch.
struct VStats {
    unsigned long long cand;       // users tested against half-planes
    unsigned long long plane_evals;// (user, half-plane) evaluations executed
    unsigned long long survivors;  // users sent to the exact count
    unsigned long long fac_checks; // (user, facility) comparisons in the exact count
    unsigned long long rechecks;   // comparisons re-decided exactly (FP64 expansion)
    unsigned long long results;
};

// ------------------------------------------------------------ exact predicate
// Sign of d2(u,f) - d2(u,q) for float inputs.  Every product of two floats is
// exact in double, and
//   d2(u,f) - d2(u,q) = fx^2+fy^2-qx^2-qy^2 - 2ux fx - 2uy fy + 2ux qx + 2uy qy
// is a sum of eight exact doubles.  Its sign comes from a nonoverlapping
// expansion grown with TwoSum (Knuth; Shewchuk 1997, Grow-Expansion): the sign
// of an expansion is the sign of its largest nonzero component.  Explicit
// round-to-nearest intrinsics keep the compiler from fusing or reordering.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e)
{
    double x = __dadd_rn(a, b);
    double bv = __dsub_rn(x, a);
    double av = __dsub_rn(x, bv);
    double br = __dsub_rn(b, bv);
    double ar = __dsub_rn(a, av);
    s = x;
    e = __dadd_rn(ar, br);
}

static __device__ __noinline__ int sign_d2diff_exact(float ux, float uy, float fx, float fy,
                                              float qx, float qy)
{
    double t[8];
    t[0] = __dmul_rn((double)fx, (double)fx);
    t[1] = __dmul_rn((double)fy, (double)fy);
    t[2] = -__dmul_rn((double)qx, (double)qx);
    t[3] = -__dmul_rn((double)qy, (double)qy);
    t[4] = -2.0 * __dmul_rn((double)ux, (double)fx);
    t[5] = -2.0 * __dmul_rn((double)uy, (double)fy);
    t[6] = 2.0 * __dmul_rn((double)ux, (double)qx);
    t[7] = 2.0 * __dmul_rn((double)uy, (double)qy);
    double e[8];
    int m = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        double q = t[i];
        for (int j = 0; j < m; ++j) {
            double s, h;
            two_sum(q, e[j], s, h);
            e[j] = h;
            q = s;
        }
        e[m++] = q;
    }
    for (int j = m - 1; j >= 0; --j)
        if (e[j] != 0.0) return e[j] > 0.0 ? 1 : -1;
    return 0;
}

// f strictly nearer to u than q, FP32 filter then exact.  The computed squared
// distances carry a relative error below (1+u)^4-1 each and the difference one
// more rounding: |err| <= 5.0001u (Df+Dq) (+ underflow, covered by 1e-30).
__device__ __forceinline__ bool closer_f32(float ux, float uy, float fx, float fy,
                                           float qx, float qy, float Dq,
                                           unsigned long long* rechecks)
{
    float dx = ux - fx, dy = uy - fy;
    float Df = fmaf(dx, dx, dy * dy);
    float d = Df - Dq;
    float bnd = fmaf(6.0f * kU32, Df + Dq, 1e-30f);
    if (d < -bnd) return true;
    if (d > bnd) return false;
    ++*rechecks;
    return sign_d2diff_exact(ux, uy, fx, fy, qx, qy) < 0;
}

// Same decision with a double-precision filter (the plain FP64 form).
__device__ __forceinline__ bool closer_f64(float ux, float uy, float fx, float fy,
                                           float qx, float qy, double Dq,
                                           unsigned long long* rechecks)
{
    double dx = (double)ux - (double)fx, dy = (double)uy - (double)fy;
    double Df = fma(dx, dx, dy * dy);
    double d = Df - Dq;
    double bnd = 8.0 * kU64 * (Df + Dq);
    if (d < -bnd) return true;
    if (d > bnd) return false;
    ++*rechecks;
    return sign_d2diff_exact(ux, uy, fx, fy, qx, qy) < 0;
}

}  // namespace rknn
