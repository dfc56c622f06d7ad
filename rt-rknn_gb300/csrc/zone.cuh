// Influence-zone kernel interface: capacities, per-warp state layout, args.
#pragma once
#include "rknn_common.cuh"
#include "verify.cuh"

namespace rknn {

constexpr int ZONE_WARPS = 1;          // warps (queries in flight) per block
// zone_kernel_cta: one block of ZCTA_THREADS threads per query; its queue
// holds at most ZCTA_PQ_MAX entries (a multiple of ZCTA_THREADS)
constexpr int ZCTA_THREADS = 256;
constexpr int ZCTA_PQ_MAX = 2048;

// Per-query capacities of the zone state.  Measured on uniform data
// (100k facilities): about 4.6k bisectors and at most ~4k^2 live vertices
// for k in 1..50.
struct ZoneCaps {
    int vc;   // vertices
    int lc;   // bisectors
    int pc;   // priority-queue entries
    int rm;   // user-cell ring scan radius (cells)
};

// Per-query state in shared memory.  Vertices and bisectors are kept as
// 16-byte records so that one load brings everything a loop needs:
//   vd   double2 (x, y)                           vertex coordinates (FP64)
//   v4   float4  (x, y, d2 to q, count | flags<<16)  the same rounded to float
//   ld   double2 (a, b)                           bisector y = a x + b (x = b if vertical)
//   l4   float4  (a, b, 3.01u|b|, flags)          the same rounded to float
//   cd   double2 / c2 float2                      candidate intersections
struct ZoneLayout {
    size_t vd, v4, cons, ld, l4, lpos;
    size_t pqk, pqc;
    size_t cd, c2, ccnt, cfl;
    size_t tk, tc, sc;
    size_t bytes;
};

__host__ __device__ inline size_t zl_align(size_t x) { return (x + 15) & ~(size_t)15; }

#if defined(RKNN_CHECKED) && defined(RKNN_CHECKED_SPARE)
constexpr size_t ZL_SPARE = 1;     // one spare element per array takes rejected accesses
#else
constexpr size_t ZL_SPARE = 0;
#endif

__host__ __device__ inline size_t zl_max(size_t a, size_t b) { return a > b ? a : b; }

__host__ __device__ inline ZoneLayout zone_layout(const ZoneCaps& c)
{
    ZoneLayout L;
    size_t o = 0;
    const size_t VC = c.vc + ZL_SPARE, LC = c.lc + ZL_SPARE, PC = c.pc + ZL_SPARE;
    const size_t CC = (size_t)c.lc + 4 + ZL_SPARE;
    const size_t W = 2 * (size_t)c.rm + 1;
    const size_t bm = ((W * W + 31) / 32 + ZL_SPARE) * 4;
    L.vd = o;   o = zl_align(o + zl_max(16 * VC, bm));     // also the epilogue's cell bitmap
    L.v4 = o;   o = zl_align(o + 16 * VC);
    L.cons = o; o = zl_align(o + 2 * VC);                  // vertex indices < 65536
    L.ld = o;   o = zl_align(o + 16 * LC);
    L.l4 = o;   o = zl_align(o + 16 * LC);
    L.lpos = o; o = zl_align(o + 4 * LC);
    L.pqk = o;  o = zl_align(o + 8 * PC);
    L.pqc = o;  o = zl_align(o + 4 * PC);
    // candidates; between bisector additions the same bytes hold the list of
    // boundary vertices (at most 4 + 4 x bisectors, uint16), and after the
    // zone is built the float half-planes (lc float4)
    L.cd = o;   o = zl_align(o + zl_max(16 * CC, 16 * LC));
    L.c2 = o;   o = zl_align(o + 8 * CC);
    L.ccnt = o; o = zl_align(o + 4 * CC);
    L.cfl = o;  o = zl_align(o + CC);
    L.tk = o;   o = zl_align(o + 8 * (32 + ZL_SPARE));
    L.tc = o;   o = zl_align(o + 4 * (32 + ZL_SPARE));
    L.sc = o;   o = zl_align(o + 128);
    L.bytes = o;
    return L;
}

// Angular-slice filter (slice_kernel): 32 slices around q, one per lane.
// caps.vc = heap entries per slice (the batch class's largest k), caps.lc =
// half-planes kept for the verification, caps.rm = user ring scan radius.
struct SliceLayout {
    size_t heap, R, lpos, bitmap, bytes;
};

__host__ __device__ inline SliceLayout slice_layout(const ZoneCaps& c)
{
    SliceLayout L;
    size_t o = 0;
    const size_t W = 2 * (size_t)c.rm + 1;
    L.heap = o;   o = zl_align(o + 4 * 32 * ((size_t)c.vc + ZL_SPARE));
    L.R = o;      o = zl_align(o + 4 * 32);
    L.lpos = o;   o = zl_align(o + 4 * ((size_t)c.lc + ZL_SPARE));
    L.bitmap = o; o = zl_align(o + 4 * ((W * W + 31) / 32 + ZL_SPARE));
    L.bytes = o;
    return L;
}

struct ZoneArgs {
    // facility index
    const float2* fxy;       // cell-sorted facility coordinates
    const int* fstart;       // facility cell starts (gf.gx*gf.gy+1)
    const float4* fmbr;      // per-cell MBR (minx, miny, maxx, maxy)
    const int* fpos;         // input index -> cell-sorted position
    Grid gf;
    int nf;
    // user index
    const int* ustart;       // user cell starts (gu.gx*gu.gy+1)
    const float2* uxy;       // cell-sorted user coordinates and ids (the slice
    const int* uid;          // filter prefetches each candidate range into L2)
    Grid gu;
    int nu;
    double sx0, sy0, sx1, sy1;   // bounding box of all points (the zone's space)
    // batch
    const int* q_in;         // facility input index per query slot
    const int* k_in;
    const int* order;        // processing order of slots (may be null)
    int nq;
    int* work_counter;
    ZoneCaps caps;
    int skip_coincident;
    int vertex_test = 0;     // 0: count k-1 and extreme boundary vertices (rknn-inf); 1: every
                             // zone-boundary vertex (count k-1, space boundary with count < k)
    int rmax;                // == caps.rm
    int seg_cap;             // segments per query slot (>= 2*rmax+2)
    // outputs (per slot)
    QDesc* qd;
    float4* planes;          // [slot][pstride]
    int* bis_pos;            // [slot][pstride] facility positions of the bisectors
    int pstride;             // >= caps.lc: row stride of planes / bis_pos
    float* slice_r;          // [slot][32]: the slice filter's bounds R(P) (slice kernel)
    int2* segs;              // [slot][seg_cap]: (user start, candidate offset)
    ZStats* zst;
    int* fault;              // checked builds: {flag, array id, index, capacity, line}
    // Fused verification (slice filter, FP32 batches): the block claims each
    // slot's result region itself and verifies the slot's users when there
    // are at most fuse_cand of them; larger slots are listed for the
    // verification kernel.
    int fuse = 0;
    int fuse_cand = 0;       // most candidates a block verifies itself
    int fuse_sc = 0;         // half-planes kept in shared memory
    int fuse_ss = 0;         // segments kept in shared memory
    int rcap = 0;            // most ids a slot's region holds
    long long* cand_off_w = nullptr;   // [slot] region start (written here)
    int* reg_len_w = nullptr;          // [slot] region length
    int* deflist = nullptr;            // slots left to the verification kernel
    int* ndef = nullptr;               // their count
    int* chunk_off_w = nullptr;        // their work-item offsets (items of vchunk users)
    int vchunk = 0;
    int done_total = 0;                // blocks of all the batch's filter launches (v.done counts them)
    VerifyArgs v;            // the verification's arguments
};

// Fused verification state after the slice filter's own shared memory:
// the slot's descriptor, region, verify-here flag, then fuse_sc half-planes
// of 32 bytes ((a, a, b, b), (c, c, w, w)) and fuse_ss segments.
struct FuseLayout {
    size_t d, r0, rlen, here, planes, segs, bytes;
};

__host__ __device__ inline FuseLayout fuse_layout(size_t base, int sc, int ss)
{
    FuseLayout L;
    size_t o = zl_align(base);
    L.d = o;      o += sizeof(QDesc);
    L.r0 = o;     o += 8;
    L.rlen = o;   o += 4;
    L.here = o;   o += 4;
    o = zl_align(o);
    L.planes = o; o += 32 * (size_t)sc;
    L.segs = o;   o += 8 * (size_t)ss;
    L.bytes = zl_align(o);
    return L;
}

// Start of the slice kernel's shared memory after its own state: NWQ warps'
// regions, then (two warps) both warps' lists and 64 bytes of shared ints.
__host__ __device__ inline size_t slice_own_bytes(size_t warp_bytes, int nwq, int kr)
{
    return (size_t)nwq * warp_bytes + (nwq == 2 ? (size_t)2 * kr * 32 * sizeof(float) + 64 : 0);
}

// zone state in shared memory, one warp (one query at a time) per block
__global__ void zone_kernel_smem(ZoneArgs a);
// the same search, one block of ZCTA_THREADS per query (small batches), and
// with blocks of ZCTA_THREADS / 2
__global__ void zone_kernel_cta(ZoneArgs a);
__global__ void zone_kernel_cta_half(ZoneArgs a);

// angular-slice filter, same arguments and outputs: slice bounds in a
// shared-memory heap (any k), or in registers for k <= 4, 8, 12, 16, 24, 32
__global__ void slice_kernel(ZoneArgs a);
__global__ void slice_kernel_r4(ZoneArgs a);
__global__ void slice_kernel_r8(ZoneArgs a);
__global__ void slice_kernel_r10(ZoneArgs a);
__global__ void slice_kernel_r12(ZoneArgs a);
__global__ void slice_kernel_r16(ZoneArgs a);
__global__ void slice_kernel_r24(ZoneArgs a);
__global__ void slice_kernel_r32(ZoneArgs a);
// the same with two warps per query (blocks of 64 threads)
__global__ void slice_kernel2_r4(ZoneArgs a);
__global__ void slice_kernel2_r8(ZoneArgs a);
__global__ void slice_kernel2_r10(ZoneArgs a);
__global__ void slice_kernel2_r12(ZoneArgs a);
__global__ void slice_kernel2_r16(ZoneArgs a);
__global__ void slice_kernel2_r24(ZoneArgs a);
__global__ void slice_kernel2_r32(ZoneArgs a);

}  // namespace rknn
