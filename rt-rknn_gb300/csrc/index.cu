// Uniform-grid index: cell id per point, stable LSD radix sort on the cell
// id (8-bit digits), cell start offsets and per-cell facility MBRs.  It
// replaces the reference's per-process R*-tree (rknn-inf/RStarTree2D.cpp,
// insert 106-114): the zone kernel treats grid cells as leaf nodes and the
// verification reads each grid row of cells as one contiguous range.
#include "index.cuh"
#include <climits>
#include <vector>

namespace rknn {

namespace {
constexpr unsigned FULL = 0xffffffffu;
constexpr int RS_THREADS = 256;
constexpr int RS_TILE = 2048;          // items per tile (8 sub-tiles of 256)

__global__ void k_cell_ids(const float2* xy, int n, Grid g, uint32_t* keys, uint32_t* vals)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 p = xy[i];
    int cx = cell_coord(p.x, g.x0, g.inv, g.gx);
    int cy = cell_coord(p.y, g.y0, g.inv, g.gy);
    keys[i] = (uint32_t)(cy * g.gx + cx);
    vals[i] = (uint32_t)i;
}

__global__ void k_rs_hist(const uint32_t* keys, int n, int shift, uint32_t* hist, int ntiles)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
    for (int i = threadIdx.x; i < RS_TILE; i += RS_THREADS) {
        int idx = base + i;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// stable scatter of one tile: sub-tiles in order, warps in order, lanes in order
__global__ void k_rs_scatter(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                             int n, int shift, const uint32_t* offs, int ntiles)
{
    __shared__ uint32_t run[256];
    __shared__ uint32_t wc[RS_THREADS / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    run[tid] = offs[tid * ntiles + blockIdx.x];
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
    for (int sub = 0; sub < RS_TILE; sub += RS_THREADS) {
        int idx = base + sub + tid;
        bool ok = idx < n;
        uint32_t key = ok ? kin[idx] : 0u, val = ok ? vin[idx] : 0u;
        uint32_t dg = ok ? (key >> shift) & 255 : 256u;
        unsigned mm = __match_any_sync(FULL, dg);
        int rank = __popc(mm & ((1u << lane) - 1));
#pragma unroll
        for (int j = 0; j < 8; ++j) wc[w][lane * 8 + j] = 0;
        __syncwarp();
        if (ok && rank == 0) wc[w][dg] = __popc(mm);
        __syncthreads();
        {
            uint32_t acc = run[tid];
#pragma unroll
            for (int j = 0; j < RS_THREADS / 32; ++j) { uint32_t c = wc[j][tid]; wc[j][tid] = acc; acc += c; }
            run[tid] = acc;
        }
        __syncthreads();
        if (ok) {
            uint32_t p = wc[w][dg] + rank;
            kout[p] = key;
            vout[p] = val;
        }
        __syncthreads();
    }
}

// exclusive scan, 1024 items per block, block totals to sums
__global__ void k_scan_block(const uint32_t* in, uint32_t* out, int n, uint32_t* sums)
{
    __shared__ uint32_t ws[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    int i = blockIdx.x * 1024 + tid;
    uint32_t v = i < n ? in[i] : 0u, x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(FULL, t, o);
            if (lane >= o) t += y;
        }
        ws[lane] = t;
    }
    __syncthreads();
    uint32_t excl = x - v + (w ? ws[w - 1] : 0u);
    if (i < n) out[i] = excl;
    if (tid == 1023 && sums) sums[blockIdx.x] = ws[31];
}

__global__ void k_scan_add(uint32_t* out, int n, const uint32_t* sums)
{
    int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n && blockIdx.x > 0) out[i] += sums[blockIdx.x];
}

__global__ void k_count(const uint32_t* keys, int n, uint32_t* counts)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&counts[keys[i]], 1u);
}

__global__ void k_gather(const float2* xy, const int* ids, const uint32_t* vals, int n,
                         float2* xy_s, int* ids_s, int* idx_s, int* pos_of)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t src = vals[i];
    xy_s[i] = xy[src];
    if (ids_s) ids_s[i] = ids ? ids[src] : (int)src;
    if (idx_s) idx_s[i] = (int)src;
    if (pos_of) pos_of[src] = i;
}

__global__ void k_mbr(const float2* xy, const int* start, int nc, float4* mbr)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    float4 r = make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
    for (int i = start[c]; i < start[c + 1]; ++i) {
        float2 p = xy[i];
        r.x = fminf(r.x, p.x); r.y = fminf(r.y, p.y);
        r.z = fmaxf(r.z, p.x); r.w = fmaxf(r.w, p.y);
    }
    mbr[c] = r;
}

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }
}  // namespace

cudaError_t scan_exclusive_u32(const uint32_t* in, uint32_t* out, int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    int nb = nblk(n, 1024);
    uint32_t* sums = nullptr;
    cudaError_t e = cudaSuccess;
    if (nb > 1) {
        e = cudaMallocAsync(&sums, sizeof(uint32_t) * nb, st);
        if (e != cudaSuccess) return e;
    }
    k_scan_block<<<nb, 1024, 0, st>>>(in, out, n, sums);
    if (nb > 1) {
        e = scan_exclusive_u32(sums, sums, nb, st);
        if (e == cudaSuccess) k_scan_add<<<nb, 1024, 0, st>>>(out, n, sums);
        cudaFreeAsync(sums, st);
    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t radix_sort_pairs(uint32_t*& keys, uint32_t*& vals, uint32_t*& tkeys, uint32_t*& tvals,
                             int n, int key_bits, cudaStream_t st)
{
    if (n <= 1) return cudaSuccess;
    const int ntiles = nblk(n, RS_TILE);
    uint32_t* hist = nullptr;
    cudaError_t e = cudaMallocAsync(&hist, sizeof(uint32_t) * 256 * (size_t)ntiles, st);
    if (e != cudaSuccess) return e;
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_rs_hist<<<ntiles, RS_THREADS, 0, st>>>(keys, n, shift, hist, ntiles);
        e = scan_exclusive_u32(hist, hist, 256 * ntiles, st);
        if (e != cudaSuccess) break;
        k_rs_scatter<<<ntiles, RS_THREADS, 0, st>>>(keys, vals, tkeys, tvals, n, shift, hist, ntiles);
        std::swap(keys, tkeys);
        std::swap(vals, tvals);
    }
    cudaFreeAsync(hist, st);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

// Sort n points into g's cells.  Outputs (device, caller-allocated):
// xy_s[n], ids_s[n] (may be null), idx_s[n] (may be null), pos_of[n] (may be
// null), start[nc+1].
cudaError_t grid_sort(const float2* d_xy, const int* d_ids, int n, const Grid& g,
                      float2* xy_s, int* ids_s, int* idx_s, int* pos_of, int* start,
                      cudaStream_t st)
{
    const int nc = g.gx * g.gy;
    cudaError_t e;
    uint32_t *k = nullptr, *v = nullptr, *tk = nullptr, *tv = nullptr, *cnt = nullptr;
    size_t bytes = sizeof(uint32_t) * (size_t)(n > 0 ? n : 1);
    if ((e = cudaMallocAsync(&k, bytes, st)) != cudaSuccess) return e;
    if ((e = cudaMallocAsync(&v, bytes, st)) != cudaSuccess) return e;
    if ((e = cudaMallocAsync(&tk, bytes, st)) != cudaSuccess) return e;
    if ((e = cudaMallocAsync(&tv, bytes, st)) != cudaSuccess) return e;
    if ((e = cudaMallocAsync(&cnt, sizeof(uint32_t) * (size_t)(nc + 1), st)) != cudaSuccess) return e;
    if (n > 0) k_cell_ids<<<nblk(n, 256), 256, 0, st>>>(d_xy, n, g, k, v);
    int bits = 0;
    while ((1ll << bits) < (long long)nc) ++bits;
    bits = ((bits + 7) / 8) * 8;
    e = radix_sort_pairs(k, v, tk, tv, n, bits, st);
    if (e == cudaSuccess) {
        cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (size_t)(nc + 1), st);
        if (n > 0) k_count<<<nblk(n, 256), 256, 0, st>>>(k, n, cnt);
        e = scan_exclusive_u32(cnt, (uint32_t*)start, nc + 1, st);
    }
    if (e == cudaSuccess && n > 0)
        k_gather<<<nblk(n, 256), 256, 0, st>>>(d_xy, d_ids, v, n, xy_s, ids_s, idx_s, pos_of);
    cudaFreeAsync(k, st);
    cudaFreeAsync(v, st);
    cudaFreeAsync(tk, st);
    cudaFreeAsync(tv, st);
    cudaFreeAsync(cnt, st);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t cell_mbrs(const float2* xy_s, const int* start, const Grid& g, float4* mbr, cudaStream_t st)
{
    int nc = g.gx * g.gy;
    k_mbr<<<nblk(nc, 256), 256, 0, st>>>(xy_s, start, nc, mbr);
    return cudaGetLastError();
}

// Grid over [x0,x1]x[y0,y1] with about `per_cell` points per cell.
Grid make_grid(double x0, double y0, double x1, double y1, long long n, double per_cell, int max_side)
{
    Grid g;
    double w = x1 - x0, h = y1 - y0;
    double ext = w > h ? w : h;
    if (!(ext > 0)) ext = 1.0;
    double ww = w > 0 ? w : ext * 1e-3, hh = h > 0 ? h : ext * 1e-3;
    double cs = n > 0 ? sqrt(ww * hh * per_cell / (double)n) : ext;
    if (!(cs > 0)) cs = ext;
    if (ext / cs > max_side) cs = ext / max_side;
    float inv = (float)(1.0 / cs);
    g.x0 = (float)x0;
    g.y0 = (float)y0;
    g.inv = inv;
    g.cs = (float)(1.0 / (double)inv);
    // cells needed so that every coordinate maps inside without clamping
    g.gx = (int)floorf(((float)x1 - g.x0) * inv) + 1;
    g.gy = (int)floorf(((float)y1 - g.y0) * inv) + 1;
    if (g.gx < 1) g.gx = 1;
    if (g.gy < 1) g.gy = 1;
    return g;
}

}  // namespace rknn
