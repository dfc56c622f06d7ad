// Grid index construction (device).
#pragma once
#include "rknn_common.cuh"

namespace rknn {

Grid make_grid(double x0, double y0, double x1, double y1, long long n, double per_cell, int max_side);

cudaError_t scan_exclusive_u32(const uint32_t* in, uint32_t* out, int n, cudaStream_t st);

cudaError_t radix_sort_pairs(uint32_t*& keys, uint32_t*& vals, uint32_t*& tkeys, uint32_t*& tvals,
                             int n, int key_bits, cudaStream_t st);

cudaError_t grid_sort(const float2* d_xy, const int* d_ids, int n, const Grid& g,
                      float2* xy_s, int* ids_s, int* idx_s, int* pos_of, int* start,
                      cudaStream_t st);

cudaError_t cell_mbrs(const float2* xy_s, const int* start, const Grid& g, float4* mbr, cudaStream_t st);

}  // namespace rknn
