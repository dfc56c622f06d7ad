// Verification kernels: half-plane filter, exact recount, result finalize.
#pragma once
#include "rknn_common.cuh"

namespace rknn {

constexpr int VERIFY_UPT = 4;                       // users per lane per chunk
constexpr int VERIFY_CHUNK = 32 * VERIFY_UPT;       // users per work item
constexpr int VERIFY_WARPS = 8;                     // warps per block
constexpr int SORT_CAP = 16384;                     // results sorted in shared memory

enum { MODE_FP64 = 0, MODE_FP32 = 1 };

struct VerifyArgs {
    const QDesc* qd;
    const float4* planes;    // [slot][lc] float half-planes relative to q
    const int* bis_pos;      // [slot][lc] facility positions (FP64 planes are rebuilt from these)
    int lc;
    const int2* segs;        // [slot][seg_cap]
    int seg_cap;
    const int* chunk_off;    // [nq+1]
    const int* cand_off;     // [nq+1] result region of each slot
    int nq;
    const float2* uxy;       // cell-sorted users
    const int* uid;          // their ids
    const float2* fxy;       // cell-sorted facilities
    const int* fstart;
    Grid gf;
    int* res_count;          // [nq]
    int* res_pool;           // results, region per slot
    int* work_counter;
    VStats* vstats;
    int mode;
    int nu, nf, ncf;         // array sizes (bounds-checked builds)
    long long pool_cap;
    int* fault;              // checked builds: {flag, array id, index, size, line}
};

__global__ void verify_kernel(VerifyArgs a);

// single block: cand_off / chunk_off from QDesc.ncand; flags slots whose
// region does not fit the pool
__global__ void plan_kernel(QDesc* qd, int nq, int* cand_off, int* chunk_off, int pool_cap);

// single block: exclusive scan of res_count into out_off
__global__ void scan_counts_kernel(const int* res_count, int nq, int* out_off);

// one block per slot: sort the slot's results into out[out_off[s] ...]
__global__ void finalize_kernel(int* res_pool, const int* cand_off, const int* res_count,
                                const int* out_off, int* out, int nq);

}  // namespace rknn
