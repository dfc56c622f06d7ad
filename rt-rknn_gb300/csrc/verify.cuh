// Verification kernels: half-plane filter, exact recount, result finalize.
#pragma once
#include "rknn_common.cuh"

namespace rknn {

constexpr int VERIFY_UPT = 4;                       // default users per lane per work item
constexpr int VERIFY_CHUNK = 32 * VERIFY_UPT;       // default users per work item
constexpr int VERIFY_WARPS = 8;                     // default warps per block
constexpr int VERIFY_SAMPLES = 4096;                // work-item offsets cached per block
constexpr int FIN_WARPS = 8;                        // finalize: slots per block (one warp each)
constexpr int FIN_WCAP = 512;                       // ids one warp sorts in registers

enum { MODE_FP64 = 0, MODE_FP32 = 1 };

struct VerifyArgs {
    const QDesc* qd;
    const float4* planes;    // [slot][lc] float half-planes relative to q
    const int* bis_pos;      // [slot][lc] facility positions (FP64 planes are rebuilt from these)
    int lc;                  // row stride of planes / bis_pos
    int stage_cap;           // half-planes staged per warp (the filter uses the first ones;
                             // fewer only means more users reach the exact recount)
    const int2* segs;        // [slot][seg_cap]
    int seg_cap;
    int seg_stage = 0;       // user segments staged per warp beside the half-planes
                             // (a slot with more reads them from global memory)
    const int* chunk_off;    // [nq+1]
    const long long* cand_off;   // [nq] start of each slot's result region in res_pool
    const int* reg_len;          // [nq] its length (ids the slot stores at most)
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
    int* dropped;            // set when a slot had more results than its region
    const float* slice_r;    // [slot][32] slice bounds (queries flagged QF_SLICE_R)
    int2* surv;              // survivors of the half-plane filter: (slot, user position)
    int surv_cap;            // 0: no list (the verification kernel recounts in-warp)
    int* surv_count;
    int* fault;              // checked builds: {flag, array id, index, size, line}
    // slots to verify: chunk_off indexes deflist[0 .. *ndef) when deflist is
    // set (the fused slice filter verified the others), else slots 0 .. nq
    const int* deflist = nullptr;
    const int* ndef = nullptr;
    long long* region_top = nullptr;   // total of the result regions (fused claims)
    int* done = nullptr;               // fused filter: its blocks finished
};

__global__ void verify_kernel(VerifyArgs a);        // 4 users per lane per work item
__global__ void verify_kernel_u2(VerifyArgs a);     // 2
__global__ void verify_kernel_u8(VerifyArgs a);     // 8

// exact recount of the listed survivors, one thread each
__global__ void recount_kernel(VerifyArgs a);

// single block: result regions (min(candidates, rcap) ids at 64-bit offsets,
// their lengths and *region_top = their total) and work-item offsets from
// QDesc.ncand; flags slots whose region does not fit the pool
__global__ void plan_kernel(QDesc* qd, int nq, long long* cand_off, int* reg_len, long long* region_top,
                            int* chunk_off, long long pool_cap, int rcap, int chunk);

// single block: exclusive scan of the stored result counts into out_off
// out_off: nq+1 offsets, then OFF_TAIL ints: the region total (low and high
// halves of *region_top), the dropped flag and the listed survivors
// (counters[2], counters[3]), so that one copy brings back all of them.
constexpr int OFF_TAIL = 4;
// out_off_host (or null): device-accessible host memory that receives a
// copy of the same nq+1+OFF_TAIL ints.
__global__ void scan_counts_kernel(const int* res_count, const int* reg_len, const long long* region_top, int nq,
                                   int* out_off, const int* counters, int* out_off_host);

// Output offsets computed by finalize_kernel itself (batches of up to
// FIN_SCAN_MAX slots, which then need no scan_counts_kernel): each block sums
// the stored ids of the slots before its own, writes its slots' offsets to
// out_off (and out_off_host) and the last block the total and the run's
// flags, as scan_counts_kernel does.
constexpr int FIN_SCAN_MAX = 4096;
struct FinScan {
    int on = 0;
    int* out_off_host = nullptr;
    const long long* region_top = nullptr;
    const int* counters = nullptr;
};

// one block per slot: sort the slot's results into out[out_off[s] ...]
// out may be device-accessible host memory of out_cap ids: a slot whose range
// would pass out_cap is left out (the caller sees the total and fails the
// batch).  zero[0 .. zero_n) (another batch's counters, unused by this one)
// is cleared for the next batch.
__global__ void finalize_kernel(int* res_pool, const long long* cand_off, const int* reg_len, const int* res_count,
                                int* out_off, int* out, int nq, long long out_cap, int* zero,
                                long long zero_n, FinScan S);

}  // namespace rknn
