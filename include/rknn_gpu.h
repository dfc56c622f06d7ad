/*
 * rknn_gpu.h - C ABI of the GB300 reverse k-nearest-neighbour engine.
 *
 * Plain C types only (no CUDA or C++ types in signatures), so any FFI can
 * bind it.  Every function returns an rknn_status; on failure
 * rknn_last_error() gives a message for the calling thread.  The library
 * never exits the process and has no CPU fallback: when the GPU path cannot
 * run, calls fail with RKNN_ERR_CUDA.
 *
 * Semantics (shared by every entry point): for a query facility q (an index
 * into the facility list, as the reference's `-q`, rknn-inf/inf.cpp:207) and
 * k >= 1, the result is the set of users u with
 *     #{ f != q : d2(u,f) < d2(u,q) } < k,
 * evaluated exactly on the float32 coordinates.  This is rknn-naive's
 * brute-force answer (rknn-naive/rknn.cpp:169-198) with the strict-< tie
 * rule of rknn-inf (rknn-inf/inf.h:77-93) and rknn-naive-gpu
 * (rknn-naive-gpu/rknn_kernel.cu:156).  Result ids are returned sorted
 * ascending.
 *
 * Reference interfaces replaced:
 *   rknn_index_create  - the per-process R*-tree build of every reference
 *                        binary (rknn-inf/inf.cpp:165-177,
 *                        RStarTree2D.cpp:106-114) plus the space bounding box
 *                        (inf.cpp:181-199)
 *   rknn_query         - one `rknn-inf -if F -k K -q Q` run after loading:
 *                        influence-zone filter (inf.cpp:201-585) and
 *                        verification (inf.h:241-249); on the GPU side it
 *                        replaces gpu_get_rknn_candidates
 *                        (rknn-inf-gpu/inf_kernel.h:22-27) and gpuReverseKNN
 *                        (rknn-naive-gpu/rknn_kernel.cuh:40-46)
 *   rknn_query_batch   - many such runs in one launch (no reference
 *                        counterpart; the reference answers one query per
 *                        process)
 */
#ifndef RKNN_GPU_H
#define RKNN_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    RKNN_OK = 0,
    RKNN_ERR_ARG = 1,       /* bad argument (null pointer, k <= 0, q out of range, ...) */
    RKNN_ERR_OOM = 2,       /* device or host allocation failed */
    RKNN_ERR_CUDA = 3,      /* CUDA error (no device, launch failure, ...) */
    RKNN_ERR_TIMEOUT = 4,   /* a bounded wait ran out */
    RKNN_ERR_CAPACITY = 5,  /* output buffer too small; required size returned */
    RKNN_ERR_STATE = 6      /* object in the wrong state for the call */
} rknn_status;

typedef enum {
    RKNN_MODE_FP64 = 0,     /* plain form: predicates filtered in double precision */
    RKNN_MODE_FP32 = 1      /* predicates filtered in float32 with a certified bound */
} rknn_mode;

typedef struct rknn_index rknn_index;

typedef struct {
    int32_t device;         /* CUDA device ordinal (default 0) */
    float fac_per_cell;     /* facilities per facility-grid cell (0: default 2) */
    float usr_per_cell;     /* users per user-grid cell (0: default 8) */
    int32_t skip_coincident;/* 1 (default): a facility at q's exact position adds no
                               bisector (the reference adds a degenerate one) */
    int32_t filter;         /* candidate filter: RKNN_FILTER_AUTO (default), _INF, _SLICE */
    int32_t slice_min_k;    /* AUTO: k classes whose largest k reaches this use the slice
                               filter, smaller ones the influence zone (0: default 1) */
    int32_t users_per_thread;   /* verification: users per lane per work item, 2/4/8 (0: 4) */
    int32_t verify_warps;       /* verification: warps per block, 4/8/16 (0: 8) */
    int32_t zone_vertex_test;   /* influence zone's vertex test (inf.cpp:268-353): 0 (default)
                                   the reference's, over vertices of count k-1 and the eight
                                   extreme space-boundary vertices (it can drop a needed
                                   facility: a superset filter); 1 every vertex of the zone's
                                   boundary: count k-1 and every space-boundary vertex of
                                   count < k (no needed facility dropped).  Results are exact
                                   either way */
    int32_t reserved[1];
} rknn_index_opts;

typedef enum {
    RKNN_FILTER_AUTO = 0,   /* angular slices from slice_min_k on (the faster filter at every
                               k measured), the influence zone below it and for k beyond the
                               slices' shared-memory room (k ~ 1400) */
    RKNN_FILTER_INF = 1,    /* always rknn-inf's influence zone (inf.cpp:201-585); beyond
                               its shared-memory capacity (k ~ 35) the zone is cut short */
    RKNN_FILTER_SLICE = 2   /* always the angular-slice filter (rknn-slice/slice.h) */
} rknn_filter;

typedef struct {
    int64_t queries;
    int64_t results;        /* result ids returned */
    int64_t bisectors;      /* influence-zone bisectors created */
    int64_t zone_vertices_max;
    int64_t zone_candidates;/* bisector intersections considered (slice filter:
                               facilities offered to the slice heaps) */
    int64_t zone_fp64;      /* intersections computed in double precision */
    int64_t candidates;     /* users tested against the half-planes */
    int64_t plane_evals;    /* (user, half-plane) evaluations */
    int64_t survivors;      /* users recounted exactly */
    int64_t fac_checks;     /* (user, facility) comparisons in the exact count */
    int64_t rechecks;       /* comparisons decided by the exact expansion */
    int64_t overflow;       /* queries whose zone hit a capacity (results still exact) */
    double device_ms;       /* device time of the last launch sequence */
    int64_t zone_cycles[8]; /* zone kernel SM cycles by phase, summed over queries: ring
                               expansion, pop + rules, vertex test, vertex count pass,
                               candidate intersections, dedup, counts/erase/append, epilogue.
                               The slice filter fills 0 facility stream, and within it 1
                               slice-bound offers, 3 ring stop tests, 4 cell ranges, 5 facility
                               items (with 1); 2 user-cell ring scan, 7 half-planes and
                               segments, 6 the verification of the query's users when
                               the filter does it (warp 0's share) */
    int64_t zone_points;    /* facilities taken from the zone search's queue */
    int64_t zone_cells;     /* facility grid cells taken from the queue */
    int64_t fused_slots;    /* queries the slice filter verified itself (FP32 batches
                               small enough for two warps a query); the rest went
                               through the verification kernel */
} rknn_query_stats;

void rknn_index_opts_default(rknn_index_opts* opts);

/* Build the device index.  fxy/uxy: interleaved x,y float32 (2*nf, 2*nu);
 * fid/uid: ids (fid may be null).  nf >= 1, nu >= 0. */
rknn_status rknn_index_create(const float* fxy, const int32_t* fid, int64_t nf,
                              const float* uxy, const int32_t* uid, int64_t nu,
                              const rknn_index_opts* opts, rknn_index** out);

rknn_status rknn_index_destroy(rknn_index* idx);

/* Number of facilities / users in the index. */
rknn_status rknn_index_size(const rknn_index* idx, int64_t* nf, int64_t* nu);

/* Binary snapshot of an index's input points: a file that loads in
 * milliseconds where the reference parses text (rknn-inf/inf.cpp:129-161)
 * and builds an R*-tree per process.  Little-endian layout:
 *   "RKNNSNP1", uint32 version (1), uint32 0, int64 nf, int64 nu,
 *   float fxy[2 nf], int32 fid[nf], float uxy[2 nu], int32 uid[nu],
 *   uint64 hash: FNV-1a (64-bit) over the preceding bytes taken as
 *   little-endian 64-bit words, the last one zero-padded.
 * The snapshot functions are host code: they need no GPU. */
rknn_status rknn_snapshot_write(const char* path, const float* fxy, const int32_t* fid, int64_t nf,
                                const float* uxy, const int32_t* uid, int64_t nu);
/* Reads a snapshot into arrays the library allocates (release each with
 * rknn_snapshot_free).  RKNN_ERR_ARG: not a snapshot, truncated, or the
 * hash does not match. */
rknn_status rknn_snapshot_read(const char* path, float** fxy, int32_t** fid, int64_t* nf,
                               float** uxy, int32_t** uid, int64_t* nu);
void rknn_snapshot_free(void* p);
/* rknn_index_create over a snapshot's points. */
rknn_status rknn_index_open(const char* path, const rknn_index_opts* opts, rknn_index** out);
/* Writes the index's input points (facility ids included) as a snapshot. */
rknn_status rknn_index_save(const rknn_index* idx, const char* path);

typedef struct {
    int64_t nf, nu;
    double x0, y0, x1, y1;          /* bounding box of all points: the zone's space */
    float fgrid_x0, fgrid_y0, fgrid_inv;   /* facility grid: cell of v is floor((v-x0)*inv) */
    int32_t fgrid_gx, fgrid_gy;
    float ugrid_x0, ugrid_y0, ugrid_inv;   /* user grid */
    int32_t ugrid_gx, ugrid_gy;
} rknn_index_info;

/* Geometry of the index (for audits against a CPU restatement). */
rknn_status rknn_index_get_info(const rknn_index* idx, rknn_index_info* info);

/* One query, one launch sequence, host buffers.  Writes up to cap ids to
 * out_ids and the result size to *n_out; returns RKNN_ERR_CAPACITY (with
 * *n_out set) when cap is too small.  stats may be null. */
rknn_status rknn_query(rknn_index* idx, int32_t q_index, int32_t k, int32_t mode,
                       int32_t* out_ids, int64_t cap, int64_t* n_out,
                       rknn_query_stats* stats);

/* One query that allocates nothing.  No counterpart in the reference.
 * For callers that cannot allocate device memory at query time (plugins in a
 * host process whose device memory all belongs to that host's own allocator,
 * serving loops that must not stall on cudaMalloc): the per-query scratch lives in a
 * fixed 16 MiB device array that the library holds on every device that
 * loads it, until exit.  Same semantics and outputs as rknn_query, host
 * buffers, synchronous.  Limits: k <= 128 (larger k: RKNN_ERR_CAPACITY) and
 * at most about 2 million candidate users for the query (otherwise
 * RKNN_ERR_CAPACITY; use rknn_query).  The first call on a device looks up
 * the array's device address; make that first call before any stream
 * capture.  Creating an index on a device drops that cached address (after
 * a cudaDeviceReset every index must be created again anyway), so the next
 * call looks it up once more.  All calls share the array: they are
 * serialized by a process-wide lock and leave the GPU idle before
 * returning, on failure too (calls that overlapped on the GPU would race on
 * it).  The index is built beforehand by rknn_index_create. */
rknn_status rknn_query_noalloc(rknn_index* idx, int32_t q_index, int32_t k, int32_t mode,
                               int32_t* out_ids, int64_t cap, int64_t* n_out);

/* nq queries in one launch sequence (CUDA graph), host buffers.  Results of
 * query i are out_ids[offsets[i] .. offsets[i+1]); offsets has nq+1 entries.
 * RKNN_ERR_CAPACITY when cap < offsets[nq] (offsets still filled). */
rknn_status rknn_query_batch(rknn_index* idx, const int32_t* q_index, const int32_t* k,
                             int32_t nq, int32_t mode, int32_t* out_ids, int64_t cap,
                             int64_t* offsets, rknn_query_stats* stats);

/* Page-locked host memory for rknn_query_batch's out_ids (and any other
 * buffer).  The batch call copies result ids straight into a page-locked
 * out_ids, in the same stream round trip as the offsets when the batch
 * returns no more ids than the previous batch plus a quarter plus 4096;
 * pageable buffers go through a staging copy.  No counterpart in the
 * reference (its host arrays are std::vector). */
rknn_status rknn_host_alloc(int64_t bytes, void** out);
rknn_status rknn_host_free(void* p);

/* Device-resident form: q_index/k are device pointers, read by the kernels
 * in place (keep them unchanged until rknn_batch_device_results returns);
 * results stay on the device (see rknn_batch_device_results).  kmax bounds every k[i] (it sizes
 * the zone state; a larger k is still answered exactly, with the zone cut
 * short).  Enqueued on the index's stream; returns without synchronizing.
 * Query indices must be valid (an out-of-range slot yields no results). */
rknn_status rknn_query_batch_device(rknn_index* idx, const int32_t* d_q_index,
                                    const int32_t* d_k, int32_t nq, int32_t kmax, int32_t mode);

/* Device pointers to the last device batch's results: ids and nq+1 int32
 * offsets.  Synchronizes the index's stream; when a query's results outgrew
 * the room the batch gave them, runs the batch again (from the caller's q
 * and k) so that the results are complete.  Valid until the next
 * query call on this index. */
rknn_status rknn_batch_device_results(rknn_index* idx, const int32_t** d_ids,
                                      const int32_t** d_offsets);

/* Wait for the index's stream. */
rknn_status rknn_sync(rknn_index* idx);

/* Use the caller's CUDA stream (a cudaStream_t passed as void*; null resets
 * to the library's own stream). */
rknn_status rknn_set_stream(rknn_index* idx, void* stream);

/* Statistics of the last query call (host or device form). */
rknn_status rknn_last_stats(rknn_index* idx, rknn_query_stats* stats);

/* Per-query zone record of the last call (for audits): bisector count and
 * the facility input indices of the bisectors in creation order. */
rknn_status rknn_last_zone(rknn_index* idx, int32_t slot, int32_t* bis_fac, int32_t cap,
                           int32_t* n_bis, int32_t* flags);

/* Profiling mode (on != 0): the next query calls launch their kernels one
 * by one, with CUDA events between them, instead of replaying a CUDA graph. */
rknn_status rknn_set_profiling(rknn_index* idx, int32_t on);

/* Device time of each kernel of the last profiled call, in milliseconds:
 * ms[0] zone (or slice filter), ms[1] plan, ms[2] verify, ms[3] exact
 * recount of the survivors, ms[4] result offsets, ms[5] finalize.  A stage
 * that the batch does not launch reads about 0: the plan when the slice
 * filter verifies its own queries (FP32 batches of up to about 1200
 * queries; ms[0] then includes that verification), the offsets for
 * batches of up to 4096 queries (finalize computes them, in ms[5]). */
rknn_status rknn_last_kernel_ms(rknn_index* idx, double* ms);

/* ---- Serving: continuous batching over a resident index ----------------
 * No counterpart in the reference (one query per process).  A server keeps
 * the index on the device and runs a worker thread.  Requests queue as they
 * are submitted; whenever one of the server's slots is free, the worker
 * forms a batch from the queue (first come first served, one mode per batch,
 * as many requests as max_batch and the slot's scratch budget admit, the
 * budget charged by each request's scratch estimate from its k) and launches
 * it on the slot's own stream while earlier batches are still running, so
 * the work of several batches overlaps on the GPU.  A request's result does
 * not depend on the batch it ran in. */
typedef struct rknn_server rknn_server;

typedef struct {
    int32_t slots;          /* batches in flight at once (default 3) */
    int32_t max_batch;      /* requests per batch (default 4096) */
    int64_t scratch_bytes;  /* device scratch one batch may use (default 256 MiB) */
    int32_t reserved[8];
} rknn_serve_opts;

typedef struct {
    int64_t submitted, completed, failed;
    int64_t batches;        /* batches launched */
    double mean_batch;      /* requests per batch */
    int32_t max_inflight;   /* most batches on the GPU at once */
    int32_t pad;
    double p50_ms, p99_ms, mean_ms, max_ms;   /* submit -> result ready */
    double throughput_qps;  /* completed / (last completion - first submission) */
} rknn_serve_stats;

void rknn_serve_opts_default(rknn_serve_opts* opts);

/* Start a server over idx (which must outlive it). */
rknn_status rknn_serve_start(rknn_index* idx, const rknn_serve_opts* opts, rknn_server** out);

/* Queue one request; *ticket identifies it in rknn_serve_wait.  Thread-safe.
 * Admission rule: a request whose scratch estimate on its own (a batch of
 * one, padded as batches are) exceeds the server's scratch_bytes is refused
 * with RKNN_ERR_CAPACITY, so no batch passes the budget; other requests are
 * combined first come first served while the batch's estimate fits. */
rknn_status rknn_serve_submit(rknn_server* srv, int32_t q_index, int32_t k, int32_t mode,
                              uint64_t* ticket);

/* Wait up to timeout_ms (< 0: no limit) for a request, then copy its sorted
 * ids and release it.  RKNN_ERR_TIMEOUT: not done yet (call again).
 * RKNN_ERR_CAPACITY: cap too small, *n_out set, request kept.  latency_ms
 * (may be null): submit to result ready.  Thread-safe. */
rknn_status rknn_serve_wait(rknn_server* srv, uint64_t ticket, int32_t timeout_ms,
                            int32_t* out_ids, int64_t cap, int64_t* n_out, double* latency_ms);

/* Open-loop load: submit n requests, request i at arrival_s[i] seconds after
 * the call starts (non-decreasing), wait for all, and write each request's
 * latency (ms) and result size.  Results themselves are dropped. */
rknn_status rknn_serve_replay(rknn_server* srv, int64_t n, const int32_t* q_index,
                              const int32_t* k, const int32_t* mode, const double* arrival_s,
                              double* latency_ms, int64_t* n_results);

/* Counters and latency percentiles of requests completed since the start
 * (or since the last call with reset != 0). */
rknn_status rknn_serve_stats_get(rknn_server* srv, int32_t reset, rknn_serve_stats* stats);

/* Failure test hook (no counterpart in the reference): the next `count`
 * batches the worker launches fail on the host, with no GPU fault involved.
 * kind 1: the batch's workspace allocation fails as a cudaMalloc would
 * (after its old arrays were released), its requests end with RKNN_ERR_OOM;
 * kind 2: the launch fails after the batch's input copy, its requests end
 * with RKNN_ERR_CUDA.  Later batches allocate afresh and run normally. */
rknn_status rknn_serve_inject_fault(rknn_server* srv, int32_t kind, int32_t count);

/* Finish queued and running requests, stop the worker, free the server. */
rknn_status rknn_serve_stop(rknn_server* srv);

/* ---- Autotuning ---------------------------------------------------------
 * No counterpart in the reference.  Times a sample batch (the caller's
 * queries, in the given mode): first every combination of facility-grid
 * density {0.25, 0.5, 1, 2, 4} and user-grid density {1, 2, 4, 8, 16}
 * (points per cell: the grids are rebuilt on the device), then with the best
 * grids every combination of users per lane {2, 4, 8} and warps per block
 * {4, 8, 16} of the verification kernel (34 settings), and leaves the index
 * set to the fastest.  Results never depend on these settings.  Not to be
 * called while a server over the index is running. */
typedef struct {
    float fac_per_cell, usr_per_cell;   /* chosen grid densities */
    int32_t users_per_thread, verify_warps;
    double default_ms;      /* device time of the sample batch with the settings on entry */
    double best_ms;         /* ... with the chosen settings */
    int32_t trials;         /* settings timed */
    int32_t reserved[5];
} rknn_tune_result;

rknn_status rknn_index_tune(rknn_index* idx, const int32_t* q_index, const int32_t* k, int32_t nq,
                            int32_t mode, rknn_tune_result* result);

/* Message of the last failure on this thread ("" if none). */
const char* rknn_last_error(void);

/* Library version string. */
const char* rknn_version(void);

#ifdef __cplusplus
}
#endif
#endif /* RKNN_GPU_H */
