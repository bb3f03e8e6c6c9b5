/*
 * openph.h — C ABI of the GB300-native OpenPH reduction library
 * (libopenph_gb300.so).  Plain pointers and sizes only.
 *
 * The reduction is over Z/2 on a filtered complex's boundary matrix: columns
 * are added left to right until every nonzero column has a distinct low (the
 * row of its last nonzero).  Every algorithm below yields the same low array
 * (the lows of a reduced matrix are unique).  All algorithms run on the GPU;
 * there is no CPU fallback: without a usable CUDA device the calls fail with
 * OPH_ERR_CUDA.
 */
#ifndef OPENPH_GB300_H
#define OPENPH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
enum {
    OPH_OK = 0,
    OPH_ERR_BAD_INPUT = 1,  /* malformed matrix or argument; nothing ran       */
    OPH_ERR_OOM = 2,        /* device memory (or the caller's budget) exhausted */
    OPH_ERR_OVERFLOW = 3,   /* column store could not grow any further          */
    OPH_ERR_TIMEOUT = 4,    /* sweep/iteration cap reached before convergence   */
    OPH_ERR_CUDA = 5,       /* CUDA runtime error (no device, launch failure)   */
    OPH_ERR_ALGO = 6        /* algorithm string not recognised                  */
};

/* algorithm ids; the strings of the reference's dispatch
 * (src/cuda/algorithms/algorithm_factory.cu:10-12, 54-78, 103-148) map to
 * these: "standard", "twist", "ph_row", "standard_parallel", "twist_parallel",
 * "ph_row_parallel", "pms". */
enum {
    OPH_ALGO_STANDARD = 0,
    OPH_ALGO_TWIST = 1,
    OPH_ALGO_PH_ROW = 2,
    OPH_ALGO_STANDARD_PARALLEL = 3,
    OPH_ALGO_TWIST_PARALLEL = 4,
    OPH_ALGO_PH_ROW_PARALLEL = 5,
    OPH_ALGO_PMS = 6
};

/* Returns the algorithm id for a reference algorithm string, or -1. */
int oph_algo_from_string(const char *algstr);
const char *oph_status_string(int status);

/* --------------------------------------------------------- drop-in entry */
/*
 * openph — the reference's C function behind the `ph` MATLAB MEX call,
 * same name, arguments and meaning (replaces src/cuda/openph.cu:29-35, called
 * from src/matlab/ph/ph.cu:71-74).
 *
 *   algstr      one of the seven reference algorithm strings
 *   h_rows_in   int32[nnz], 1-based row of each nonzero
 *   h_cols_in   int32[nnz], 1-based column of each nonzero, non-decreasing;
 *               rows ascending inside a column
 *   m           number of columns (= rows)
 *   col_width   accepted and ignored: column capacity is adaptive, no fixed
 *               slot count is needed
 *   h_low_true  int32[m] 1-based true lows (0 = none) used only by the
 *               progress trackers; may be all zeros or NULL
 *   nnz         number of nonzeros
 *   h_low       out int32[m]: 1-based low of each reduced column, 0 if zero
 *   h_ess       out int32[m]: 1 if the column is estimated essential
 *   err_linf, err_lone, err_redu, err_ess, time_track
 *               out float[m+1] progress trackers (index 0 = initial state,
 *               1..num_iters-1 = after each iteration); each may be NULL
 *   num_iters   out int32[1]
 *   gpu_number  CUDA device ordinal (the reference hard-codes 0 in the MEX)
 *
 * Like the reference, this returns nothing; errors are reported on stderr
 * and leave h_low all zeros.  Use oph_openph for a status code.
 */
void openph(char *algstr, int *h_rows_in, int *h_cols_in, int m, int col_width, int *h_low_true, int nnz,
            int *h_low, int *h_ess, float *err_linf, float *err_lone, float *err_redu, float *err_ess,
            float *time_track, int *num_iters, int gpu_number);

/* openph with a status code (OPH_OK on success). */
int oph_openph(const char *algstr, const int *h_rows_in, const int *h_cols_in, int m, int col_width,
               const int *h_low_true, int nnz, int *h_low, int *h_ess, float *err_linf, float *err_lone,
               float *err_redu, float *err_ess, float *time_track, int *num_iters, int gpu_number);

/* ------------------------------------------------------- context-based API */
typedef struct oph_context oph_context;

typedef struct {
    int32_t num_iters;       /* iterations as the reference counts them        */
    int32_t sweeps;          /* pms sweeps (0 for the sequential variants)     */
    int64_t additions;       /* column additions performed on the device       */
    int64_t slots_moved;     /* sum over additions of |P| + |T| + |T xor P|    */
    int64_t pool_bytes;      /* column-store bytes in use at the end           */
    int32_t regrows;         /* times the column store had to grow             */
    float device_ms;         /* device time of the reduction (CUDA events)     */
    int32_t dual;            /* 1 when pms reduced the anti-transpose, 2 when
                                some blocks of D were reduced on D' and the
                                others on D                                   */
} oph_info;

/* A context owns one CUDA stream on one device plus cached device buffers;
 * calls on one context are serialised on its stream, distinct contexts may be
 * used from distinct host threads.  No global device symbols are used. */
int oph_context_create(int device, oph_context **out);
int oph_context_destroy(oph_context *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order work. */
void *oph_context_stream(oph_context *ctx);
/* Cap on device bytes the context may hold (0 = no cap). */
int oph_context_set_budget(oph_context *ctx, int64_t bytes);

/*
 * oph_reduce — reduce one boundary matrix given as host 0-based CSC.
 *   colptr int64[m+1], rows int32[colptr[m]] (ascending inside each column)
 *   low    out int32[m], 0-based, -1 = zero or cleared column
 *   ess    out int32[m] (may be NULL)
 *   arglow out int32[m], arglow[i] = column whose low is i, or -1 (may be NULL)
 */
int oph_reduce(oph_context *ctx, int algo, int64_t m, const int64_t *colptr, const int32_t *rows, int32_t *low,
               int32_t *ess, int32_t *arglow, oph_info *info);

/*
 * oph_reduce_device — the same on device-resident buffers, asynchronously on
 * the context's stream except for the host reads of the convergence flag.
 * d_colptr/d_rows/d_low/d_ess/d_arglow are device pointers (d_ess and
 * d_arglow may be NULL).
 */
int oph_reduce_device(oph_context *ctx, int algo, int64_t m, const int64_t *d_colptr, const int32_t *d_rows,
                      int32_t *d_low, int32_t *d_ess, int32_t *d_arglow, oph_info *info);

/*
 * oph_reduce_batch — reduce `count` independent matrices in one pass over a
 * segmented store.  Instance b owns columns [col_off[b], col_off[b+1]) of the
 * concatenation; colptr (int64[col_off[count]+1]) indexes the concatenated
 * rows, and each instance's row indices are LOCAL (0-based within the
 * instance).  low/ess are concatenated per-instance local outputs.
 * Host buffers; ess may be NULL.
 */
int oph_reduce_batch(oph_context *ctx, int algo, int32_t count, const int64_t *col_off, const int64_t *colptr,
                     const int32_t *rows, int32_t *low, int32_t *ess, oph_info *info);

/* the same on device buffers (asynchronous on the context's stream) */
int oph_reduce_batch_device(oph_context *ctx, int algo, int32_t count, const int64_t *d_col_off,
                            const int64_t *d_colptr, const int32_t *d_rows, int64_t total_m, int64_t total_nnz,
                            int32_t *d_low, int32_t *d_ess, oph_info *info);

/* ---------------------------------------------------------------- serving */
/*
 * A reduction server with continuous batching: requests are reduced by a
 * worker thread that advances every admitted request with each pms sweep over
 * one block-diagonal column space, admits queued requests between sweeps
 * while they fit in the device arena (budget_bytes of HBM, allocated up
 * front), and releases each request as soon as it has converged.  At most
 * max_active requests are on the device at once.  Each request is reduced on
 * the matrix a single-matrix pms reduction would choose for it (OPH_DUAL_AUTO
 * below: a Rips-like request through its anti-transpose, built at
 * admission; a request split by block as two parts side by side, the D part
 * joining after the D' part's first sweep), and the results are identical to
 * that reduction's.  A chain of additions in the bitmap tiers stops after 128
 * additions a sweep (environment variable OPH_SERVE_CHAIN_CAP, read at
 * creation; 0 for no limit) and goes on in the next sweep, so no sweep of
 * every active request waits on one long chain.
 */
typedef struct oph_server oph_server;

typedef struct {
    double latency_ms;   /* submit -> result on the host          */
    double queue_ms;     /* submit -> admitted to the device        */
    double submit_ms;    /* host monotonic clock at submit (ms)     */
    double done_ms;      /* host monotonic clock at completion (ms) */
    int32_t sweeps;      /* sweeps the request took part in         */
    int32_t status;      /* OPH_OK or the failure                   */
    int64_t m;
} oph_request_info;

typedef struct {
    int64_t completed, pending, active, sweeps, regrows;
    int64_t pool_bytes_in_use, columns_in_use, arena_bytes;
    int64_t dual_admitted;  /* requests with a part reduced through their
                               anti-transpose (split by block or whole)   */
} oph_server_counters;

int oph_server_create(int device, int64_t budget_bytes, int32_t max_active, oph_server **out);
/* Queue a 0-based CSC matrix; returns a ticket.  The matrix is copied to
 * the device (the caller may free its buffers on return) and checked and
 * graded there, so the submitting thread does no per-entry work.
 * OPH_ERR_OOM if it can never fit the arena, OPH_ERR_BAD_INPUT if
 * malformed.  Queued copies live outside the arena until admission. */
int oph_server_submit(oph_server *srv, int64_t m, const int64_t *colptr, const int32_t *rows, int64_t *ticket);
/* The same for a 0-based CSC already in device memory on the server's device
 * (d_colptr[m + 1] with d_colptr[0] == 0, d_rows[nnz]): the server copies it
 * device to device and checks it there before returning (the caller's
 * buffers may be freed then), and its admission reads that copy in place —
 * no host copy and no host-to-device transfer of the input.  Pairs with
 * oph_rips_device / oph_lower_star_device.  No counterpart in the reference. */
int oph_server_submit_device(oph_server *srv, int64_t m, const int64_t *d_colptr, const int32_t *d_rows,
                             int64_t *ticket);
/* Wait for a ticket (timeout_ms < 0: forever); copies low/ess (0-based,
 * -1 = none; either may be NULL) and frees the ticket. */
int oph_server_wait(oph_server *srv, int64_t ticket, int32_t *low, int32_t *ess, oph_request_info *info,
                    int64_t timeout_ms);
int oph_server_stats(oph_server *srv, oph_server_counters *out);
/* Finishes the queued requests, stops the worker, frees the arena. */
int oph_server_destroy(oph_server *srv);

/* ------------------------------------------------------------ diagnostics */
typedef struct {
    float phase2_narrow_ms;   /* Phase II narrow-tier kernel, summed over launches */
    float phase2_wide_ms;     /* Phase II wide + global tiers                      */
    float phase1_ms;          /* Phase I kernels                                   */
    float setup_ms;           /* store set-up, alpha/beta, Phase 0                 */
    int32_t phase2_launches;  /* narrow-tier launches that did work                */
    int32_t kernel_launches;  /* every kernel launched by the last reduction       */
    int64_t tier_additions[4];/* column additions done by each Phase II tier       */
    int64_t tier_slots[4];    /* sum of |P| + |T| + |T xor P| per tier (tiers 0-1:
                                 only with OPH_PROFILE_SLOTS)                      */
    float tier_ms[3];         /* tiers 1, 2 and 3 apart (their sum is
                                 phase2_wide_ms)                                   */
} oph_profile;

#define OPH_PROFILE_EVENTS 1  /* per-phase CUDA-event timing                     */
#define OPH_PROFILE_SLOTS 2   /* exact |T| tracking in the lazy tiers 0 and 1,   */
                              /* for tier_slots (slower: not for timed runs)     */
/* Select profiling for later reductions on ctx: an OR of OPH_PROFILE_*
 * (0, the default, turns it off). */
int oph_context_set_profile(oph_context *ctx, int on);
/* Per-phase device times and launch counts of the last reduction on ctx. */
int oph_last_profile(oph_context *ctx, oph_profile *out);

/*
 * oph_reduce_pms_noalloc — pms on device buffers WITHOUT allocating any
 * device memory.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc — a host framework whose caching allocator owns the
 * GPU's memory (MATLAB GPU arrays, PyTorch), or a real-time pipeline that
 * cannot afford cudaMalloc's implicit synchronisation.  Every working array
 * comes from one fixed 32 MiB device array inside the library, held by every
 * GPU that loads it until exit; a matrix whose working set does not fit
 * (roughly 200,000 columns of a 2-complex) is rejected with OPH_ERR_OOM, and
 * a column store that would have to grow returns OPH_ERR_OVERFLOW (use
 * oph_reduce_device for those).  A malformed CSC is rejected with
 * OPH_ERR_BAD_INPUT before anything is written.
 * d_colptr (int64[m+1]) and d_rows are the 0-based CSC on the device; d_low
 * and d_ess (may be NULL) receive 0-based lows (-1 = none) and the essential
 * flags, as oph_reduce_device produces them.  `stream` is a cudaStream_t
 * (NULL = the legacy default stream).  The call is synchronous (it returns
 * when the results are in place, and reads sizes and status back to the
 * host), so it must not be issued on a stream under capture.  The first call
 * on a device looks up the array's address (cudaGetSymbolAddress) and keeps
 * it for the process: not for use after a cudaDeviceReset.  All calls share
 * the array: calls that overlap on the GPU race, so serialise them.
 */
int oph_reduce_pms_noalloc(int64_t m, const int64_t *d_colptr, const int32_t *d_rows, int32_t *d_low,
                           int32_t *d_ess, void *stream);

/* Autotuning of the pms Phase II narrow tier (lanes per column and shared
 * staging capacity).  oph_context_autotune reduces the given host CSC matrix
 * once per candidate (after one warm-up) and keeps the fastest for later
 * reductions on ctx; oph_context_autotune_batch does the same on a batch.
 * lanes/cap/best_ms receive the choice (each may be NULL). */
int oph_context_autotune(oph_context *ctx, int64_t m, const int64_t *colptr, const int32_t *rows, int32_t *lanes,
                         int32_t *cap, float *best_ms);
int oph_context_autotune_batch(oph_context *ctx, int32_t count, const int64_t *col_off, const int64_t *colptr,
                               const int32_t *rows, int32_t *lanes, int32_t *cap, float *best_ms);
/* Set the narrow-tier configuration directly (must be a candidate). */
int oph_context_set_tier0(oph_context *ctx, int32_t lanes, int32_t cap);

/* Which matrix pms reduces (no counterpart in the reference, whose pms
 * always reduces D).  The low pairs of D and of its anti-transpose D'
 * (entry (i, j) of D at (m-1-j, m-1-i)) determine each other, so reducing
 * D' gives the same low and ess; it moves the work from the top dimension,
 * which twist and pms on D must reduce column by column, to the bottom one.
 *   OPH_DUAL_AUTO    D' when the input is graded (every column's rows from
 *                    one dimension bucket, distinct buckets from distinct
 *                    ones), has at least 2^17 columns and its top bucket
 *                    holds at least 8 times the columns of the bottom one
 *                    (Rips complexes); else, from 2^17 columns, a choice
 *                    per block (one dimension's columns with their rows,
 *                    which reduce independently of the others): D' for a
 *                    block whose row simplices have at most two cofaces on
 *                    average (the triangles of a triangulated surface, as in
 *                    lower-star images), D for the others; else D
 *   OPH_DUAL_NEVER   always D
 *   OPH_DUAL_ALWAYS  D' whenever the input is graded
 *   OPH_DUAL_BLOCKS  the per-block choice at any size
 * Reductions with per-sweep trackers (oph_openph with tracker outputs)
 * always reduce D, whose progress the trackers describe.  Default AUTO. */
#define OPH_DUAL_AUTO 0
#define OPH_DUAL_NEVER 1
#define OPH_DUAL_ALWAYS 2
#define OPH_DUAL_BLOCKS 3
int oph_context_set_dual(oph_context *ctx, int32_t mode);

/* Testing hooks: cap the sweep count (0 = default) and the initial column
 * store size in bytes (0 = default), to exercise the timeout and regrow
 * paths without faulting anything. */
int oph_context_set_limits(oph_context *ctx, int32_t max_sweeps, int64_t initial_pool_bytes);

/* ------------------------------------------------- complexes on the device
 * The reference reads boundary matrices produced on the host by Javaplex
 * (example_factory.m:17-114, stream2cmo.m:1-26); no counterpart in its C
 * code.  These build the filtered complex straight into device buffers, in
 * the reduction's input layout (0-based CSC, columns in filtration order
 * (value, dimension, vertex tuple), rows ascending), identical to the host
 * generators of openph_gb300 (gen/ophgen.c: oph_rips, oph_lower_star).
 * Call once with d_colptr == NULL for the sizes (*m, *nnz), allocate
 * d_colptr[m + 1], d_rows[nnz] and optionally d_value[m] (FP64 filtration
 * values), then call again with them.  Work runs on the context's stream and
 * is complete on return; scratch is allocated from the stream's memory pool
 * and released before returning. */
#define OPH_GEN_MAX_POINTS 16384
/* Vietoris-Rips complex of dimension <= 2 of n points (d_points: n x d FP64,
 * row-major, on the device) with edges of length <= threshold (+inf: the
 * full 2-skeleton); value = the largest pairwise Euclidean distance. */
int oph_rips_device(oph_context *ctx, const double *d_points, int n, int d, double threshold, int64_t *m,
                    int64_t *nnz, int64_t *d_colptr, int32_t *d_rows, double *d_value);
/* Lower-star filtration of an h x w FP32 image (row-major, on the device) on
 * the Freudenthal triangulation (diagonals (y,x)-(y+1,x+1)); value of a
 * simplex = the largest value of its vertices.  h, w >= 2, h * w < 2^20. */
int oph_lower_star_device(oph_context *ctx, const float *d_image, int h, int w, int64_t *m, int64_t *nnz,
                          int64_t *d_colptr, int32_t *d_rows, double *d_value);

#ifdef __cplusplus
}
#endif

#endif /* OPENPH_GB300_H */
