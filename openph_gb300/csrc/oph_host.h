// Host-side internals shared by the translation units of libopenph_gb300.
#pragma once
#include <vector>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "openph.h"
#include "oph_device.cuh"

#define OPH_CUDA_TRY(expr)                                                                         \
    do {                                                                                           \
        cudaError_t _e = (expr);                                                                   \
        if (_e != cudaSuccess) {                                                                   \
            fprintf(stderr, "openph_gb300: %s failed: %s (%s:%d)\n", #expr, cudaGetErrorString(_e), \
                    __FILE__, __LINE__);                                                           \
            return OPH_ERR_CUDA;                                                                   \
        }                                                                                          \
    } while (0)

namespace oph {

// A grow-only device buffer owned by a context.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

// Device views of one reduction's working state (single matrix or a
// block-diagonal batch).  All indices are global column ids; a batch instance
// b owns columns [inst_off[b], inst_off[b+1]) and its rows are shifted into
// that range, so the batch is one block-diagonal boundary matrix.
struct Work {
    int64_t m = 0, nnz = 0;
    const int64_t *colptr = nullptr;  // m+1
    const int32_t *rows = nullptr;    // nnz (global row ids)
    int32_t *low = nullptr;           // m
    int8_t *classes = nullptr;        // m: 0 unknown, -1 pivot (negative), 1 cleared (positive)
    uint8_t *clear = nullptr;         // m: row marked for clearing
    int8_t *dim = nullptr;            // m: nnz(col) - 1, the reference's "dimension"
    int32_t *first = nullptr;         // m: first column (in order) holding each low
    int32_t *beta = nullptr;          // m
    int32_t *worklist = nullptr;      // m
    int32_t *widelist = nullptr;      // m
    int64_t *seg = nullptr;           // m: segment of each column
    PivRec *rec = nullptr;            // m: per-row pivot records (left[] inside)
    int32_t *agg = nullptr;           // tiles * MAXC (tile maxima, then exclusive prefixes)
    int64_t ntiles = 0;
    int *pool = nullptr;              // column store
    DevStatus *st = nullptr;
    bool ascending = false;           // pms: buckets in ascending order (the anti-transpose)
    bool checked = false;             // colptr/rows already passed the structural check
    const uint8_t *preclear = nullptr;  // pms: columns cleared before Phase 0 (m bytes), or none
    const int64_t *inst_off = nullptr;  // a batch: its instances' column offsets (device, inst_count + 1)
    int inst_count = 0;
};

struct Context;

// setup.cu
// init_store: the column store (pool) and a fresh status block for w;
// setup_store: init_store, then the columns of w's CSC into the store, low,
// dim, and with need_beta the pivot records, left[] and beta.
int init_store(Context *ctx, Work &w);
int setup_store(Context *ctx, Work &w, bool need_beta);
int coo1_to_csc(Context *ctx, const int *d_rows1, const int *d_cols1, int64_t nnz, int64_t m, int64_t *d_colptr,
                int32_t *d_rows0);
// Structural check of a device CSC (k_check_csc), synchronous: OPH_OK or
// OPH_ERR_BAD_INPUT.  With d_inst_off, rows are local to their instance, and
// d_rows_out (if set) receives them shifted into the instance's columns.
int check_csc(Context *ctx, const int64_t *d_colptr, const int32_t *d_rows, int64_t m, int64_t nnz,
              const int64_t *d_inst_off = nullptr, int count = 0, int32_t *d_rows_out = nullptr);
int grow_pool(Context *ctx, Work &w);

// pms.cu
int run_pms(Context *ctx, Work &w, oph_info *info);

// variants.cu
int run_sequential(Context *ctx, Work &w, int algo, int32_t *d_ess, oph_info *info);

// dual.cu: pms on the anti-transpose.  dual_choose grades w's buckets and
// decides (*bad_input: malformed CSC); dual_setup builds the anti-transpose
// of w straight into wd's column store (wd shares w's per-column arrays),
// with D's buckets reversed, left[], beta and the pivot records; dual_lows
// maps wd's lows back to D's.
// The automatic choice: D' for matrices of at least DUAL_MIN_M columns whose
// top bucket holds DUAL_RATIO times the bottom one's columns (below that
// size the few more sweeps and the transpose cost more than D's additions);
// else, at that size, a choice per block (a bucket's columns with their
// rows): D' for the blocks whose row simplices have at most two cofaces on
// average, D for the others (DUAL_CHOICE_SPLIT when both occur).
constexpr unsigned long long DUAL_RATIO = 8;
constexpr int64_t DUAL_MIN_M = 1 << 17;
enum { DUAL_CHOICE_D = 0, DUAL_CHOICE_DUAL = 1, DUAL_CHOICE_SPLIT = 2 };
int dual_choose(Context *ctx, const Work &w, int mode, int *choice, bool *bad_input);
int dual_setup(Context *ctx, const Work &w, Work &wd);
// DUAL_CHOICE_SPLIT (after dual_choose, whose grading they read): the D'
// columns of the D-reduced blocks pre-cleared; then D's columns of the
// D'-reduced blocks and every row the D' reduction paired; then the lows of
// the D'-reduced blocks' columns taken from low_dual (D'-reduced, mapped).
int split_preclear_dual(Context *ctx, const Work &w, uint8_t *clear);
int split_preclear_primal(Context *ctx, int64_t m, const int32_t *low_dual, uint8_t *clear);
int split_merge(Context *ctx, int32_t *low, const int32_t *low_dual, int64_t m);
// The two pre-clears on any stream, for callers with their own buffers (the
// request server): grade_tmp is dual_grade's tmp, clear the m columns' flags
// (set, never reset).
void split_clear_dual(cudaStream_t s, int sm_count, const void *grade_tmp, const int64_t *colptr,
                      const int32_t *rows, int64_t m, uint8_t *clear);
void split_clear_primal(cudaStream_t s, int sm_count, const void *grade_tmp, int64_t m, const int32_t *low_dual,
                        uint8_t *clear);
// The same pieces for callers with their own buffers (the request server):
// dual_grade grades a device CSC (synchronous; tmp of dual_grade_tmp_bytes);
// host_prefers_dual makes the automatic choice on a host CSC;
// dual_build_store writes the anti-transpose of a device CSC of m columns
// into the column store at pool (its segments recorded as seg_base + offset,
// its rows shifted by roff), with low, seg, dim, the pivot records and beta
// of its columns (each array given from the matrix's first column; tmp of
// dual_tmp_bytes).
size_t dual_grade_tmp_bytes(int64_t m);
int dual_grade(cudaStream_t s, int sm_count, const int64_t *colptr, const int32_t *rows, int64_t m, int64_t nnz,
               int mode, void *tmp, int *choice, bool *bad_input, int *launches);
// each column's bucket and the per-block choice inside dual_grade's tmp
void dual_split_arrays(void *tmp, int64_t m, const int8_t **bucket, const uint8_t **split);
bool host_prefers_dual(int64_t m, const int64_t *colptr, const int32_t *rows);
size_t dual_tmp_bytes(int64_t m, int64_t nnz);
int dual_build_store(cudaStream_t s, int sm_count, const int64_t *colptr, const int32_t *rows, int64_t m,
                     int64_t nnz, int *pool, int64_t seg_base, int roff, int64_t *seg, int32_t *low, int8_t *dim,
                     PivRec *rec, int32_t *beta, void *tmp, int *launches);
int dual_lows(Context *ctx, const Work &wd, int32_t **low);

// capi.cu
void *ctx_alloc(Context *ctx, int slot, size_t bytes);
int ctx_sync_status(Context *ctx, Work &w, DevStatus *out);

// Per-sweep progress trackers of a pms reduction (the reference's track(),
// src/cuda/algorithms/tracker.cu:92-134, called once per iteration by
// pms.cu:16,106).  Set on the context for one reduction by oph_openph when
// the caller passes low_true and tracker arrays.
struct Tracking {
    const int32_t *low_true = nullptr;  // device, 0-based (-1 = none)
    const int32_t *ess_true = nullptr;  // device
    uint8_t *ess_hat = nullptr;         // device, m: running essential estimate
    double *acc = nullptr;              // device, 4 per slot: sum |low - low_true|,
                                        //   max |.|, #unclassified, sum ess_hat
    int slots = 0;                      // slot 0 = before Phase 0, slot k = after sweep k
    std::vector<float> sweep_ms;        // device time of each sweep that ran
};

// Per-iteration progress of the standard and twist walks (the reference's
// track_host after every column, standard.cu:44-49, twist.cu:68-71).  In
// those algorithms a column is reduced completely at its one visit, so the
// state after iteration k follows from the visit order, the initial lows and
// the final lows (twist also clears the low of each new pivot's row); the
// walker only stamps the end of every iteration (globaltimer, ns), and the
// host replays the rest.
struct SeqTracking {
    std::vector<int32_t> low0;  // the lows before the walk
    std::vector<int8_t> dim;    // nnz - 1 per column (twist's visit order)
    std::vector<long long> ns;  // end of iteration k (k = 0: the walk's start)
    long long iters = 0;        // entries: 1 + iterations
    // the row forms: each row that had additions, as the walker logged it
    // ({row, pivot, k, end ns (two ints)} and k {column, new low} pairs),
    // and the walk's start; rows_ok is false when the log ran out of room
    std::vector<int> ev;
    long long ev_t0 = 0;
    bool rows_ok = false;
};

struct Context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    DevBuf bufs[48];  // indexed by Slot
    DevStatus *h_status = nullptr;  // pinned mirror
    int max_sweeps = 0;             // 0 = default
    int64_t initial_pool_bytes = 0; // 0 = default
    int64_t budget = 0;
    int64_t pool_ints = 0;          // current pool capacity
    int profile = 0;                // record per-phase events
    int count_slots = 0;            // exact |P| + |T| + |T xor P| in every tier
    cudaEvent_t *pev = nullptr;     // profiling events (pairs)
    int pev_n = 0;
    oph_profile prof{};             // last reduction
    int launches = 0;               // kernels launched by the current reduction
    int tier0 = 0;                  // Phase II tier-0 candidate (autotuned)
    int dual = OPH_DUAL_AUTO;       // which matrix pms reduces
    Tracking *track = nullptr;      // per-sweep trackers for the current reduction
    SeqTracking *seq_track = nullptr;  // per-iteration trackers of a standard / twist walk
    // two pms sweeps (the list ping-pong's two parities) captured as one CUDA
    // graph and replayed instead of 2 x 11 launches; sweep_key holds the
    // launch arguments it was captured with
    cudaGraphExec_t sweep_graph = nullptr;
    std::vector<unsigned char> sweep_key;
    // the whole sweep loop as one graph: a conditional WHILE node whose body
    // runs two sweeps and sets the loop condition from the device status
    // (converged, overflow, error, sweep cap), so the host waits once per
    // reduction instead of once per batch of sweeps; loop_key as sweep_key
    cudaGraphExec_t loop_graph = nullptr;
    std::vector<unsigned char> loop_key;
};

// buffer slots of Context::bufs
enum Slot {
    S_STATUS, S_COLPTR, S_ROWS, S_LOW, S_CLASSES, S_CLEAR, S_DIM, S_FIRST, S_LEFT, S_BETA, S_WORK, S_WIDE, S_SEG,
    S_ROWPIV, S_AGG, S_POOL, S_POOL2, S_ESS, S_ARGLOW, S_COO_R, S_COO_C, S_LOWTRUE, S_TRACK, S_INSTOFF, S_TMP,
    S_ULIST, S_KAGG, S_ESSHAT, S_SLIST, S_DGRADE, S_DCOLPTR, S_DSORT, S_DTEMP, S_DLOW, S_BITMAP, S_CHECK, S_IASC, S_IBUCKET, S_IOPEN, S_RANGES, S_SEQNS, S_PRECLEAR, S_NSLOTS
};

}  // namespace oph

// The C ABI's opaque context is the library's Context.
struct oph_context : public oph::Context {};
