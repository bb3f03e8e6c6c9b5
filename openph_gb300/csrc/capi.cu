// C ABI of libopenph_gb300 (include/openph.h): contexts, device workspace,
// input conversion, algorithm dispatch and output finalisation.
//
// Reference counterparts: openph() (src/cuda/openph.cu:29-237) and
// algorithm_factory() (src/cuda/algorithms/algorithm_factory.cu:1-151).
// Unlike the reference, device buffers are cached per context instead of
// ~17 cudaMalloc/cudaFree pairs per call, every call runs on the context's
// own stream, and nothing uses global __device__ symbols, so distinct
// contexts are independent.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "oph_host.h"
#include "pms.cuh"

using namespace oph;


namespace oph {

void *ctx_alloc(Context *ctx, int slot, size_t bytes) {
    DevBuf &b = ctx->bufs[slot];
    if (bytes == 0) bytes = 16;
    bytes = (bytes + 255) & ~(size_t)255;
    if (b.bytes >= bytes) return b.ptr;
    if (ctx->budget > 0) {
        size_t total = 0;
        for (int i = 0; i < S_NSLOTS; i++) total += (i == slot) ? 0 : ctx->bufs[i].bytes;
        if ((int64_t)(total + bytes) > ctx->budget) return nullptr;
    }
    if (b.ptr) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(b.ptr);
        b.ptr = nullptr;
        b.bytes = 0;
    }
    if (cudaMalloc(&b.ptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        b.ptr = nullptr;
        return nullptr;
    }
    b.bytes = bytes;
    return b.ptr;
}

// --------------------------------------------------------------- kernels
enum EssMode { ESS_PAIRS = 0, ESS_ROW_PARALLEL = 1, ESS_RUNNING = 2 };

// Output pass 1: low (0- or 1-based, optionally local to its batch instance),
// ess initial values, arglow cleared.
__global__ void k_finalize1(const int32_t *__restrict__ low, int64_t m, int one_based, int ess_mode,
                            const int64_t *__restrict__ inst_off, int count, int32_t *__restrict__ out_low,
                            int32_t *__restrict__ ess, int32_t *__restrict__ arglow) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        int l = low[j];
        int64_t base = 0;
        if (inst_off) {
            int lo = 0, hi = count;
            while (hi - lo > 1) {
                int mid = (lo + hi) >> 1;
                if (inst_off[mid] <= j) lo = mid; else hi = mid;
            }
            base = inst_off[lo];
        }
        if (out_low) out_low[j] = l >= 0 ? (int32_t)(l - base) + one_based : (one_based ? 0 : -1);
        if (ess) {
            if (ess_mode == ESS_PAIRS) ess[j] = l >= 0 ? 0 : 1;
            else if (ess_mode == ESS_ROW_PARALLEL) ess[j] = 1;
            else if (l >= 0) ess[j] = 0;
        }
        if (arglow) arglow[j] = -1;
    }
}

// Output pass 2: the row of every nonzero low is paired (ess 0), arglow.
__global__ void k_finalize2(const int32_t *__restrict__ low, int64_t m, const int64_t *__restrict__ inst_off,
                            int count, int32_t *__restrict__ ess, int32_t *__restrict__ arglow) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        int l = low[j];
        if (l < 0) continue;
        if (ess) ess[l] = 0;
        if (arglow) {
            int64_t base = 0;
            if (inst_off) {
                int lo = 0, hi = count;
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (inst_off[mid] <= j) lo = mid; else hi = mid;
                }
                base = inst_off[lo];
            }
            arglow[l] = (int32_t)(j - base);
        }
    }
}

// Tracker entries kept per reduction (the reference's arrays hold m + 1).
constexpr int64_t MAX_TRACKED = 1 << 16;

__global__ void k_fill_i32(int32_t *p, int64_t n, int32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// Tracker sums for the reference's progress outputs (tracker.cu:92-134):
// acc[0] = sum |low - low_true|, acc[1] = max |.|, acc[2] = sum ess,
// acc[3] = sum ess_true, acc[4] = sum |low_true + 1| (1-based norm),
// acc[5] = max |low_true + 1|.  Lows 0-based; low_true 0-based (-1 = none).
__global__ void k_tracker(const int32_t *__restrict__ low, const int32_t *__restrict__ low_true,
                          const int32_t *__restrict__ ess, const int32_t *__restrict__ ess_true, int64_t m,
                          double *acc) {
    double s = 0, mx = 0, se = 0, st = 0, nt = 0, mt = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        double d = fabs((double)low[j] - (double)low_true[j]);
        s += d;
        mx = fmax(mx, d);
        se += ess[j];
        st += ess_true[j];
        double t = fabs((double)low_true[j] + 1.0);
        nt += t;
        mt = fmax(mt, t);
    }
    atomicAdd(&acc[0], s);
    atomicAdd(&acc[2], se);
    atomicAdd(&acc[3], st);
    atomicAdd(&acc[4], nt);
    // maxima of non-negative doubles compare as their bit patterns
    atomicMax((unsigned long long *)&acc[1], (unsigned long long)__double_as_longlong(mx));
    atomicMax((unsigned long long *)&acc[5], (unsigned long long)__double_as_longlong(mt));
}

// ess_true from low_true (compute_ess_true, src/cuda/kernels.cu:54-62).
__global__ void k_ess_true(const int32_t *__restrict__ low_true, int64_t m, int32_t *__restrict__ ess_true, int pass) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        int l = low_true[j];
        if (pass == 0) ess_true[j] = l >= 0 ? 0 : 1;
        else if (l >= 0 && l < m) ess_true[l] = 0;
    }
}

__global__ void k_shift_down(const int *__restrict__ in, int64_t m, int32_t *__restrict__ out) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        out[j] = in[j] - 1;
}

int ctx_sync_status(Context *ctx, Work &w, DevStatus *out) {
    OPH_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, w.st, sizeof(DevStatus), cudaMemcpyDeviceToHost, ctx->stream));
    OPH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (out) *out = *ctx->h_status;
    return OPH_OK;
}

static int grid_for(Context *ctx, int64_t n) {
    int64_t g = (n + 255) / 256;
    int64_t cap = (int64_t)ctx->sm_count * 16;
    if (g > cap) g = cap;
    return g < 1 ? 1 : (int)g;
}

// Allocates the per-column working arrays of a reduction of m columns.
static int alloc_work(Context *ctx, Work &w, int64_t m) {
    const int64_t mm = m > 0 ? m : 1;
    w.m = m;
    w.low = (int32_t *)ctx_alloc(ctx, S_LOW, sizeof(int32_t) * mm);
    w.classes = (int8_t *)ctx_alloc(ctx, S_CLASSES, mm);
    w.clear = (uint8_t *)ctx_alloc(ctx, S_CLEAR, mm);
    w.dim = (int8_t *)ctx_alloc(ctx, S_DIM, mm);
    w.first = (int32_t *)ctx_alloc(ctx, S_FIRST, sizeof(int32_t) * mm);
    w.beta = (int32_t *)ctx_alloc(ctx, S_BETA, sizeof(int32_t) * mm);
    w.worklist = (int32_t *)ctx_alloc(ctx, S_WORK, sizeof(int32_t) * mm);
    w.widelist = (int32_t *)ctx_alloc(ctx, S_WIDE, sizeof(int32_t) * mm);
    w.seg = (int64_t *)ctx_alloc(ctx, S_SEG, sizeof(int64_t) * mm);
    w.rec = (PivRec *)ctx_alloc(ctx, S_ROWPIV, sizeof(PivRec) * mm);
    w.ntiles = (m + 2047) / 2048;
    w.agg = (int32_t *)ctx_alloc(ctx, S_AGG, sizeof(int32_t) * MAXC * (w.ntiles + 1) + 64);
    w.st = (DevStatus *)ctx_alloc(ctx, S_STATUS, sizeof(DevStatus));
    if (!w.low || !w.classes || !w.clear || !w.dim || !w.first || !w.beta || !w.worklist || !w.widelist ||
        !w.seg || !w.rec || !w.agg || !w.st)
        return OPH_ERR_OOM;
    return OPH_OK;
}

struct Outputs {
    int32_t *low = nullptr;     // device, m
    int one_based = 0;
    int32_t *ess = nullptr;     // device, m (may be null)
    int32_t *arglow = nullptr;  // device, m (may be null)
    const int64_t *inst_off = nullptr;
    int count = 0;
};

// pms with some blocks of D reduced on D' and the others on D (dual_choose's
// DUAL_CHOICE_SPLIT): D' first, its columns of the D-reduced blocks
// pre-cleared; then D, with its columns of the D'-reduced blocks and every
// row the D' reduction paired pre-cleared; the lows put together in w.low.
static int reduce_split(Context *ctx, Work &w, oph_info *info) {
    const int64_t m = w.m;
    uint8_t *pre = (uint8_t *)ctx_alloc(ctx, S_PRECLEAR, m);
    if (!pre) return OPH_ERR_OOM;
    Work wd;
    int rc;
    if ((rc = dual_setup(ctx, w, wd)) || (rc = split_preclear_dual(ctx, w, pre))) return rc;
    DevStatus hs;
    if ((rc = ctx_sync_status(ctx, wd, &hs))) return rc;
    if (hs.error) return OPH_ERR_BAD_INPUT;
    wd.preclear = pre;
    oph_info a{}, b{};
    if ((rc = run_pms(ctx, wd, &a))) return rc;
    int32_t *mapped = nullptr;
    if ((rc = dual_lows(ctx, wd, &mapped)) || (rc = split_preclear_primal(ctx, m, mapped, pre))) return rc;
    if ((rc = setup_store(ctx, w, true))) return rc;
    ctx->launches += 3;
    if ((rc = ctx_sync_status(ctx, w, &hs))) return rc;
    if (hs.error || hs.max_dim > MAXC - 2) return OPH_ERR_BAD_INPUT;
    w.preclear = pre;
    rc = run_pms(ctx, w, &b);
    w.preclear = nullptr;
    if (rc || (rc = split_merge(ctx, w.low, mapped, m))) return rc;
    info->sweeps = a.sweeps + b.sweeps;
    info->num_iters = info->sweeps + 1;  // as for pms on one matrix: sweeps + 1
    info->additions = a.additions + b.additions;
    info->slots_moved = a.slots_moved + b.slots_moved;
    info->pool_bytes = std::max(a.pool_bytes, b.pool_bytes);
    info->regrows = a.regrows + b.regrows;
    info->device_ms = a.device_ms + b.device_ms;
    info->dual = 2;
    return OPH_OK;
}

// Runs `algo` on the CSC already in w.colptr / w.rows and writes outputs.
static int reduce_core(Context *ctx, int algo, Work &w, const Outputs &o, oph_info *info) {
    cudaStream_t s = ctx->stream;
    const int64_t m = w.m;
    const bool pms = algo == OPH_ALGO_PMS;
    ctx->launches = 0;
    ctx->prof = oph_profile{};
    if (ctx->profile) cudaEventRecord(ctx->ev[2], s);
    // pms on the anti-transpose where that moves the work to a far smaller
    // dimension bucket (not with per-sweep trackers, which follow D's own
    // reduction); wr is the matrix reduced
    int rc;
    // nothing indexes through colptr / rows before they pass the structural
    // check: here, or in the grading of dual_choose, which makes the same
    // checks (bounds first) whenever it runs
    const bool grades = pms && !ctx->track && ctx->dual != OPH_DUAL_NEVER && m > 0;
    if (!w.checked && !grades && (rc = check_csc(ctx, w.colptr, w.rows, m, w.nnz, nullptr, 0))) return rc;
    int choice = DUAL_CHOICE_D;
    if (pms && !ctx->track) {
        bool bad = false;
        if ((rc = dual_choose(ctx, w, ctx->dual, &choice, &bad))) return rc;
        if (bad) return OPH_ERR_BAD_INPUT;
    }
    const bool dual = choice == DUAL_CHOICE_DUAL;
    const bool split = choice == DUAL_CHOICE_SPLIT && m > 0;
    Work wd;
    if (split) {
        // reduce_split builds both stores itself
    } else if (dual) {
        // D' built straight into its column store, with its buckets, left[]
        // and beta
        if ((rc = dual_setup(ctx, w, wd))) return rc;
    } else {
        if ((rc = setup_store(ctx, w, pms))) return rc;
        ctx->launches += pms ? 3 : 1;
    }
    Work &wr = dual ? wd : w;
    if (ctx->profile) {
        cudaEventRecord(ctx->ev[3], s);
        cudaEventSynchronize(ctx->ev[3]);
        cudaEventElapsedTime(&ctx->prof.setup_ms, ctx->ev[2], ctx->ev[3]);
    }
    DevStatus hs;
    if (!split) {
        if ((rc = ctx_sync_status(ctx, wr, &hs))) return rc;
        if (hs.error) return OPH_ERR_BAD_INPUT;
        // the Phase I scan keeps one running maximum per dimension bucket -1 ..
        // MAXC-2 (D's buckets, checked by dual_choose when D' is reduced)
        if (pms && !dual && hs.max_dim > MAXC - 2) return OPH_ERR_BAD_INPUT;
    }
    const int row_quirk = algo == OPH_ALGO_PH_ROW;
    if (row_quirk && o.ess) k_fill_i32<<<grid_for(ctx, m), 256, 0, s>>>(o.ess, m, 1);
    oph_info local{};
    if (m > 0) {
        if (split) {
            rc = reduce_split(ctx, w, &local);
        } else if (pms) {
            rc = run_pms(ctx, wr, &local);
        } else {
            rc = run_sequential(ctx, w, algo, row_quirk ? o.ess : nullptr, &local);
        }
        if (rc) return rc;
    } else {
        local.num_iters = 1;
    }
    const int ess_mode = algo == OPH_ALGO_PH_ROW_PARALLEL ? ESS_ROW_PARALLEL : (row_quirk ? ESS_RUNNING : ESS_PAIRS);
    if (dual && m > 0) {
        // D's lows, back in w.low for the outputs and the trackers
        int32_t *mapped = nullptr;
        if ((rc = dual_lows(ctx, wd, &mapped))) return rc;
        OPH_CUDA_TRY(cudaMemcpyAsync(w.low, mapped, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice, s));
    }
    if (!split) local.dual = dual ? 1 : 0;
    if (m > 0) {
        k_finalize1<<<grid_for(ctx, m), 256, 0, s>>>(w.low, m, o.one_based, ess_mode, o.inst_off, o.count, o.low,
                                                     o.ess, o.arglow);
        k_finalize2<<<grid_for(ctx, m), 256, 0, s>>>(w.low, m, o.inst_off, o.count, o.ess, o.arglow);
        ctx->launches += 2;
        OPH_CUDA_TRY(cudaGetLastError());
    }
    ctx->prof.kernel_launches = ctx->launches;
    if (info) *info = local;
    return OPH_OK;
}

static int check_algo(int algo) { return algo >= OPH_ALGO_STANDARD && algo <= OPH_ALGO_PMS ? OPH_OK : OPH_ERR_ALGO; }

}  // namespace oph

// =================================================================== C ABI
extern "C" {

__attribute__((visibility("default"))) int oph_algo_from_string(const char *algstr) {
    if (!algstr) return -1;
    static const char *names[] = {"standard", "twist", "ph_row", "standard_parallel", "twist_parallel",
                                  "ph_row_parallel", "pms"};
    for (int i = 0; i < 7; i++)
        if (strcmp(algstr, names[i]) == 0) return i;
    return -1;
}

__attribute__((visibility("default"))) const char *oph_status_string(int status) {
    switch (status) {
        case OPH_OK: return "ok";
        case OPH_ERR_BAD_INPUT: return "malformed boundary matrix or argument";
        case OPH_ERR_OOM: return "out of device memory (or over the context budget)";
        case OPH_ERR_OVERFLOW: return "column store cannot grow any further";
        case OPH_ERR_TIMEOUT: return "iteration cap reached before convergence";
        case OPH_ERR_CUDA: return "CUDA runtime error";
        case OPH_ERR_ALGO: return "algorithm not recognised";
        default: return "unknown status";
    }
}

__attribute__((visibility("default"))) int oph_context_create(int device, oph_context **out) {
    if (!out) return OPH_ERR_BAD_INPUT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return OPH_ERR_CUDA;
    }
    if (device < 0 || device >= n) return OPH_ERR_BAD_INPUT;
    OPH_CUDA_TRY(cudaSetDevice(device));
    oph_context *ctx = new oph_context();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost((void **)&ctx->h_status, sizeof(DevStatus)) != cudaSuccess) {
        delete ctx;
        return OPH_ERR_CUDA;
    }
    for (auto &e : ctx->ev) cudaEventCreate(&e);
    *out = ctx;
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_context_destroy(oph_context *ctx) {
    if (!ctx) return OPH_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto &b : ctx->bufs)
        if (b.ptr) cudaFree(b.ptr);
    for (auto &e : ctx->ev) cudaEventDestroy(e);
    for (int i = 0; i < ctx->pev_n; i++) cudaEventDestroy(ctx->pev[i]);
    free(ctx->pev);
    if (ctx->sweep_graph) cudaGraphExecDestroy(ctx->sweep_graph);
    if (ctx->loop_graph) cudaGraphExecDestroy(ctx->loop_graph);
    if (ctx->h_status) cudaFreeHost(ctx->h_status);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return OPH_OK;
}

__attribute__((visibility("default"))) void *oph_context_stream(oph_context *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

__attribute__((visibility("default"))) int oph_context_set_budget(oph_context *ctx, int64_t bytes) {
    if (!ctx || bytes < 0) return OPH_ERR_BAD_INPUT;
    ctx->budget = bytes;
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_context_set_limits(oph_context *ctx, int32_t max_sweeps,
                                                                  int64_t initial_pool_bytes) {
    if (!ctx || max_sweeps < 0 || initial_pool_bytes < 0) return OPH_ERR_BAD_INPUT;
    ctx->max_sweeps = max_sweeps;
    ctx->initial_pool_bytes = initial_pool_bytes;
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_context_set_profile(oph_context *ctx, int on) {
    if (!ctx) return OPH_ERR_BAD_INPUT;
    if (on & ~3) return OPH_ERR_BAD_INPUT;
    ctx->profile = on & 1;
    ctx->count_slots = (on >> 1) & 1;
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_last_profile(oph_context *ctx, oph_profile *out) {
    if (!ctx || !out) return OPH_ERR_BAD_INPUT;
    *out = ctx->prof;
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_reduce_device(oph_context *ctx, int algo, int64_t m,
                                                             const int64_t *d_colptr, const int32_t *d_rows,
                                                             int32_t *d_low, int32_t *d_ess, int32_t *d_arglow,
                                                             oph_info *info) {
    if (!ctx || m < 0 || m >= (1ll << 29) || !d_colptr || (m > 0 && !d_low)) return OPH_ERR_BAD_INPUT;
    if (check_algo(algo)) return OPH_ERR_ALGO;
    OPH_CUDA_TRY(cudaSetDevice(ctx->device));
    int64_t nnz = 0;
    OPH_CUDA_TRY(cudaMemcpyAsync(&nnz, d_colptr + m, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    OPH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (nnz < 0 || (nnz > 0 && !d_rows)) return OPH_ERR_BAD_INPUT;
    Work w;
    int rc = alloc_work(ctx, w, m);
    if (rc) return rc;
    w.nnz = nnz;
    w.colptr = d_colptr;
    w.rows = d_rows;
    Outputs o;
    o.low = d_low;
    o.ess = d_ess;
    o.arglow = d_arglow;
    rc = reduce_core(ctx, algo, w, o, info);
    if (rc) return rc;
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_reduce(oph_context *ctx, int algo, int64_t m, const int64_t *colptr,
                                                      const int32_t *rows, int32_t *low, int32_t *ess,
                                                      int32_t *arglow, oph_info *info) {
    if (!ctx || m < 0 || m >= (1ll << 29) || !colptr || (m > 0 && !low)) return OPH_ERR_BAD_INPUT;
    if (check_algo(algo)) return OPH_ERR_ALGO;
    const int64_t nnz = colptr[m];
    if (nnz < 0 || colptr[0] != 0 || (nnz > 0 && !rows)) return OPH_ERR_BAD_INPUT;
    OPH_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    int64_t *d_colptr = (int64_t *)ctx_alloc(ctx, S_COLPTR, sizeof(int64_t) * (m + 1));
    int32_t *d_rows = (int32_t *)ctx_alloc(ctx, S_ROWS, sizeof(int32_t) * (nnz > 0 ? nnz : 1));
    int32_t *d_out = (int32_t *)ctx_alloc(ctx, S_ESS, sizeof(int32_t) * 3 * (m > 0 ? m : 1));
    if (!d_colptr || !d_rows || !d_out) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cudaMemcpyAsync(d_colptr, colptr, sizeof(int64_t) * (m + 1), cudaMemcpyHostToDevice, s));
    if (nnz > 0) OPH_CUDA_TRY(cudaMemcpyAsync(d_rows, rows, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, s));
    Work w;
    int rc = alloc_work(ctx, w, m);
    if (rc) return rc;
    w.nnz = nnz;
    w.colptr = d_colptr;
    w.rows = d_rows;
    Outputs o;
    o.low = d_out;
    o.ess = ess ? d_out + m : nullptr;
    o.arglow = arglow ? d_out + 2 * m : nullptr;
    rc = reduce_core(ctx, algo, w, o, info);
    if (rc) return rc;
    if (m > 0) {
        OPH_CUDA_TRY(cudaMemcpyAsync(low, d_out, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
        if (ess) OPH_CUDA_TRY(cudaMemcpyAsync(ess, d_out + m, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
        if (arglow) OPH_CUDA_TRY(cudaMemcpyAsync(arglow, d_out + 2 * m, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
    }
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    return OPH_OK;
}

static int batch_core(oph_context *ctx, int algo, int32_t count, const int64_t *d_col_off, const int64_t *d_colptr,
                      const int32_t *d_rows_local, int64_t total_m, int64_t total_nnz, int32_t *d_low, int32_t *d_ess,
                      oph_info *info) {
    cudaStream_t s = ctx->stream;
    ctx->launches = 0;
    // instance offsets, colptr and local rows checked, and the rows shifted
    // into their instances' column ranges, in one pass (a checked entry is
    // the only one written)
    int32_t *d_rows_g = (int32_t *)ctx_alloc(ctx, S_COO_R, sizeof(int32_t) * (total_nnz > 0 ? total_nnz : 1));
    if (!d_rows_g) return OPH_ERR_OOM;
    int rc = check_csc(ctx, d_colptr, d_rows_local, total_m, total_nnz, d_col_off, count, d_rows_g);
    if (rc) return rc;
    Work w;
    rc = alloc_work(ctx, w, total_m);
    if (rc) return rc;
    w.nnz = total_nnz;
    w.colptr = d_colptr;
    w.rows = d_rows_g;
    w.checked = true;
    w.inst_off = d_col_off;
    w.inst_count = count;
    Outputs o;
    o.low = d_low;
    o.ess = d_ess;
    o.inst_off = d_col_off;
    o.count = count;
    return reduce_core(ctx, algo, w, o, info);
}

__attribute__((visibility("default"))) int oph_reduce_batch_device(oph_context *ctx, int algo, int32_t count,
                                                                   const int64_t *d_col_off, const int64_t *d_colptr,
                                                                   const int32_t *d_rows, int64_t total_m,
                                                                   int64_t total_nnz, int32_t *d_low, int32_t *d_ess,
                                                                   oph_info *info) {
    if (!ctx || count < 1 || total_m < 0 || total_m >= (1ll << 29) || total_nnz < 0 || !d_col_off || !d_colptr ||
        (total_m > 0 && !d_low))
        return OPH_ERR_BAD_INPUT;
    if (check_algo(algo)) return OPH_ERR_ALGO;
    OPH_CUDA_TRY(cudaSetDevice(ctx->device));
    return batch_core(ctx, algo, count, d_col_off, d_colptr, d_rows, total_m, total_nnz, d_low, d_ess, info);
}

__attribute__((visibility("default"))) int oph_reduce_batch(oph_context *ctx, int algo, int32_t count,
                                                            const int64_t *col_off, const int64_t *colptr,
                                                            const int32_t *rows, int32_t *low, int32_t *ess,
                                                            oph_info *info) {
    if (!ctx || count < 1 || !col_off || !colptr) return OPH_ERR_BAD_INPUT;
    if (check_algo(algo)) return OPH_ERR_ALGO;
    const int64_t total_m = col_off[count];
    if (total_m < 0 || total_m >= (1ll << 29) || col_off[0] != 0 || (total_m > 0 && !low)) return OPH_ERR_BAD_INPUT;
    for (int b = 0; b < count; b++)
        if (col_off[b + 1] < col_off[b]) return OPH_ERR_BAD_INPUT;
    const int64_t total_nnz = colptr[total_m];
    if (total_nnz < 0 || (total_nnz > 0 && !rows)) return OPH_ERR_BAD_INPUT;
    OPH_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    int64_t *d_off = (int64_t *)ctx_alloc(ctx, S_INSTOFF, sizeof(int64_t) * (count + 1));
    int64_t *d_colptr = (int64_t *)ctx_alloc(ctx, S_COLPTR, sizeof(int64_t) * (total_m + 1));
    int32_t *d_rows = (int32_t *)ctx_alloc(ctx, S_ROWS, sizeof(int32_t) * (total_nnz > 0 ? total_nnz : 1));
    int32_t *d_out = (int32_t *)ctx_alloc(ctx, S_ESS, sizeof(int32_t) * 2 * (total_m > 0 ? total_m : 1));
    if (!d_off || !d_colptr || !d_rows || !d_out) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cudaMemcpyAsync(d_off, col_off, sizeof(int64_t) * (count + 1), cudaMemcpyHostToDevice, s));
    OPH_CUDA_TRY(cudaMemcpyAsync(d_colptr, colptr, sizeof(int64_t) * (total_m + 1), cudaMemcpyHostToDevice, s));
    if (total_nnz > 0)
        OPH_CUDA_TRY(cudaMemcpyAsync(d_rows, rows, sizeof(int32_t) * total_nnz, cudaMemcpyHostToDevice, s));
    int rc = batch_core(ctx, algo, count, d_off, d_colptr, d_rows, total_m, total_nnz, d_out,
                        ess ? d_out + total_m : nullptr, info);
    if (rc) return rc;
    if (total_m > 0) {
        OPH_CUDA_TRY(cudaMemcpyAsync(low, d_out, sizeof(int32_t) * total_m, cudaMemcpyDeviceToHost, s));
        if (ess) OPH_CUDA_TRY(cudaMemcpyAsync(ess, d_out + total_m, sizeof(int32_t) * total_m, cudaMemcpyDeviceToHost, s));
    }
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    return OPH_OK;
}

// ----------------------------------------------------------- drop-in path
static std::mutex g_ctx_mu;
static oph_context *g_ctx[64];

static oph_context *default_context(int device, int *rc) {
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    if (device < 0 || device >= 64) { *rc = OPH_ERR_BAD_INPUT; return nullptr; }
    if (!g_ctx[device]) {
        *rc = oph_context_create(device, &g_ctx[device]);
        if (*rc) return nullptr;
    }
    *rc = OPH_OK;
    return g_ctx[device];
}

}  // extern "C"

// The state behind the reference's tracker sums (track_host,
// tracker.cu:136-172): the lows against low_true (sum and maximum of the
// differences, the maximum through a count of every difference), the
// unclassified columns, the essential estimate; changed one entry at a time.
struct TrackState {
    const std::vector<int32_t> &lt;
    std::vector<int32_t> low;
    std::vector<int8_t> cls, ess;
    std::vector<int64_t> hist;
    double l1 = 0;
    int64_t mx = 0, uncl = 0, esum = 0;
    TrackState(const std::vector<int32_t> &low0, const std::vector<int32_t> &low_true)
        : lt(low_true), low(low0), cls(low0.size(), 0), ess(low0.size(), 1), hist(low0.size() + 2, 0) {
        const int64_t m = (int64_t)low.size();
        uncl = esum = m;
        for (int64_t c = 0; c < m; c++) {
            const int64_t d = diff(c);
            hist[d]++;
            l1 += (double)d;
            mx = std::max(mx, d);
        }
    }
    int64_t diff(int64_t c) const { return (int64_t)std::llabs((long long)low[c] - (long long)lt[c]); }
    void set_low(int64_t c, int32_t v) {
        if (low[c] == v) return;
        const int64_t d0 = diff(c);
        hist[d0]--;
        l1 -= (double)d0;
        low[c] = v;
        const int64_t d1 = diff(c);
        hist[d1]++;
        l1 += (double)d1;
        if (d1 > mx) mx = d1;
        while (mx > 0 && hist[mx] == 0) mx--;
    }
    void set_cls(int64_t c, int8_t v) {
        if (cls[c] == 0 && v != 0) uncl--;
        cls[c] = v;
    }
    void clear_ess(int64_t c) {
        if (ess[c]) {
            ess[c] = 0;
            esum--;
        }
    }
    void entry(std::vector<double> &out, int64_t k) const {
        out[4 * k] = l1;
        out[4 * k + 1] = (double)mx;
        out[4 * k + 2] = (double)uncl;
        out[4 * k + 3] = (double)esum;
    }
};

// The reference's per-iteration trackers of a standard or twist reduction
// (after every column: standard.cu:44-49, twist.cu:68-71; on the device for
// the parallel forms, standard_parallel.cu:40-43, twist_parallel.cu:75-78),
// replayed on the host from the walk: the state after iteration k is every
// visited column at its final low, twist's cleared rows at -1, every other
// column at its initial low.  classes and ess follow each form's own
// updates: the CPU forms classify the visited column (a zero column as 1)
// and clear ess at the pair (reduce_col_host's clearing of the intermediate
// lows only clears rows that are already some earlier pivot's low); the
// parallel forms re-apply update_classes (pivot pairs only) and ess_hat
// (every current low, and the pairs) after each column, kernels.cu:93-124.
// Out: 4 sums per entry, as Tracking::acc.
static void replay_seq_trackers(const SeqTracking &tk, int algo, const std::vector<int32_t> &low_fin,
                                const std::vector<int32_t> &low_true, std::vector<double> &out) {
    const int64_t m = (int64_t)low_fin.size();
    const bool twist = algo == OPH_ALGO_TWIST || algo == OPH_ALGO_TWIST_PARALLEL;
    const bool par = algo == OPH_ALGO_STANDARD_PARALLEL || algo == OPH_ALGO_TWIST_PARALLEL;
    TrackState st(tk.low0, low_true);
    out.assign(4 * (size_t)tk.iters, 0.0);
    st.entry(out, 0);
    int64_t k = 1;
    auto visit = [&](int64_t j) {
        const int32_t l = low_fin[j];
        st.set_low(j, l);
        if (twist && l >= 0) st.set_low(l, -1);
        if (l >= 0) {
            st.set_cls(j, -1);
            st.set_cls(l, 1);
            st.clear_ess(j);
            st.clear_ess(l);
        } else if (!par) {
            st.set_cls(j, 1);
        }
        if (par) {
            if (k == 1) {
                for (int64_t c = 0; c < m; c++)
                    if (st.low[c] >= 0) st.clear_ess(st.low[c]);
            } else if (l >= 0) {
                st.clear_ess(l);
            }
        }
        if (k < tk.iters) st.entry(out, k);
        k++;
    };
    if (twist) {
        int maxd = -1;
        for (int64_t c = 0; c < m; c++) maxd = std::max(maxd, (int)tk.dim[c]);
        for (int d = maxd; d >= 1; d--)
            for (int64_t j = 0; j < m; j++)
                if (tk.dim[j] == d) visit(j);
    } else {
        for (int64_t j = 0; j < m; j++) visit(j);
    }
}

// The same for the row forms (after every row i = m-1 .. 0: ph_row.cu:65-113,
// ph_row_parallel.cu:44-83), from the walker's log of the rows that had
// additions: each neighbour of the row's pivot took the pivot once and
// moved to its logged new low.  The CPU form clears the row and the pivot
// pair from ess before each addition and marks a neighbour that is now the
// first column ever to hold its new low as a pair (a new low of -1 marks
// nothing; the reference reads pivots[-1] there), in column order, and after
// the last row marks every pair and classifies the remaining essentials
// (ph_row.cu:91-103); the parallel form never fills arglow (classes stay 0)
// and clears ess at every current low after each row.  time: the time
// between two logged rows is shared evenly by the rows between them.
static void replay_row_trackers(const SeqTracking &tk, int algo, const std::vector<int32_t> &low_true,
                                std::vector<double> &out, std::vector<float> &ms) {
    const int64_t m = (int64_t)tk.low0.size();
    const bool par = algo == OPH_ALGO_PH_ROW_PARALLEL;
    TrackState st(tk.low0, low_true);
    std::vector<int32_t> pivots(m, -1);
    for (int64_t j = 0; j < m; j++) {
        const int32_t l = st.low[j];
        if (l >= 0 && (pivots[l] == -1 || j < pivots[l])) pivots[l] = (int32_t)j;
    }
    out.assign(4 * (size_t)(m + 1), 0.0);
    ms.assign((size_t)(m + 1), 0.0f);
    st.entry(out, 0);
    size_t e = 0;
    long long tprev = tk.ev_t0;
    int64_t kprev = 0;
    std::vector<std::pair<int32_t, int32_t>> nb;
    for (int64_t k = 1; k <= m; k++) {
        const int64_t i = m - k;
        nb.clear();
        if (e + 5 <= tk.ev.size() && tk.ev[e] == (int)i) {
            const int piv = tk.ev[e + 1], cnt = tk.ev[e + 2];
            const long long t = (long long)(uint32_t)tk.ev[e + 3] | ((long long)tk.ev[e + 4] << 32);
            for (int q = 0; q < cnt; q++) nb.emplace_back(tk.ev[e + 5 + 2 * q], tk.ev[e + 6 + 2 * q]);
            e += 5 + 2 * (size_t)cnt;
            std::sort(nb.begin(), nb.end());
            for (const auto &pr : nb) {
                const int32_t j = pr.first, nl = pr.second;
                if (!par) {
                    if (st.low[j] > -1) st.clear_ess(st.low[j]);
                    st.clear_ess(piv);
                    st.clear_ess(st.low[piv]);
                }
                st.set_low(j, nl);
                if (!par && nl >= 0) {
                    if (pivots[nl] == -1 || j < pivots[nl]) pivots[nl] = j;
                    if (pivots[nl] == j) {
                        st.set_cls(j, -1);
                        st.set_cls(nl, 1);
                        st.clear_ess(j);
                        st.clear_ess(nl);
                    }
                }
            }
            for (int64_t q = kprev + 1; q <= k; q++) ms[q] = (float)((t - tprev) * 1e-6 / (double)(k - kprev));
            tprev = t;
            kprev = k;
        }
        if (par) {
            if (k == 1) {
                for (int64_t c = 0; c < m; c++)
                    if (st.low[c] >= 0) st.clear_ess(st.low[c]);
            } else {
                for (const auto &pr : nb)
                    if (pr.second >= 0) st.clear_ess(pr.second);
            }
        } else if (i == 0) {
            for (int64_t c = 0; c < m; c++)
                if (st.low[c] > -1) {
                    st.clear_ess(c);
                    st.clear_ess(st.low[c]);
                    st.set_cls(c, -1);
                    st.set_cls(st.low[c], 1);
                }
            for (int64_t c = 0; c < m; c++)
                if (st.ess[c] == 1 && st.cls[c] == 0) st.set_cls(c, 2);
        }
        st.entry(out, k);
    }
}

extern "C" {

__attribute__((visibility("default"))) int oph_openph(const char *algstr, const int *h_rows_in, const int *h_cols_in,
                                                      int m, int col_width, const int *h_low_true, int nnz, int *h_low,
                                                      int *h_ess, float *err_linf, float *err_lone, float *err_redu,
                                                      float *err_ess, float *time_track, int *num_iters,
                                                      int gpu_number) {
    (void)col_width;  // capacity is adaptive
    const int algo = oph_algo_from_string(algstr);
    if (algo < 0) return OPH_ERR_ALGO;
    if (m < 0 || nnz < 0 || (nnz > 0 && (!h_rows_in || !h_cols_in)) || (m > 0 && !h_low)) return OPH_ERR_BAD_INPUT;
    // the reference clamps an out-of-range ordinal to 0 (functions.cu:49-56)
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return OPH_ERR_CUDA;
    }
    if (gpu_number < 0 || gpu_number >= ndev) gpu_number = 0;
    int rc = OPH_OK;
    oph_context *ctx = default_context(gpu_number, &rc);
    if (!ctx) return rc;
    OPH_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int64_t mm = m > 0 ? m : 1;
    int *d_r1 = (int *)ctx_alloc(ctx, S_COO_R, sizeof(int) * (nnz > 0 ? nnz : 1));
    int *d_c1 = (int *)ctx_alloc(ctx, S_COO_C, sizeof(int) * (nnz > 0 ? nnz : 1));
    int64_t *d_colptr = (int64_t *)ctx_alloc(ctx, S_COLPTR, sizeof(int64_t) * (m + 1));
    int32_t *d_rows = (int32_t *)ctx_alloc(ctx, S_ROWS, sizeof(int32_t) * (nnz > 0 ? nnz : 1));
    int32_t *d_out = (int32_t *)ctx_alloc(ctx, S_ESS, sizeof(int32_t) * 2 * mm);
    int32_t *d_lt = (int32_t *)ctx_alloc(ctx, S_LOWTRUE, sizeof(int32_t) * 2 * mm);
    double *d_acc = nullptr;
    if (!d_r1 || !d_c1 || !d_colptr || !d_rows || !d_out || !d_lt) return OPH_ERR_OOM;
    if (nnz > 0) {
        OPH_CUDA_TRY(cudaMemcpyAsync(d_r1, h_rows_in, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
        OPH_CUDA_TRY(cudaMemcpyAsync(d_c1, h_cols_in, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
    }
    Work w;
    rc = alloc_work(ctx, w, m);
    if (rc) return rc;
    // the status block must be clean before the conversion kernel reports into it
    OPH_CUDA_TRY(cudaMemsetAsync(w.st, 0, sizeof(DevStatus), s));
    rc = coo1_to_csc(ctx, d_r1, d_c1, nnz, m, d_colptr, d_rows);
    if (rc) return rc;
    DevStatus hs;
    if ((rc = ctx_sync_status(ctx, w, &hs))) return rc;
    if (hs.error) return OPH_ERR_BAD_INPUT;
    w.nnz = nnz;
    w.colptr = d_colptr;
    w.rows = d_rows;
    w.checked = true;  // the COO conversion validated every entry
    const bool track = h_low_true && (err_linf || err_lone || err_redu || err_ess);
    int32_t *lt0 = d_lt, *esst = d_lt + mm;
    if (track && m > 0) {
        // low_true arrives 1-based and is compared 0-based like the
        // reference (openph.cu:99-122); ess_true follows from it
        OPH_CUDA_TRY(cudaMemcpyAsync(lt0, h_low_true, sizeof(int) * m, cudaMemcpyHostToDevice, s));
        k_shift_down<<<grid_for(ctx, m), 256, 0, s>>>(lt0, m, lt0);
        k_ess_true<<<grid_for(ctx, m), 256, 0, s>>>(lt0, m, esst, 0);
        k_ess_true<<<grid_for(ctx, m), 256, 0, s>>>(lt0, m, esst, 1);
    }
    // pms records an entry per sweep (pms.cu:16,106); standard and twist an
    // entry per column (below); the row forms the initial and final state
    Tracking tr;
    const bool per_sweep = track && m > 0 && algo == OPH_ALGO_PMS;
    if (per_sweep) {
        tr.low_true = lt0;
        tr.ess_true = esst;
        tr.slots = (int)std::min<int64_t>(m + 1, MAX_TRACKED);
        tr.ess_hat = (uint8_t *)ctx_alloc(ctx, S_ESSHAT, (size_t)m);
        tr.acc = (double *)ctx_alloc(ctx, S_TRACK, sizeof(double) * (16 + 4 * (size_t)tr.slots));
        if (!tr.ess_hat || !tr.acc) return OPH_ERR_OOM;
        tr.acc += 16;
        ctx->track = &tr;
    } else if (track && m > 0) {
        d_acc = (double *)ctx_alloc(ctx, S_TRACK, sizeof(double) * (16 + 4 * 2));
        if (!d_acc) return OPH_ERR_OOM;
    }
    // the sequential algorithms record an entry per column (standard, twist)
    // or row (the row forms), replayed on the host after the walk
    SeqTracking stk;
    const bool per_col = track && m > 0 && algo != OPH_ALGO_PMS;
    if (per_col) ctx->seq_track = &stk;
    Outputs o;
    o.low = d_out;
    o.one_based = 1;
    o.ess = d_out + mm;
    oph_info info{};
    rc = reduce_core(ctx, algo, w, o, &info);
    ctx->track = nullptr;
    ctx->seq_track = nullptr;
    if (rc) return rc;
    if (m > 0) {
        OPH_CUDA_TRY(cudaMemcpyAsync(h_low, d_out, sizeof(int) * m, cudaMemcpyDeviceToHost, s));
        if (h_ess) OPH_CUDA_TRY(cudaMemcpyAsync(h_ess, d_out + mm, sizeof(int) * m, cudaMemcpyDeviceToHost, s));
    }
    const int it = info.num_iters > 0 ? info.num_iters : 1;
    double acc[16] = {0};
    std::vector<double> entries;
    if (track && m > 0) {
        // the final state, with the final essential estimate
        double *fin = per_sweep ? tr.acc - 16 : d_acc;
        OPH_CUDA_TRY(cudaMemsetAsync(fin, 0, sizeof(double) * 16, s));
        k_tracker<<<grid_for(ctx, m), 256, 0, s>>>(w.low, lt0, d_out + mm, esst, m, fin);
        OPH_CUDA_TRY(cudaMemcpyAsync(acc, fin, sizeof(double) * 16, cudaMemcpyDeviceToHost, s));
        if (per_sweep) {
            entries.resize(4 * (size_t)tr.slots);
            OPH_CUDA_TRY(cudaMemcpyAsync(entries.data(), tr.acc, sizeof(double) * entries.size(),
                                         cudaMemcpyDeviceToHost, s));
        }
    }
    std::vector<int32_t> h_low0, h_lt;  // the final lows (0-based) and low_true, for the replay
    if (per_col && stk.iters > 0) {
        h_low0.resize(m);
        h_lt.resize(m);
        OPH_CUDA_TRY(cudaMemcpyAsync(h_low0.data(), w.low, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
        OPH_CUDA_TRY(cudaMemcpyAsync(h_lt.data(), lt0, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
    }
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    if (num_iters) *num_iters = it;
    const int last = it - 1 < m ? it - 1 : m;
    const bool rows = algo == OPH_ALGO_PH_ROW || algo == OPH_ALGO_PH_ROW_PARALLEL;
    const bool replayed = per_col && stk.iters == it &&
                          (rows ? stk.rows_ok : (int64_t)stk.ns.size() == it);
    std::vector<float> row_ms;
    if (replayed) {
        if (rows) replay_row_trackers(stk, algo, h_lt, entries, row_ms);
        else replay_seq_trackers(stk, algo, h_low0, h_lt, entries);
    }
    if (time_track && m >= 1) {
        time_track[0] = 0.0f;
        if (replayed) {
            for (int k = 1; k <= last; k++)
                time_track[k] = rows ? row_ms[k] : (float)((stk.ns[k] - stk.ns[k - 1]) * 1e-6);
        } else if (per_sweep) {
            for (int k = 1; k < last && k - 1 < (int)tr.sweep_ms.size(); k++) time_track[k] = tr.sweep_ms[k - 1];
            time_track[last] = (int)tr.sweep_ms.size() >= last ? tr.sweep_ms[last - 1] : info.device_ms;
        } else {
            time_track[last] = info.device_ms;
        }
    }
    if (track && m > 0) {
        // normalised like openph.cu:184-193 (by the 1-based low_true's norms);
        // err_ess = ess_true / ess_hat, 1 when equal (tracker.cu:124-133)
        const double n1 = acc[4], ninf = acc[5], esst_sum = acc[3];
        auto put = [&](int k, double lone, double linf, double unclassified, double ess_hat) {
            if (err_lone) err_lone[k] = (float)(lone / n1);
            if (err_linf) err_linf[k] = (float)(linf / ninf);
            if (err_redu) err_redu[k] = (float)(unclassified / (double)m);
            if (err_ess) err_ess[k] = ess_hat == esst_sum ? 1.0f : (float)(esst_sum / ess_hat);
        };
        if (replayed) {
            // every entry, the last included, as the algorithm leaves it
            for (int k = 0; k <= last; k++)
                put(k, entries[4 * k], entries[4 * k + 1], entries[4 * k + 2], entries[4 * k + 3]);
        } else {
            if (per_sweep)
                for (int k = 0; k < last && k < tr.slots; k++)
                    put(k, entries[4 * k], entries[4 * k + 1], entries[4 * k + 2], entries[4 * k + 3]);
            // the last entry: the final lows, every column classified
            put(last, acc[0], acc[1], 0.0, acc[2]);
        }
    }
    return OPH_OK;
}

__attribute__((visibility("default"))) void openph(char *algstr, int *h_rows_in, int *h_cols_in, int m,
                                                   int col_width, int *h_low_true, int nnz, int *h_low, int *h_ess,
                                                   float *err_linf, float *err_lone, float *err_redu, float *err_ess,
                                                   float *time_track, int *num_iters, int gpu_number) {
    int rc = oph_openph(algstr, h_rows_in, h_cols_in, m, col_width, h_low_true, nnz, h_low, h_ess, err_linf,
                        err_lone, err_redu, err_ess, time_track, num_iters, gpu_number);
    if (rc != OPH_OK) {
        if (rc == OPH_ERR_ALGO) printf("Not recognised");
        else fprintf(stderr, "openph: %s\n", oph_status_string(rc));
        if (h_low)
            for (int i = 0; i < m; i++) h_low[i] = 0;
    }
}

}  // extern "C"

// ----------------------------------------------------------------- autotune
static int autotune_run(oph_context *ctx, int32_t *lanes, int32_t *cap, float *best_ms,
                        int (*run)(oph_context *, void *), void *arg) {
    int best = -1;
    float best_t = 0;
    for (int v = 0; v < T0_CANDIDATES; v++) {
        ctx->tier0 = v;
        int rc = run(ctx, arg);  // warm-up (and set-up of the candidate)
        if (rc) return rc;
        cudaEventRecord(ctx->ev[4], ctx->stream);
        rc = run(ctx, arg);
        if (rc) return rc;
        cudaEventRecord(ctx->ev[5], ctx->stream);
        cudaEventSynchronize(ctx->ev[5]);
        float t = 0;
        cudaEventElapsedTime(&t, ctx->ev[4], ctx->ev[5]);
        if (best < 0 || t < best_t) { best = v; best_t = t; }
    }
    ctx->tier0 = best;
    int l = 0, c = 0;
    t0_candidate(best, &l, &c);
    if (lanes) *lanes = l;
    if (cap) *cap = c;
    if (best_ms) *best_ms = best_t;
    return OPH_OK;
}

struct TuneOne { int64_t m; const int64_t *colptr; const int32_t *rows; int32_t *low; };
struct TuneBatch { int32_t count; const int64_t *col_off, *colptr; const int32_t *rows; int32_t *low; };

extern "C" {

__attribute__((visibility("default"))) int oph_context_set_dual(oph_context *ctx, int32_t mode) {
    if (!ctx || mode < OPH_DUAL_AUTO || mode > OPH_DUAL_BLOCKS) return OPH_ERR_BAD_INPUT;
    ctx->dual = mode;
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_context_set_tier0(oph_context *ctx, int32_t lanes, int32_t cap) {
    if (!ctx) return OPH_ERR_BAD_INPUT;
    for (int v = 0; v < T0_CANDIDATES; v++) {
        int l, c;
        t0_candidate(v, &l, &c);
        if (l == lanes && c == cap) {
            ctx->tier0 = v;
            return OPH_OK;
        }
    }
    return OPH_ERR_BAD_INPUT;
}

__attribute__((visibility("default"))) int oph_context_autotune(oph_context *ctx, int64_t m, const int64_t *colptr,
                                                                const int32_t *rows, int32_t *lanes, int32_t *cap,
                                                                float *best_ms) {
    if (!ctx || m < 0 || !colptr) return OPH_ERR_BAD_INPUT;
    std::vector<int32_t> low(m > 0 ? m : 1);
    TuneOne t{m, colptr, rows, low.data()};
    return autotune_run(ctx, lanes, cap, best_ms,
                        [](oph_context *c, void *p) {
                            TuneOne *a = (TuneOne *)p;
                            return oph_reduce(c, OPH_ALGO_PMS, a->m, a->colptr, a->rows, a->low, nullptr, nullptr,
                                              nullptr);
                        },
                        &t);
}

__attribute__((visibility("default"))) int oph_context_autotune_batch(oph_context *ctx, int32_t count,
                                                                      const int64_t *col_off, const int64_t *colptr,
                                                                      const int32_t *rows, int32_t *lanes,
                                                                      int32_t *cap, float *best_ms) {
    if (!ctx || count < 1 || !col_off || !colptr) return OPH_ERR_BAD_INPUT;
    std::vector<int32_t> low(col_off[count] > 0 ? col_off[count] : 1);
    TuneBatch t{count, col_off, colptr, rows, low.data()};
    return autotune_run(ctx, lanes, cap, best_ms,
                        [](oph_context *c, void *p) {
                            TuneBatch *a = (TuneBatch *)p;
                            return oph_reduce_batch(c, OPH_ALGO_PMS, a->count, a->col_off, a->colptr, a->rows,
                                                    a->low, nullptr, nullptr);
                        },
                        &t);
}

}  // extern "C"
