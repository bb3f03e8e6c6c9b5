// Set-up of a reduction on the device: input conversion, the adaptive column
// store, the initial low array, dimension buckets and the alpha/beta tables.
//
// Reference counterparts (all replaced, none ported):
//   create_rows / create_rows_mp  src/cuda/functions.cu:68-91, src/cuda/kernels.cu:25-38
//   compute_low                   src/cuda/kernels.cu:40-52
//   compute_simplex_dimensions_h  src/cuda/dimensions.cu:54-104 (host, single thread)
//   create_beta_h / create_beta   src/cuda/algorithms/pms/beta.cu:2-26 (host, single thread)
//   assert_col_order              src/cuda/functions.cu:27-35 (warning only)
#include <algorithm>

#include "oph_host.h"

namespace oph {

// 1-based COO (column-major) -> 0-based CSC.  Validates ranges, column order
// and strictly ascending rows inside a column; any violation sets st->error.
__global__ void k_coo1_to_csc(const int *__restrict__ r1, const int *__restrict__ c1, int64_t nnz, int64_t m,
                              int64_t *__restrict__ colptr, int32_t *__restrict__ rows0, DevStatus *st) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        int r = r1[k], c = c1[k];
        bool bad = r < 1 || r > m || c < 1 || c > m;
        int pc = 0;
        if (k > 0) {
            pc = c1[k - 1];
            if (pc > c) bad = true;
            else if (pc == c && r1[k - 1] >= r) bad = true;
        }
        if (bad) { atomicExch(&st->error, 1); continue; }
        rows0[k] = r - 1;
        if (k == 0 || pc != c)
            for (int64_t q = (k == 0 ? 0 : pc); q < c; q++) colptr[q] = k;  // columns pc+1 .. c (1-based)
        if (k == nnz - 1)
            for (int64_t q = c; q <= m; q++) colptr[q] = nnz;
    }
}

// Structural check of a 0-based CSC before any kernel indexes through it:
// colptr[0] == 0, colptr non-decreasing within [0, nnz], rows strictly
// ascending inside a column and below the column count of their matrix —
// m, or, for a batch (inst_off != nullptr), the size of the column's
// instance, whose offsets must run from 0 to m without decreasing.  Only
// reads; any violation sets *bad.  Bounds come first: no row is read
// outside [0, nnz) and no offset outside [0, count].  With rows_out (a
// batch), every checked entry is also written there shifted into its
// instance's column range (the rows of a batch as one block-diagonal matrix).
__global__ void k_check_csc(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                            int64_t nnz, const int64_t *__restrict__ inst_off, int count, int *bad,
                            int32_t *__restrict__ rows_out) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    if (tid == 0 && (colptr[0] != 0 || colptr[m] != nnz)) atomicExch(bad, 1);
    if (inst_off) {
        for (int64_t b = tid; b < count; b += stride)
            if (inst_off[b] > inst_off[b + 1] || (b == 0 && inst_off[0] != 0) ||
                (b == count - 1 && inst_off[count] != m))
                atomicExch(bad, 1);
    }
    for (int64_t j = tid; j < m; j += stride) {
        const int64_t lo = colptr[j], hi = colptr[j + 1];
        if (lo < 0 || hi < lo || hi > nnz) {
            atomicExch(bad, 1);
            continue;
        }
        int64_t lim = m, base = 0;
        if (inst_off) {
            int a = 0, z = count;  // last b with inst_off[b] <= j (bounded steps whatever the offsets)
            while (z - a > 1) {
                const int mid = (a + z) >> 1;
                if (inst_off[mid] <= j) a = mid; else z = mid;
            }
            base = inst_off[a];
            lim = inst_off[a + 1] - base;
        }
        int prev = -1;
        for (int64_t k = lo; k < hi; k++) {
            const int r = rows[k];
            if (r <= prev || r >= lim) {
                atomicExch(bad, 1);
                break;
            }
            prev = r;
            if (rows_out) rows_out[k] = r + (int32_t)base;
        }
    }
}

// Per column: segment (start = 8j + 4*ceil(colptr[j]/4), which leaves room for
// the 4-int header and rounds every capacity up to a multiple of 4 without a
// prefix scan), rows copied in, low = last row, dim = nnz - 1.  Rows must be
// strictly ascending and < m.
__global__ void k_setup_columns(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                                int *__restrict__ pool, int64_t *__restrict__ seg, int32_t *__restrict__ low,
                                int8_t *__restrict__ dim, DevStatus *st) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = colptr[j], b = colptr[j + 1];
        int64_t s = 8 * j + 4 * ((a + 3) >> 2);
        int64_t e = 8 * (j + 1) + 4 * ((b + 3) >> 2);
        int n = (int)(b - a);
        seg[j] = s;
        pool[s] = n;
        pool[s + 1] = (int)(e - s - SEG_HDR);
        pool[s + 2] = 0;
        pool[s + 3] = 0;
        int prev = -1;
        bool bad = n < 0;
        for (int64_t k = a; k < b; k++) {
            int r = rows[k];
            if (r <= prev || r >= m) bad = true;
            pool[s + SEG_HDR + (k - a)] = r;
            prev = r;
        }
        if (bad) atomicExch(&st->error, 1);
        low[j] = n > 0 ? rows[b - 1] : -1;
        dim[j] = (int8_t)(n - 1 > 126 ? 126 : n - 1);
        if (n - 1 > MAXC - 2) atomicMax(&st->max_dim, n - 1);
    }
}

// left[i] = first column holding row i (atomicMin over the entries, into
// the pivot records, which start as the 0x7f byte pattern).
__global__ void k_left(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                       PivRec *__restrict__ rec) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        for (int64_t k = colptr[j]; k < colptr[j + 1]; k++) atomicMin(&rec[rows[k]].left, (int)j);
}

// beta[j] = largest row whose first column is j; each record is then set to
// "no pivot" with its left (-1 where no column holds the row).
__global__ void k_beta(PivRec *__restrict__ rec, int64_t m, int32_t *__restrict__ beta) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        int l = rec[i].left;
        if (l == FIRST_NONE) l = -1;
        else atomicMax(&beta[l], (int)i);
        int4 *r = reinterpret_cast<int4 *>(rec + i);
        r[0] = make_int4(-1, 0, l, (int)SEG4_NONE);
        r[1] = make_int4(-1, -1, -1, -1);
    }
}

static int grid_for(Context *ctx, int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)ctx->sm_count * 16;
    if (g > cap) g = cap;
    return g < 1 ? 1 : (int)g;
}

int check_csc(Context *ctx, const int64_t *d_colptr, const int32_t *d_rows, int64_t m, int64_t nnz,
              const int64_t *d_inst_off, int count, int32_t *d_rows_out) {
    int *d_bad = (int *)ctx_alloc(ctx, S_CHECK, sizeof(int));
    if (!d_bad) return OPH_ERR_OOM;
    cudaStream_t s = ctx->stream;
    OPH_CUDA_TRY(cudaMemsetAsync(d_bad, 0, sizeof(int), s));
    k_check_csc<<<grid_for(ctx, std::max<int64_t>(m, count), 256), 256, 0, s>>>(d_colptr, d_rows, m, nnz,
                                                                                d_inst_off, count, d_bad, d_rows_out);
    ctx->launches++;
    OPH_CUDA_TRY(cudaGetLastError());
    int bad = 0;
    OPH_CUDA_TRY(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    return bad ? OPH_ERR_BAD_INPUT : OPH_OK;
}

int coo1_to_csc(Context *ctx, const int *d_rows1, const int *d_cols1, int64_t nnz, int64_t m, int64_t *d_colptr,
                int32_t *d_rows0) {
    if (nnz == 0) {
        OPH_CUDA_TRY(cudaMemsetAsync(d_colptr, 0, sizeof(int64_t) * (m + 1), ctx->stream));
        return OPH_OK;
    }
    DevStatus *st = (DevStatus *)ctx->bufs[S_STATUS].ptr;
    k_coo1_to_csc<<<grid_for(ctx, nnz, 256), 256, 0, ctx->stream>>>(d_rows1, d_cols1, nnz, m, d_colptr, d_rows0, st);
    OPH_CUDA_TRY(cudaGetLastError());
    return OPH_OK;
}

// Initial pool: the packed segments plus room for growth.
static int64_t initial_pool_ints(Context *ctx, int64_t m, int64_t nnz) {
    int64_t packed = 8 * (m + 1) + 4 * ((nnz + 3) / 4) + 64;
    if (ctx->initial_pool_bytes > 0) {
        int64_t want = ctx->initial_pool_bytes / 4;
        return want > packed ? want : packed;
    }
    return packed * 4 + (16 << 20);
}

int init_store(Context *ctx, Work &w) {
    const int64_t m = w.m;
    int64_t pool_ints = initial_pool_ints(ctx, m, w.nnz);
    // tail padding: narrow-tier kernels read up to a group's width past a
    // segment start
    w.pool = (int *)ctx_alloc(ctx, S_POOL, sizeof(int) * (pool_ints + POOL_PAD));
    if (!w.pool) return OPH_ERR_OOM;
    ctx->pool_ints = pool_ints;
    const int64_t used = 8 * (m + 1) + 4 * ((w.nnz + 3) / 4) + 64;
    DevStatus init{};
    init.pool_used = (unsigned long long)((used + 3) & ~3ll);
    init.pool_size = (unsigned long long)pool_ints;
    init.max_dim = -1;
    OPH_CUDA_TRY(cudaMemcpyAsync(w.st, &init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
    return OPH_OK;
}

int setup_store(Context *ctx, Work &w, bool need_beta) {
    const int64_t m = w.m;
    int rc = init_store(ctx, w);
    if (rc) return rc;
    if (m == 0) return OPH_OK;
    if (need_beta) {
        OPH_CUDA_TRY(cudaMemsetAsync(w.rec, 0x7f, sizeof(PivRec) * m, ctx->stream));
        OPH_CUDA_TRY(cudaMemsetAsync(w.beta, 0xff, sizeof(int32_t) * m, ctx->stream));
    }
    k_setup_columns<<<grid_for(ctx, m, 256), 256, 0, ctx->stream>>>(w.colptr, w.rows, m, w.pool, w.seg, w.low,
                                                                    w.dim, w.st);
    if (need_beta) k_left<<<grid_for(ctx, m, 256), 256, 0, ctx->stream>>>(w.colptr, w.rows, m, w.rec);
    OPH_CUDA_TRY(cudaGetLastError());
    if (need_beta) {
        k_beta<<<grid_for(ctx, m, 256), 256, 0, ctx->stream>>>(w.rec, m, w.beta);
        OPH_CUDA_TRY(cudaGetLastError());
    }
    return OPH_OK;
}

// Grow the column store after an overflow: a larger pool, the used prefix
// copied over (segment offsets are pool-relative, so nothing else changes),
// the overflow flag cleared.
int grow_pool(Context *ctx, Work &w) {
    DevStatus hs;
    OPH_CUDA_TRY(cudaMemcpyAsync(&hs, w.st, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
    OPH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    int64_t used = (int64_t)(hs.pool_used < hs.pool_size ? hs.pool_used : hs.pool_size);
    int64_t want = ctx->pool_ints * 2;
    if (want < used + (16 << 20)) want = used + (16 << 20);
    if (want >= MAX_POOL_INTS) return OPH_ERR_OVERFLOW;
    int *np = (int *)ctx_alloc(ctx, S_POOL2, sizeof(int) * (want + POOL_PAD));
    if (!np) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cudaMemcpyAsync(np, w.pool, sizeof(int) * used, cudaMemcpyDeviceToDevice, ctx->stream));
    // swap the two pool slots so the larger one becomes the pool
    DevBuf t = ctx->bufs[S_POOL];
    ctx->bufs[S_POOL] = ctx->bufs[S_POOL2];
    ctx->bufs[S_POOL2] = t;
    w.pool = np;
    ctx->pool_ints = want;
    unsigned long long fields[2] = {(unsigned long long)used, (unsigned long long)want};
    OPH_CUDA_TRY(cudaMemcpyAsync(&w.st->pool_used, fields, sizeof(fields), cudaMemcpyHostToDevice, ctx->stream));
    int zero = 0;
    OPH_CUDA_TRY(cudaMemcpyAsync(&w.st->overflow, &zero, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    OPH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return OPH_OK;
}

}  // namespace oph
