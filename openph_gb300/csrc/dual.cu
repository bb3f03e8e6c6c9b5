// pms on the anti-transposed matrix (the coboundary matrix of the reversed
// filtration), for complexes whose top dimension dwarfs the bottom one.
//
// For any Z/2 matrix D of m columns and its anti-transpose D' (entry (i, j)
// of D is entry (m-1-j, m-1-i) of D'), every lower-left submatrix of D' is
// the transpose of one of D, with the same rank; the low pairs of a reduced
// matrix are read off those ranks (low(j) = i iff
// r(i, j) - r(i+1, j) - r(i, j-1) + r(i+1, j-1) = 1, r(i, j) the rank of rows
// >= i of columns <= j), so
//     low_D(j) = i   <=>   low_D'(m-1-i) = m-1-j,
// and a column unpaired in D is unpaired in D'.  This is the duality of
// persistent homology and cohomology (de Silva, Morozov and
// Vejdemo-Johansson, "Dualities in persistent (co)homology", 2011), which
// Ripser (Bauer, 2021) uses to the same end.  low and ess are a function of
// those pairs, so reducing D' gives the reference's outputs bit for bit.
//
// The work moves: twist on D must reduce every column of the top dimension
// (nothing clears them), pms on D' every column of the bottom one.  A Rips
// complex truncated at triangles has ~10^4 times more triangles than
// vertices: 216M additions on the 5M-column torus, against a few thousand on
// D'.  A lower-star image is the other way round and stays on D.
//
// pms needs its dimension buckets graded (rows of distinct buckets disjoint).
// D' is given the buckets of D's columns (reversed), which are graded on D'
// exactly when every column of D takes its rows from one bucket and distinct
// buckets take them from distinct buckets; k_dual_grade checks that on the
// device, together with the structural checks of the set-up, and a matrix
// that fails stays on D.
#include <cub/device/device_radix_sort.cuh>

#include "oph_host.h"

namespace oph {

constexpr int TAB_NONE = -1000;  // no column of this bucket has rows yet

__device__ __forceinline__ int bucket_of(int64_t n) { return (int)(n - 1 > 126 ? 126 : n - 1); }

// Buckets of D: per-bucket column counts, the bucket the rows of each
// bucket's columns come from (tab, TAB_NONE if none, conflicts set *mixed),
// and the structural checks (colptr monotone within [0, nnz], rows strictly
// ascending and < m: *bad).
__global__ void k_dual_grade(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                             int64_t nnz, const int8_t *__restrict__ bucket, unsigned long long *count, int *tab,
                             int *mixed, int *bad) {
    __shared__ unsigned long long s_count[MAXC];
    __shared__ int s_tab[MAXC];
    __shared__ int s_flags[2];
    if (threadIdx.x < MAXC) {
        s_count[threadIdx.x] = 0;
        s_tab[threadIdx.x] = TAB_NONE;
    }
    if (threadIdx.x < 2) s_flags[threadIdx.x] = 0;
    __syncthreads();
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t lo = colptr[j], hi = colptr[j + 1];
        if (lo < 0 || hi < lo || hi > nnz) {  // bounds first: nothing is read past rows[nnz)
            s_flags[1] = 1;
            continue;
        }
        const int b = bucket_of(hi - lo);
        if (b + 1 >= MAXC) {  // a bucket the Phase I scan does not keep
            s_flags[0] = 1;
            continue;
        }
        atomicAdd(&s_count[b + 1], 1ull);
        int rb = TAB_NONE, prev = -1;
        for (int64_t k = lo; k < hi; k++) {
            const int r = rows[k];
            if (r <= prev || r >= m) {
                s_flags[1] = 1;
                break;
            }
            prev = r;
            const int br = bucket[r];
            if (k == lo) rb = br;
            else if (br != rb) s_flags[0] = 1;
        }
        if (rb != TAB_NONE) {
            const int old = atomicCAS(&s_tab[b + 1], TAB_NONE, rb);
            if (old != TAB_NONE && old != rb) s_flags[0] = 1;
        }
    }
    __syncthreads();
    if (threadIdx.x < MAXC) {
        if (s_count[threadIdx.x]) atomicAdd(&count[threadIdx.x], s_count[threadIdx.x]);
        const int t = s_tab[threadIdx.x];
        if (t != TAB_NONE) {
            const int old = atomicCAS(&tab[threadIdx.x], TAB_NONE, t);
            if (old != TAB_NONE && old != t) atomicExch(mixed, 1);
        }
    }
    if (threadIdx.x == 0) {
        if (s_flags[0]) atomicExch(mixed, 1);
        if (s_flags[1]) atomicExch(bad, 1);
    }
}

// Each column's bucket, one byte, for k_dual_grade's row lookups (a column
// whose colptr is out of bounds gets any value: k_dual_grade rejects it).
__global__ void k_dual_buckets(const int64_t *__restrict__ colptr, int64_t m, int8_t *__restrict__ bucket) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        bucket[j] = (int8_t)bucket_of(colptr[j + 1] - colptr[j]);
}

// left of D' without atomics: row m-1-j of D' first appears in column
// m-1-low_D(j) (the largest row of D's column j), for every nonempty j.
__global__ void k_dual_left(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                            PivRec *__restrict__ rec) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = colptr[j + 1];
        if (b > colptr[j]) rec[m - 1 - j].left = (int)(m - 1 - rows[b - 1]);
    }
}


// Sort keys of D': entry k of D (row r, column j) becomes key m-1-r (its
// column in D'), value m-1-j (its row), written at nnz-1-k so that a stable
// sort by key leaves the rows of each column of D' ascending.
__global__ void k_dual_keys(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                            int64_t nnz, uint32_t *__restrict__ key, int32_t *__restrict__ val) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        for (int64_t k = colptr[j]; k < colptr[j + 1]; k++) {
            key[nnz - 1 - k] = (uint32_t)(m - 1 - rows[k]);
            val[nnz - 1 - k] = (int32_t)(m - 1 - j);
        }
}

// colptr of D' from the sorted keys (each column's first entry writes the
// pointers of the empty columns before it).
__global__ void k_dual_colptr(const uint32_t *__restrict__ key, int64_t nnz, int64_t m, int64_t *__restrict__ colptr) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = key[k];
        const int64_t pc = k > 0 ? (int64_t)key[k - 1] : -1;
        if (pc != c)
            for (int64_t q = pc + 1; q <= c; q++) colptr[q] = k;
        if (k == nnz - 1)
            for (int64_t q = c + 1; q <= m; q++) colptr[q] = nnz;
    }
}

// The buckets of D' (those of D, reversed), over the ones the set-up derived
// from D' itself.
__global__ void k_dual_dims(const int64_t *__restrict__ colptr, int64_t m, int8_t *__restrict__ dim) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < m; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = m - 1 - c;
        dim[c] = (int8_t)bucket_of(colptr[i + 1] - colptr[i]);
    }
}

__global__ void k_dual_low_clear(int32_t *__restrict__ low, int64_t m) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        low[j] = -1;
}

// low_D(m-1-r) = m-1-c for every low r = low_D'(c).
__global__ void k_dual_low(const int32_t *__restrict__ low_d, int64_t m, int32_t *__restrict__ low) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < m; c += (int64_t)gridDim.x * blockDim.x) {
        const int r = low_d[c];
        if (r >= 0) low[m - 1 - r] = (int32_t)(m - 1 - c);
    }
}

static int grid_of(Context *ctx, int64_t n) {
    int64_t g = (n + 255) / 256, cap = (int64_t)ctx->sm_count * 16;
    return (int)std::max<int64_t>(1, std::min(g, cap));
}

void dual_left(Context *ctx, const Work &wd) {
    k_dual_left<<<grid_of(ctx, wd.m), 256, 0, ctx->stream>>>(wd.src_colptr, wd.src_rows, wd.m, wd.rec);
    ctx->launches++;
}

int dual_choose(Context *ctx, const Work &w, int mode, bool *use, bool *bad_input) {
    *use = false;
    *bad_input = false;
    if (mode == OPH_DUAL_NEVER || w.m == 0) return OPH_OK;
    cudaStream_t s = ctx->stream;
    struct Grade {
        unsigned long long count[MAXC];
        int tab[MAXC];
        int mixed, bad;
    };
    Grade *d = (Grade *)ctx_alloc(ctx, S_DGRADE, sizeof(Grade));
    if (!d) return OPH_ERR_OOM;
    Grade init{};
    for (int b = 0; b < MAXC; b++) init.tab[b] = TAB_NONE;
    OPH_CUDA_TRY(cudaMemcpyAsync(d, &init, sizeof(Grade), cudaMemcpyHostToDevice, s));
    // the buckets go through w.dim, which the set-up rewrites afterwards
    k_dual_buckets<<<grid_of(ctx, w.m), 256, 0, s>>>(w.colptr, w.m, w.dim);
    k_dual_grade<<<grid_of(ctx, w.m), 256, 0, s>>>(w.colptr, w.rows, w.m, w.nnz, w.dim, d->count, d->tab,
                                                    &d->mixed, &d->bad);
    ctx->launches += 2;
    OPH_CUDA_TRY(cudaGetLastError());
    Grade g;
    OPH_CUDA_TRY(cudaMemcpyAsync(&g, d, sizeof(Grade), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    if (g.bad) {
        *bad_input = true;
        return OPH_OK;
    }
    if (g.mixed) return OPH_OK;
    // distinct buckets must take their rows from distinct buckets
    for (int a = 0; a < MAXC; a++)
        for (int b = a + 1; b < MAXC; b++)
            if (g.tab[a] != TAB_NONE && g.tab[a] == g.tab[b]) return OPH_OK;
    int lo = -1, hi = -1;
    for (int b = 0; b < MAXC; b++)
        if (g.count[b]) {
            if (lo < 0) lo = b;
            hi = b;
        }
    if (mode == OPH_DUAL_ALWAYS) *use = true;
    else *use = w.m >= DUAL_MIN_M && lo >= 0 && hi > lo && g.count[lo] * DUAL_RATIO <= g.count[hi];
    return OPH_OK;
}

int dual_build(Context *ctx, const Work &w, Work &wd) {
    cudaStream_t s = ctx->stream;
    const int64_t m = w.m, nnz = w.nnz;
    int64_t *colptr = (int64_t *)ctx_alloc(ctx, S_DCOLPTR, sizeof(int64_t) * (m + 1));
    const size_t n1 = (size_t)(nnz > 0 ? nnz : 1);
    char *kv = (char *)ctx_alloc(ctx, S_DSORT, n1 * 4 * sizeof(int32_t));
    if (!colptr || !kv) return OPH_ERR_OOM;
    uint32_t *k0 = (uint32_t *)kv, *k1 = k0 + n1;
    int32_t *v0 = (int32_t *)(k1 + n1), *v1 = v0 + n1;
    wd = w;
    wd.colptr = colptr;
    wd.ascending = true;
    wd.src_colptr = w.colptr;
    wd.src_rows = w.rows;
    if (nnz == 0) {
        OPH_CUDA_TRY(cudaMemsetAsync(colptr, 0, sizeof(int64_t) * (m + 1), s));
        wd.rows = v0;
        return OPH_OK;
    }
    k_dual_keys<<<grid_of(ctx, m), 256, 0, s>>>(w.colptr, w.rows, m, nnz, k0, v0);
    int bits = 1;
    while (bits < 32 && (1ll << bits) < m) bits++;
    cub::DoubleBuffer<uint32_t> dk(k0, k1);
    cub::DoubleBuffer<int32_t> dv(v0, v1);
    size_t tb = 0;
    OPH_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, dk, dv, nnz, 0, bits, s));
    void *tmp = ctx_alloc(ctx, S_DTEMP, tb > 0 ? tb : 1);
    if (!tmp) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cub::DeviceRadixSort::SortPairs(tmp, tb, dk, dv, nnz, 0, bits, s));
    k_dual_colptr<<<grid_of(ctx, nnz), 256, 0, s>>>(dk.Current(), nnz, m, colptr);
    ctx->launches += 3 + (bits + 7) / 8;
    OPH_CUDA_TRY(cudaGetLastError());
    wd.rows = dv.Current();
    wd.entry_col = dk.Current();
    return OPH_OK;
}

void dual_dims(Context *ctx, const Work &w, Work &wd) {
    k_dual_dims<<<grid_of(ctx, w.m), 256, 0, ctx->stream>>>(w.colptr, w.m, wd.dim);
    ctx->launches++;
}

int dual_lows(Context *ctx, const Work &wd, int32_t **low) {
    cudaStream_t s = ctx->stream;
    const int64_t m = wd.m;
    int32_t *out = (int32_t *)ctx_alloc(ctx, S_DLOW, sizeof(int32_t) * (m > 0 ? m : 1));
    if (!out) return OPH_ERR_OOM;
    k_dual_low_clear<<<grid_of(ctx, m), 256, 0, s>>>(out, m);
    k_dual_low<<<grid_of(ctx, m), 256, 0, s>>>(wd.low, m, out);
    ctx->launches += 2;
    OPH_CUDA_TRY(cudaGetLastError());
    *low = out;
    return OPH_OK;
}

}  // namespace oph
