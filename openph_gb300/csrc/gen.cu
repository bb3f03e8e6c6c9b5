// Complexes built on the device: the Vietoris-Rips complex of a point cloud
// and the lower-star filtration of an image, as the sorted CSC boundary
// matrix the reduction consumes, with no host pass over the simplices.
//
// The input stand-ins of the reference's benchmarks (Javaplex streams,
// example_factory.m:17-114, stream2cmo.m:1-26) are generated on the host by
// gen/ophgen.c; these kernels produce the identical matrix (same filtration
// values, same order, same rows) from the points or the image already in
// HBM.  The order is (value, dimension, vertex tuple): every simplex gets a
// 128-bit key, the order-preserving bits of its FP64 value followed by a
// word holding its dimension and vertex ids, and one radix sort of the keys
// is the filtration order.  The key alone names the simplex, so the sorted
// keys are decoded back into columns: a position table per vertex and per
// edge turns each simplex's facets into row indices.
//
// Distances are summed in the host generator's order with separately
// rounded multiplies and adds (no FMA) and a correctly rounded square root,
// so every value, and with it the order, is bit-identical to the host's.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda/std/tuple>

#include "oph_host.h"

namespace oph {

namespace {

struct SKey {
    unsigned long long vb;   // order-preserving bits of the filtration value
    unsigned long long lex;  // dimension << 60 | a << 40 | b << 20 | c
};
struct SKeyDecomposer {
    __host__ __device__ cuda::std::tuple<unsigned long long &, unsigned long long &> operator()(SKey &k) const {
        return {k.vb, k.lex};
    }
};

__device__ __forceinline__ unsigned long long dbits(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dvalue(unsigned long long b) {
    const unsigned long long u = (b & 0x8000000000000000ull) ? (b & 0x7fffffffffffffffull) : ~b;
    return __longlong_as_double((long long)u);
}
__device__ __forceinline__ unsigned long long lexkey(int dim, unsigned a, unsigned b, unsigned c) {
    return ((unsigned long long)dim << 60) | ((unsigned long long)a << 40) | ((unsigned long long)b << 20) | c;
}

// ------------------------------------------------------------------ Rips
// Distances of every pair (upper triangle) and the adjacency bitsets: bit c
// of row a (words of 32) is set when a != c and |p_a - p_c| <= thr.
__global__ void k_rips_dist(const double *__restrict__ pts, int n, int d, double thr, double *__restrict__ D,
                            unsigned *__restrict__ adj, int words) {
    const int64_t pairs = (int64_t)n * n;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < pairs; q += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / n), b = (int)(q % n);
        if (b <= a) continue;
        double s = 0.0;
        for (int t = 0; t < d; t++) {
            const double x = __dsub_rn(pts[(int64_t)a * d + t], pts[(int64_t)b * d + t]);
            s = __dadd_rn(s, __dmul_rn(x, x));
        }
        const double v = __dsqrt_rn(s);
        D[(int64_t)a * n + b] = v;
        D[(int64_t)b * n + a] = v;
        if (v <= thr) {
            atomicOr(&adj[(int64_t)a * words + (b >> 5)], 1u << (b & 31));
            atomicOr(&adj[(int64_t)b * words + (a >> 5)], 1u << (a & 31));
        }
    }
}

// Bits of row r above column c (exclusive), within word w.
__device__ __forceinline__ unsigned above(int w, int c) {
    const int lo = w * 32;
    if (c < lo) return 0xffffffffu;
    if (c >= lo + 31) return 0u;
    return 0xffffffffu << ((c - lo) + 1);
}

// Edges per row (b > a), one thread per row.
__global__ void k_rips_deg(const unsigned *__restrict__ adj, int n, int words, long long *__restrict__ deg) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
        long long s = 0;
        for (int w = a >> 5; w < words; w++) s += __popc(adj[(int64_t)a * words + w] & above(w, a));
        deg[a] = s;
    }
}

// Triangles above every edge (a, b): common neighbours c > b.  One warp per
// row a walks its edges; lane-strided over the words.
__global__ void k_rips_tri_count(const unsigned *__restrict__ adj, int n, int words,
                                 const long long *__restrict__ eoff, long long *__restrict__ tcnt) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int a = wid; a < n; a += nw) {
        long long e = eoff[a];
        const unsigned *ra = adj + (int64_t)a * words;
        for (int wb = a >> 5; wb < words; wb++) {
            unsigned bits = ra[wb] & above(wb, a);
            while (bits) {
                const int b = wb * 32 + __ffs(bits) - 1;
                bits &= bits - 1;
                const unsigned *rb = adj + (int64_t)b * words;
                long long s = 0;
                for (int w = (b >> 5) + lane; w < words; w += 32) s += __popc(ra[w] & rb[w] & above(w, b));
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) tcnt[e] = s;
                e++;
            }
        }
    }
}

// Keys of every simplex: vertices at [0, n), edges at n + edge index, and
// the triangles of edge e at n + E + toff[e].
__global__ void k_rips_keys(const unsigned *__restrict__ adj, const double *__restrict__ D, int n, int words,
                            const long long *__restrict__ eoff, const long long *__restrict__ toff, long long E,
                            SKey *__restrict__ keys) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int a = wid; a < n; a += nw) {
        if (lane == 0) keys[a] = SKey{dbits(0.0), lexkey(0, a, 0, 0)};
        long long e = eoff[a];
        const unsigned *ra = adj + (int64_t)a * words;
        for (int wb = a >> 5; wb < words; wb++) {
            unsigned bits = ra[wb] & above(wb, a);
            while (bits) {
                const int b = wb * 32 + __ffs(bits) - 1;
                bits &= bits - 1;
                const double dab = D[(int64_t)a * n + b];
                if (lane == 0) keys[n + e] = SKey{dbits(dab), lexkey(1, a, b, 0)};
                const unsigned *rb = adj + (int64_t)b * words;
                long long t = n + E + toff[e];
                // common neighbours c > b in increasing c, lane-parallel by word
                for (int w0 = b >> 5; w0 < words; w0 += 32) {
                    const int w = w0 + lane;
                    const unsigned cm = w < words ? (ra[w] & rb[w] & above(w, b)) : 0u;
                    int cnt = __popc(cm);
                    int pre = cnt;
                    for (int o = 1; o < 32; o <<= 1) {
                        const int u = __shfl_up_sync(0xffffffffu, pre, o);
                        if (lane >= o) pre += u;
                    }
                    const int total = __shfl_sync(0xffffffffu, pre, 31);
                    long long slot = t + pre - cnt;
                    unsigned bitsc = cm;
                    while (bitsc) {
                        const int c = w * 32 + __ffs(bitsc) - 1;
                        bitsc &= bitsc - 1;
                        double v = dab;
                        const double dac = D[(int64_t)a * n + c], dbc = D[(int64_t)b * n + c];
                        if (dac > v) v = dac;
                        if (dbc > v) v = dbc;
                        keys[slot++] = SKey{dbits(v), lexkey(2, a, b, c)};
                    }
                    t += total;
                }
                e++;
            }
        }
    }
}

// Sorted keys -> position tables (vertex id, and edge (a, b) as a * n + b).
__global__ void k_rips_pos(const SKey *__restrict__ keys, int64_t m, int n, int32_t *__restrict__ vpos,
                           int32_t *__restrict__ epos) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long L = keys[r].lex;
        const int dim = (int)(L >> 60);
        const int a = (int)((L >> 40) & 0xfffff), b = (int)((L >> 20) & 0xfffff);
        if (dim == 0) vpos[a] = (int32_t)r;
        else if (dim == 1) epos[(int64_t)a * n + b] = (int32_t)r;
    }
}

// Column sizes and values.
__global__ void k_col_sizes(const SKey *__restrict__ keys, int64_t m, int64_t *__restrict__ cnt,
                            double *__restrict__ value) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        const int dim = (int)(keys[r].lex >> 60);
        cnt[r] = dim > 0 ? dim + 1 : 0;
        if (value) value[r] = dvalue(keys[r].vb);
    }
}

__device__ __forceinline__ void sort3(int32_t &x, int32_t &y, int32_t &z) {
    int32_t t;
    if (x > y) { t = x; x = y; y = t; }
    if (y > z) { t = y; y = z; z = t; }
    if (x > y) { t = x; x = y; y = t; }
}

__global__ void k_rips_rows(const SKey *__restrict__ keys, int64_t m, int n, const int32_t *__restrict__ vpos,
                            const int32_t *__restrict__ epos, const int64_t *__restrict__ colptr,
                            int32_t *__restrict__ rows) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long L = keys[r].lex;
        const int dim = (int)(L >> 60);
        const int a = (int)((L >> 40) & 0xfffff), b = (int)((L >> 20) & 0xfffff), c = (int)(L & 0xfffff);
        const int64_t k = colptr[r];
        if (dim == 1) {
            int32_t x = vpos[a], y = vpos[b];
            rows[k] = min(x, y);
            rows[k + 1] = max(x, y);
        } else if (dim == 2) {
            int32_t x = epos[(int64_t)a * n + b], y = epos[(int64_t)a * n + c], z = epos[(int64_t)b * n + c];
            sort3(x, y, z);
            rows[k] = x;
            rows[k + 1] = y;
            rows[k + 2] = z;
        }
    }
}

// ------------------------------------------------------------ lower star
// Vertex (y, x) = y * w + x; edges H(y, x) = (y,x)-(y,x+1), V = (y,x)-(y+1,x),
// D = (y,x)-(y+1,x+1); triangles per square: upper (y,x),(y,x+1),(y+1,x+1)
// and lower (y,x),(y+1,x),(y+1,x+1).
__global__ void k_ls_keys(const float *__restrict__ img, int h, int w, SKey *__restrict__ keys) {
    const int64_t V = (int64_t)h * w, EH = (int64_t)h * (w - 1), EV = (int64_t)(h - 1) * w,
                  ED = (int64_t)(h - 1) * (w - 1);
    const int64_t m = V + EH + EV + ED + 2 * ED;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x) {
        int64_t t = q;
        SKey k;
        if (t < V) {
            k = SKey{dbits((double)img[t]), lexkey(0, (unsigned)t, 0, 0)};
        } else if ((t -= V) < EH + EV + ED) {
            unsigned a, b;
            if (t < EH) {
                const int y = (int)(t / (w - 1)), x = (int)(t % (w - 1));
                a = y * w + x; b = a + 1;
            } else if ((t -= EH) < EV) {
                const int y = (int)(t / w), x = (int)(t % w);
                a = y * w + x; b = a + w;
            } else {
                t -= EV;
                const int y = (int)(t / (w - 1)), x = (int)(t % (w - 1));
                a = y * w + x; b = a + w + 1;
            }
            const double va = (double)img[a], vb = (double)img[b];
            k = SKey{dbits(va > vb ? va : vb), lexkey(1, a, b, 0)};
        } else {
            t -= EH + EV + ED;
            const int64_t sq = t >> 1;
            const int up = (t & 1) == 0;  // the host emits the upper triangle first
            const int y = (int)(sq / (w - 1)), x = (int)(sq % (w - 1));
            const unsigned a = y * w + x, b = up ? a + 1 : a + w, c = a + w + 1;
            double v = (double)img[a];
            if ((double)img[b] > v) v = (double)img[b];
            if ((double)img[c] > v) v = (double)img[c];
            k = SKey{dbits(v), lexkey(2, a, b, c)};
        }
        keys[q] = k;
    }
}

__device__ __forceinline__ int64_t ls_edge(unsigned a, unsigned b, int h, int w) {
    const int64_t V = (int64_t)h * w, EH = (int64_t)h * (w - 1), EV = (int64_t)(h - 1) * w;
    const int y = (int)(a / w), x = (int)(a % w);
    if (b == a + 1) return V + (int64_t)y * (w - 1) + x;
    if (b == a + (unsigned)w) return V + EH + (int64_t)y * w + x;
    return V + EH + EV + (int64_t)y * (w - 1) + x;
}

__global__ void k_ls_pos(const SKey *__restrict__ keys, int64_t m, int h, int w, int32_t *__restrict__ pos) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long L = keys[r].lex;
        const int dim = (int)(L >> 60);
        const unsigned a = (unsigned)((L >> 40) & 0xfffff), b = (unsigned)((L >> 20) & 0xfffff);
        if (dim == 0) pos[a] = (int32_t)r;
        else if (dim == 1) pos[ls_edge(a, b, h, w)] = (int32_t)r;
    }
}

__global__ void k_ls_rows(const SKey *__restrict__ keys, int64_t m, int h, int w, const int32_t *__restrict__ pos,
                          const int64_t *__restrict__ colptr, int32_t *__restrict__ rows) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long L = keys[r].lex;
        const int dim = (int)(L >> 60);
        const unsigned a = (unsigned)((L >> 40) & 0xfffff), b = (unsigned)((L >> 20) & 0xfffff),
                       c = (unsigned)(L & 0xfffff);
        const int64_t k = colptr[r];
        if (dim == 1) {
            const int32_t x = pos[a], y = pos[b];
            rows[k] = min(x, y);
            rows[k + 1] = max(x, y);
        } else if (dim == 2) {
            int32_t x = pos[ls_edge(a, b, h, w)], y = pos[ls_edge(b, c, h, w)], z = pos[ls_edge(a, c, h, w)];
            sort3(x, y, z);
            rows[k] = x;
            rows[k + 1] = y;
            rows[k + 2] = z;
        }
    }
}

int grid_of(Context *ctx, int64_t n) {
    const int64_t g = (n + 255) / 256, cap = (int64_t)ctx->sm_count * 16;
    return (int)std::max<int64_t>(1, std::min(g, cap));
}

// Scratch of one generator call, released on every exit.
struct Scratch {
    cudaStream_t s;
    std::vector<void *> ptrs;
    explicit Scratch(cudaStream_t st) : s(st) {}
    void *get(size_t bytes) {
        void *p = nullptr;
        if (cudaMallocAsync(&p, bytes ? bytes : 16, s) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        ptrs.push_back(p);
        return p;
    }
    ~Scratch() {
        for (void *p : ptrs) cudaFreeAsync(p, s);
    }
};

// Sort the keys, then sizes, values and column pointers; returns the
// sorted keys (in k0 or k1).
int sort_and_colptr(Context *ctx, Scratch &sc, SKey *k0, SKey *k1, int64_t m, int64_t *d_colptr, double *d_value,
                    SKey **sorted) {
    cudaStream_t s = ctx->stream;
    cub::DoubleBuffer<SKey> db(k0, k1);
    size_t tb = 0;
    OPH_CUDA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, tb, db, m, SKeyDecomposer{}, 0, 128, s));
    void *tmp = sc.get(tb);
    if (!tmp) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cub::DeviceRadixSort::SortKeys(tmp, tb, db, m, SKeyDecomposer{}, 0, 128, s));
    *sorted = db.Current();
    // colptr = exclusive scan of the column sizes, colptr[m] = nnz
    int64_t *cnt = (int64_t *)sc.get(sizeof(int64_t) * (size_t)(m + 1));
    if (!cnt) return OPH_ERR_OOM;
    k_col_sizes<<<grid_of(ctx, m), 256, 0, s>>>(*sorted, m, cnt, d_value);
    OPH_CUDA_TRY(cudaMemsetAsync(cnt + m, 0, sizeof(int64_t), s));
    size_t sb = 0;
    OPH_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, sb, cnt, d_colptr, m + 1, s));
    void *st = sc.get(sb);
    if (!st) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cub::DeviceScan::ExclusiveSum(st, sb, cnt, d_colptr, m + 1, s));
    return OPH_OK;
}

}  // namespace

}  // namespace oph

using namespace oph;

extern "C" {

__attribute__((visibility("default"))) int oph_rips_device(oph_context *ctx, const double *d_points, int n, int d,
                                                           double threshold, int64_t *m_out, int64_t *nnz_out,
                                                           int64_t *d_colptr, int32_t *d_rows, double *d_value) {
    if (!ctx || n <= 0 || n > OPH_GEN_MAX_POINTS || d <= 0 || !d_points || threshold != threshold)
        return OPH_ERR_BAD_INPUT;
    OPH_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    Scratch sc(s);
    const int words = (n + 31) / 32;
    double *D = (double *)sc.get(sizeof(double) * (size_t)n * n);
    unsigned *adj = (unsigned *)sc.get(sizeof(unsigned) * (size_t)n * words);
    long long *deg = (long long *)sc.get(sizeof(long long) * (size_t)(n + 1));
    long long *eoff = (long long *)sc.get(sizeof(long long) * (size_t)(n + 1));
    if (!D || !adj || !deg || !eoff) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cudaMemsetAsync(adj, 0, sizeof(unsigned) * (size_t)n * words, s));
    k_rips_dist<<<grid_of(ctx, (int64_t)n * n), 256, 0, s>>>(d_points, n, d, threshold, D, adj, words);
    k_rips_deg<<<grid_of(ctx, n), 256, 0, s>>>(adj, n, words, deg);
    OPH_CUDA_TRY(cudaMemsetAsync(deg + n, 0, sizeof(long long), s));
    size_t sb = 0;
    OPH_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, sb, deg, eoff, n + 1, s));
    void *st = sc.get(sb);
    if (!st) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cub::DeviceScan::ExclusiveSum(st, sb, deg, eoff, n + 1, s));
    long long E = 0;
    OPH_CUDA_TRY(cudaMemcpyAsync(&E, eoff + n, sizeof(long long), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    long long *tcnt = (long long *)sc.get(sizeof(long long) * (size_t)(E + 1));
    long long *toff = (long long *)sc.get(sizeof(long long) * (size_t)(E + 1));
    if (!tcnt || !toff) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cudaMemsetAsync(tcnt, 0, sizeof(long long) * (size_t)(E + 1), s));
    const int wgrid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 7) / 8, (int64_t)ctx->sm_count * 8));
    if (E > 0) k_rips_tri_count<<<wgrid, 256, 0, s>>>(adj, n, words, eoff, tcnt);
    size_t sb2 = 0;
    OPH_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, sb2, tcnt, toff, E + 1, s));
    void *st2 = sc.get(sb2);
    if (!st2) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cub::DeviceScan::ExclusiveSum(st2, sb2, tcnt, toff, E + 1, s));
    long long T = 0;
    OPH_CUDA_TRY(cudaMemcpyAsync(&T, toff + E, sizeof(long long), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    const int64_t m = n + E + T, nnz = 2 * E + 3 * T;
    if (m >= (1ll << 31)) return OPH_ERR_BAD_INPUT;
    if (m_out) *m_out = m;
    if (nnz_out) *nnz_out = nnz;
    if (!d_colptr) return OPH_OK;  // sizes only
    if (!d_rows && nnz > 0) return OPH_ERR_BAD_INPUT;
    SKey *k0 = (SKey *)sc.get(sizeof(SKey) * (size_t)m), *k1 = (SKey *)sc.get(sizeof(SKey) * (size_t)m);
    int32_t *vpos = (int32_t *)sc.get(sizeof(int32_t) * (size_t)n);
    int32_t *epos = (int32_t *)sc.get(sizeof(int32_t) * (size_t)n * n);
    if (!k0 || !k1 || !vpos || !epos) return OPH_ERR_OOM;
    k_rips_keys<<<wgrid, 256, 0, s>>>(adj, D, n, words, eoff, toff, E, k0);
    SKey *sorted = nullptr;
    int rc = sort_and_colptr(ctx, sc, k0, k1, m, d_colptr, d_value, &sorted);
    if (rc) return rc;
    k_rips_pos<<<grid_of(ctx, m), 256, 0, s>>>(sorted, m, n, vpos, epos);
    k_rips_rows<<<grid_of(ctx, m), 256, 0, s>>>(sorted, m, n, vpos, epos, d_colptr, d_rows);
    OPH_CUDA_TRY(cudaGetLastError());
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_lower_star_device(oph_context *ctx, const float *d_image, int h,
                                                                 int w, int64_t *m_out, int64_t *nnz_out,
                                                                 int64_t *d_colptr, int32_t *d_rows,
                                                                 double *d_value) {
    if (!ctx || h < 2 || w < 2 || (int64_t)h * w >= (1ll << 20) || !d_image) return OPH_ERR_BAD_INPUT;
    const int64_t V = (int64_t)h * w, ED = (int64_t)(h - 1) * (w - 1);
    const int64_t E = (int64_t)h * (w - 1) + (int64_t)(h - 1) * w + ED, T = 2 * ED;
    const int64_t m = V + E + T, nnz = 2 * E + 3 * T;
    if (m_out) *m_out = m;
    if (nnz_out) *nnz_out = nnz;
    if (!d_colptr) return OPH_OK;
    if (!d_rows) return OPH_ERR_BAD_INPUT;
    OPH_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    Scratch sc(s);
    SKey *k0 = (SKey *)sc.get(sizeof(SKey) * (size_t)m), *k1 = (SKey *)sc.get(sizeof(SKey) * (size_t)m);
    int32_t *pos = (int32_t *)sc.get(sizeof(int32_t) * (size_t)(V + E));
    if (!k0 || !k1 || !pos) return OPH_ERR_OOM;
    k_ls_keys<<<grid_of(ctx, m), 256, 0, s>>>(d_image, h, w, k0);
    SKey *sorted = nullptr;
    int rc = sort_and_colptr(ctx, sc, k0, k1, m, d_colptr, d_value, &sorted);
    if (rc) return rc;
    k_ls_pos<<<grid_of(ctx, m), 256, 0, s>>>(sorted, m, h, w, pos);
    k_ls_rows<<<grid_of(ctx, m), 256, 0, s>>>(sorted, m, h, w, pos, d_colptr, d_rows);
    OPH_CUDA_TRY(cudaGetLastError());
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    return OPH_OK;
}

}  // extern "C"
