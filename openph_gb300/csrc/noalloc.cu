// oph_reduce_pms_noalloc: the pms reduction for callers that cannot allocate
// device memory.
//
// Some callers own all of the device's memory, or must not call cudaMalloc
// at all: a host framework whose caching allocator holds the GPU (MATLAB's
// GPU arrays, PyTorch's caching allocator), or a real-time pipeline where
// cudaMalloc's implicit device synchronisation is not acceptable.  For them
// this entry point reduces a small matrix with every working array carved out
// of one fixed file-scope device array (NOALLOC_SCRATCH_BYTES, held by every
// GPU that loads the library until the process exits).  The caller passes
// the device input and output buffers and a stream; nothing here calls
// cudaMalloc, cudaFree, cudaMallocHost or any allocating library routine.
//
// The call is synchronous: it reads the input's size and the convergence
// status back to the host and waits on the stream, so it must not be issued
// on a stream that is being captured into a CUDA graph.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (once per device, with that device current) and
// keeps it for the life of the process; a cudaDeviceReset invalidates it, so
// the entry point is not for use after a device reset.  All calls share the
// one array: calls that overlap on the GPU (two streams, two threads) race
// and corrupt each other, so serialise them.  Each call re-initialises every
// part of the array it reads, so nothing from the previous call leaks into
// the next.
#include <algorithm>
#include <mutex>

#include "pms.cuh"

namespace oph {

// kernels of the single-matrix path (setup.cu, capi.cu), launched unchanged
__global__ void k_setup_columns(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                                int *__restrict__ pool, int64_t *__restrict__ seg, int32_t *__restrict__ low,
                                int8_t *__restrict__ dim, DevStatus *st);
__global__ void k_check_csc(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                            int64_t nnz, const int64_t *__restrict__ inst_off, int count, int *bad,
                            int32_t *__restrict__ rows_out);
__global__ void k_left(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                       PivRec *__restrict__ rec);
__global__ void k_beta(PivRec *__restrict__ rec, int64_t m, int32_t *__restrict__ beta);
__global__ void k_finalize1(const int32_t *__restrict__ low, int64_t m, int one_based, int ess_mode,
                            const int64_t *__restrict__ inst_off, int count, int32_t *__restrict__ out_low,
                            int32_t *__restrict__ ess, int32_t *__restrict__ arglow);
__global__ void k_finalize2(const int32_t *__restrict__ low, int64_t m, const int64_t *__restrict__ inst_off,
                            int count, int32_t *__restrict__ ess, int32_t *__restrict__ arglow);

constexpr size_t NOALLOC_SCRATCH_BYTES = 32u << 20;

// The scratch.  Host code must not use this name as an address (it is a host
// stand-in); the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_mu;
void *g_addr[64];
int g_sm[64];

// Device address of the scratch on the current device (looked up once).
int scratch_address(int dev, unsigned char **out, int *sm) {
    if (dev < 0 || dev >= 64) return OPH_ERR_BAD_INPUT;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "openph_gb300: cudaGetSymbolAddress of the no-allocation scratch failed: %s\n",
                    cudaGetErrorString(e));
            cudaGetLastError();
            return OPH_ERR_CUDA;
        }
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return OPH_ERR_CUDA;
        g_sm[dev] = n;
        g_addr[dev] = p;
    }
    *out = (unsigned char *)g_addr[dev];
    *sm = g_sm[dev];
    return OPH_OK;
}

// Bump carving of the scratch, 256-byte aligned.
struct Carver {
    unsigned char *base;
    size_t off = 0;
    template <class T>
    T *take(size_t count) {
        off = (off + 255) & ~(size_t)255;
        T *p = reinterpret_cast<T *>(base + off);
        off += sizeof(T) * count;
        return p;
    }
};

}  // namespace

}  // namespace oph

using namespace oph;

extern "C" __attribute__((visibility("default"))) int oph_reduce_pms_noalloc(int64_t m, const int64_t *d_colptr,
                                                                             const int32_t *d_rows, int32_t *d_low,
                                                                             int32_t *d_ess, void *stream) {
    if (m < 0 || m >= (1ll << 29) || !d_colptr || (m > 0 && !d_low)) return OPH_ERR_BAD_INPUT;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sm = 0;
    OPH_CUDA_TRY(cudaGetDevice(&dev));
    unsigned char *scratch = nullptr;
    int rc = scratch_address(dev, &scratch, &sm);
    if (rc) return rc;
    int64_t nnz = 0;
    OPH_CUDA_TRY(cudaMemcpyAsync(&nnz, d_colptr + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    if (nnz < 0 || (nnz > 0 && !d_rows)) return OPH_ERR_BAD_INPUT;
    if (m == 0) return OPH_OK;

    // carve the working arrays; the column store gets what is left, and must
    // hold twice the packed input
    Carver c{scratch};
    PmsArgs a{};
    DevStatus *st = c.take<DevStatus>(1);
    a.m = m;
    a.low = c.take<int32_t>(m);
    a.classes = c.take<int8_t>(m);
    a.clear = c.take<uint8_t>(m);
    int8_t *dim = c.take<int8_t>(m);
    a.dim = dim;
    a.first = c.take<int32_t>(m);
    int32_t *beta = c.take<int32_t>(m);
    a.beta = beta;
    a.worklist = c.take<int32_t>(m);
    a.widelist = c.take<int32_t>(m);
    a.slist = c.take<int32_t>(m);
    a.seg = c.take<int64_t>(m);
    a.rec = c.take<PivRec>(m);
    a.ntiles = (m + 2047) / 2048;
    a.agg = c.take<int32_t>((size_t)MAXC * (a.ntiles + 1));
    c.off = (c.off + 255) & ~(size_t)255;
    const int64_t packed = 8 * (m + 1) + 4 * ((nnz + 3) / 4) + 64;
    const int64_t pool_ints =
        c.off < NOALLOC_SCRATCH_BYTES ? (int64_t)((NOALLOC_SCRATCH_BYTES - c.off) / sizeof(int)) - POOL_PAD : 0;
    if (pool_ints < 2 * packed) {
        fprintf(stderr,
                "openph_gb300: oph_reduce_pms_noalloc: %lld columns / %lld nonzeros need more than its fixed "
                "%zu-byte scratch\n",
                (long long)m, (long long)nnz, NOALLOC_SCRATCH_BYTES);
        return OPH_ERR_OOM;
    }
    a.pool = c.take<int>((size_t)pool_ints + POOL_PAD);
    a.st = st;

    // a fresh status block (the array keeps the previous call's contents)
    DevStatus init{};
    init.pool_used = (unsigned long long)((packed + 3) & ~3ll);
    init.pool_size = (unsigned long long)pool_ints;
    init.max_dim = -1;
    OPH_CUDA_TRY(cudaMemcpyAsync(st, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, (int64_t)sm * 16));
    // the caller's CSC is checked (read only) before any kernel writes
    // through its offsets or rows
    DevStatus hs;
    k_check_csc<<<grid, 256, 0, s>>>(d_colptr, d_rows, m, nnz, nullptr, 0, &st->error, nullptr);
    OPH_CUDA_TRY(cudaGetLastError());
    OPH_CUDA_TRY(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs.error) return OPH_ERR_BAD_INPUT;
    k_setup_columns<<<grid, 256, 0, s>>>(d_colptr, d_rows, m, a.pool, a.seg, a.low, dim, st);
    OPH_CUDA_TRY(cudaMemsetAsync(a.rec, 0x7f, sizeof(PivRec) * m, s));
    OPH_CUDA_TRY(cudaMemsetAsync(beta, 0xff, sizeof(int32_t) * m, s));
    k_left<<<grid, 256, 0, s>>>(d_colptr, d_rows, m, a.rec);
    k_beta<<<grid, 256, 0, s>>>(a.rec, m, beta);
    OPH_CUDA_TRY(cudaGetLastError());
    OPH_CUDA_TRY(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs.error || hs.max_dim > MAXC - 2) return OPH_ERR_BAD_INPUT;

    OPH_CUDA_TRY(cudaMemsetAsync(a.first, 0x7f, sizeof(int32_t) * m, s));
    OPH_CUDA_TRY(cudaMemsetAsync(a.classes, 0, m, s));
    OPH_CUDA_TRY(cudaMemsetAsync(a.clear, 0, m, s));
    // launch geometry from a context on the stack (it owns no resources)
    Context ctx;
    ctx.device = dev;
    ctx.sm_count = sm;
    ctx.stream = s;
    SweepGrids g{};
    if ((rc = sweep_grids(&ctx, m, a.ntiles, &g))) return rc;
    launch_phase0(a, 0, m, g.m, s);
    for (int sweeps = 0;;) {
        for (int b = 0; b < 8; b++) launch_sweep(a, g, s);
        sweeps += 8;
        OPH_CUDA_TRY(cudaGetLastError());
        OPH_CUDA_TRY(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
        OPH_CUDA_TRY(cudaStreamSynchronize(s));
        // the store cannot grow here (growing would allocate): report it
        if (hs.overflow) return OPH_ERR_OVERFLOW;
        if (hs.converged) break;
        if (sweeps >= (1 << 20)) return OPH_ERR_TIMEOUT;
    }
    k_finalize1<<<grid, 256, 0, s>>>(a.low, m, 0, 0, nullptr, 0, d_low, d_ess, nullptr);
    k_finalize2<<<grid, 256, 0, s>>>(a.low, m, nullptr, 0, d_ess, nullptr);
    OPH_CUDA_TRY(cudaGetLastError());
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    return OPH_OK;
}
