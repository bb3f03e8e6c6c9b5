// pms — parallel multi-scale reduction of a Z/2 boundary matrix, GB300 form.
//
// Reference: src/cuda/algorithms/pms/pms.cu:1-118 (driver),
// pms_functions.cu:6-140 (kernels), beta.cu:2-26 (alpha/beta pivots).
//
// Sweep structure kept from the reference: Phase 0 once, then sweeps of
//   Phase I  — pivot discovery by dimension + twist clearing, and
//   Phase II — left-to-right additions by known pivots + the beta check,
// until no two columns share a low.  What changes:
//   * Phase I (the reference's one-thread-per-dimension serial walk,
//     transverse_dimensions, pms_functions.cu:55-85) is restated as
//     data-parallel passes:  first[row] = min column with that low (atomicMin);
//     a column's low is "repeated" iff first[low] != column; ceil(j) = the
//     exclusive prefix max of repeated lows over earlier columns of j's
//     dimension bucket (a tiled scan); j is a pivot iff it is first for its
//     low, unclassified, and low > ceil(j).  Identical marks to the serial walk
//     on graded matrices (rows of distinct buckets are disjoint).
//   * Phase II runs a compacted worklist of unresolved columns through a
//     persistent work queue; the column being reduced stays in shared memory
//     across its whole chain of additions and is written back once; pivots are
//     staged into shared memory; columns wider than the narrow tier go to a
//     wide tier (one warp per column, larger shared buffers), and beyond that
//     to a global-memory tier.
//   * Convergence is tested on the device (the count of repeated lows from
//     Phase I); kernels of a converged sweep return at once, so the host reads
//     one status word per batch of sweeps instead of one per sweep.
#include <algorithm>

#include "oph_host.h"

namespace oph {

constexpr int P1_THREADS = 256;
constexpr int P1_ITEMS = 8;
constexpr int P1_TILE = P1_THREADS * P1_ITEMS;

struct PmsArgs {
    int64_t m;
    int32_t *low;
    int8_t *classes;
    uint8_t *clear;
    const int8_t *dim;
    int32_t *first;
    const int32_t *left;
    const int32_t *beta;
    int32_t *worklist;
    int32_t *widelist;
    int64_t *seg;
    unsigned long long *rowpiv;
    int32_t *agg;
    int64_t ntiles;
    int *pool;
    DevStatus *st;
};

// ---------------------------------------------------------------- Phase 0
// mark_pivots_and_clear (pms_functions.cu:33-53): low_j == beta_j >= 0 means
// row low_j first appears in column j, so j is a final pivot; the column of
// row low_j is positive and is cleared (the clear is applied by Phase I).
__global__ void k_phase0(PmsArgs a) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < a.m; j += (int64_t)gridDim.x * blockDim.x) {
        int lj = a.low[j];
        if (lj >= 0 && lj == a.beta[j]) {
            a.classes[j] = -1;
            a.rowpiv[lj] = pack_pivot((int)j, a.seg[j]);
            a.clear[lj] = 1;
        }
    }
}

// --------------------------------------------------------------- Phase I
// (a) apply pending clears (clear_positives, pms_functions.cu:131-140) and
//     record the first column of every low.
__global__ void k_p1_first(PmsArgs a) {
    if (a.st->converged) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.st->reps = 0;
        a.st->wl_count = 0;
        a.st->wl_cursor = 0;
        a.st->wide_count = 0;
        a.st->wide_cursor = 0;
    }
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < a.m; j += (int64_t)gridDim.x * blockDim.x) {
        int lj = a.low[j];
        if (a.clear[j]) {
            a.clear[j] = 0;
            a.classes[j] = 1;
            if (lj >= 0) a.low[j] = -1;
            lj = -1;
        }
        if (lj >= 0) {
            // a column whose low already has a pivot to its left is a repeat:
            // the pivot itself records first[low], so only the others race
            const unsigned long long w = a.rowpiv[lj];
            if (w == NO_PIVOT || pivot_col(w) >= (int)j) atomicMin(&a.first[lj], (int)j);
        }
    }
}

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// (b) per-tile maxima of repeated lows, per dimension bucket; counts repeats.
__global__ void __launch_bounds__(P1_THREADS) k_p1_tiles(PmsArgs a) {
    if (a.st->converged) return;
    __shared__ int sm[P1_THREADS / 32][MAXC];
    __shared__ int sreps;
    if (threadIdx.x == 0) sreps = 0;
    int mx[MAXC];
#pragma unroll
    for (int d = 0; d < MAXC; d++) mx[d] = -1;
    int reps = 0;
    const int64_t base = (int64_t)blockIdx.x * P1_TILE + (int64_t)threadIdx.x * P1_ITEMS;
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++) {
        int64_t j = base + t;
        if (j < a.m) {
            int lj = a.low[j];
            if (lj >= 0 && a.first[lj] != (int)j) {
                int b = a.dim[j] + 1;
#pragma unroll
                for (int d = 0; d < MAXC; d++)
                    if (d == b) mx[d] = max(mx[d], lj);
                reps++;
            }
        }
    }
    __syncthreads();
    if (reps) atomicAdd(&sreps, reps);
#pragma unroll
    for (int d = 0; d < MAXC; d++) {
        int v = warp_max(mx[d]);
        if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5][d] = v;
    }
    __syncthreads();
    if (threadIdx.x < MAXC) {
        int v = -1;
        for (int w = 0; w < P1_THREADS / 32; w++) v = max(v, sm[w][threadIdx.x]);
        a.agg[blockIdx.x * MAXC + threadIdx.x] = v;
    }
    if (threadIdx.x == 0 && sreps) atomicAdd(&a.st->reps, sreps);
}

// (c) exclusive prefix max of the tile maxima, one warp per bucket; decides
//     convergence (no repeated low anywhere).
__global__ void k_p1_scan(PmsArgs a) {
    if (a.st->converged) return;
    if (a.st->reps == 0) {
        if (threadIdx.x == 0) a.st->converged = 1;
        return;
    }
    const int d = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (d >= MAXC) return;
    const int64_t n = a.ntiles;
    const int64_t chunk = (n + 31) / 32;
    const int64_t lo = lane * chunk, hi = min(n, lo + chunk);
    int local = -1;
    for (int64_t t = lo; t < hi; t++) local = max(local, a.agg[t * MAXC + d]);
    // exclusive scan of the lane maxima
    int incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl = max(incl, v);
    }
    int run = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) run = -1;
    for (int64_t t = lo; t < hi; t++) {
        int v = a.agg[t * MAXC + d];
        a.agg[t * MAXC + d] = run;
        run = max(run, v);
    }
}

// (d) mark pivots: first for its low, unclassified, low above the running
//     ceiling of repeated lows in its bucket.
__global__ void __launch_bounds__(P1_THREADS) k_p1_mark(PmsArgs a) {
    if (a.st->converged) return;
    __shared__ int sm[P1_THREADS / 32][MAXC];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * P1_TILE + (int64_t)threadIdx.x * P1_ITEMS;
    int lows[P1_ITEMS], bkt[P1_ITEMS];
    bool rep[P1_ITEMS];
    int mx[MAXC];
#pragma unroll
    for (int d = 0; d < MAXC; d++) mx[d] = -1;
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++) {
        int64_t j = base + t;
        lows[t] = -1; bkt[t] = 0; rep[t] = false;
        if (j < a.m) {
            int lj = a.low[j];
            lows[t] = lj;
            bkt[t] = a.dim[j] + 1;
            if (lj >= 0 && a.first[lj] != (int)j) {
                rep[t] = true;
#pragma unroll
                for (int d = 0; d < MAXC; d++)
                    if (d == bkt[t]) mx[d] = max(mx[d], lj);
            }
        }
    }
    // block-exclusive prefix of the per-thread maxima, per bucket
    int pre[MAXC];
#pragma unroll
    for (int d = 0; d < MAXC; d++) {
        int incl = mx[d];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl = max(incl, v);
        }
        int ex = __shfl_up_sync(0xffffffffu, incl, 1);
        pre[d] = lane == 0 ? -1 : ex;
        if (lane == 31) sm[wid][d] = incl;
    }
    __syncthreads();
#pragma unroll
    for (int d = 0; d < MAXC; d++) {
        int c = a.agg[blockIdx.x * MAXC + d];
        for (int w = 0; w < wid; w++) c = max(c, sm[w][d]);
        pre[d] = max(pre[d], c);
    }
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++) {
        int64_t j = base + t;
        if (j >= a.m) break;
        int lj = lows[t];
        if (lj < 0) continue;
        int ceil = -1;
#pragma unroll
        for (int d = 0; d < MAXC; d++)
            if (d == bkt[t]) ceil = pre[d];
        if (rep[t]) {
#pragma unroll
            for (int d = 0; d < MAXC; d++)
                if (d == bkt[t]) pre[d] = max(pre[d], lj);
        } else if (a.classes[j] == 0 && lj > ceil) {
            a.classes[j] = -1;
            a.rowpiv[lj] = pack_pivot((int)j, a.seg[j]);
            a.clear[lj] = 1;
        }
    }
}

// (e) reset first[], apply the clears of this Phase I, and compact the
//     unresolved columns (unclassified, nonzero low) into the worklist.
__global__ void k_p1_worklist(PmsArgs a) {
    if (a.st->converged) return;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j0 = blockIdx.x * (int64_t)blockDim.x; j0 < a.m; j0 += stride) {
        int64_t j = j0 + threadIdx.x;
        bool want = false;
        if (j < a.m) {
            int lj = a.low[j];
            // reset first[] for the next sweep: once per row, by its winner
            if (lj >= 0 && a.first[lj] == (int)j) a.first[lj] = FIRST_NONE;
            if (a.clear[j]) {
                a.clear[j] = 0;
                a.classes[j] = 1;
                if (lj >= 0) a.low[j] = -1;
                lj = -1;
            }
            want = lj >= 0 && a.classes[j] == 0;
        }
        warp_append(want, (int)j, a.worklist, &a.st->wl_count);
    }
}

// -------------------------------------------------------------- Phase II
// phase_ii (pms_functions.cu:87-112) for one column j by a group of G lanes.
// A/B/C are the group's shared buffers of `cap` ints (A: the column, B: merge
// output, C: the staged pivot).  Returns false if j was handed to the next
// tier (too wide) — its state is written back first — or if a pool
// allocation failed (nothing of j is changed then).
template <int G, class Tile>
__device__ void reduce_column(const Tile &tile, const PmsArgs &a, int j, int *A, int *B, int *C, int cap,
                              int32_t *handoff, int *handoff_cnt, long long &adds, long long &slots) {
    const int lane = tile.thread_rank();
    int lj = a.low[j];
    unsigned long long w = ld_acquire(&a.rowpiv[lj]);
    if (w == NO_PIVOT || pivot_col(w) >= j) return;
    const long long sj = a.seg[j];
    int n = a.pool[sj];
    const int capj = a.pool[sj + 1];
    if (n > cap) {
        if (lane == 0) handoff[atomicAdd(handoff_cnt, 1)] = j;
        return;
    }
    group_copy<G>(tile, A, a.pool + sj + SEG_HDR, n);
    bool made_pivot = false, handed = false;
    for (;;) {
        const long long sp = pivot_seg(w);
        const int np = a.pool[sp];
        if (n + np > cap) { handed = true; break; }
        group_copy<G>(tile, C, a.pool + sp + SEG_HDR, np);
        const int nn = merge_xor<G>(tile, A, n, C, np, B);
        slots += n + np + nn;
        adds++;
        n = nn;
        int *t = A; A = B; B = t;
        lj = n ? A[n - 1] : -1;
        if (lj < 0) break;
        if (a.left[lj] == j) made_pivot = true;
        if (lane == 0) a.clear[lj] = 1;
        if (made_pivot) break;
        w = ld_acquire(&a.rowpiv[lj]);
        if (w == NO_PIVOT || pivot_col(w) >= j) break;
    }
    // write the column back: in place when it fits, else a fresh segment
    long long dst = sj;
    int dcap = capj;
    if (n > capj) {
        dcap = round4(max(2 * n, 16));
        long long off = 0;
        if (lane == 0) off = pool_alloc(a.st, SEG_HDR + dcap);
        off = tile.shfl(off, 0);
        if (off < 0) return;  // pool exhausted: j keeps its pre-sweep state
        dst = off;
    }
    group_copy<G>(tile, a.pool + dst + SEG_HDR, A, n);
    if (lane == 0) {
        a.pool[dst] = n;
        a.pool[dst + 1] = dcap;
        a.seg[j] = dst;
        a.low[j] = lj;
    }
    if (made_pivot) {
        fence_acq_rel();
        tile.sync();
        if (lane == 0) {
            a.classes[j] = -1;
            st_release(&a.rowpiv[lj], pack_pivot(j, dst));
        }
    } else if (handed) {
        if (lane == 0) handoff[atomicAdd(handoff_cnt, 1)] = j;
    }
    tile.sync();
}

// Narrow tier: G lanes per column, the column in shared memory (A/B, CAP
// ints each), the pivot in registers when it has at most G entries (the
// common case: most pivots are apparent pairs with 3 entries) and read from
// the store otherwise.  Each addition is two dependent round trips: the pivot
// word (with left[] alongside) and the pivot's header + rows in one go.
// Reads up to G ints past a segment's start, which the pool's tail padding
// keeps in bounds.
template <int G, class Tile>
__device__ void reduce_column_narrow(const Tile &tile, const PmsArgs &a, int j, int *A, int *B, int cap,
                                     long long &adds, long long &slots) {
    const int lane = tile.thread_rank();
    int lj = a.low[j];
    unsigned long long w = ld_acquire(&a.rowpiv[lj]);
    if (w == NO_PIVOT || pivot_col(w) >= j) return;
    const long long sj = a.seg[j];
    int n = a.pool[sj];
    const int capj = a.pool[sj + 1];
    if (n > cap) {
        if (lane == 0) a.widelist[atomicAdd(&a.st->wide_count, 1)] = j;
        return;
    }
    group_copy<G>(tile, A, a.pool + sj + SEG_HDR, n);
    bool made_pivot = false, handed = false;
    for (;;) {
        const long long sp = pivot_seg(w);
        const int np = a.pool[sp];
        const int pv = a.pool[sp + SEG_HDR + lane];
        if (n + np > cap) { handed = true; break; }
        int nn;
        if (np <= G) nn = merge_xor_small<G>(tile, A, n, pv, np, B);
        else nn = merge_xor<G>(tile, A, n, a.pool + sp + SEG_HDR, np, B);
        slots += n + np + nn;
        adds++;
        n = nn;
        int *t = A; A = B; B = t;
        lj = n ? A[n - 1] : -1;
        if (lj < 0) break;
        const int lf = a.left[lj];
        w = ld_acquire(&a.rowpiv[lj]);
        if (lane == 0) a.clear[lj] = 1;
        if (lf == j) { made_pivot = true; break; }
        if (w == NO_PIVOT || pivot_col(w) >= j) break;
    }
    long long dst = sj;
    int dcap = capj;
    if (n > capj) {
        dcap = round4(max(2 * n, 16));
        long long off = 0;
        if (lane == 0) off = pool_alloc(a.st, SEG_HDR + dcap);
        off = tile.shfl(off, 0);
        if (off < 0) return;  // pool exhausted: j keeps its pre-sweep state
        dst = off;
    }
    group_copy<G>(tile, a.pool + dst + SEG_HDR, A, n);
    if (lane == 0) {
        a.pool[dst] = n;
        a.pool[dst + 1] = dcap;
        a.seg[j] = dst;
        a.low[j] = lj;
    }
    if (made_pivot) {
        fence_acq_rel();
        tile.sync();
        if (lane == 0) {
            a.classes[j] = -1;
            st_release(&a.rowpiv[lj], pack_pivot(j, dst));
        }
    } else if (handed) {
        if (lane == 0) a.widelist[atomicAdd(&a.st->wide_count, 1)] = j;
    }
    tile.sync();
}

template <int G, int CAP>
__global__ void __launch_bounds__(256) k_p2_narrow(PmsArgs a) {
    if (a.st->converged) return;
    extern __shared__ int smem[];
    auto tile = cg::tiled_partition<G>(cg::this_thread_block());
    const int gid = threadIdx.x / G;
    int *buf = smem + (size_t)gid * 2 * CAP;
    const int count = a.st->wl_count;
    long long adds = 0, slots = 0;
    for (;;) {
        int idx = 0;
        if (tile.thread_rank() == 0) idx = atomicAdd(&a.st->wl_cursor, 1);
        idx = tile.shfl(idx, 0);
        if (idx >= count) break;
        reduce_column_narrow<G>(tile, a, a.worklist[idx], buf, buf + CAP, CAP, adds, slots);
    }
    if (tile.thread_rank() == 0 && adds) {
        atomicAdd(&a.st->additions, (unsigned long long)adds);
        atomicAdd(&a.st->slots, (unsigned long long)slots);
    }
}

// Wide tier: one warp per column with large shared buffers; columns wider
// still fall through to the global tier (handoff list = worklist, reused).
template <int CAP>
__global__ void __launch_bounds__(32) k_p2_wide(PmsArgs a) {
    if (a.st->converged) return;
    extern __shared__ int smem[];
    auto tile = cg::tiled_partition<32>(cg::this_thread_block());
    const int count = a.st->wide_count;
    long long adds = 0, slots = 0;
    for (;;) {
        int idx = 0;
        if (tile.thread_rank() == 0) idx = atomicAdd(&a.st->wide_cursor, 1);
        idx = tile.shfl(idx, 0);
        if (idx >= count) break;
        reduce_column<32>(tile, a, a.widelist[idx], smem, smem + CAP, smem + 2 * CAP, CAP, a.worklist,
                          &a.st->wl_count, adds, slots);
    }
    if (tile.thread_rank() == 0 && adds) {
        atomicAdd(&a.st->additions, (unsigned long long)adds);
        atomicAdd(&a.st->slots, (unsigned long long)slots);
    }
}

// Global tier: one warp per column, buffers bump-allocated in the pool.
__global__ void __launch_bounds__(32) k_p2_global(PmsArgs a) {
    if (a.st->converged) return;
    auto tile = cg::tiled_partition<32>(cg::this_thread_block());
    const int lane = tile.thread_rank();
    const int count = a.st->wl_count;
    long long adds = 0, slots = 0;
    for (int idx = blockIdx.x; idx < count; idx += gridDim.x) {
        const int j = a.worklist[idx];
        int lj = a.low[j];
        unsigned long long w = ld_acquire(&a.rowpiv[lj]);
        if (w == NO_PIVOT || pivot_col(w) >= j) continue;
        const long long sj = a.seg[j];
        int n = a.pool[sj];
        const int capj = a.pool[sj + 1];
        const int *A = a.pool + sj + SEG_HDR;
        int *X = nullptr, *Y = nullptr;
        int bcap = 0;
        bool made_pivot = false, failed = false;
        for (;;) {
            const long long sp = pivot_seg(w);
            const int np = a.pool[sp];
            if (n + np > bcap) {
                int ncap = round4(max(2 * (n + np), 1024));
                long long off = 0;
                if (lane == 0) off = pool_alloc(a.st, 2ll * ncap);
                off = tile.shfl(off, 0);
                if (off < 0) { failed = true; break; }
                int *NX = a.pool + off, *NY = NX + ncap;
                group_copy<32>(tile, NX, A, n);
                A = NX; X = NX; Y = NY; bcap = ncap;
            }
            int *out = (A == X) ? Y : X;
            const int nn = merge_xor<32>(tile, A, n, a.pool + sp + SEG_HDR, np, out);
            slots += n + np + nn;
            adds++;
            n = nn;
            A = out;
            lj = n ? A[n - 1] : -1;
            if (lj < 0) break;
            if (a.left[lj] == j) made_pivot = true;
            if (lane == 0) a.clear[lj] = 1;
            if (made_pivot) break;
            w = ld_acquire(&a.rowpiv[lj]);
            if (w == NO_PIVOT || pivot_col(w) >= j) break;
        }
        if (failed) continue;
        long long dst = sj;
        int dcap = capj;
        if (n > capj) {
            dcap = round4(max(2 * n, 16));
            long long off = 0;
            if (lane == 0) off = pool_alloc(a.st, SEG_HDR + dcap);
            off = tile.shfl(off, 0);
            if (off < 0) continue;
            dst = off;
        }
        if (A != a.pool + dst + SEG_HDR) group_copy<32>(tile, a.pool + dst + SEG_HDR, A, n);
        if (lane == 0) {
            a.pool[dst] = n;
            a.pool[dst + 1] = dcap;
            a.seg[j] = dst;
            a.low[j] = lj;
        }
        if (made_pivot) {
            fence_acq_rel();
            tile.sync();
            if (lane == 0) {
                a.classes[j] = -1;
                st_release(&a.rowpiv[lj], pack_pivot(j, dst));
            }
        }
        tile.sync();
    }
    if (lane == 0 && adds) {
        atomicAdd(&a.st->additions, (unsigned long long)adds);
        atomicAdd(&a.st->slots, (unsigned long long)slots);
    }
}

// Resets the global-tier queue before the wide kernel hands columns over.
__global__ void k_reset_global_queue(DevStatus *st) {
    if (st->converged) return;
    st->wl_count = 0;
}

__global__ void k_count_sweep(DevStatus *st) {
    if (!st->converged) st->sweeps++;
}

// ------------------------------------------------------------------ driver
#ifndef OPH_NARROW_G
#define OPH_NARROW_G 8
#endif
#ifndef OPH_NARROW_CAP
#define OPH_NARROW_CAP 128
#endif
constexpr int NARROW_G = OPH_NARROW_G;
constexpr int NARROW_CAP = OPH_NARROW_CAP;
constexpr int WIDE_CAP = 8192;

int run_pms(Context *ctx, Work &w, oph_info *info) {
    const int64_t m = w.m;
    PmsArgs a{};
    a.m = m; a.low = w.low; a.classes = w.classes; a.clear = w.clear; a.dim = w.dim; a.first = w.first;
    a.left = w.left; a.beta = w.beta; a.worklist = w.worklist; a.widelist = w.widelist; a.seg = w.seg;
    a.rowpiv = w.rowpiv; a.agg = w.agg; a.ntiles = w.ntiles; a.pool = w.pool; a.st = w.st;
    cudaStream_t s = ctx->stream;

    static bool attr_done[64] = {};
    const size_t narrow_smem = (size_t)(256 / NARROW_G) * 2 * NARROW_CAP * sizeof(int);
    const size_t wide_smem = (size_t)3 * WIDE_CAP * sizeof(int);
    if (!attr_done[ctx->device & 63]) {
        OPH_CUDA_TRY(cudaFuncSetAttribute(k_p2_narrow<NARROW_G, NARROW_CAP>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)narrow_smem));
        OPH_CUDA_TRY(cudaFuncSetAttribute(k_p2_wide<WIDE_CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)wide_smem));
        attr_done[ctx->device & 63] = true;
    }
    int nb_narrow = 0;
    OPH_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb_narrow, k_p2_narrow<NARROW_G, NARROW_CAP>, 256,
                                                               narrow_smem));
    if (nb_narrow < 1) nb_narrow = 1;
    const int grid_narrow = ctx->sm_count * nb_narrow;
    int nb_wide = 0;
    OPH_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb_wide, k_p2_wide<WIDE_CAP>, 32, wide_smem));
    if (nb_wide < 1) nb_wide = 1;
    const int grid_wide = ctx->sm_count * nb_wide;
    const int grid_m = (int)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, (int64_t)ctx->sm_count * 16));
    const int grid_t = (int)std::max<int64_t>(1, w.ntiles);

    OPH_CUDA_TRY(cudaMemsetAsync(w.first, 0x7f, sizeof(int32_t) * m, s));
    OPH_CUDA_TRY(cudaMemsetAsync(w.rowpiv, 0xff, sizeof(unsigned long long) * m, s));
    OPH_CUDA_TRY(cudaMemsetAsync(w.classes, 0, m, s));
    OPH_CUDA_TRY(cudaMemsetAsync(w.clear, 0, m, s));

    cudaEventRecord(ctx->ev[0], s);
    k_phase0<<<grid_m, 256, 0, s>>>(a);
    ctx->launches++;
    OPH_CUDA_TRY(cudaGetLastError());

    // profiling: 4 events per sweep (before Phase I, before/after the narrow
    // tier, after the wide and global tiers), reused batch after batch
    constexpr int MAX_BATCH = 16;
    if (ctx->profile && ctx->pev_n < 4 * MAX_BATCH + 2) {
        ctx->pev = (cudaEvent_t *)realloc(ctx->pev, sizeof(cudaEvent_t) * (4 * MAX_BATCH + 2));
        for (int i = ctx->pev_n; i < 4 * MAX_BATCH + 2; i++) cudaEventCreate(&ctx->pev[i]);
        ctx->pev_n = 4 * MAX_BATCH + 2;
    }
    if (ctx->profile) cudaEventRecord(ctx->pev[4 * MAX_BATCH], s);  // end of Phase 0

    const int max_sweeps = ctx->max_sweeps > 0 ? ctx->max_sweeps : 1 << 20;
    int sweeps_launched = 0;
    int batch = 2;
    DevStatus hs{};
    int rc = OPH_OK;
    float p2_ms = 0, p2w_ms = 0, p1_ms = 0;
    int p2_launches = 0;
    int regrows = 0;
    for (;;) {
        const int nb = std::min(batch, max_sweeps - sweeps_launched);
        for (int b = 0; b < nb; b++) {
            if (ctx->profile) cudaEventRecord(ctx->pev[4 * b], s);
            k_p1_first<<<grid_m, 256, 0, s>>>(a);
            k_p1_tiles<<<grid_t, P1_THREADS, 0, s>>>(a);
            k_p1_scan<<<1, 32 * MAXC, 0, s>>>(a);
            k_p1_mark<<<grid_t, P1_THREADS, 0, s>>>(a);
            k_p1_worklist<<<grid_m, 256, 0, s>>>(a);
            if (ctx->profile) cudaEventRecord(ctx->pev[4 * b + 1], s);
            k_p2_narrow<NARROW_G, NARROW_CAP><<<grid_narrow, 256, narrow_smem, s>>>(a);
            if (ctx->profile) cudaEventRecord(ctx->pev[4 * b + 2], s);
            k_reset_global_queue<<<1, 1, 0, s>>>(w.st);
            k_p2_wide<WIDE_CAP><<<grid_wide, 32, wide_smem, s>>>(a);
            k_p2_global<<<ctx->sm_count * 4, 32, 0, s>>>(a);
            k_count_sweep<<<1, 1, 0, s>>>(w.st);
            if (ctx->profile) cudaEventRecord(ctx->pev[4 * b + 3], s);
            ctx->launches += 10;
        }
        sweeps_launched += nb;
        OPH_CUDA_TRY(cudaGetLastError());
        OPH_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, w.st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
        OPH_CUDA_TRY(cudaStreamSynchronize(s));
        hs = *ctx->h_status;
        if (ctx->profile) {
            // sweeps past convergence return at once; count only working ones
            const int worked = std::max(0, std::min(nb, hs.sweeps - (sweeps_launched - nb)));
            for (int b = 0; b < nb; b++) {
                float t1 = 0, t2 = 0, t3 = 0;
                cudaEventElapsedTime(&t1, ctx->pev[4 * b], ctx->pev[4 * b + 1]);
                cudaEventElapsedTime(&t2, ctx->pev[4 * b + 1], ctx->pev[4 * b + 2]);
                cudaEventElapsedTime(&t3, ctx->pev[4 * b + 2], ctx->pev[4 * b + 3]);
                p1_ms += t1;
                p2_ms += t2;
                p2w_ms += t3;
            }
            p2_launches += worked;
        }
        if (hs.error) { rc = OPH_ERR_BAD_INPUT; break; }
        if (hs.overflow) {
            // a column could not be written back: grow the store and run the
            // sweep again from the consistent state the kernels left
            int g = grow_pool(ctx, w);
            if (g != OPH_OK) { rc = g; break; }
            a.pool = w.pool;
            regrows++;
            if (hs.converged) break;
            continue;
        }
        if (hs.converged) break;
        if (sweeps_launched >= max_sweeps) { rc = OPH_ERR_TIMEOUT; break; }
        batch = std::min(batch * 2, MAX_BATCH);
    }
    cudaEventRecord(ctx->ev[1], s);
    OPH_CUDA_TRY(cudaEventSynchronize(ctx->ev[1]));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    if (ctx->profile) {
        float p0 = 0;
        cudaEventElapsedTime(&p0, ctx->ev[0], ctx->pev[4 * MAX_BATCH]);
        ctx->prof.phase2_narrow_ms = p2_ms;
        ctx->prof.phase2_wide_ms = p2w_ms;
        ctx->prof.phase1_ms = p1_ms;
        ctx->prof.setup_ms += p0;
        ctx->prof.phase2_launches = p2_launches;
    }
    if (info) {
        info->sweeps = hs.sweeps;
        info->num_iters = std::max(hs.sweeps, 1) + 1;
        info->additions = (int64_t)hs.additions;
        info->slots_moved = (int64_t)hs.slots;
        info->pool_bytes = (int64_t)hs.pool_used * 4;
        info->regrows = regrows;
        info->device_ms = ms;
    }
    return rc;
}

}  // namespace oph
