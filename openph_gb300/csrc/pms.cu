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
//   * Phase II takes the unresolved columns that can add this sweep from a
//     work queue, each column on chip for its whole chain of additions and
//     written back once, through tiers by column length: a column per lane
//     (the scalar tier, <= 48 rows), 8 lanes per column (tier 0, <= 128 rows,
//     three-row pivots added in place), a warp per column (tier 1, <= 512
//     rows, pending toggles in registers), a CTA per column (tier 2, merge
//     path in shared memory; tier 3, the column as a bitmap of its rows).  A
//     pivot of at most four rows comes with the one 32-byte record read that
//     also gives the beta check; the flags every chain would rewrite are
//     written only on change.
//   * On the anti-transpose (dual.cu) Phase II takes the dimension buckets in
//     ascending order, so that each bucket's pivots clear the next bucket's
//     columns before they are reduced (twist's order).
//   * Phase I visits a compacted list of the unresolved columns; the first
//     holds only the columns with a low (k_list_*): a zero column never adds
//     or repeats, and on the anti-transpose of a Rips complex the zero top
//     dimension is almost all of the matrix.
//   * Columns can arrive cleared (Work::preclear: the per-block form, where
//     another part reduces them); Phase 0 skips those, Phase I zeroes them.
//   * Convergence is tested on the device (the count of repeated lows from
//     Phase I); kernels of a converged sweep return at once, so the host reads
//     one status word per batch of sweeps, and the sweeps of a batch are
//     replayed from a captured CUDA graph.
#include <algorithm>
#include <cstring>

#include "oph_host.h"
#include "pms.cuh"

namespace oph {

// OPH_COUNTS=1: diagnostic counters of the Phase II tiers (DevStatus::diag,
// printed with OPH_TRACE=2).
#ifndef OPH_COUNTS
#define OPH_COUNTS 0
#endif

constexpr int P1_THREADS = 256;
constexpr int P1_ITEMS = 8;
constexpr int P1_TILE = P1_THREADS * P1_ITEMS;



// ---------------------------------------------------------------- Phase 0
// mark_pivots_and_clear (pms_functions.cu:33-53): low_j == beta_j >= 0 means
// row low_j first appears in column j, so j is a final pivot; the column of
// row low_j is positive and is cleared (the clear is applied by Phase I).
// A column cleared before Phase 0 publishes nothing (one this kernel clears
// meanwhile is positive, so it is no pivot either way).
__global__ void k_phase0(PmsArgs a, int64_t c0, int64_t c1) {
    for (int64_t j = c0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < c1; j += (int64_t)gridDim.x * blockDim.x) {
        int lj = a.low[j];
        if (lj >= 0 && lj == a.beta[j] && !a.clear[j]) {
            a.classes[j] = -1;
            const long long sj = a.seg[j];
            rec_publish<false>(a.rec, lj, (int)j, a.pool[sj], sj, a.pool + sj + SEG_HDR);
            a.clear[lj] = 1;
        }
    }
}

// --------------------------------------------------------------- Phase I
// The columns a Phase I pass visits: with a compacted list, its U entries in
// column order (only unresolved columns can repeat a low or become new
// pivots: a pivot always holds the first occurrence of its low and a cleared
// or zero column has none); without one, all m columns.
__device__ __forceinline__ int64_t p1_count(const PmsArgs &a) { return a.ulist ? (int64_t)*a.ucur : a.m; }
__device__ __forceinline__ int64_t p1_col(const PmsArgs &a, int64_t idx) {
    return a.ulist ? (int64_t)a.ulist[idx] : idx;
}
// A compacted list that fits one tile: Phase I runs as one block
// (k_p1_small) and the grid-wide Phase I kernels return at once.
__device__ __forceinline__ bool p1_small(const PmsArgs &a) { return a.ulist && *a.ucur <= P1_TILE; }

// Another column to the left holds the same low: a published pivot, or an
// earlier column recorded in first[].
__device__ __forceinline__ bool is_repeat(const PmsArgs &a, int64_t j, int lj) {
    const int pc = a.rec[lj].col;
    return (pc >= 0 && pc < (int)j) || a.first[lj] != (int)j;
}

// (a) apply pending clears (clear_positives, pms_functions.cu:131-140) and
//     record the first column of every low.
__device__ __forceinline__ void p1_reset(const PmsArgs &a) {
    a.st->reps = 0;
    a.st->wl_count = 0;
    for (int t = 0; t < 5; t++) { a.st->t_count[t] = 0; a.st->t_cursor[t] = 0; }
    a.st->s_cursor = 0;
    a.st->s_out = 0;
    if (OPH_COUNTS) a.st->diag[5] = 0;  // the eager tier's longest chain, per sweep
}
__device__ __forceinline__ void p1_first_range(const PmsArgs &a, int64_t i0, int64_t stride) {
    const int64_t n = p1_count(a);
    for (int64_t idx = i0; idx < n; idx += stride) {
        const int64_t j = p1_col(a, idx);
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
            const int pc = a.rec[lj].col;
            // many columns can share a low: skip the atomic when first[]
            // already holds a smaller column (a stale read only costs the
            // atomic that would have been issued anyway)
            if ((pc < 0 || pc >= (int)j) && a.first[lj] > (int)j)
                atomicMin(&a.first[lj], (int)j);
        }
    }
}
__global__ void k_p1_first(PmsArgs a) {
    if (a.st->converged || p1_small(a)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) p1_reset(a);
    p1_first_range(a, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// (b) per-tile maxima of repeated lows, per dimension bucket; counts repeats
//     (per instance too, when the columns belong to several).
__device__ __forceinline__ void k_p1_tiles_tile(PmsArgs a, const int64_t n, const int64_t tile) {
    __shared__ int sm[P1_THREADS / 32][MAXC];
    __shared__ int sreps;
    if (threadIdx.x == 0) sreps = 0;
    int mx[MAXC];
#pragma unroll
    for (int d = 0; d < MAXC; d++) mx[d] = -1;
    int reps = 0;
    int cur_inst = -1, cur_reps = 0;  // per-instance counts, flushed on change
    const int64_t base = (int64_t)tile * P1_TILE + (int64_t)threadIdx.x * P1_ITEMS;
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++) {
        const int64_t idx = base + t;
        if (idx < n) {
            const int64_t j = p1_col(a, idx);
            const int lj = a.low[j];
            if (lj >= 0 && is_repeat(a, j, lj)) {
                const int b = a.dim[j] + 1;
#pragma unroll
                for (int d = 0; d < MAXC; d++)
                    if (d == b) mx[d] = max(mx[d], lj);
                reps++;
                if (a.ireps) {
                    const int ib = a.inst[j];
                    if (ib != cur_inst) {
                        if (cur_reps) atomicAdd(&a.ireps[cur_inst], cur_reps);
                        cur_inst = ib;
                        cur_reps = 0;
                    }
                    cur_reps++;
                }
            }
        }
    }
    if (cur_reps) atomicAdd(&a.ireps[cur_inst], cur_reps);
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
        a.agg[tile * MAXC + threadIdx.x] = v;
    }
    if (threadIdx.x == 0 && sreps) atomicAdd(&a.st->reps, sreps);
}
// One pass over the list's tiles, a grid-stride loop: the grid is sized
// for the machine, not for the matrix (a grid of one block per tile of
// the full matrix costs ~0.3 ms of empty blocks per sweep at 3.5e8 columns).
__global__ void __launch_bounds__(P1_THREADS) k_p1_tiles(PmsArgs a) {
    if (a.st->converged || p1_small(a)) return;
    const int64_t n = p1_count(a);
    for (int64_t tile = blockIdx.x; tile * P1_TILE < n; tile += gridDim.x) {
        k_p1_tiles_tile(a, n, tile);
        __syncthreads();  // the next tile reuses the shared arrays
    }
}

// (c) exclusive prefix max of the tile maxima, one warp per bucket; decides
//     convergence (no repeated low anywhere).
__global__ void k_p1_scan(PmsArgs a) {
    if (a.st->converged || p1_small(a)) return;
    if (a.st->reps == 0) {
        if (threadIdx.x == 0) a.st->converged = 1;
        return;
    }
    const int d = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (d >= MAXC) return;
    const int64_t n = (p1_count(a) + P1_TILE - 1) / P1_TILE;
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
//     ceiling of repeated lows in its bucket.  With a compacted list, also
//     count per tile the columns that stay unresolved.
__device__ __forceinline__ void k_p1_mark_tile(PmsArgs a, const int64_t n, const int64_t tile) {
    __shared__ int sm[P1_THREADS / 32][MAXC];
    __shared__ int skeep;
    __shared__ int sunres[MAXC];
    if (threadIdx.x == 0) skeep = 0;
    if (threadIdx.x < MAXC) sunres[threadIdx.x] = 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t base = (int64_t)tile * P1_TILE + (int64_t)threadIdx.x * P1_ITEMS;
    int lows[P1_ITEMS], bkt[P1_ITEMS];
    bool rep[P1_ITEMS];
    int mx[MAXC];
#pragma unroll
    for (int d = 0; d < MAXC; d++) mx[d] = -1;
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++) {
        const int64_t idx = base + t;
        lows[t] = -1; bkt[t] = 0; rep[t] = false;
        if (idx < n) {
            const int64_t j = p1_col(a, idx);
            const int lj = a.low[j];
            lows[t] = lj;
            bkt[t] = a.dim[j] + 1;
            if (lj >= 0 && is_repeat(a, j, lj)) {
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
        int c = a.agg[tile * MAXC + d];
        for (int w = 0; w < wid; w++) c = max(c, sm[w][d]);
        pre[d] = max(pre[d], c);
    }
    int keep = 0;
    int icur = -1, icnt[MAXC];  // per-instance bucket counts (a.ibucket)
#pragma unroll
    for (int d = 0; d < MAXC; d++) icnt[d] = 0;
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++) {
        const int64_t idx = base + t;
        if (idx >= n) break;
        const int64_t j = p1_col(a, idx);
        const int lj = lows[t];
        if (lj < 0) continue;
        int ceil = -1;
#pragma unroll
        for (int d = 0; d < MAXC; d++)
            if (d == bkt[t]) ceil = pre[d];
        const int cls = a.classes[j];
        bool kept = false;
        if (rep[t]) {
#pragma unroll
            for (int d = 0; d < MAXC; d++)
                if (d == bkt[t]) pre[d] = max(pre[d], lj);
            kept = cls == 0;
        } else if (cls == 0 && lj > ceil) {
            a.classes[j] = -1;
            const long long sj = a.seg[j];
            rec_publish<false>(a.rec, lj, (int)j, a.pool[sj], sj, a.pool + sj + SEG_HDR);
            a.clear[lj] = 1;
        } else {
            kept = cls == 0;
        }
        keep += kept;
        if (kept && a.ascending) atomicAdd(&sunres[bkt[t]], 1);
        if (kept && a.ibucket) {
            const int ib = a.inst[j];
            if (a.iasc[ib]) {
                if (ib != icur) {  // flush the previous instance's counts
                    if (icur >= 0)
#pragma unroll
                        for (int d = 0; d < MAXC; d++)
                            if (icnt[d]) atomicAdd(&a.ibucket[icur * MAXC + d], icnt[d]);
#pragma unroll
                    for (int d = 0; d < MAXC; d++) icnt[d] = 0;
                    icur = ib;
                }
#pragma unroll
                for (int d = 0; d < MAXC; d++)
                    if (d == bkt[t]) icnt[d]++;
            }
        }
    }
    if (a.ibucket) {
        // the warp's threads on one instance add their counts once
        const unsigned peers = __match_any_sync(0xffffffffu, icur);
        const bool leader = lane == __ffs(peers) - 1;
#pragma unroll
        for (int d = 0; d < MAXC; d++) {
            const int c = __reduce_add_sync(peers, icnt[d]);
            if (leader && icur >= 0 && c) atomicAdd(&a.ibucket[icur * MAXC + d], c);
        }
    }
    if (a.ulist) {
        if (keep) atomicAdd(&skeep, keep);
        __syncthreads();
        if (threadIdx.x == 0) a.kagg[tile] = skeep;
        if (a.ascending && threadIdx.x < MAXC && sunres[threadIdx.x])
            atomicAdd(&a.st->bucket_unres[threadIdx.x], sunres[threadIdx.x]);
    }
}
// One pass over the list's tiles, a grid-stride loop: the grid is sized
// for the machine, not for the matrix (a grid of one block per tile of
// the full matrix costs ~0.3 ms of empty blocks per sweep at 3.5e8 columns).
__global__ void __launch_bounds__(P1_THREADS) k_p1_mark(PmsArgs a) {
    if (a.st->converged || p1_small(a)) return;
    const int64_t n = p1_count(a);
    for (int64_t tile = blockIdx.x; tile * P1_TILE < n; tile += gridDim.x) {
        k_p1_mark_tile(a, n, tile);
        __syncthreads();  // the next tile reuses the shared arrays
    }
}

// The end of (e): the next list's length, and the bucket each instance (or
// the matrix) opens to Phase II: the lowest with unresolved columns (counts
// of this sweep's k_p1_mark, cleared for the next one).  One block.
__device__ __forceinline__ void p1_kscan_tail(const PmsArgs &a, int total) {
    if (threadIdx.x == 0) {
        *a.unext = total;
        if (a.ascending) {
            int open = MAXC;
            for (int d = MAXC - 1; d >= 0; d--) {
                if (a.st->bucket_unres[d] > 0) open = d;
                a.st->bucket_unres[d] = 0;
            }
            a.st->bucket_open = open;
        }
    }
    if (a.iopen) {
        for (int b = threadIdx.x; b < a.nslots; b += blockDim.x) {
            int open = MAXC;
            for (int d = MAXC - 1; d >= 0; d--) {
                if (a.ibucket[b * MAXC + d] > 0) open = d;
                a.ibucket[b * MAXC + d] = 0;
            }
            a.iopen[b] = a.iasc[b] ? open : MAXC;
        }
    }
}

// (e) compacted list: exclusive scan of the per-tile counts (one block).
__global__ void k_p1_kscan(PmsArgs a) {
    if (a.st->converged || p1_small(a)) return;
    __shared__ int wsum[32];
    const int64_t n = (p1_count(a) + P1_TILE - 1) / P1_TILE;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int carry = 0;
    for (int64_t b0 = 0; b0 < n; b0 += blockDim.x) {
        const int64_t t = b0 + threadIdx.x;
        const int v = t < n ? a.kagg[t] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        int before = carry, total = 0;
        for (int w = 0; w < nw; w++) {
            if (w < wid) before += wsum[w];
            total += wsum[w];
        }
        if (t < n) a.kagg[t] = before + incl - v;
        carry += total;
        __syncthreads();
    }
    p1_kscan_tail(a, carry);
}

// (f) compacted list: the columns that stay unresolved, in order, into the
//     next list, and into the Phase II queue; first[] reset (once per row, by
//     its winner).  Clears marked in (d) are applied by the next Phase I
//     (Phase II skips such columns).
// Whether unresolved column j can add anything in this sweep's Phase II: its
// low lj has a pivot to its left now (published by Phase 0 / I), or one can
// be published during Phase II.  The latter happens only through the beta
// check, by the first column holding row lj (left[lj]), when that column is
// left of j, unresolved and its chain still above lj.  Other columns would
// find no pivot on their visit; leaving them out of the queue changes no
// addition.
#ifndef OPH_P2_FILTER
#define OPH_P2_FILTER 1
#endif
__device__ __forceinline__ bool p2_ready(const PmsArgs &a, int j) {
    if (a.clear[j]) return false;  // positive: cleared by the next Phase I
    const int lj = a.low[j];
    const int4 h = __ldcg(reinterpret_cast<const int4 *>(&a.rec[lj]));
    if (h.x >= 0 && h.x < j) return true;
    const int p = h.z;
    if (p < 0 || p >= j) return false;
    return a.classes[p] == 0 && a.low[p] > lj;
}

__device__ __forceinline__ void k_p1_scatter_tile(PmsArgs a, const int64_t n, const int64_t tile) {
    __shared__ int wsum[P1_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t base = (int64_t)tile * P1_TILE + (int64_t)threadIdx.x * P1_ITEMS;
    int cols[P1_ITEMS];
    unsigned keepmask = 0;
    int cnt = 0;
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++) {
        const int64_t idx = base + t;
        cols[t] = -1;
        if (idx < n) {
            const int64_t j = p1_col(a, idx);
            const int lj = a.low[j];
            if (lj >= 0 && a.first[lj] == (int)j) a.first[lj] = FIRST_NONE;
            if (lj >= 0 && a.classes[j] == 0) {
                cols[t] = (int)j;
                keepmask |= 1u << t;
                cnt++;
            }
        }
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    int off = a.kagg[tile] + incl - cnt;
    for (int w = 0; w < wid; w++) off += wsum[w];
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++)
        if (keepmask & (1u << t)) a.ulist_next[off++] = cols[t];
    // Phase II takes these columns from a queue filled by warp-aggregated
    // appends: concurrently reduced columns then come from all over the
    // matrix instead of one neighbourhood (which contends on shared pivots).
    // Only columns that can add this sweep are queued (p2_ready), and in
    // ascending order only those of the open buckets.
    const int open = a.ascending ? __ldcg(&a.st->bucket_open) : MAXC;
#pragma unroll
    for (int t = 0; t < P1_ITEMS; t++) {
        const bool kept = (keepmask >> t) & 1u;
        const bool want = kept && a.dim[cols[t]] + 1 <= (a.iopen ? a.iopen[a.inst[cols[t]]] : open) &&
                          (!OPH_P2_FILTER || p2_ready(a, cols[t]));
        warp_append(want, cols[t], a.worklist, &a.st->t_count[0]);
    }
}
// One pass over the list's tiles, a grid-stride loop: the grid is sized
// for the machine, not for the matrix (a grid of one block per tile of
// the full matrix costs ~0.3 ms of empty blocks per sweep at 3.5e8 columns).
__global__ void __launch_bounds__(P1_THREADS) k_p1_scatter(PmsArgs a) {
    if (a.st->converged || p1_small(a)) return;
    const int64_t n = p1_count(a);
    for (int64_t tile = blockIdx.x; tile * P1_TILE < n; tile += gridDim.x) {
        k_p1_scatter_tile(a, n, tile);
        __syncthreads();  // the next tile reuses the shared arrays
    }
}

// Phase I of a compacted list that fits one tile, as one block: (a)-(f) in
// order with block barriers between them, the tile's scan prefix being the
// empty one.  Six grid launches of mostly idle blocks become one.
__global__ void __launch_bounds__(P1_THREADS) k_p1_small(PmsArgs a) {
    if (a.st->converged || !p1_small(a)) return;
    const int64_t n = p1_count(a);
    if (threadIdx.x == 0) p1_reset(a);
    __syncthreads();
    p1_first_range(a, threadIdx.x, blockDim.x);
    __syncthreads();
    __shared__ int s_reps;
    k_p1_tiles_tile(a, n, 0);
    __syncthreads();
    if (threadIdx.x == 0) s_reps = atomicAdd(&a.st->reps, 0);  // thread 0 added the tile's count
    __syncthreads();
    if (s_reps == 0) {  // no repeated low: converged
        if (threadIdx.x == 0) a.st->converged = 1;
        return;
    }
    if (threadIdx.x < MAXC) a.agg[threadIdx.x] = -1;  // nothing before the first tile
    __syncthreads();
    k_p1_mark_tile(a, n, 0);
    __syncthreads();
    int keep = 0;
    if (threadIdx.x == 0) {  // the tile's count, written by thread 0; its offset is 0
        keep = a.kagg[0];
        a.kagg[0] = 0;
    }
    p1_kscan_tail(a, keep);  // reads `keep` on thread 0 only
    __syncthreads();
    k_p1_scatter_tile(a, n, 0);
}

// (e') without a compacted list: reset first[], apply the clears of this
//      Phase I, and queue the unresolved columns (any order) for Phase II.
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
        warp_append(want, (int)j, a.worklist, &a.st->t_count[0]);
    }
}

// -------------------------------------------------------------- Phase II
// Pool allocation for column j: the global bump pointer, or the pool region
// of j's instance when the columns belong to several instances.
__device__ __forceinline__ long long col_alloc(const PmsArgs &a, int j, long long ints) {
    if (!a.inst) return pool_alloc(a.st, ints);
    const int b = a.inst[j];
    const unsigned long long off = atomicAdd(&a.ipool[2 * b], (unsigned long long)ints);
    if (off + (unsigned long long)ints > a.ipool[2 * b + 1]) {
        atomicExch(&a.iover[b], 1);
        atomicExch(&a.st->overflow, 1);
        return -1;
    }
    return (long long)off;
}

// Phase II tiers.  A column is reduced with its rows on chip across its whole
// chain of additions; a column that would outgrow its tier is written back
// and queued for the next tier:
//   scalar  a lane per column,  48 rows      (32 columns per warp; k_p2_scalar)
//   tier 0  8 lanes per column, CAP 128      (4 columns per warp)
//   tier 1  a warp per column,  CAP 512      (pivot staged in shared memory
//                                             when wider than the warp)
//   tier 2  a CTA per column,   CAP 8192     (block-wide merge path)
//   tier 3  a CTA per column,   a bitmap of its rows (no limit; the merge
//                               path in pool buffers when the bitmap's window
//                               cannot hold a row)
// The queues ping-pong between the worklist and widelist arrays (the scalar
// tier hands on through slist).  Each addition costs one dependent round trip
// when the pivot has at most four entries (its record carries them, with
// left[] for the beta check) and two otherwise; reading G ints past a segment
// start stays in bounds through the pool's tail padding.
// In the lane groups, pivots of at most G entries are held one per lane and
// merged without staging: three rows read from their record in place
// (merge3_inplace: only the rows above the first insertion point move), other
// pivots of at most four entries by runs (merge_xor_seg, a loop over the
// pivot's entries), wider ones up to G by per-element threshold search
// (merge_xor_thr, a loop over A's chunks).
#ifndef OPH_INPLACE3
#define OPH_INPLACE3 1
#endif
// Which of tiers 0 (bit 0) and 1 (bit 1) reduce lazy columns
// (reduce_column_lazy); the others merge eagerly on every addition
// (reduce_column_smem).
#ifndef OPH_LAZY
#define OPH_LAZY 2
#endif
// Mark column lj positive (cleared by the next Phase I).  Every chain through
// row lj marks it again; with CHECK the flag is read (alongside the record)
// and written only while still 0, so the hot flags are not rewritten by
// thousands of warps (unconditional stores to a few hot L2 sectors left half
// of the SMs at a fifth of the others' rate).
template <bool CHECK = true>
__device__ __forceinline__ void mark_clear(const PmsArgs &a, int lj, bool leader) {
    if (!leader) return;
    if (!CHECK || !a.clear[lj]) a.clear[lj] = 1;
}
template <int G, class Tile>
__device__ void reduce_column_smem(const Tile &tile, const PmsArgs &a, int j, int *A, int *B, int *C, int cap,
                                   int32_t *out_list, int *out_cnt, long long &adds, long long &slots) {
    const int lane = tile.thread_rank();
    if (a.clear[j]) return;  // positive: cleared by the next Phase I
    int lj = a.low[j];
    if (lj < 0) return;
    int4 h, e;
    rec_load(&a.rec[lj], h, e);
    if (h.x < 0 || h.x >= j) return;  // no pivot to the left of j yet
    const long long sj = a.seg[j];
    int n = a.pool[sj];
    const int capj = a.pool[sj + 1];
    if (n > cap) {
        if (lane == 0) out_list[atomicAdd(out_cnt, 1)] = j;
        return;
    }
    group_copy<G>(tile, A, a.pool + sj + SEG_HDR, n);
    bool made_pivot = false, handed = false;
    for (;;) {
        // the pivot's rows: from the record when it holds them all, else from
        // the pivot's segment after an acquire of the record
        int np, pv;
        const int *P = nullptr;
        if (rec_complete(h, e)) {
            np = h.y;
            pv = rec_entry(e, lane & 3);
        } else {
            const int4 h2 = rec_header(&a.rec[lj], h);
            np = h2.y;
            P = a.pool + 4ll * (unsigned)h2.w + SEG_HDR;
            pv = P[lane];
        }
        if (n + np > cap) { handed = true; break; }
        int nn;
        bool swap = true;
        if (OPH_INPLACE3 && np == 3 && !P) {
            // the common apparent pair: its rows are in the record
            nn = merge3_inplace<G>(tile, A, n, e.x, e.y);
            swap = false;
        } else if (np <= 4) {
            nn = merge_xor_seg<G>(tile, A, n, pv, np, B);
        } else if (np <= G) {
            nn = merge_xor_thr<G>(tile, A, n, pv, np, B);
        } else if (C) {
            group_copy<G>(tile, C, P, np);
            nn = merge_xor<G>(tile, A, n, C, np, B);
        } else {
            nn = merge_xor<G>(tile, A, n, P, np, B);
        }
        slots += n + np + nn;
        adds++;
        n = nn;
        if (swap) {
            int *t = A; A = B; B = t;
        }
        lj = n ? A[n - 1] : -1;
        if (lj < 0) break;
        rec_load(&a.rec[lj], h, e);
        mark_clear(a, lj, lane == 0);
        if (h.z == j) { made_pivot = true; break; }  // the beta check: row lj first appears in j
        if (h.x < 0 || h.x >= j) break;
    }
    long long dst = sj;
    int dcap = capj;
    if (n > capj) {
        dcap = round4(max(n + (n >> 1), 16));
        long long off = 0;
        if (lane == 0) off = col_alloc(a, j, SEG_HDR + dcap);
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
            rec_publish(a.rec, lj, j, n, dst, A);
        }
    } else if (handed) {
        if (lane == 0) out_list[atomicAdd(out_cnt, 1)] = j;
    }
    tile.sync();
}

// The same chain of additions on a lazy column.  The column under reduction
// is T = A xor D: A ascending in shared memory (the column as of the last
// flush, less the entries popped off its top), D ascending in registers
// (lane k < dn holds D[k]), the pending toggles, at most G of them.  Adding
// a pivot P (whose last entry is low(T)) pops low(T) off whichever of A and
// D holds it and toggles P's other entries in D: a ballot gives each one's
// rank and a one-lane shuffle makes or closes its slot.  Equal tops of A and
// D cancel as they surface.  D is merged into A (merge_xor_thr) only when a
// pivot would not fit in what is left of D and when the chain ends, so an
// addition costs O(|P|) register work instead of an O(|T|) copy: on the
// long top-dimension chains of Rips complexes a flush comes every 6 (G = 8)
// to 38 (G = 32) additions.  Pivots wider than G are merged eagerly into A.
// With STATS the exact |T| is carried through every addition (membership of
// each toggled row in A by binary search) for the |P| + |T| + |T xor P|
// counters; without it only additions are counted.
struct LazyDiag {
    unsigned long long c[8];
};
template <int G, bool STATS, class Tile>
__device__ void reduce_column_lazy(const Tile &tile, const PmsArgs &a, int j, int *A, int *B, int *C, int cap,
                                   int32_t *out_list, int *out_cnt, long long &adds, long long &slots,
                                   LazyDiag &dg) {
    const int lane = tile.thread_rank();
    if (a.clear[j]) return;  // positive: cleared by the next Phase I
    int lj = a.low[j];
    if (lj < 0) return;
    int4 h, e;
    rec_load(&a.rec[lj], h, e);
    if (h.x < 0 || h.x >= j) return;  // no pivot to the left of j yet
    const long long sj = a.seg[j];
    int n = a.pool[sj];
    const int capj = a.pool[sj + 1];
    if (n > cap) {
        if (lane == 0) out_list[atomicAdd(out_cnt, 1)] = j;
        return;
    }
    group_copy<G>(tile, A, a.pool + sj + SEG_HDR, n);
    if (OPH_COUNTS) { dg.c[6]++; dg.c[7] += n; }
    int dn = 0, dv = 0;
    int tsize = n;  // |T|, kept with STATS
    bool made_pivot = false, handed = false;
    for (;;) {
        int np, pv;
        const int *P = nullptr;
        if (rec_complete(h, e)) {
            np = h.y;
            pv = rec_entry(e, lane & 3);
        } else {
            const int4 h2 = rec_header(&a.rec[lj], h);
            np = h2.y;
            P = a.pool + 4ll * (unsigned)h2.w + SEG_HDR;
            pv = P[lane];
        }
        if (n + dn + np > cap) { handed = true; break; }
        if (OPH_COUNTS) dg.c[np - 1 > G ? 3 : np > 4 ? 2 : P ? 1 : 0]++;
        // pop low(T): the larger of the two (settled, so different) tops
        if (n > 0 && A[n - 1] == lj) n--;
        else dn--;
        const int k = np - 1;  // P's entries below the low
        int common = 1;        // |T and P|, with STATS
        if (STATS && k <= G) {
            for (int t = 0; t < k; t++) {
                const int x = tile.shfl(pv, t);
                const bool inD = tile.ballot(lane < dn && dv == x) != 0u;
                const int r = lower_bound(A, n, x);
                const bool inA = r < n && A[r] == x;
                common += inA != inD;
            }
        }
        if (k > G - dn && dn > 0) {  // no room in D: flush it into A
            if (OPH_COUNTS) dg.c[4]++;
            n = merge_xor_thr<G>(tile, A, n, dv, dn, B);
            int *t = A; A = B; B = t;
            dn = 0;
        }
        if (k > G) {
            // a wide pivot, merged into A directly (staged when there is room)
            const int *src = P;
            if (C) {
                group_copy<G>(tile, C, P, k);
                src = C;
            }
            const int nn = merge_xor<G>(tile, A, n, src, k, B);
            if (STATS) common += (n + k - nn) / 2;
            n = nn;
            int *t = A; A = B; B = t;
        } else if (k <= 4) {
            for (int t = 0; t < k; t++) {
                const int x = tile.shfl(pv, t);
                const bool valid = lane < dn;
                const int r = __popc(tile.ballot(valid && dv < x));
                if (tile.ballot(valid && dv == x)) {
                    const int v = tile.shfl_down(dv, 1);
                    if (lane >= r) dv = v;
                    dn--;
                } else {
                    const int v = tile.shfl_up(dv, 1);
                    if (lane > r) dv = v;
                    if (lane == r) dv = x;
                    dn++;
                }
            }
        } else {
            // D xor P' through shared memory (B is free between flushes)
            if (lane < dn) B[lane] = dv;
            tile.sync();
            const int nd = merge_xor_thr<G>(tile, B, dn, pv, k, B + G);
            dv = lane < nd ? B[G + lane] : 0;
            tile.sync();
            dn = nd;
        }
        if (STATS) {
            const int nt = tsize + np - 2 * common;
            slots += tsize + np + nt;
            tsize = nt;
        }
        adds++;
        // settle: equal tops of A and D cancel; the larger top is the low
        for (;;) {
            const int at = n > 0 ? A[n - 1] : -1;
            const int dt = tile.shfl(dv, dn > 0 ? dn - 1 : 0);
            if (dn > 0 && at == dt) {
                n--;
                dn--;
                if (OPH_COUNTS) dg.c[5]++;
                continue;
            }
            lj = dn > 0 ? max(at, dt) : at;
            break;
        }
        if (lj < 0) break;
        rec_load(&a.rec[lj], h, e);
        mark_clear(a, lj, lane == 0);
        if (h.z == j) { made_pivot = true; break; }  // the beta check: row lj first appears in j
        if (h.x < 0 || h.x >= j) break;
    }
    if (dn > 0) {
        n = merge_xor_thr<G>(tile, A, n, dv, dn, B);
        int *t = A; A = B; B = t;
    }
    long long dst = sj;
    int dcap = capj;
    if (n > capj) {
        dcap = round4(max(n + (n >> 1), 16));
        long long off = 0;
        if (lane == 0) off = col_alloc(a, j, SEG_HDR + dcap);
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
            rec_publish(a.rec, lj, j, n, dst, A);
        }
    } else if (handed) {
        if (lane == 0) out_list[atomicAdd(out_cnt, 1)] = j;
    }
    tile.sync();
}

__device__ __forceinline__ void tier_stats(const PmsArgs &a, int tier, long long adds, long long slots) {
    if (adds) {
        atomicAdd(&a.st->additions, (unsigned long long)adds);
        atomicAdd(&a.st->slots, (unsigned long long)slots);
        atomicAdd(&a.st->tier_adds[tier], (unsigned long long)adds);
        atomicAdd(&a.st->tier_slots[tier], (unsigned long long)slots);
    }
}

// ------------------------------------------------------------ scalar tier
// Short columns, one per lane: the first Phase II pass over the queue.  A
// lane holds its column in shared memory interleaved with the other lanes'
// (row k of the lane's column at col[32 k]; whatever rows the lanes touch,
// their accesses fall in distinct banks) and adds pivots of at most four
// rows, read from their records, by scalar toggles: rank the row, then
// shift the rows above it by one.  32 columns per warp, no lane idle on
// another's work.  A column that would outgrow TS_CAP rows, or meets a pivot
// not held whole in its record, is written back and handed to tier 0.
#ifndef OPH_TS_CAP
#define OPH_TS_CAP 48
#endif
constexpr int TS_CAP = OPH_TS_CAP;
constexpr int TS_BLOCK = 256;
#ifndef OPH_SCALAR
#define OPH_SCALAR 1
#endif

// Toggle row x in the lane's column of m1 rows; returns the new length.
__device__ __forceinline__ int ts_toggle(int *col, int m1, int x) {
    int lo = 0, len = m1;
    while (len > 0) {
        const int h = len >> 1;
        if (col[(lo + h) * 32] < x) { lo += h + 1; len -= h + 1; }
        else len = h;
    }
    if (lo < m1 && col[lo * 32] == x) {
        for (int k = lo; k < m1 - 1; k++) col[k * 32] = col[(k + 1) * 32];
        return m1 - 1;
    }
    for (int k = m1; k > lo; k--) col[k * 32] = col[(k - 1) * 32];
    col[lo * 32] = x;
    return m1 + 1;
}

#ifndef OPH_TS_REFILL
#define OPH_TS_REFILL 24
#endif
constexpr int TS_REFILL = OPH_TS_REFILL;
// The queue a scalar pass takes its columns from, and the list it hands on to.
struct ScalarQ {
    const int32_t *in;
    const int *in_count;
    int *cursor;
    int32_t *out;
    int *out_count;
};

// CAP rows per lane in BLOCK * CAP ints of dynamic shared memory.
template <int CAP, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_p2_scalar(PmsArgs a, ScalarQ sq) {
    if (a.st->converged) return;
    extern __shared__ int sm[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int *col = sm + wid * CAP * 32 + lane;
    const int count = *sq.in_count;
    long long adds = 0, slots = 0;
    bool active = false, exhausted = false;
    int j = -1, n = 0, lj = -1, capj = 0;
    long long sj = 0;
    int4 h = make_int4(0, 0, 0, 0), e = h;
    LazyDiag dg{};  // OPH_COUNTS: [0] additions, [1] handed over at load, [2] mid-chain, [3] steps, [4] loads, [5] rows
    int fin = 0;  // a finished column awaiting write-back: 1 hand off, 2 stop, 3 became a pivot
    for (;;) {
        if (OPH_COUNTS) dg.c[3]++;
        // Book-keeping (write-backs and refills) diverges from the additions,
        // so it waits until at least TS_REFILL lanes have no column to add to
        // (or none has): finished lanes keep their column in shared memory
        // until then, and the long paths run with many lanes at once.
        const unsigned waiting = __ballot_sync(0xffffffffu, !active);
        if (__popc(waiting) >= TS_REFILL || waiting == 0xffffffffu) {
            bool handoff = false;
            if (fin) {
                long long dst = sj;
                int dcap = capj;
                bool stored = true;
                if (n > capj) {
                    dcap = round4(max(n + (n >> 1), 16));
                    dst = col_alloc(a, j, SEG_HDR + dcap);
                    stored = dst >= 0;  // pool exhausted: j keeps its pre-sweep state
                }
                if (stored) {
                    int *d = a.pool + dst + SEG_HDR;
                    for (int k = 0; k < n; k++) d[k] = col[k * 32];
                    a.pool[dst] = n;
                    a.pool[dst + 1] = dcap;
                    a.seg[j] = dst;
                    a.low[j] = lj;
                    if (fin == 3) {
                        int top[4];
                        const int k0 = n > 4 ? n - 4 : 0;
                        for (int k = 0; k < 4; k++) top[k] = k0 + k < n ? col[(k0 + k) * 32] : -1;
                        a.classes[j] = -1;
                        rec_publish_top(a.rec, lj, j, n, dst, top);
                    }
                    handoff = fin == 1;
                }
                fin = 0;
            }
            warp_append(handoff, j, sq.out, sq.out_count);
            handoff = false;
            // lanes without a column take the next ones from the queue
            const bool need = !active && !exhausted;
            const unsigned nm = __ballot_sync(0xffffffffu, need);
            if (nm) {
                const int leader = __ffs(nm) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(sq.cursor, __popc(nm));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (need) {
                    const int idx = base + __popc(nm & ((1u << lane) - 1u));
                    if (idx >= count) {
                        exhausted = true;
                    } else {
                        j = sq.in[idx];
                        lj = a.low[j];
                        bool ok = lj >= 0 && !a.clear[j];
                        if (ok) {
                            rec_load(&a.rec[lj], h, e);
                            ok = h.x >= 0 && h.x < j;  // a pivot to the left of j
                        }
                        if (ok) {
                            sj = a.seg[j];
                            n = a.pool[sj];
                            capj = a.pool[sj + 1];
                            // a column this tier cannot add its first pivot to
                            // goes to tier 0 untouched
                            if (n > CAP || !rec_complete(h, e) || n + h.y - 2 > CAP) {
                                handoff = true;
                                if (OPH_COUNTS) dg.c[1]++;
                            } else {
                                // 16-byte loads issued together (a segment starts
                                // on 16 bytes, its capacity a multiple of four)
                                const int4 *src = reinterpret_cast<const int4 *>(a.pool + sj + SEG_HDR);
#pragma unroll 12
                                for (int q = 0; q < CAP / 4; q++)
                                    if (4 * q < n) {
                                        const int4 v = __ldcg(src + q);
                                        col[(4 * q) * 32] = v.x;
                                        col[(4 * q + 1) * 32] = v.y;
                                        col[(4 * q + 2) * 32] = v.z;
                                        col[(4 * q + 3) * 32] = v.w;
                                    }
                                active = true;
                                if (OPH_COUNTS) { dg.c[4]++; dg.c[5] += n; }
                            }
                        }
                    }
                }
            }
            warp_append(handoff, j, sq.out, sq.out_count);
            if (__all_sync(0xffffffffu, !active && exhausted)) break;
        }
        // one addition on every column that has a pivot to add
        if (active) {
            const int np = h.y;
            if (!rec_complete(h, e) || n + np - 2 > CAP) {
                fin = 1;
                if (OPH_COUNTS) dg.c[2]++;
            } else {
                int m1 = n - 1;  // the low cancels
                for (int t = np - 2; t >= 0; t--) m1 = ts_toggle(col, m1, rec_entry(e, t));
                slots += n + np + m1;
                adds++;
                if (OPH_COUNTS) dg.c[0]++;
                n = m1;
                lj = n > 0 ? col[(n - 1) * 32] : -1;
                if (lj < 0) {
                    fin = 2;
                } else {
                    rec_load(&a.rec[lj], h, e);
                    mark_clear(a, lj, true);
                    if (h.z == j) fin = 3;  // the beta check: row lj first appears in j
                    else if (h.x < 0 || h.x >= j) fin = 2;
                }
            }
            if (fin) active = false;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        adds += __shfl_xor_sync(0xffffffffu, adds, o);
        slots += __shfl_xor_sync(0xffffffffu, slots, o);
    }
    if (lane == 0) {
        tier_stats(a, 0, adds, slots);
        if (adds) atomicAdd(&a.st->s_adds, (unsigned long long)adds);
    }
    if (OPH_COUNTS)
        for (int q = 0; q < 6; q++)
            if (dg.c[q]) atomicAdd(&a.st->sdiag[q], dg.c[q]);
}

// Tiers 0 and 1: groups of G lanes, each group with A/B buffers of CAP ints
// and, with STAGE, a C buffer into which a pivot wider than the group is
// staged; without it (tier 0) such a pivot is searched in the store.
template <int G, int CAP, int BLOCK, bool STAGE, bool LAZY>
__device__ __forceinline__ void p2_tier_body(const PmsArgs &a, int tier) {
    if (a.st->converged) return;
    extern __shared__ int smem[];
    auto tile = cg::tiled_partition<G>(cg::this_thread_block());
    const int gid = threadIdx.x / G;
    int *buf = smem + (size_t)gid * (STAGE ? 3 : 2) * CAP;
    int32_t *in_list = tier == 0 ? a.t0_list : (tier & 1) ? a.widelist : a.worklist;
    int32_t *out_list = (tier & 1) ? a.worklist : a.widelist;
    const int count = tier == 0 ? *a.t0_count : a.st->t_count[tier];
    long long adds = 0, slots = 0;
    LazyDiag dg{};
    for (;;) {
        int idx = 0;
        if (tile.thread_rank() == 0) idx = atomicAdd(&a.st->t_cursor[tier], 1);
        idx = tile.shfl(idx, 0);
        if (idx >= count) break;
        {
            int *C = STAGE ? buf + 2 * CAP : nullptr;
            int *qn = &a.st->t_count[tier + 1];
            if (!LAZY) {
                const long long before = adds;
                reduce_column_smem<G>(tile, a, in_list[idx], buf, buf + CAP, C, CAP, out_list, qn, adds, slots);
                if (OPH_COUNTS) {  // eager tier: visits, longest chain, columns that added
                    const unsigned long long c = (unsigned long long)(adds - before);
                    dg.c[4]++;
                    dg.c[5] = c > dg.c[5] ? c : dg.c[5];
                    dg.c[6] += c > 0;
                }
            }
            else if (a.stats)
                reduce_column_lazy<G, true>(tile, a, in_list[idx], buf, buf + CAP, C, CAP, out_list, qn, adds, slots,
                                            dg);
            else
                reduce_column_lazy<G, false>(tile, a, in_list[idx], buf, buf + CAP, C, CAP, out_list, qn, adds, slots,
                                             dg);
        }
    }
    if (tile.thread_rank() == 0) {
        tier_stats(a, tier, adds, slots);
        if (OPH_COUNTS) {
            for (int q = 0; q < 8; q++) {
                if (!dg.c[q]) continue;
                if (!LAZY && q == 5) atomicMax(&a.st->diag[8 * (tier & 1) + q], dg.c[q]);
                else atomicAdd(&a.st->diag[8 * (tier & 1) + q], dg.c[q]);
            }
#if OPH_COUNTS
            unsigned smid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            if (adds) atomicAdd(&a.st->diag_sm[smid & 255], (unsigned long long)adds);
#endif
        }
    }
}

// Tier 0 (the autotuned narrow tier) with its occupancy target: resident
// columns hide the record reads of the chains, so the register budget is
// held to what T0_MINB blocks of BLOCK threads per SM allow.
#ifndef OPH_T0_MINB
#define OPH_T0_MINB 0
#endif
template <int G, int CAP, int BLOCK, bool STAGE, bool LAZY>
#if OPH_T0_MINB > 0
__global__ void __launch_bounds__(BLOCK, OPH_T0_MINB) k_p2_tier(PmsArgs a, int tier) {
#else
__global__ void __launch_bounds__(BLOCK) k_p2_tier(PmsArgs a, int tier) {
#endif
    p2_tier_body<G, CAP, BLOCK, STAGE, LAZY>(a, tier);
}
// Tier 1 (a warp per column; its shared buffers bound the occupancy).
template <int G, int CAP, int BLOCK, bool STAGE, bool LAZY>
__global__ void __launch_bounds__(BLOCK) k_p2_tier1(PmsArgs a, int tier) {
    p2_tier_body<G, CAP, BLOCK, STAGE, LAZY>(a, tier);
}

// The shared-memory window of tier 3 (per CTA): 96 KB, 786,432 rows below a
// column's low (a larger window left too little L1 for the pivots' rows: the
// 5M-column torus lost 6%, and the lower-star image and the batch gained
// nothing).  A column whose rows all lie in it is reduced there:
// an addition then costs O(|P|) shared toggles and a shared search for the
// next low, where the merge path rewrites all of T and the global bitmap
// pays an L2 round trip for each.
#ifndef OPH_SBM_WORDS
#define OPH_SBM_WORDS 24576
#endif
constexpr int SBM_WORDS = OPH_SBM_WORDS;
constexpr size_t SBM_BYTES = sizeof(uint32_t) * SBM_WORDS;

// True when column j's rows (first T0, low lj) lie in a shared window.
__device__ __forceinline__ bool fits_sbm(int T0, int lj) { return (long long)lj - T0 < 32ll * SBM_WORDS - 32; }

// The start of a CTA's column: its low and that row's pivot record, read by
// one thread and shared, so that every thread of the CTA takes the same
// branches around its barriers (the clear flag and the record can change
// under other chains between two threads' reads).  True when an addition is
// due: not cleared, a low whose pivot lies to the left.
__device__ __forceinline__ bool col_start(const PmsArgs &a, int j, int &lj, int4 &h, int4 &e) {
    __shared__ __align__(16) int4 s_he[2];
    __shared__ int s_lj;
    if (threadIdx.x == 0) {
        const int l = a.clear[j] ? -1 : a.low[j];
        int4 hh = make_int4(-1, 0, 0, 0), ee = make_int4(-1, -1, -1, -1);
        if (l >= 0) rec_load_acq(&a.rec[l], hh, ee);
        s_lj = l;
        s_he[0] = hh;
        s_he[1] = ee;
    }
    __syncthreads();  // rewritten only by the next column's call, behind the caller's queue barriers
    lj = s_lj;
    h = s_he[0];
    e = s_he[1];
    return lj >= 0 && h.x >= 0 && h.x < j;
}

// Tiers 2 and 3: the whole CTA on one column.  With cap > 0 the column and
// the staged pivot live in shared memory (A/B/C of cap ints); with cap == 0
// they live in pool-allocated buffers that grow as needed.
__device__ void reduce_column_block(const PmsArgs &a, int j, int *sA, int *sB, int *sC, int cap, int *scratch,
                                    int32_t *out_list, int *out_cnt, long long &adds, long long &slots) {
    __shared__ long long s_off;
    __shared__ int s_small[4];
    __shared__ __align__(16) int4 s_rec[2];
    const int tid = threadIdx.x;
    int lj;
    int4 h, e;
    if (!col_start(a, j, lj, h, e)) return;
    const long long sj = a.seg[j];
    int n = a.pool[sj];
    const int capj = a.pool[sj + 1];
    const bool smem_mode = cap > 0;
    if (smem_mode && n > cap) {
        if (tid == 0) out_list[atomicAdd(out_cnt, 1)] = j;
        return;
    }
    int *A, *B;
    int bcap;
    if (smem_mode) {
        A = sA; B = sB; bcap = cap;
        block_copy(A, a.pool + sj + SEG_HDR, n);
    } else {
        bcap = round4(max(2 * n, 4096));
        if (tid == 0) s_off = col_alloc(a, j, 2ll * bcap);
        __syncthreads();
        if (s_off < 0) return;
        A = a.pool + s_off; B = A + bcap;
        block_copy(A, a.pool + sj + SEG_HDR, n);
    }
    bool made_pivot = false, handed = false;
    // The record came with acquire (rec_load_acq), so a wide pivot's rows are
    // read straight from its segment.  When the next low is known before the
    // merge (the larger of the column's and the pivot's second rows, when
    // they differ), thread 0 fetches its record during the copy and the
    // merge and settles it after: one round trip per addition off the chain.
    int t1 = n >= 2 ? A[n - 2] : -1;
    for (;;) {
        const int np = h.y;
        const bool inrec = np <= 4;
        const int p2 = np >= 2 ? (inrec ? rec_entry(e, np - 2) : e.z) : -1;
        const bool known = t1 != p2 || t1 < 0;
        const int pnext = known ? max(t1, p2) : -1;
        int4 hh = make_int4(-1, 0, 0, 0), ee = make_int4(-1, -1, -1, -1);
        if (tid == 0 && pnext >= 0) rec_fetch(&a.rec[pnext], hh, ee);
        const int *P;
        if (inrec) {
            if (tid < np) s_small[tid] = rec_entry(e, tid);
            __syncthreads();
            P = s_small;
        } else {
            P = a.pool + 4ll * (unsigned)h.w + SEG_HDR;
        }
        if (n + np > bcap) {
            if (smem_mode) { handed = true; break; }
            const int ncap = round4(2 * (n + np));
            if (tid == 0) s_off = col_alloc(a, j, 2ll * ncap);
            __syncthreads();
            if (s_off < 0) return;  // j keeps its pre-sweep state
            int *NA = a.pool + s_off;
            block_copy(NA, A, n);
            A = NA; B = NA + ncap; bcap = ncap;
        }
        if (smem_mode && P != s_small) {
            block_copy(sC, P, np);
            P = sC;
        }
        const int nn = merge_xor_path(A, n, P, np, B, scratch);
        slots += n + np + nn;
        adds++;
        n = nn;
        int *t = A; A = B; B = t;
        lj = n ? A[n - 1] : -1;
        if (lj < 0) break;
        if (known && lj == pnext) {
            if (tid == 0) {
                rec_settle(&a.rec[lj], hh, ee);
                s_rec[0] = hh;
                s_rec[1] = ee;
            }
        } else if (tid == 0) {
            rec_load_acq(&a.rec[lj], hh, ee);
            s_rec[0] = hh;
            s_rec[1] = ee;
        }
        __syncthreads();  // rewritten only after the next merge's barriers
        h = s_rec[0];
        e = s_rec[1];
        mark_clear<false>(a, lj, tid == 0);  // few columns: no hot flags
        if (h.z == j) { made_pivot = true; break; }
        if (h.x < 0 || h.x >= j) break;
        t1 = n >= 2 ? A[n - 2] : -1;
    }
    long long dst = sj;
    int dcap = capj;
    if (n > capj) {
        dcap = round4(max(n + (n >> 1), 16));
        if (tid == 0) s_off = col_alloc(a, j, SEG_HDR + dcap);
        __syncthreads();
        if (s_off < 0) return;
        dst = s_off;
    }
    block_copy(a.pool + dst + SEG_HDR, A, n);
    if (tid == 0) {
        a.pool[dst] = n;
        a.pool[dst + 1] = dcap;
        a.seg[j] = dst;
        a.low[j] = lj;
    }
    if (made_pivot) {
        fence_acq_rel();
        __syncthreads();
        if (tid == 0) {
            a.classes[j] = -1;
            rec_publish(a.rec, lj, j, n, dst, A);
        }
    } else if (handed) {
        if (tid == 0) out_list[atomicAdd(out_cnt, 1)] = j;
    }
    __syncthreads();
}

template <int CAP, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_p2_block(PmsArgs a, int tier) {
    if (a.st->converged) return;
    extern __shared__ int smem[];
    __shared__ int scratch[2 * (BLOCK / 32)];
    __shared__ int s_idx, s_route;
    int32_t *in_list = tier == 0 ? a.t0_list : (tier & 1) ? a.widelist : a.worklist;
    int32_t *out_list = (tier & 1) ? a.worklist : a.widelist;
    const int count = tier == 0 ? *a.t0_count : a.st->t_count[tier];
    long long adds = 0, slots = 0;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(&a.st->t_cursor[tier], 1);
        __syncthreads();
        const int idx = s_idx;
        __syncthreads();
        if (idx >= count) break;
        const int j = in_list[idx];
        if (tier == 2) {
            // a column whose rows fit tier 3's shared window is reduced there:
            // its additions toggle bits instead of rewriting the column (one
            // thread decides: clear[j] may change under other chains)
            if (threadIdx.x == 0) {
                const int lj = a.low[j];
                const long long sj = a.seg[j];
                s_route = lj >= 0 && !a.clear[j] && fits_sbm(a.pool[sj] > 0 ? a.pool[sj + SEG_HDR] : lj, lj);
                if (s_route) out_list[atomicAdd(&a.st->t_count[3], 1)] = j;
            }
            __syncthreads();
            const bool routed = s_route;
            __syncthreads();
            if (routed) continue;
        }
        reduce_column_block(a, j, smem, smem + CAP, smem + 2 * CAP, CAP, scratch, out_list,
                            tier < 3 ? &a.st->t_count[tier + 1] : nullptr, adds, slots);
    }
    if (threadIdx.x == 0) tier_stats(a, tier, adds, slots);
}

// ------------------------------------------------------------ bitmap tier
// Tier 3's columns (longer than tier 2's shared buffers) as a bitmap over
// rows [w0, w0 + 32 * bm_words) in a per-CTA scratch in global memory: an
// addition toggles the pivot's bits, O(|P|) work where a merge rewrites all
// of T (the reduced cochains of a Rips complex's anti-transpose run to ~10^5
// rows against pivots of a few hundred); the next low is the highest set bit
// below the old one; the rows are written back in order, and the words
// cleared, once, when the chain ends.  A row below w0 (a window smaller than
// the matrix) sends the column to the merge path instead.
constexpr int64_t BM_MAX_WORDS = 1 << 18;
constexpr int BM_BLOCK = 1024;
// A 16-byte load of bitmap words: through L2 for the global bitmap (other
// blocks never touch a CTA's scratch, but L1 is not kept coherent with the
// atomics), plain for the shared one.
template <bool SM>
__device__ __forceinline__ uint4 bm_load4(const uint32_t *p) {
    if (SM) return *reinterpret_cast<const uint4 *>(p);
    return __ldcg(reinterpret_cast<const uint4 *>(p));
}
template <bool SM>
__device__ __forceinline__ uint32_t bm_load(const uint32_t *p) {
    if (SM) return *p;
    return __ldcg(p);
}


// Rows of words [lo, top] in ascending order into dst (when not null), the
// words zeroed; every set bit lies in that range.  Four words per thread
// (lo rounded down to a multiple of 4, the per-CTA scratch a multiple of 4
// words long).  Returns the number of rows.
template <bool SM>
__device__ int bitmap_extract(uint32_t *bm, int lo, int top, int w0, int *dst, int *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int out = 0;
    for (int base = lo & ~3; base <= top; base += 4 * (int)blockDim.x) {
        const int w = base + 4 * (int)threadIdx.x;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (w <= top) v = bm_load4<SM>(bm + w);
        const int c = __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) red[wid] = incl;
        __syncthreads();
        int before = 0, total = 0;
        for (int q = 0; q < nw; q++) {
            if (q < wid) before += red[q];
            total += red[q];
        }
        __syncthreads();
        if (c) {
            int pos = out + before + incl - c;
            if (dst) {
                const uint32_t words[4] = {v.x, v.y, v.z, v.w};
                for (int q = 0; q < 4; q++)
                    for (uint32_t b = words[q]; b; b &= b - 1) dst[pos++] = w0 + (w + q) * 32 + (__ffs(b) - 1);
            }
            *reinterpret_cast<uint4 *>(bm + w) = make_uint4(0u, 0u, 0u, 0u);
        }
        out += total;
    }
    __syncthreads();
    return out;
}

// The highest set bit of the bitmap strictly below bit `pos` (relative to
// the window), -1 when there is none: a warp's search from the top, 128
// words a step, 16-byte loads (the words above pos's own are clear or
// masked).
template <bool SM>
__device__ __forceinline__ int bm_below(const uint32_t *bm, int pos) {
    const int lane = threadIdx.x & 31;
    if (pos <= 0) return -1;
    const int wl = (pos - 1) >> 5;
    const uint32_t ml = 0xffffffffu >> (31 - ((pos - 1) & 31));  // bits 0 .. (pos - 1) & 31
    for (int c0 = wl & ~3; c0 >= 0; c0 -= 128) {
        const int w = c0 - 4 * lane;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (w >= 0) v = bm_load4<SM>(bm + w);
        const uint32_t q0 = w > wl ? 0u : w == wl ? v.x & ml : v.x;
        const uint32_t q1 = w + 1 > wl ? 0u : w + 1 == wl ? v.y & ml : v.y;
        const uint32_t q2 = w + 2 > wl ? 0u : w + 2 == wl ? v.z & ml : v.z;
        const uint32_t q3 = w + 3 > wl ? 0u : w + 3 == wl ? v.w & ml : v.w;
        const int hi = q3 ? (w + 3) * 32 + 31 - __clz(q3)
                     : q2 ? (w + 2) * 32 + 31 - __clz(q2)
                     : q1 ? (w + 1) * 32 + 31 - __clz(q1)
                     : q0 ? w * 32 + 31 - __clz(q0) : -1;
        const unsigned nz = __ballot_sync(0xffffffffu, hi >= 0);
        if (nz) return __shfl_sync(0xffffffffu, hi, __ffs(nz) - 1);  // the lowest lane holds the highest words
    }
    return -1;
}

// Named barrier among the first `count` threads of the CTA (id 1; 0 is
// __syncthreads): a chain's warps meet without its prefetching warp.
__device__ __forceinline__ void bar_named(int count) { asm volatile("bar.sync 1, %0;" ::"r"(count) : "memory"); }

// A bitmap window seen through `word(w)`: a pointer to its word w, in the
// CTA's own shared memory (tier 3) or in the slice of a cluster that holds it
// (tier 4, distributed shared memory).

// The highest set bit strictly below window row `pos`, -1 when there is
// none: a warp's search from the top, 128 words a step.
template <class W>
__device__ __forceinline__ int bits_below(W word, int pos) {
    const int lane = threadIdx.x & 31;
    if (pos <= 0) return -1;
    const int wl = (pos - 1) >> 5;
    const uint32_t ml = 0xffffffffu >> (31 - ((pos - 1) & 31));
    for (int c0 = wl & ~3; c0 >= 0; c0 -= 128) {
        const int w = c0 - 4 * lane;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (w >= 0) v = *reinterpret_cast<const uint4 *>(word(w));
        const uint32_t q0 = w > wl ? 0u : w == wl ? v.x & ml : v.x;
        const uint32_t q1 = w + 1 > wl ? 0u : w + 1 == wl ? v.y & ml : v.y;
        const uint32_t q2 = w + 2 > wl ? 0u : w + 2 == wl ? v.z & ml : v.z;
        const uint32_t q3 = w + 3 > wl ? 0u : w + 3 == wl ? v.w & ml : v.w;
        const int hi = q3 ? (w + 3) * 32 + 31 - __clz(q3)
                     : q2 ? (w + 2) * 32 + 31 - __clz(q2)
                     : q1 ? (w + 1) * 32 + 31 - __clz(q1)
                     : q0 ? w * 32 + 31 - __clz(q0) : -1;
        const unsigned nz = __ballot_sync(0xffffffffu, hi >= 0);
        if (nz) return __shfl_sync(0xffffffffu, hi, __ffs(nz) - 1);  // the lowest lane holds the highest words
    }
    return -1;
}

// The prefetching warp of a chain.  In a large matrix the pivot records and
// pivot rows a chain visits sit in HBM, not L2, and each addition waits on
// the record of its low and then on the pivot's rows.  Most next lows of a
// long column are among its highest set bits below the current low (84% on
// the anti-transpose of a Rips torus, 75% within the highest 16), so this
// warp, outside the chain's barriers, follows the low the chain publishes
// (`cur`): each round it takes the 32 highest set bits below it (lane k the
// k-th, from a racy view of the bitmap: only what is prefetched depends on
// it), reads their records (bringing them into L2) and prefetches the rows of
// their pivots.  It stops when `done` is set, or after a bounded number of
// rounds.
template <class W>
__device__ void chain_prefetcher(const PmsArgs &a, W word, int w0, const volatile int *cur, const volatile int *done,
                                 int *tmp) {
    const int lane = threadIdx.x & 31;
    int last = -2;
    for (int round = 0; round < (1 << 20); round++) {
        const int d = __shfl_sync(0xffffffffu, *done, 0);
        if (d) break;
        const int lj = __shfl_sync(0xffffffffu, *cur, 0);
        if (lj == last || lj < 0) {
            __nanosleep(100);
            continue;
        }
        last = lj;
        // the 32 highest set bits below the low, at most four steps of 128
        // words down
        tmp[lane] = -1;
        __syncwarp();
        const int pos = lj - w0;
        const int wl = (pos - 1) >> 5;
        const uint32_t ml = 0xffffffffu >> (31 - ((pos - 1) & 31));
        int got = 0;
        for (int c0 = wl & ~3, st = 0; pos > 0 && c0 >= 0 && st < 4 && got < 32; c0 -= 128, st++) {
            const int w = c0 - 4 * lane;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (w >= 0) v = *reinterpret_cast<const uint4 *>(word(w));
            const uint32_t q0 = w > wl ? 0u : w == wl ? v.x & ml : v.x;
            const uint32_t q1 = w + 1 > wl ? 0u : w + 1 == wl ? v.y & ml : v.y;
            const uint32_t q2 = w + 2 > wl ? 0u : w + 2 == wl ? v.z & ml : v.z;
            const uint32_t q3 = w + 3 > wl ? 0u : w + 3 == wl ? v.w & ml : v.w;
            const int c = __popc(q0) + __popc(q1) + __popc(q2) + __popc(q3);
            int incl = c;  // lane 0 holds the highest words: ranks run up the lanes
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += u;
            }
            int r = got + incl - c;
            const uint32_t qs[4] = {q3, q2, q1, q0};
#pragma unroll
            for (int k = 0; k < 4; k++)
                for (uint32_t x = qs[k]; x && r < 32; r++) {
                    const int hb = 31 - __clz(x);
                    x &= ~(1u << hb);
                    tmp[r] = (w + 3 - k) * 32 + hb;
                }
            got += __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
        }
        const int my = tmp[lane];
        __syncwarp();
        if (my >= 0) {
            const int4 hc = __ldcg(reinterpret_cast<const int4 *>(&a.rec[w0 + my]));
            if (hc.x >= 0 && hc.y > 4 && (unsigned)hc.w != SEG4_NONE) {
                const int *P = a.pool + 4ll * (unsigned)hc.w + SEG_HDR;
                const int lines = min((4 * hc.y + 127) >> 7, 16);
                for (int q = 0; q < lines; q++) prefetch_l2(P + 32 * q);
            }
        }
    }
}

struct ChainResult {
    int n, lj, lo;     // the column's length and low after the chain, its lowest row ever set
    bool made, fell;   // it became the pivot of its low / a pivot row lay below the window
};

// The chain of additions into bitmap column j (tiers 3 and 4), run by the
// whole CTA (1024 threads) once the column's rows are set in the window
// [w0, ...) that `word` reaches: warps 0 .. 30 toggle the pivot's rows (one
// each), warp 0 then counts the column, finds the next low (bits_below) and
// reads that row's pivot record; two barriers of those 31 warps per
// addition.  Warp 31 prefetches ahead of them (chain_prefetcher).  A pivot
// row below the window undoes that addition's toggles and ends the chain
// (`fell`): the caller hands the column to the merge path.  After
// a.chain_cap additions (if set) the chain stops with the column unresolved,
// its low's pivot known: the next sweep's Phase I sees a repeat and hands it
// back.  n, lj: the column's length and low; lo: its lowest row.
template <class W>
__device__ ChainResult bitmap_chain(const PmsArgs &a, int j, int lj, int n, int lo, int w0, W word,
                                    long long &adds, long long &slots) {
    __shared__ int s_red[32], s_fb[32];
    __shared__ int s_small[4];
    __shared__ int s_lo;
    __shared__ volatile int s_cur, s_done;  // the chain's low and its end, for the prefetching warp
    __shared__ int s_ctmp[32];              // the prefetching warp's candidates
    __shared__ __align__(16) int4 s_rec[2][2];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    const int ntg = blockDim.x - 32;
    int4 h, e;
    if (tid == 0) {
        rec_load_acq(&a.rec[lj], h, e);
        s_rec[1][0] = h;
        s_rec[1][1] = e;
        s_lo = lo;
        s_cur = lj;
        s_done = 0;
    }
    __syncthreads();  // s_rec[1] is next written by the second addition
    h = s_rec[1][0];
    e = s_rec[1][1];
    bool made = false, fell = false;
    if (wid == nw - 1) {
        chain_prefetcher(a, word, w0, &s_cur, &s_done, s_ctmp);
    } else if (h.x >= 0 && h.x < j) {
        for (int par = 0, steps = 1;; par ^= 1, steps++) {
            const int np = h.y;
            const int *P = np <= 4 ? nullptr : a.pool + 4ll * (unsigned)h.w + SEG_HDR;
            int d = 0;
            bool below = false;
            for (int k = tid; k < np; k += ntg) {
                const int row = P ? __ldcg(P + k) : rec_entry(e, k);
                const int r = row - w0;
                if (r < 0) {
                    below = true;
                    continue;
                }
                if (k == 0) s_lo = min(s_lo, row);  // only thread 0 writes it
                const uint32_t bit = 1u << (r & 31);
                d += (atomicXor(word(r >> 5), bit) & bit) ? -1 : 1;
            }
            d = __reduce_add_sync(0xffffffffu, d);
            const bool fb = __any_sync(0xffffffffu, below);
            if (lane == 0) {
                s_red[wid] = d;
                s_fb[wid] = fb;
            }
            bar_named(ntg);
            if (wid == 0) {
                const int tt = __reduce_add_sync(0xffffffffu, lane < nw - 1 ? s_red[lane] : 0);
                const int f = __any_sync(0xffffffffu, lane < nw - 1 && s_fb[lane]);
                const int nn = n + tt;
                const int b = (!f && nn > 0) ? bits_below(word, lj - w0) : -1;
                const int next = b >= 0 ? w0 + b : -1;
                if (lane == 0) {
                    if (next >= 0) {
                        s_cur = next;  // for the prefetching warp
                        int4 hh, ee;
                        rec_load_acq(&a.rec[next], hh, ee);
                        s_rec[par][0] = hh;
                        s_rec[par][1] = ee;
                    }
                    s_small[0] = nn;
                    s_small[1] = next;  // -1: zero column
                    s_small[2] = f;     // a pivot row below the window
                }
            }
            bar_named(ntg);
            const int nn = s_small[0], next = s_small[1];
            if (s_small[2]) {
                // undo the toggles: the column is as before this addition
                for (int k = tid; k < np; k += ntg) {
                    const int r = (P ? __ldcg(P + k) : rec_entry(e, k)) - w0;
                    if (r >= 0) atomicXor(word(r >> 5), 1u << (r & 31));
                }
                fell = true;
                break;
            }
            slots += n + np + nn;
            adds++;
            n = nn;
            if (next < 0) {
                n = 0;
                lj = -1;
                break;
            }
            lj = next;
            h = s_rec[par][0];
            e = s_rec[par][1];
            mark_clear<false>(a, lj, tid == 0);
            if (h.z == j) {  // the beta check: row lj first appears in j
                made = true;
                break;
            }
            if (h.x < 0 || h.x >= j || steps == a.chain_cap) break;
        }
    }
    if (tid == 0) s_done = 1;
    __syncthreads();  // every warp, the prefetcher included, past the chain (and any undo)
    ChainResult res;
    res.n = n;
    res.lj = lj;
    res.lo = s_lo;
    res.made = made;
    res.fell = fell;
    // every thread took the chain warps' values: warp 31 ran no additions,
    // so its n and lj come from the shared result below
    __shared__ int s_out[2];
    if (tid == 0) {
        s_out[0] = n;
        s_out[1] = (made ? 1 : 0) | (fell ? 2 : 0);
        s_small[3] = lj;
    }
    __syncthreads();
    res.n = s_out[0];
    res.lj = s_small[3];
    res.made = (s_out[1] & 1) != 0;
    res.fell = (s_out[1] & 2) != 0;
    __syncthreads();  // s_out and s_small are rewritten by the next column's chain
    return res;
}

// Returns true when the column needs the merge path (its state written back
// first).
//
// One addition: the pivot's rows toggle their bits (warps 0 .. 30), warp 0
// then counts the column and finds its next low and the set bit below that;
// two CTA barriers.  The chain's latency is the round trips to L2, so they
// are taken off it where the data allow:
// * the record of the low is read with acquire in one round trip
//   (rec_load_acq), and a wide pivot's rows are loaded in one more, the
//   window check riding on the toggles (a row below the window undoes them);
// * the next low is most often known before the toggles: with t1 the
//   column's set bit below its low and p2 the pivot's second-highest row
//   (the record holds the pivot's top rows), it is max(t1, p2) unless the
//   two are equal and cancel.  Warp 31 then fetches that row's record while
//   the other warps load and toggle the pivot, so an addition costs about
//   one round trip instead of two.
template <bool SM>
__device__ bool reduce_column_bitmap(const PmsArgs &a, int j, uint32_t *bm, int64_t bm_words, long long &adds,
                                     long long &slots) {
    __shared__ int s_red[32], s_fb[32];
    __shared__ int s_small[4];
    __shared__ int s_lo;
    __shared__ __align__(16) int4 s_rec[2][2];  // per parity of the addition: the prefetched record
    __shared__ long long s_off;
    const int tid = threadIdx.x;
    int lj;
    int4 h, e;
    if (!col_start(a, j, lj, h, e)) return false;
    const long long sj = a.seg[j];
    int n = a.pool[sj];
    const int capj = a.pool[sj + 1];
    const int *T = a.pool + sj + SEG_HDR;
    const long long nbits = 32ll * bm_words;
    // the window's first row: a multiple of 32 with lj - w0 < nbits
    const int w0 = (long long)lj + 1 > nbits ? (int)(((long long)lj + 1 - nbits + 31) & ~31ll) : 0;
    if (n > 0 && T[0] < w0) return true;
    int t1 = n >= 2 ? T[n - 2] : -1;  // the set bit below the low
    const int lo0 = n > 0 ? T[0] : lj;  // no set bit below it
    if (tid == 0) s_lo = lo0;
    for (int k = tid; k < n; k += blockDim.x) {
        const int r = T[k] - w0;
        atomicOr(bm + (r >> 5), 1u << (r & 31));
    }
    __syncthreads();
    bool made_pivot = false, fell_back = false;
    if constexpr (SM) {
        // the shared window: the chain with its prefetching warp
        (void)t1;
        const ChainResult ch = bitmap_chain(a, j, lj, n, lo0, w0, [&](int w) { return bm + w; }, adds, slots);
        n = ch.n;
        lj = ch.lj;
        made_pivot = ch.made;
        fell_back = ch.fell;
        if (tid == 0) s_lo = ch.lo;
        __syncthreads();
    } else {
        const int lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
        const int ntg = blockDim.x - 32;  // toggling threads: every warp but the last
        for (int par = 0, steps = 1;; par ^= 1, steps++) {
            const int np = h.y;
            const int *P = np <= 4 ? nullptr : a.pool + 4ll * (unsigned)h.w + SEG_HDR;
            const int p2 = np >= 2 ? (P ? e.z : rec_entry(e, np - 2)) : -1;
            const bool known = t1 != p2 || t1 < 0;
            const int pnext = known ? max(t1, p2) : -1;  // -1 when known: T = P, the sum is zero
            if (wid == nw - 1) {
                if (lane == 0 && pnext >= 0) {
                    int4 hh, ee;
                    rec_load_acq(&a.rec[pnext], hh, ee);
                    s_rec[par][0] = hh;
                    s_rec[par][1] = ee;
                }
            } else {
                int d = 0;
                bool below = false;
                for (int k = tid; k < np; k += ntg) {
                    const int r = (P ? __ldcg(P + k) : rec_entry(e, k)) - w0;
                    if (r < 0) {
                        below = true;
                        continue;
                    }
                    if (k == 0) s_lo = min(s_lo, r + w0);  // only thread 0 writes it
                    const uint32_t bit = 1u << (r & 31);
                    d += (atomicXor(bm + (r >> 5), bit) & bit) ? -1 : 1;
                }
                d = __reduce_add_sync(0xffffffffu, d);
                const bool fb = __any_sync(0xffffffffu, below);
                if (lane == 0) {
                    s_red[wid] = d;
                    s_fb[wid] = fb;
                }
            }
            __syncthreads();
            if (wid == 0) {
                const int t = __reduce_add_sync(0xffffffffu, lane < nw - 1 ? s_red[lane] : 0);
                const int f = __any_sync(0xffffffffu, lane < nw - 1 && s_fb[lane]);
                const int nn = n + t;
                int next = -1, nb = -1;
                if (!f && nn > 0) {
                    // lj's bit went with the pivot's top: the next low lies below it
                    next = known ? (pnext >= 0 ? pnext - w0 : -1) : bm_below<SM>(bm, lj - w0);
                    if (nn > 1 && next >= 0) nb = bm_below<SM>(bm, next);
                }
                if (lane == 0) {
                    if (!f && next >= 0 && !(known && w0 + next == pnext)) {
                        int4 hh, ee;
                        rec_load_acq(&a.rec[w0 + next], hh, ee);
                        s_rec[par][0] = hh;
                        s_rec[par][1] = ee;
                    }
                    s_small[0] = nn;
                    s_small[1] = next;  // -1: zero column (or, never, no bit left)
                    s_small[2] = nb;    // the set bit below it
                    s_small[3] = f;     // the pivot reaches below the window
                }
            }
            __syncthreads();
            const int nn = s_small[0], next = s_small[1], nb = s_small[2];
            if (s_small[3]) {
                // undo the toggles: the column is back to its state before this
                // addition, which the merge path takes over
                if (wid < nw - 1)
                    for (int k = tid; k < np; k += ntg) {
                        const int r = (P ? __ldcg(P + k) : rec_entry(e, k)) - w0;
                        if (r >= 0) atomicXor(bm + (r >> 5), 1u << (r & 31));
                    }
                __syncthreads();
                fell_back = true;
                break;
            }
            slots += n + np + nn;
            adds++;
            n = nn;
            if (next < 0) {
                n = 0;
                lj = -1;
                break;
            }
            lj = w0 + next;
            t1 = nb >= 0 ? w0 + nb : -1;
            h = s_rec[par][0];
            e = s_rec[par][1];
            mark_clear<false>(a, lj, tid == 0);
            if (h.z == j) { made_pivot = true; break; }  // the beta check: row lj first appears in j
            if (h.x < 0 || h.x >= j || steps == a.chain_cap) break;
        }
    }
    const int lo_row = s_lo;
    long long dst = sj;
    int dcap = capj;
    bool stored = true;
    if (n > capj) {
        dcap = round4(max(n + (n >> 1), 16));
        if (tid == 0) s_off = col_alloc(a, j, SEG_HDR + dcap);
        __syncthreads();
        stored = s_off >= 0;  // pool exhausted: j keeps its pre-sweep state
        dst = s_off;
    }
    const int top = n > 0 ? (lj - w0) >> 5 : -1;
    bitmap_extract<SM>(bm, (lo_row - w0) >> 5, top, w0, stored ? a.pool + dst + SEG_HDR : nullptr, s_red);
    if (!stored) return false;
    if (tid == 0) {
        a.pool[dst] = n;
        a.pool[dst + 1] = dcap;
        a.seg[j] = dst;
        a.low[j] = lj;
    }
    if (made_pivot) {
        fence_acq_rel();
        __syncthreads();
        if (tid == 0) {
            a.classes[j] = -1;
            rec_publish(a.rec, lj, j, n, dst, a.pool + dst + SEG_HDR);
        }
    }
    __syncthreads();
    return fell_back;
}

// Tier 3: the bitmap path (per-CTA scratch at bm + blockIdx.x * bm_words),
// or the merge path in pool buffers when there is no scratch or the window
// does not reach a column's rows.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_p2_bitmap(PmsArgs a, int tier) {
    if (a.st->converged) return;
    const int count = a.st->t_count[tier];
    if (count == 0) return;
    extern __shared__ __align__(16) uint32_t sbm[];  // SBM_WORDS, zero between columns
    __shared__ int scratch[2 * (BLOCK / 32)];
    __shared__ int s_idx, s_fit;
    const int32_t *in_list = (tier & 1) ? a.widelist : a.worklist;
    uint32_t *bm = a.bm ? a.bm + (size_t)blockIdx.x * a.bm_words : nullptr;
    for (int q = 4 * threadIdx.x; q < SBM_WORDS; q += 4 * BLOCK)
        *reinterpret_cast<uint4 *>(sbm + q) = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    long long adds = 0, slots = 0;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(&a.st->t_cursor[tier], 1);
        __syncthreads();
        const int idx = s_idx;
        __syncthreads();
        if (idx >= count) break;
        const int j = in_list[idx];
        // the shared window when the column's rows fit it, else (or when a
        // pivot reaches below it) the global bitmap, else the merge path
        if (threadIdx.x == 0) {
            const int lj = a.low[j];
            const long long sj = a.seg[j];
            s_fit = lj < 0 ? -1 : fits_sbm(a.pool[sj] > 0 ? a.pool[sj + SEG_HDR] : lj, lj);
        }
        __syncthreads();
        if (s_fit < 0) continue;  // nothing left to add (s_fit is rewritten behind the next barrier pair)
        const bool fit = s_fit;
        bool fell = true;
        if (fit) fell = reduce_column_bitmap<true>(a, j, sbm, SBM_WORDS, adds, slots);
        if (fell && a.cluster_tier) {
            // wider than the shared window: the cluster tier's, next
            if (threadIdx.x == 0) a.worklist[atomicAdd(&a.st->t_count[4], 1)] = j;
            continue;
        }
        if (fell && bm) fell = reduce_column_bitmap<false>(a, j, bm, a.bm_words, adds, slots);
        if (fell) reduce_column_block(a, j, nullptr, nullptr, nullptr, 0, scratch, nullptr, nullptr, adds, slots);
    }
    if (threadIdx.x == 0) tier_stats(a, tier, adds, slots);
}

// ------------------------------------------------------------ cluster tier
// Tier 4: a column whose rows span more than one CTA's shared window (on a
// Rips complex's anti-transpose the longest reduced cochains reach across
// the whole matrix) is held as a bitmap spread over the shared memory of a
// cluster of CL CTAs, CTA r holding rows [w0 + r CL_ROWS, w0 + (r+1) CL_ROWS).
// Every CTA of the cluster loads its slice of the column and writes its part
// of the result back; the chain of additions in between runs on the first
// CTA, whose threads toggle the pivot's bits and search for the next low
// through distributed shared memory (a few hundred cycles an access, where
// the global bitmap costs an L2 round trip per toggle round and search step).
#ifndef OPH_CL
#define OPH_CL 8
#endif
constexpr int CL_SIZE = OPH_CL;
constexpr int CL_WORDS = 49152;         // bitmap words per CTA (192 KB)
constexpr int CL_ROWS = 32 * CL_WORDS;  // rows per CTA
constexpr size_t CL_BYTES = sizeof(uint32_t) * CL_WORDS;
constexpr int CL_BLOCK = 1024;

// Word w of the cluster bitmap (slice w / CL_WORDS), through the CTA's own
// shared memory when it holds that slice.
__device__ __forceinline__ uint32_t *cl_word(const cg::cluster_group &cl, uint32_t *cbm, int w, int rank) {
    const int q = w / CL_WORDS;
    return (q == rank ? cbm : cl.map_shared_rank(cbm, q)) + (w - q * CL_WORDS);
}

struct ClState {  // the leader's decision on the next queued column, copied into every CTA
    int idx;      // queue position (>= the queue's count: no work left)
    int go;       // 0: nothing to do, 1: the cluster bitmap, 2: the merge path (rows below the window)
    int j, lj, n, w0, lo;
    int chain;    // the CTA that runs the chain: the one holding the low's slice
};
struct ClResult {  // the leader's chain, copied into every CTA
    int n, lj, lo, made, fell, stored, dcap, pad;
    long long dst;
};

template <int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(CL_BLOCK) k_p2_cluster(PmsArgs a, int tier) {
    if (a.st->converged) return;
    const int count = a.st->t_count[tier];
    if (count == 0) return;  // both read alike by every CTA: written by an earlier kernel
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = CL_BLOCK / 32;
    extern __shared__ __align__(16) uint32_t cbm[];  // CL_WORDS, zero between columns
    __shared__ ClState s_cs[2];      // per parity of the loop: written by the leader into every CTA
    __shared__ ClResult s_res[2];
    __shared__ int s_cnt[2][CL];     // (leader) set bits per slice
    __shared__ int s_red[32];
    __shared__ int scratch[2 * (CL_BLOCK / 32)];
    const int32_t *in_list = (tier & 1) ? a.widelist : a.worklist;
    for (int q = 4 * tid; q < CL_WORDS; q += 4 * CL_BLOCK)
        *reinterpret_cast<uint4 *>(cbm + q) = make_uint4(0u, 0u, 0u, 0u);
    cl.sync();  // every CTA of the cluster running, its slice zeroed
    long long adds = 0, slots = 0;
    for (int it = 0;; it ^= 1) {
        if (rank == 0 && tid == 0) {
            ClState c{};
            c.idx = atomicAdd(&a.st->t_cursor[tier], 1);
            if (c.idx < count) {
                const int j = in_list[c.idx];
                const int lj = a.clear[j] ? -1 : a.low[j];
                c.j = j;
                if (lj >= 0) {
                    int4 h, e;
                    rec_load_acq(&a.rec[lj], h, e);
                    if (h.x >= 0 && h.x < j) {
                        const long long sj = a.seg[j];
                        const long long nbits = (long long)CL * CL_ROWS;
                        c.lj = lj;
                        c.n = a.pool[sj];
                        c.w0 = (long long)lj + 1 > nbits ? (int)(((long long)lj + 1 - nbits + 127) & ~127ll) : 0;
                        c.lo = c.n > 0 ? a.pool[sj + SEG_HDR] : lj;
                        c.go = c.lo < c.w0 ? 2 : 1;
                        c.chain = min((lj - c.w0) / CL_ROWS, CL - 1);
                    }
                }
            }
            for (int q = 0; q < CL; q++) *cl.map_shared_rank(&s_cs[it], q) = c;
        }
        cl.sync();
        const ClState c = s_cs[it];
        if (c.idx >= count) break;
        if (c.go == 0) continue;
        if (c.go == 2) {
            if (rank == 0)
                reduce_column_block(a, c.j, nullptr, nullptr, nullptr, 0, scratch, nullptr, nullptr, adds, slots);
            continue;
        }
        const int j = c.j, w0 = c.w0;
        const long long sj = a.seg[j];
        const int capj = a.pool[sj + 1];
        const int *T = a.pool + sj + SEG_HDR;
        // every CTA: its slice of the column
        {
            const int r0 = rank * CL_ROWS;
            for (int k = tid; k < c.n; k += CL_BLOCK) {
                const int r = T[k] - w0 - r0;
                if ((unsigned)r < (unsigned)CL_ROWS) atomicOr(cbm + (r >> 5), 1u << (r & 31));
            }
        }
        cl.sync();
        if (rank == c.chain) {
            // the chain, on the CTA that holds the low's slice: its searches
            // and most of its toggles fall there (the low of a long chain
            // stays within one slice); the pivot rows elsewhere are toggled
            // through distributed shared memory
            const ChainResult ch = bitmap_chain(
                a, j, c.lj, c.n, c.lo, w0, [&](int w) { return cl_word(cl, cbm, w, rank); }, adds, slots);
            const int n = ch.n, lj = ch.lj;
            const bool made = ch.made, fell = ch.fell;
            // the result, and the column's new segment when it outgrew its own
            if (tid == 0) {
                ClResult r{};
                r.n = n;
                r.lj = lj;
                r.lo = ch.lo;
                r.made = made;
                r.fell = fell;
                r.stored = 1;
                r.dst = sj;
                r.dcap = capj;
                if (n > capj) {
                    r.dcap = round4(max(n + (n >> 1), 16));
                    r.dst = col_alloc(a, j, SEG_HDR + r.dcap);
                    r.stored = r.dst >= 0;  // pool exhausted: j keeps its pre-sweep state
                }
                for (int q = 0; q < CL; q++) *cl.map_shared_rank(&s_res[it], q) = r;
            }
        }
        cl.sync();
        // every CTA: its slice of the result, after the set bits of the
        // slices below it, then the words zeroed
        const ClResult r = s_res[it];
        const int lo_w = (r.lo - w0) >> 5, top_w = r.n > 0 ? (r.lj - w0) >> 5 : -1;
        const int s0 = rank * CL_WORDS;
        const int a_w = max(lo_w, s0) - s0, b_w = min(top_w, s0 + CL_WORDS - 1) - s0;
        {
            int cnt = 0;
            for (int w = (a_w & ~3) + 4 * tid; w <= b_w; w += 4 * CL_BLOCK) {
                const uint4 v = *reinterpret_cast<const uint4 *>(cbm + w);
                cnt += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
            }
            for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            if (lane == 0) s_red[wid] = cnt;
            __syncthreads();
            if (tid == 0) {
                int tot = 0;
                for (int q = 0; q < nw; q++) tot += s_red[q];
                *cl.map_shared_rank(&s_cnt[it][rank], 0) = tot;
            }
        }
        cl.sync();
        int off = 0;
        {
            const int *cnts = cl.map_shared_rank(&s_cnt[it][0], 0);
            for (int q = 0; q < rank; q++) off += cnts[q];
        }
        bitmap_extract<true>(cbm, a_w, b_w, w0 + rank * CL_ROWS, r.stored ? a.pool + r.dst + SEG_HDR + off : nullptr,
                             s_red);
        __threadfence();  // this slice's rows visible before the chain's CTA publishes the column
        cl.sync();
        if (rank == c.chain) {
            if (r.stored) {
                if (tid == 0) {
                    a.pool[r.dst] = r.n;
                    a.pool[r.dst + 1] = r.dcap;
                    a.seg[j] = r.dst;
                    a.low[j] = r.lj;
                    if (r.made) {
                        a.classes[j] = -1;
                        fence_acq_rel();
                        rec_publish(a.rec, r.lj, j, r.n, r.dst, a.pool + r.dst + SEG_HDR);
                    }
                }
                if (r.fell) {
                    __syncthreads();
                    reduce_column_block(a, j, nullptr, nullptr, nullptr, 0, scratch, nullptr, nullptr, adds, slots);
                }
            }
            __syncthreads();
        }
    }
    if (tid == 0) tier_stats(a, 3, adds, slots);  // counted with the bitmap tier
    cl.sync();  // no CTA leaves while another may still reach its shared memory
}

__global__ void k_count_sweep(DevStatus *st) {
    if (!st->converged) st->sweeps++;
}

// ------------------------------------------------------------------ driver
#ifndef OPH_T0_G
#define OPH_T0_G 8
#endif
#ifndef OPH_T0_CAP
#define OPH_T0_CAP 128
#endif
#ifndef OPH_T1_CAP
#define OPH_T1_CAP 512
#endif
#ifndef OPH_T1_G
#define OPH_T1_G 32
#endif
constexpr int T0_G = OPH_T0_G, T0_CAP = OPH_T0_CAP, T0_BLOCK = 256;
constexpr int T1_G = OPH_T1_G, T1_CAP = OPH_T1_CAP, T1_BLOCK = 256;
constexpr bool T1_STAGE = true;
constexpr bool T0_LAZY = (OPH_LAZY & 1) != 0, T1_LAZY = (OPH_LAZY & 2) != 0;
// Threads per column in the CTA tiers.
#ifndef OPH_BLOCK_THREADS
#define OPH_BLOCK_THREADS 256
#endif
constexpr int T2_CAP = 8192, T2_BLOCK = OPH_BLOCK_THREADS;

// Occupancy-filling grid for a kernel with `smem` bytes of dynamic shared
// memory (attribute set once per device).
template <class K>
static int fill_grid(Context *ctx, K kernel, int block, size_t smem, int *done) {
    if (!done[ctx->device & 63]) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return -1;
        done[ctx->device & 63] = 1;
    }
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, block, smem) != cudaSuccess) return -1;
    return ctx->sm_count * (nb < 1 ? 1 : nb);
}

// Tier-0 candidates for the autotuner: lanes per column x shared capacity.
// Candidate 0 is the default.
struct T0Cand {
    int lanes, cap;
};
static const T0Cand kT0[T0_CANDIDATES] = {{8, 128}, {4, 128}, {8, 64}, {8, 256}, {16, 128}, {16, 256}, {32, 128}};

template <int G, int CAP>
static int t0_grid(Context *ctx, size_t *smem) {
    static int done[64];
    *smem = (size_t)(T0_BLOCK / G) * 2 * CAP * sizeof(int);
    return fill_grid(ctx, k_p2_tier<G, CAP, T0_BLOCK, false, T0_LAZY>, T0_BLOCK, *smem, done);
}
template <int G, int CAP>
static void t0_launch(const PmsArgs &a, const SweepGrids &g, cudaStream_t s) {
    k_p2_tier<G, CAP, T0_BLOCK, false, T0_LAZY><<<g.g0, T0_BLOCK, g.s0, s>>>(a, 0);
}
static int t0_grid_of(Context *ctx, int v, size_t *smem) {
    switch (v) {
        case 1: return t0_grid<4, 128>(ctx, smem);
        case 2: return t0_grid<8, 64>(ctx, smem);
        case 3: return t0_grid<8, 256>(ctx, smem);
        case 4: return t0_grid<16, 128>(ctx, smem);
        case 5: return t0_grid<16, 256>(ctx, smem);
        case 6: return t0_grid<32, 128>(ctx, smem);
        default: return t0_grid<8, 128>(ctx, smem);
    }
}
static void launch_t0(const PmsArgs &a, const SweepGrids &g, cudaStream_t s) {
    switch (g.v0) {
        case 1: t0_launch<4, 128>(a, g, s); break;
        case 2: t0_launch<8, 64>(a, g, s); break;
        case 3: t0_launch<8, 256>(a, g, s); break;
        case 4: t0_launch<16, 128>(a, g, s); break;
        case 5: t0_launch<16, 256>(a, g, s); break;
        case 6: t0_launch<32, 128>(a, g, s); break;
        default: t0_launch<8, 128>(a, g, s); break;
    }
}

int t0_candidate(int v, int *lanes, int *cap) {
    if (v < 0 || v >= T0_CANDIDATES) return -1;
    *lanes = kT0[v].lanes;
    *cap = kT0[v].cap;
    return 0;
}

// The cluster tier's grid: as many clusters as can be resident at once (at
// most 16), each CL_SIZE CTAs of 1024 threads and CL_BYTES of shared memory;
// 0 when the device runs no such cluster.
static int cluster_grid(Context *ctx) {
    static int done[64], grid[64];
    const int d = ctx->device & 63;
    if (done[d]) return grid[d];
    done[d] = 1;
    grid[d] = 0;
    if (cudaFuncSetAttribute(k_p2_cluster<CL_SIZE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CL_BYTES) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(CL_SIZE * 16, 1, 1);
    cfg.blockDim = dim3(CL_BLOCK, 1, 1);
    cfg.dynamicSmemBytes = CL_BYTES;
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, k_p2_cluster<CL_SIZE>, &cfg) != cudaSuccess || nc < 1) {
        cudaGetLastError();
        return 0;
    }
    grid[d] = CL_SIZE * std::min(nc, 16);
    return grid[d];
}

int sweep_grids(Context *ctx, int64_t m, int64_t ntiles, SweepGrids *g) {
    static int done1[64], done2[64], dones[64];
    g->ss = (size_t)TS_BLOCK * TS_CAP * sizeof(int);
    g->gs = fill_grid(ctx, k_p2_scalar<TS_CAP, TS_BLOCK>, TS_BLOCK, g->ss, dones);

    g->v0 = (ctx->tier0 >= 0 && ctx->tier0 < T0_CANDIDATES) ? ctx->tier0 : 0;
    g->s1 = (size_t)(T1_BLOCK / T1_G) * (T1_STAGE ? 3 : 2) * T1_CAP * sizeof(int);
    g->s2 = (size_t)3 * T2_CAP * sizeof(int);
    g->g0 = t0_grid_of(ctx, g->v0, &g->s0);
    g->g1 = fill_grid(ctx, k_p2_tier1<T1_G, T1_CAP, T1_BLOCK, T1_STAGE, T1_LAZY>, T1_BLOCK, g->s1, done1);
    g->g2 = fill_grid(ctx, k_p2_block<T2_CAP, T2_BLOCK>, T2_BLOCK, g->s2, done2);
    g->g3 = ctx->sm_count;  // tier 3: one 1024-thread CTA per SM
    static int done3[64];
    if (!done3[ctx->device & 63]) {
        if (cudaFuncSetAttribute(k_p2_bitmap<BM_BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SBM_BYTES) != cudaSuccess)
            g->g3 = -1;
        else
            done3[ctx->device & 63] = 1;
    }
    g->g4 = cluster_grid(ctx);
    g->m = (int)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, (int64_t)ctx->sm_count * 16));
    g->t = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)ctx->sm_count * 8));
    if (g->g0 < 0 || g->g1 < 0 || g->g2 < 0 || g->gs < 0 || g->g3 < 0) {
        fprintf(stderr, "openph_gb300: Phase II kernel set-up failed: %s\n", cudaGetErrorString(cudaGetLastError()));
        return OPH_ERR_CUDA;
    }
    return OPH_OK;
}

void launch_phase0(const PmsArgs &a, int64_t c0, int64_t c1, int grid, cudaStream_t s) {
    k_phase0<<<grid, 256, 0, s>>>(a, c0, c1);
}

__global__ void k_iota(int32_t *p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (int32_t)i;
}

// The first Phase I list: the columns with a low, in order.  A zero column
// never adds, repeats a low or becomes a pivot, so Phase I has nothing to do
// for it (on the anti-transpose of a Rips complex that is every column of
// the top dimension, most of the matrix).  Per tile of P1_TILE columns:
// the count, their exclusive scan (one block), then the ordered scatter.
__global__ void __launch_bounds__(P1_THREADS) k_list_count(PmsArgs a, int64_t m) {
    __shared__ int s_cnt;
    for (int64_t t = blockIdx.x; t * P1_TILE < m; t += gridDim.x) {
        if (threadIdx.x == 0) s_cnt = 0;
        __syncthreads();
        const int64_t base = t * P1_TILE + (int64_t)threadIdx.x * P1_ITEMS;
        int c = 0;
#pragma unroll
        for (int k = 0; k < P1_ITEMS; k++) c += base + k < m && a.low[base + k] >= 0;
        c = __reduce_add_sync(0xffffffffu, c);
        if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_cnt, c);
        __syncthreads();
        if (threadIdx.x == 0) a.kagg[t] = s_cnt;
        __syncthreads();
    }
}
__global__ void k_list_scan(PmsArgs a, int64_t ntiles) {
    __shared__ int wsum[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int carry = 0;
    for (int64_t b0 = 0; b0 < ntiles; b0 += blockDim.x) {
        const int64_t t = b0 + threadIdx.x;
        const int v = t < ntiles ? a.kagg[t] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        int before = carry, total = 0;
        for (int w = 0; w < nw; w++) {
            if (w < wid) before += wsum[w];
            total += wsum[w];
        }
        if (t < ntiles) a.kagg[t] = before + incl - v;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) a.st->ucount[0] = carry;
}
__global__ void __launch_bounds__(P1_THREADS) k_list_scatter(PmsArgs a, int64_t m) {
    __shared__ int wsum[P1_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t t = blockIdx.x; t * P1_TILE < m; t += gridDim.x) {
        const int64_t base = t * P1_TILE + (int64_t)threadIdx.x * P1_ITEMS;
        unsigned keep = 0;
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < P1_ITEMS; k++)
            if (base + k < m && a.low[base + k] >= 0) {
                keep |= 1u << k;
                cnt++;
            }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        int off = a.kagg[t] + incl - cnt;
        for (int w = 0; w < wid; w++) off += wsum[w];
#pragma unroll
        for (int k = 0; k < P1_ITEMS; k++)
            if (keep & (1u << k)) a.ulist[off++] = (int32_t)(base + k);
        __syncthreads();  // wsum is rewritten by the next tile
    }
}

// ---------------------------------------------------------------- trackers
// The reference's essential estimate after an iteration (ess_hat,
// src/cuda/algorithms/kernels.cu:114-124): a row that is some column's low,
// and both ends of every known pivot pair, are not essential.  Kept as one
// byte per column, all ones before Phase 0.
__global__ void k_track_ess(PmsArgs a, uint8_t *__restrict__ ess_hat) {
    if (a.st->converged) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < a.m; j += (int64_t)gridDim.x * blockDim.x) {
        const int lj = a.low[j];
        if (lj >= 0) ess_hat[lj] = 0;
        const int pc = a.rec[j].col;
        if (pc >= 0) {
            ess_hat[pc] = 0;
            ess_hat[j] = 0;
        }
    }
}

// The sums behind one tracker entry (tracker.cu:92-134): sum and maximum of
// |low - low_true| (0-based, -1 = none), columns still unclassified
// (classes == 0), and the size of the essential estimate.
__global__ void k_track_sum(PmsArgs a, const int32_t *__restrict__ low_true, const uint8_t *__restrict__ ess_hat,
                            double *acc, int check_converged) {
    if (check_converged && a.st->converged) return;
    double s = 0, mx = 0, un = 0, es = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < a.m; j += (int64_t)gridDim.x * blockDim.x) {
        const double d = fabs((double)a.low[j] - (double)low_true[j]);
        s += d;
        mx = fmax(mx, d);
        un += a.classes[j] == 0 ? 1.0 : 0.0;
        es += ess_hat[j];
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        un += __shfl_xor_sync(0xffffffffu, un, o);
        es += __shfl_xor_sync(0xffffffffu, es, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], s);
        // maxima of non-negative doubles compare as their bit patterns
        atomicMax((unsigned long long *)&acc[1], (unsigned long long)__double_as_longlong(mx));
        atomicAdd(&acc[2], un);
        atomicAdd(&acc[3], es);
    }
}

// ev (optional, 6 events): before Phase I, after Phase I, after each tier.
static void launch_sweep_ev(const PmsArgs &a0, const SweepGrids &g, cudaStream_t s, cudaEvent_t *ev, int parity) {
    PmsArgs a = a0;
    if (a0.ulist) {
        // the list read this sweep and the one it compacts into
        int32_t *L[2] = {a0.ulist, a0.ulist_next};
        int *C[2] = {&a0.st->ucount[0], &a0.st->ucount[1]};
        a.ulist = L[parity & 1];
        a.ulist_next = L[(parity + 1) & 1];
        a.ucur = C[parity & 1];
        a.unext = C[(parity + 1) & 1];
    }
    if (a.slist) {
        // the scalar tier takes the queue first and hands tier 0 the rest
        a.t0_list = a.slist;
        a.t0_count = &a0.st->s_out;
    } else {
        a.t0_list = a.worklist;
        a.t0_count = &a0.st->t_count[0];
    }
    if (ev) cudaEventRecord(ev[0], s);
    if (a.ulist) k_p1_small<<<1, P1_THREADS, 0, s>>>(a);
    k_p1_first<<<g.m, 256, 0, s>>>(a);
    k_p1_tiles<<<g.t, P1_THREADS, 0, s>>>(a);
    k_p1_scan<<<1, 32 * MAXC, 0, s>>>(a);
    k_p1_mark<<<g.t, P1_THREADS, 0, s>>>(a);
    if (a.ulist) {
        k_p1_kscan<<<1, 1024, 0, s>>>(a);
        k_p1_scatter<<<g.t, P1_THREADS, 0, s>>>(a);
    } else {
        k_p1_worklist<<<g.m, 256, 0, s>>>(a);
    }
    if (ev) cudaEventRecord(ev[1], s);
    if (a.slist) {
        DevStatus *st = a0.st;
        k_p2_scalar<TS_CAP, TS_BLOCK><<<g.gs, TS_BLOCK, g.ss, s>>>(
            a, ScalarQ{a.worklist, &st->t_count[0], &st->s_cursor, a.slist, &st->s_out});
    }
    launch_t0(a, g, s);
    if (ev) cudaEventRecord(ev[2], s);
    k_p2_tier1<T1_G, T1_CAP, T1_BLOCK, T1_STAGE, T1_LAZY><<<g.g1, T1_BLOCK, g.s1, s>>>(a, 1);
    if (ev) cudaEventRecord(ev[3], s);
    k_p2_block<T2_CAP, T2_BLOCK><<<g.g2, T2_BLOCK, g.s2, s>>>(a, 2);
    if (ev) cudaEventRecord(ev[4], s);
    k_p2_bitmap<BM_BLOCK><<<g.g3, BM_BLOCK, SBM_BYTES, s>>>(a, 3);
    if (a.cluster_tier) k_p2_cluster<CL_SIZE><<<g.g4, CL_BLOCK, CL_BYTES, s>>>(a, 4);
    k_count_sweep<<<1, 1, 0, s>>>(a.st);
    if (ev) cudaEventRecord(ev[5], s);
}

// The tracker entry of sweep `slot` (1-based), skipped once converged.
static void launch_track(const PmsArgs &a, const SweepGrids &g, cudaStream_t s, Tracking *t, int slot) {
    if (!t || slot >= t->slots) return;
    k_track_ess<<<g.m, 256, 0, s>>>(a, t->ess_hat);
    k_track_sum<<<g.m, 256, 0, s>>>(a, t->low_true, t->ess_hat, t->acc + 4 * slot, 1);
}

void launch_sweep(const PmsArgs &a, const SweepGrids &g, cudaStream_t s, int parity, cudaEvent_t *ev) {
    launch_sweep_ev(a, g, s, ev, parity);
}

// Kernels one sweep launches (launch_sweep_ev): Phase I (the one-block
// kernel and six grid kernels with the compacted list, else five), the scalar tier, tiers 0-3, the cluster tier
// when it runs, the counter.
static int kernels_per_sweep(const PmsArgs &a) {
    return (a.ulist ? 7 : 5) + (a.slist ? 1 : 0) + 4 + (a.cluster_tier ? 1 : 0) + 1;
}

// Sweeps replayed from a captured CUDA graph (0: launched one by one).
#ifndef OPH_GRAPHS
#define OPH_GRAPHS 1
#endif

// The graph of two sweeps (parities 0 and 1) for these arguments, captured on
// first use and again whenever an argument changes (a regrown store moves the
// pool).  Returns false, with nothing left captured, when capture fails; the
// caller then launches the sweeps directly.
static bool sweep_pair_graph(Context *ctx, const PmsArgs &a, const SweepGrids &g) {
    std::vector<unsigned char> key(sizeof(PmsArgs) + sizeof(SweepGrids));
    memcpy(key.data(), &a, sizeof(PmsArgs));
    memcpy(key.data() + sizeof(PmsArgs), &g, sizeof(SweepGrids));
    if (ctx->sweep_graph && key == ctx->sweep_key) return true;
    if (ctx->sweep_graph) {
        cudaGraphExecDestroy(ctx->sweep_graph);
        ctx->sweep_graph = nullptr;
    }
    cudaStream_t s = ctx->stream;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    launch_sweep_ev(a, g, s, nullptr, 0);
    launch_sweep_ev(a, g, s, nullptr, 1);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->sweep_graph, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ctx->sweep_graph = nullptr;
        return false;
    }
    ctx->sweep_key = std::move(key);
    return true;
}

// The loop condition of the sweep-loop graph: another pair of sweeps while
// the reduction has not converged, no column store allocation failed, no
// error was raised and the sweep cap is not reached.
__global__ void k_loop_cond(cudaGraphConditionalHandle h, const DevStatus *st, int cap) {
    const bool more = !st->converged && !st->overflow && !st->error && st->sweeps < cap;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

// The whole sweep loop as one graph (a conditional WHILE node around two
// sweeps and k_loop_cond), built on first use and again whenever an argument
// changes.  Returns false, with nothing left built, when the driver refuses
// any step; the caller then runs the host loop.
static bool sweep_loop_graph(Context *ctx, const PmsArgs &a, const SweepGrids &g, int cap) {
    std::vector<unsigned char> key(sizeof(PmsArgs) + sizeof(SweepGrids) + sizeof(int));
    memcpy(key.data(), &a, sizeof(PmsArgs));
    memcpy(key.data() + sizeof(PmsArgs), &g, sizeof(SweepGrids));
    memcpy(key.data() + sizeof(PmsArgs) + sizeof(SweepGrids), &cap, sizeof(int));
    if (ctx->loop_graph && key == ctx->loop_key) return true;
    if (ctx->loop_graph) {
        cudaGraphExecDestroy(ctx->loop_graph);
        ctx->loop_graph = nullptr;
    }
    cudaStream_t s = ctx->stream;
    cudaGraph_t graph = nullptr;
    if (cudaGraphCreate(&graph, 0) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    bool ok = false;
    do {
        cudaGraphConditionalHandle h;
        // the body runs at least once per launch (the handle starts at 1)
        if (cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault) != cudaSuccess) break;
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        if (cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &p) != cudaSuccess) break;
        cudaGraph_t body = p.conditional.phGraph_out[0];
        if (cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
            cudaSuccess)
            break;
        launch_sweep_ev(a, g, s, nullptr, 0);
        launch_sweep_ev(a, g, s, nullptr, 1);
        k_loop_cond<<<1, 1, 0, s>>>(h, a.st, cap);
        cudaGraph_t captured = nullptr;
        if (cudaStreamEndCapture(s, &captured) != cudaSuccess) break;
        if (cudaGraphInstantiate(&ctx->loop_graph, graph, 0) != cudaSuccess) {
            ctx->loop_graph = nullptr;
            break;
        }
        ok = true;
    } while (0);
    cudaGraphDestroy(graph);
    if (!ok) {
        cudaGetLastError();
        return false;
    }
    ctx->loop_key = std::move(key);
    return true;
}

int run_pms(Context *ctx, Work &w, oph_info *info) {
    const int64_t m = w.m;
    PmsArgs a{};
    a.m = m; a.low = w.low; a.classes = w.classes; a.clear = w.clear; a.dim = w.dim; a.first = w.first;
    a.beta = w.beta; a.worklist = w.worklist; a.widelist = w.widelist; a.seg = w.seg;
    a.rec = w.rec; a.agg = w.agg; a.ntiles = w.ntiles; a.pool = w.pool; a.st = w.st;
    a.stats = ctx->count_slots;
    // Phase I over a compacted list of the unresolved columns: every column
    // at first, then only those still unresolved after each sweep
#ifndef OPH_PHASE1_LIST
#define OPH_PHASE1_LIST 1
#endif
    if (OPH_SCALAR) {
        a.slist = (int32_t *)ctx_alloc(ctx, S_SLIST, sizeof(int32_t) * (m > 0 ? m : 1));
        if (!a.slist) return OPH_ERR_OOM;
    }
    if (OPH_PHASE1_LIST) {
        a.ulist = (int32_t *)ctx_alloc(ctx, S_ULIST, sizeof(int32_t) * 2 * (m > 0 ? m : 1));
        a.kagg = (int32_t *)ctx_alloc(ctx, S_KAGG, sizeof(int32_t) * (w.ntiles + 1));
        if (!a.ulist || !a.kagg) return OPH_ERR_OOM;
        a.ulist_next = a.ulist + m;
        a.ascending = w.ascending ? 1 : 0;
    }
    cudaStream_t s = ctx->stream;
    SweepGrids g{};
    int rc = sweep_grids(ctx, m, w.ntiles, &g);
    if (rc) return rc;
    // tier 3's bitmaps: a window of the whole matrix up to 2^23 rows per CTA,
    // zeroed here (each column leaves its words zeroed)
    a.bm_words = std::min<int64_t>(((m + 32) / 32 + 3) & ~3ll, BM_MAX_WORDS);
    a.cluster_tier = g.g4 > 0 && !getenv("OPH_NO_CLUSTER");
    a.bm = (uint32_t *)ctx_alloc(ctx, S_BITMAP, sizeof(uint32_t) * (size_t)a.bm_words * g.g3);
    if (!a.bm) return OPH_ERR_OOM;
    OPH_CUDA_TRY(cudaMemsetAsync(a.bm, 0, sizeof(uint32_t) * (size_t)a.bm_words * g.g3, s));
    if (a.ulist && ctx->track) {
        // the trackers count the zero columns that Phase I classifies
        k_iota<<<g.m, 256, 0, s>>>(a.ulist, m);
        const int mi = (int)m;
        OPH_CUDA_TRY(cudaMemcpyAsync(&w.st->ucount[0], &mi, sizeof(int), cudaMemcpyHostToDevice, s));
    } else if (a.ulist) {
        const int64_t lt = (m + P1_TILE - 1) / P1_TILE;
        const int gl = (int)std::max<int64_t>(1, std::min<int64_t>(lt, (int64_t)ctx->sm_count * 8));
        k_list_count<<<gl, P1_THREADS, 0, s>>>(a, m);
        k_list_scan<<<1, 1024, 0, s>>>(a, lt);
        k_list_scatter<<<gl, P1_THREADS, 0, s>>>(a, m);
        ctx->launches += 2;
    }

    OPH_CUDA_TRY(cudaMemsetAsync(w.first, 0x7f, sizeof(int32_t) * m, s));
    OPH_CUDA_TRY(cudaMemsetAsync(w.classes, 0, m, s));
    if (w.preclear) OPH_CUDA_TRY(cudaMemcpyAsync(w.clear, w.preclear, m, cudaMemcpyDeviceToDevice, s));
    else OPH_CUDA_TRY(cudaMemsetAsync(w.clear, 0, m, s));

    Tracking *tr = ctx->track;
    if (tr) {
        // entry 0: the state before Phase 0, every column its own estimate
        OPH_CUDA_TRY(cudaMemsetAsync(tr->ess_hat, 1, m, s));
        OPH_CUDA_TRY(cudaMemsetAsync(tr->acc, 0, sizeof(double) * 4 * tr->slots, s));
        k_track_sum<<<g.m, 256, 0, s>>>(a, tr->low_true, tr->ess_hat, tr->acc, 0);
        tr->sweep_ms.clear();
    }
    cudaEventRecord(ctx->ev[0], s);
    launch_phase0(a, 0, m, g.m, s);
    ctx->launches++;
    OPH_CUDA_TRY(cudaGetLastError());

    // per-phase events: 6 per sweep, reused batch after batch
    // sweeps launched between two reads of the status (doubling from 2): a
    // batch that overshoots convergence launches sweeps that return at once
    constexpr int MAX_BATCH = 4;
    const int nev = 6 * MAX_BATCH + 1;
    if ((ctx->profile || ctx->track || getenv("OPH_TRACE")) && ctx->pev_n < nev) {
        ctx->pev = (cudaEvent_t *)realloc(ctx->pev, sizeof(cudaEvent_t) * nev);
        for (int i = ctx->pev_n; i < nev; i++) cudaEventCreate(&ctx->pev[i]);
        ctx->pev_n = nev;
    }
    // OPH_TRACE=1: one sweep per batch, per-tier queue sizes, additions and
    // times printed to stderr (diagnostics only)
    static const int trace = getenv("OPH_TRACE") ? atoi(getenv("OPH_TRACE")) : 0;
    const bool timed = ctx->profile || trace || tr;
    if (timed) cudaEventRecord(ctx->pev[6 * MAX_BATCH], s);  // end of Phase 0

    const int max_sweeps = ctx->max_sweeps > 0 ? ctx->max_sweeps : 1 << 20;
    int sweeps_launched = 0;
    int batch = trace ? 1 : 2;
    DevStatus hs{};
    float p2_ms = 0, p2w_ms = 0, p1_ms = 0, wt_ms[3] = {0, 0, 0};
    int p2_launches = 0, regrows = 0;
    // the device-resident loop: one graph launch runs sweeps until the
    // reduction converges (or a column store allocation fails, or the cap),
    // one status read per launch
    static const bool loop_on = !getenv("OPH_HOST_LOOP");
    while (OPH_GRAPHS && loop_on && !timed && sweep_loop_graph(ctx, a, g, max_sweeps)) {
        OPH_CUDA_TRY(cudaGraphLaunch(ctx->loop_graph, s));
        OPH_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, w.st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
        OPH_CUDA_TRY(cudaStreamSynchronize(s));
        const int before = sweeps_launched;
        hs = *ctx->h_status;
        // every pair the body ran: the sweeps counted plus the one that
        // found convergence, rounded up to pairs
        const int pairs = std::max(1, (hs.sweeps - before + 2) / 2);
        sweeps_launched = std::max(hs.sweeps, before + 2 * pairs);
        ctx->launches += pairs * (2 * kernels_per_sweep(a) + 1);
        if (hs.error) { rc = OPH_ERR_BAD_INPUT; break; }
        if (hs.overflow) {
            int gr = grow_pool(ctx, w);
            if (gr != OPH_OK) { rc = gr; break; }
            a.pool = w.pool;
            regrows++;
            if (hs.converged) break;
            continue;
        }
        if (hs.converged) break;
        if (hs.sweeps >= max_sweeps) { rc = OPH_ERR_TIMEOUT; break; }
    }
    for (; !hs.converged && rc == OPH_OK;) {
        const int nb = std::min(batch, max_sweeps - sweeps_launched);
        DevStatus before = hs;
        int b = 0;
        if (OPH_GRAPHS && !timed && (sweeps_launched & 1) == 0 && nb >= 2 && sweep_pair_graph(ctx, a, g)) {
            for (; b + 2 <= nb; b += 2) {
                OPH_CUDA_TRY(cudaGraphLaunch(ctx->sweep_graph, s));
                ctx->launches += 2 * kernels_per_sweep(a);
            }
        }
        for (; b < nb; b++) {
            launch_sweep_ev(a, g, s, timed ? ctx->pev + 6 * b : nullptr, sweeps_launched + b);
            launch_track(a, g, s, tr, sweeps_launched + b + 1);
            ctx->launches += kernels_per_sweep(a);
        }
        sweeps_launched += nb;
        OPH_CUDA_TRY(cudaGetLastError());
        OPH_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, w.st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
        OPH_CUDA_TRY(cudaStreamSynchronize(s));
        hs = *ctx->h_status;
        if (timed) {
            const int worked = std::max(0, std::min(nb, hs.sweeps - (sweeps_launched - nb)));
            for (int b = 0; b < nb; b++) {
                float t[5];
                for (int q = 0; q < 5; q++) cudaEventElapsedTime(&t[q], ctx->pev[6 * b + q], ctx->pev[6 * b + q + 1]);
                p1_ms += t[0];
                p2_ms += t[1];
                p2w_ms += t[2] + t[3] + t[4];
                for (int q = 0; q < 3; q++) wt_ms[q] += t[2 + q];
                if (tr && b < worked) tr->sweep_ms.push_back(t[0] + t[1] + t[2] + t[3] + t[4]);
                if (trace && b < worked)
                    fprintf(stderr, "sweep %d: unresolved %d queued t0=%d (to tier 0: %d) t1=%d t2=%d t3=%d | adds "
                                    "scalar=%llu t0=%llu t1=%llu t2=%llu t3=%llu | ms p1=%.3f t0=%.3f t1=%.3f t2=%.3f "
                                    "t3=%.3f | open %d\n", hs.sweeps,
                            a.ulist ? hs.ucount[hs.sweeps & 1] : -1, hs.t_count[0], a.slist ? hs.s_out : -1,
                            hs.t_count[1], hs.t_count[2], hs.t_count[3], hs.s_adds - before.s_adds,
                            hs.tier_adds[0] - before.tier_adds[0] - (hs.s_adds - before.s_adds),
                            hs.tier_adds[1] - before.tier_adds[1], hs.tier_adds[2] - before.tier_adds[2],
                            hs.tier_adds[3] - before.tier_adds[3], t[0], t[1], t[2], t[3], t[4],
                            a.ascending ? hs.bucket_open - 1 : -2);
            }
            p2_launches += worked;
#if OPH_COUNTS
            if (trace > 2 && worked) {
                fprintf(stderr, "  additions per SM:");
                for (int q = 0; q < 256; q++)
                    if (hs.diag_sm[q] - before.diag_sm[q]) fprintf(stderr, " %d:%llu", q, hs.diag_sm[q] - before.diag_sm[q]);
                fprintf(stderr, "\n");
            }
#endif
            if (trace > 1 && worked && a.slist) {
                const unsigned long long *d = hs.sdiag, *e = before.sdiag;
                fprintf(stderr, "  scalar tier: additions %llu, handed at load %llu / mid-chain %llu, lane-steps %llu, "
                                "columns loaded %llu (rows %llu)\n", d[0] - e[0], d[1] - e[1], d[2] - e[2],
                        d[3] - e[3], d[4] - e[4], d[5] - e[5]);
            }
            if (trace > 1 && worked && !T0_LAZY) {
                const unsigned long long *d = hs.diag, *e = before.diag;
                fprintf(stderr, "  tier 0 (eager): visits %llu, columns that added %llu, longest chain %llu\n",
                        d[4] - e[4], d[6] - e[6], d[5]);
            }
            if (trace > 1 && worked) {
                for (int t = T0_LAZY ? 0 : 1; t < 2; t++) {
                    const unsigned long long *d = hs.diag + 8 * t, *e = before.diag + 8 * t;
                    fprintf(stderr, "  tier %d: adds rec %llu seg<=4 %llu mid %llu wide %llu | flushes %llu cancels %llu | "
                                    "columns %llu rows in %llu\n", t, d[0] - e[0], d[1] - e[1], d[2] - e[2],
                            d[3] - e[3], d[4] - e[4], d[5] - e[5], d[6] - e[6], d[7] - e[7]);
                }
            }
        }
        if (hs.error) { rc = OPH_ERR_BAD_INPUT; break; }
        if (hs.overflow) {
            // a column could not be written back: grow the store and run the
            // sweep again from the consistent state the kernels left
            int gr = grow_pool(ctx, w);
            if (gr != OPH_OK) { rc = gr; break; }
            a.pool = w.pool;
            regrows++;
            if (hs.converged) break;
            continue;
        }
        if (hs.converged) break;
        if (sweeps_launched >= max_sweeps) { rc = OPH_ERR_TIMEOUT; break; }
        if (!trace) batch = std::min(batch * 2, MAX_BATCH);
    }
    cudaEventRecord(ctx->ev[1], s);
    OPH_CUDA_TRY(cudaEventSynchronize(ctx->ev[1]));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    if (ctx->profile) {
        float p0 = 0;
        cudaEventElapsedTime(&p0, ctx->ev[0], ctx->pev[6 * MAX_BATCH]);
        ctx->prof.phase2_narrow_ms = p2_ms;
        ctx->prof.phase2_wide_ms = p2w_ms;
        for (int q = 0; q < 3; q++) ctx->prof.tier_ms[q] = wt_ms[q];
        ctx->prof.phase1_ms = p1_ms;
        ctx->prof.setup_ms += p0;
        ctx->prof.phase2_launches = p2_launches;
        for (int t = 0; t < 4; t++) {
            ctx->prof.tier_additions[t] = (int64_t)hs.tier_adds[t];
            ctx->prof.tier_slots[t] = (int64_t)hs.tier_slots[t];
        }
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
