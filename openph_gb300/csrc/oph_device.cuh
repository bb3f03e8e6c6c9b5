// Device-side building blocks shared by every reduction kernel.
//
// Column store.  Every column lives in a "segment" of a single int32 pool:
//   pool[s + 0] = length, pool[s + 1] = capacity, pool[s + 2..3] unused,
//   pool[s + 4 ..] = row indices, ascending.
// Segments start on 16-byte boundaries (s is a multiple of 4) so rows can be
// moved with 128-bit loads.  seg[j] is column j's segment.  A column that
// outgrows its capacity moves to a fresh segment bump-allocated at the end of
// the pool (`pool_used`); the pool grows on the host when the bump pointer
// would pass its end (the kernels stop cleanly and report `overflow`).  This
// replaces the reference's fixed m x p slot store (src/cuda/openph.cu:41-90,
// src/cuda/kernels.cu:25-38): no slot count is supplied.
//
// Pivot table.  rowpiv[i] publishes the column whose (final) low is row i,
// packed with that column's segment so a reader reaches the pivot's rows in
// one dependent load: (col << 35) | (segment >> 2).  ~0 = no pivot.  It is
// written with release semantics after the column's rows are in place and
// read with acquire semantics (the reference's arglow[] has neither,
// src/cuda/algorithms/pms/pms_functions.cu:87-112).
#pragma once
#include <cooperative_groups.h>
#include <cstdint>
#include <cuda_runtime.h>

namespace cg = cooperative_groups;

namespace oph {

constexpr int SEG_HDR = 4;
constexpr unsigned long long NO_PIVOT = ~0ull;
constexpr int PIV_SHIFT = 35;
constexpr unsigned long long PIV_OFF_MASK = (1ull << PIV_SHIFT) - 1;
constexpr int FIRST_NONE = 0x7f7f7f7f;  // byte pattern 0x7f: "no column yet"
constexpr int MAXC = 8;                 // dimension buckets handled by the Phase I scan (-1 .. 6)
constexpr int POOL_PAD = 1024;          // ints of readable padding past the pool's end

// Device-resident status block of one reduction.
struct DevStatus {
    unsigned long long pool_used;  // ints in use (bump pointer)
    unsigned long long pool_size;  // ints available
    unsigned long long additions;  // column additions performed
    unsigned long long slots;      // sum of |P| + |T| + |T xor P|
    int overflow;                  // a bump allocation failed; state is consistent, re-run
    int error;                     // malformed input (1) or internal error
    int converged;                 // pms: no repeated low left
    int sweeps;                    // pms sweeps run
    int wl_count;                  // Phase II worklist size
    int wl_cursor;                 // Phase II work-queue cursor
    int wide_count;                // columns handed to the wide path
    int wide_cursor;
    int reps;                      // repeated lows seen by the last Phase I
    int resume_dim;                // sequential walkers: where to resume after a regrow
    long long resume_pos;          //   (column or row index; -1 = finished)
    int max_dim;                   // largest nnz(col) - 1 seen by the set-up
    int pad;
};

__device__ __forceinline__ unsigned long long pack_pivot(int col, long long seg) {
    return ((unsigned long long)col << PIV_SHIFT) | ((unsigned long long)seg >> 2);
}
__device__ __forceinline__ int pivot_col(unsigned long long w) { return (int)(w >> PIV_SHIFT); }
__device__ __forceinline__ long long pivot_seg(unsigned long long w) { return (long long)((w & PIV_OFF_MASK) << 2); }

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ int round4(int n) { return (n + 3) & ~3; }

// Bump allocation of `ints` (a multiple of 4) from the pool; -1 on exhaustion.
__device__ __forceinline__ long long pool_alloc(DevStatus *st, long long ints) {
    unsigned long long off = atomicAdd(&st->pool_used, (unsigned long long)ints);
    if (off + (unsigned long long)ints > st->pool_size) {
        atomicExch(&st->overflow, 1);
        return -1;
    }
    return (long long)off;
}

// First index in a[0..n) whose value is >= x (a ascending).
__device__ __forceinline__ int lower_bound(const int *a, int n, int x) {
    int lo = 0;
    while (n > 0) {
        int h = n >> 1;
        if (a[lo + h] < x) { lo += h + 1; n -= h + 1; }
        else n = h;
    }
    return lo;
}

// Symmetric difference of two ascending lists (Z/2 column addition) by a
// group of G lanes.  Every output element is placed by rank: an element x of
// A lands at  i + #{P < x} - 2 * #{common values < x},  and symmetrically for
// P; common values are dropped.  Each lane handles every G-th element, ranks
// by binary search in the other list, and the common-value counts come from
// group ballots.  A, P and B may live in shared or global memory (generic
// pointers); B must not alias A or P.  Returns |A xor P|.
template <int G, class Tile>
__device__ __forceinline__ int merge_xor(const Tile &tile, const int *A, int nA, const int *P, int nP, int *B) {
    const int lane = tile.thread_rank();
    const unsigned lt = (1u << lane) - 1u;
    int carry = 0;
    for (int base = 0; base < nA; base += G) {
        int i = base + lane;
        bool v = i < nA;
        int x = v ? A[i] : 0;
        int r = v ? lower_bound(P, nP, x) : 0;
        bool dup = v && r < nP && P[r] == x;
        unsigned b = tile.ballot(dup);
        if (v && !dup) B[i + r - 2 * (carry + __popc(b & lt))] = x;
        carry += __popc(b);
    }
    const int common = carry;
    carry = 0;
    for (int base = 0; base < nP; base += G) {
        int k = base + lane;
        bool v = k < nP;
        int x = v ? P[k] : 0;
        int r = v ? lower_bound(A, nA, x) : 0;
        bool dup = v && r < nA && A[r] == x;
        unsigned b = tile.ballot(dup);
        if (v && !dup) B[k + r - 2 * (carry + __popc(b & lt))] = x;
        carry += __popc(b);
    }
    tile.sync();
    return nA + nP - 2 * common;
}

// The same symmetric difference when the pivot P has at most G entries and is
// held one element per lane (lane k < nP holds P[k] in `pv`).  Lane k ranks
// P[k] in A by binary search; every element x of A is then shifted by
//   sum over k of [P[k] < x] * (P[k] common ? -1 : +1)
// (the pivot broadcast by shuffles), and dropped if it equals some P[k].
// No staging of P and no second pass over it.  Returns |A xor P|.
template <int G, class Tile>
__device__ __forceinline__ int merge_xor_small(const Tile &tile, const int *A, int nA, int pv, int nP, int *B) {
    const int lane = tile.thread_rank();
    const unsigned lt = (1u << lane) - 1u;
    int r = 0;
    bool pdup = false;
    if (lane < nP) {
        r = lower_bound(A, nA, pv);
        pdup = r < nA && A[r] == pv;
    }
    const unsigned dmask = tile.ballot(pdup);
    if (lane < nP && !pdup) B[lane + r - 2 * __popc(dmask & lt)] = pv;
    for (int base = 0; base < nA; base += G) {
        const int i = base + lane;
        const bool v = i < nA;
        const int x = v ? A[i] : 0;
        int shift = 0;
        bool drop = false;
        for (int k = 0; k < nP; k++) {
            const int pk = tile.shfl(pv, k);
            const int s = ((dmask >> k) & 1u) ? -1 : 1;
            shift += pk < x ? s : 0;
            drop |= pk == x;
        }
        if (v && !drop) B[i + shift] = x;
    }
    tile.sync();
    return nA + nP - 2 * __popc(dmask);
}

// Group copy of n ints; 128-bit moves when both ends are 16-byte aligned.
template <int G, class Tile>
__device__ __forceinline__ void group_copy(const Tile &tile, int *dst, const int *src, int n) {
    const int lane = tile.thread_rank();
    if ((((uintptr_t)dst | (uintptr_t)src) & 15) == 0) {
        int n4 = n >> 2;
        const int4 *s4 = reinterpret_cast<const int4 *>(src);
        int4 *d4 = reinterpret_cast<int4 *>(dst);
        for (int q = lane; q < n4; q += G) d4[q] = s4[q];
        for (int q = (n4 << 2) + lane; q < n; q += G) dst[q] = src[q];
    } else {
        for (int q = lane; q < n; q += G) dst[q] = src[q];
    }
    tile.sync();
}

// Warp-aggregated append of `item` to list[] (count in *cnt) when `want`.
__device__ __forceinline__ void warp_append(bool want, int item, int *list, int *cnt) {
    unsigned mask = __activemask();
    unsigned b = __ballot_sync(mask, want);
    if (!b) return;
    int leader = __ffs(b) - 1;
    int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == leader) base = atomicAdd(cnt, __popc(b));
    base = __shfl_sync(mask, base, leader);
    if (want) list[base + __popc(b & ((1u << lane) - 1u))] = item;
}

}  // namespace oph
