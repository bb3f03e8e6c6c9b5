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
// Pivot records.  rec[i] (32 bytes, one L2 sector) describes row i:
//   col   the column whose final low is row i (the reference's arglow[i],
//         src/cuda/algorithms/pms/pms_functions.cu:87-112), -1 = none yet
//   np    that column's length, seg4 its segment / 4
//   e[4]  its four highest rows, ascending (all its rows, then markers,
//         when it has at most four)
//   left  the first input column holding row i (beta.cu:2-15)
// so one 32-byte read per column addition yields the beta check, the pivot
// test and, for a pivot of at most four entries (most pivots are apparent
// pairs of three), the pivot's rows too: one dependent round trip per
// addition instead of three.  For a wider pivot the highest rows tell a
// reader the next low of the sum before it has read the pivot's segment
// (the larger of the column's and the pivot's second rows, when they
// differ).  Every field changes at most once per
// reduction, from a marker (col -1, np 0, seg4 SEG4_NONE, e -1) to its final
// value; the publisher writes col last behind a fence.  A reader that sees
// col set but needs the segment takes an acquire load of col (ordering its
// reads of the segment) and re-reads np / seg4 only if its first read still
// showed a marker (rec_header), or reads the header with acquire in the
// first place (rec_load_acq: one round trip).
#pragma once
#include <cooperative_groups.h>
#include <cstdint>
#include <cuda_runtime.h>

namespace cg = cooperative_groups;

namespace oph {

constexpr int SEG_HDR = 4;
constexpr long long MAX_POOL_INTS = (4ll << 32) - 64;  // segment / 4 is held in 32 bits,
constexpr unsigned SEG4_NONE = 0xffffffffu;           //   this value marking "not yet published"
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
    int wl_count;                  // Phase II worklist size (tier 0 input)
    int s_cursor;                  // scalar tier: work-queue cursor
    int s_out;                     //   and the columns it hands to tier 0
    int t_count[5];                // Phase II tier queues: columns queued per tier (tier 4: the
    int t_cursor[5];               //   cluster tier) and the work-queue cursor of each tier
    int reps;                      // repeated lows seen by the last Phase I
    int resume_dim;                // sequential walkers: where to resume after a regrow
    long long resume_pos;          //   (column or row index; -1 = finished)
    long long resume_iter;         //   and the iteration count reached (trackers)
    int max_dim;                   // largest nnz(col) - 1 seen by the set-up
    int pad;
    int ucount[2];                     // compacted Phase I: list sizes (ping-pong)
    unsigned long long tier_adds[4];   // additions performed by each Phase II tier
    unsigned long long tier_slots[4];  // |P| + |T| + |T xor P| summed per tier
    unsigned long long s_adds;         // the scalar tier's share of tier_adds[0]
    int bucket_open;                   // ascending order: highest bucket (dim + 1) Phase II takes
    int bucket_unres[MAXC];            //   and the unresolved columns per bucket (this sweep)
    // diagnostics of the lazy tiers 0 and 1 (filled only in OPH_COUNTS builds),
    // per tier t at [8t ..]: additions by a pivot held in its record, by a
    // pivot of <= 4 rows read from its segment, by one of 5 .. G + 1 rows, by
    // a wider one; flushes of pending toggles before the chain's end; top
    // cancellations; columns entered; their rows on entry
    unsigned long long diag[16];
    unsigned long long sdiag[8];   // the scalar tier's (OPH_COUNTS builds)
#if defined(OPH_COUNTS) && OPH_COUNTS
    unsigned long long diag_sm[256];  // Phase II additions per SM
#endif
};

__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

struct __align__(32) PivRec {
    int col;
    int np;
    int left;
    unsigned seg4;
    int e[4];
};

// The record of a row, read through L2 (two 16-byte loads of one sector).
__device__ __forceinline__ void rec_load(const PivRec *r, int4 &h, int4 &e) {
    const int4 *p = reinterpret_cast<const int4 *>(r);
    h = __ldcg(p);
    e = __ldcg(p + 1);
}

__device__ __forceinline__ int ld_acquire_i32(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int4 ld_acquire_v4(const int4 *p) {
    int4 v;
    asm volatile("ld.acquire.gpu.global.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
}
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
__device__ __forceinline__ int4 ld_relaxed_v4(const int4 *p) {
    int4 v;
    asm volatile("ld.relaxed.gpu.global.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
}
__device__ __forceinline__ void st_release_i32(int *p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// True when a relaxed record read already holds the whole pivot (np <= 4,
// every needed entry past its marker).
__device__ __forceinline__ bool rec_complete(const int4 &h, const int4 &e) {
    const int np = h.y;
    return np >= 1 && np <= 4 && e.x >= 0 && (np < 2 || e.y >= 0) && (np < 3 || e.z >= 0) && (np < 4 || e.w >= 0);
}
// np and seg4 of a published record after the acquire of its col: the
// relaxed read's values when neither is a marker (each changes once), else
// a fresh read.
__device__ __forceinline__ int4 rec_header(const PivRec *r, const int4 &h) {
    ld_acquire_i32(&r->col);
    if (h.y > 0 && (unsigned)h.w != SEG4_NONE) return h;
    return __ldcg(reinterpret_cast<const int4 *>(r));
}
__device__ __forceinline__ int rec_entry(const int4 &e, int k) {
    return k == 0 ? e.x : k == 1 ? e.y : k == 2 ? e.z : e.w;
}
// The record of a row in one round trip, its header read with acquire: when
// col is set, every field is final and the pivot's segment may be read.
// The entries go first (relaxed, not held back by the acquire); an entry
// still showing its marker, or a header field that does, is read again
// after the acquire, when the publisher's writes are visible.
__device__ __forceinline__ bool rec_torn(const int4 &h, const int4 &e) {
    const int need = h.y < 4 ? h.y : 4;
    return h.y <= 0 || (unsigned)h.w == SEG4_NONE || e.x < 0 || (need > 1 && e.y < 0) || (need > 2 && e.z < 0) ||
           (need > 3 && e.w < 0);
}
__device__ __forceinline__ void rec_load_acq(const PivRec *r, int4 &h, int4 &e) {
    const int4 *p = reinterpret_cast<const int4 *>(r);
    e = __ldcg(p + 1);
    h = ld_acquire_v4(p);
    if (h.x >= 0 && rec_torn(h, e)) {
        h = __ldcg(p);
        e = __ldcg(p + 1);
    }
}
// A record fetched ahead without holding the fetching thread back: a strong
// relaxed read now (rec_fetch), and, where it is used, an acquire fence when
// it showed a pivot (rec_settle): the pair acts as rec_load_acq.
__device__ __forceinline__ void rec_fetch(const PivRec *r, int4 &h, int4 &e) {
    const int4 *p = reinterpret_cast<const int4 *>(r);
    e = ld_relaxed_v4(p + 1);
    h = ld_relaxed_v4(p);
}
__device__ __forceinline__ void rec_settle(const PivRec *r, int4 &h, int4 &e) {
    if (h.x < 0) return;
    fence_acq_rel();
    if (rec_torn(h, e)) {
        const int4 *p = reinterpret_cast<const int4 *>(r);
        h = __ldcg(p);
        e = __ldcg(p + 1);
    }
}

// Publish column `col` (length n, segment seg) as the pivot of row `row`;
// `top` holds its min(n, 4) highest rows, ascending.  Called by one thread
// after the column's rows are visible to it (its own writes, or writes
// ordered before by a barrier).  ORDERED = false when the readers run in a
// later kernel (Phase 0 / I).
template <bool ORDERED = true>
__device__ __forceinline__ void rec_publish_top(PivRec *rec, int row, int col, int n, long long seg, const int *top) {
    PivRec *r = rec + row;
    r->np = n;
    r->seg4 = (unsigned)(seg >> 2);
    for (int k = 0; k < 4; k++) r->e[k] = k < n ? top[k] : -1;
    if (ORDERED) {
        fence_acq_rel();
        st_release_i32(&r->col, col);
    } else {
        r->col = col;
    }
}
// The same from the column's n rows.
template <bool ORDERED = true>
__device__ __forceinline__ void rec_publish(PivRec *rec, int row, int col, int n, long long seg, const int *rows) {
    rec_publish_top<ORDERED>(rec, row, col, n, seg, rows + (n > 4 ? n - 4 : 0));
}

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

// Symmetric difference for a pivot of at most G entries held one per lane,
// by segments: the pivot's entries, ranked in A (lanes k < nP, binary
// search), cut A into nP + 1 runs that are copied with a constant shift each;
// a pivot entry absent from A is written between its runs, one present in A
// removes that element and shifts the following runs down by one.  Per
// element of A this is a load, a store and an add.  Returns |A xor P|.
template <int G, class Tile>
__device__ __forceinline__ int merge_xor_seg(const Tile &tile, const int *A, int nA, int pv, int nP, int *B) {
    const int lane = tile.thread_rank();
    int r = 0;
    bool pdup = false;
    if (lane < nP) {
        r = lower_bound(A, nA, pv);
        pdup = r < nA && A[r] == pv;
    }
    const unsigned dmask = tile.ballot(pdup);
    int src = 0, shift = 0;
    for (int k = 0; k < nP; k++) {
        const int rk = tile.shfl(r, k);
        const int pk = tile.shfl(pv, k);
        for (int q = src + lane; q < rk; q += G) B[q + shift] = A[q];
        if ((dmask >> k) & 1u) {
            src = rk + 1;
            shift -= 1;
        } else {
            if (lane == 0) B[rk + shift] = pk;
            src = rk;
            shift += 1;
        }
    }
    for (int q = src + lane; q < nA; q += G) B[q + shift] = A[q];
    tile.sync();
    return nA + nP - 2 * __popc(dmask);
}

// Move A[a..b) to A[a + t..b + t) in place, 0 < t < G: chunks from the top
// down, each loaded by the whole group before any lane stores.
template <int G, class Tile>
__device__ __forceinline__ void shift_up(const Tile &tile, int *A, int a, int b, int t) {
    const int lane = tile.thread_rank();
    for (int hi = b; hi > a; hi -= G) {
        const int q = hi - G + lane;
        const int v = q >= a ? A[q] : 0;
        tile.sync();
        if (q >= a) A[q + t] = v;
    }
}
// The same with -G < t < 0: chunks from the bottom up.
template <int G, class Tile>
__device__ __forceinline__ void shift_down(const Tile &tile, int *A, int a, int b, int t) {
    const int lane = tile.thread_rank();
    for (int lo = a; lo < b; lo += G) {
        const int q = lo + lane;
        const int v = q < b ? A[q] : 0;
        tile.sync();
        if (q < b) A[q + t] = v;
    }
}

// Add a pivot of three rows {x0, x1, low} (x0 < x1 < low = A[n - 1]) to A in
// place.  The low cancels; x0 and x1 each insert or cancel, so A splits into
// a prefix that stays, a middle run that moves by one and a top run that
// moves by two or stays.  Returns the new length.  A needs room for n + 1.
template <int G, class Tile>
__device__ __forceinline__ int merge3_inplace(const Tile &tile, int *A, int n, int x0, int x1) {
    const int lane = tile.thread_rank();
    const int m1 = n - 1;
    int r = 0;
    if (lane < 2) r = lower_bound(A, m1, lane ? x1 : x0);
    const int r0 = tile.shfl(r, 0), r1 = tile.shfl(r, 1);
    const bool d0 = r0 < m1 && A[r0] == x0;
    const bool d1 = r1 < m1 && A[r1] == x1;
    tile.sync();
    if (!d0) {
        if (!d1) shift_up<G>(tile, A, r1, m1, 2);
        shift_up<G>(tile, A, r0, r1, 1);
    } else {
        shift_down<G>(tile, A, r0 + 1, r1, -1);
        if (d1) shift_down<G>(tile, A, r1 + 1, m1, -2);
    }
    tile.sync();
    if (lane == 0) {
        if (!d0) A[r0] = x0;
        if (!d1) A[r1 + (d0 ? -1 : 1)] = x1;
    }
    tile.sync();
    return n + 1 - 2 * ((int)d0 + (int)d1);
}

// The same for a pivot of more entries (still at most G, one per lane): the
// runs are found per element instead of per pivot entry.  With thr_k = the
// first index of A that lies past P[k] (r_k, plus one when P[k] is in A, as
// that element is dropped), the element at index i moves by
// c - 2 * (common entries among the first c), c = #{k : thr_k <= i}, and c is
// found by a binary search over the thresholds held in lanes (uniform trip
// count, so every lane takes part in every shuffle).  Returns |A xor P|.
template <int G, class Tile>
__device__ __forceinline__ int merge_xor_thr(const Tile &tile, const int *A, int nA, int pv, int nP, int *B) {
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
    const int thr = r + (pdup ? 1 : 0);
    int top = 1;
    while (top * 2 <= nP) top *= 2;
    for (int base = 0; base < nA; base += G) {
        const int i = base + lane;
        int c = 0;
        for (int step = top; step > 0; step >>= 1) {
            const int t = tile.shfl(thr, min(c + step - 1, G - 1));
            if (c + step <= nP && t <= i) c += step;
        }
        const int rc = tile.shfl(r, min(c, G - 1));
        if (i < nA) {
            const bool drop = c < nP && ((dmask >> c) & 1u) && rc == i;
            const int shift = c - 2 * __popc(dmask & ((c >= 32) ? 0xffffffffu : ((1u << c) - 1u)));
            if (!drop) B[i + shift] = A[i];
        }
    }
    tile.sync();
    return nA + nP - 2 * __popc(dmask);
}

// Block-wide symmetric difference by merge path, for long columns.  The
// union of A and P in sorted order (ties: A's copy first) is cut into
// blockDim.x equal ranges; each thread finds its range's start by a binary
// search on the diagonal and merges it sequentially.  A common value is A[i]
// immediately followed by P[j], so taking A[i] cancels when P[j] == A[i] and
// taking P[j] cancels when A[i - 1] == P[j]: no thread needs its neighbours.
// A first pass counts each thread's kept elements, a block scan turns the
// counts into offsets, a second pass writes.  Per thread: one search and
// 2 (nA + nP) / blockDim.x merge steps, instead of a search per element.
// `scratch` holds blockDim.x / 32 ints; B must not alias A or P.
__device__ __forceinline__ int merge_xor_path(const int *A, int nA, const int *P, int nP, int *B, int *scratch) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    const int L = nA + nP;
    const int K = (L + nt - 1) / nt;
    const int d0 = min(tid * K, L), d1 = min(d0 + K, L);
    int lo = max(0, d0 - nP), hi = min(d0, nA);
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (A[mid] <= P[d0 - mid - 1]) lo = mid + 1;
        else hi = mid;
    }
    const int i0 = lo, j0 = d0 - lo;
    int cnt = 0;
    {
        int i = i0, j = j0;
        for (int d = d0; d < d1; d++) {
            const int a = i < nA ? A[i] : 0x7fffffff, p = j < nP ? P[j] : 0x7fffffff;
            if (i < nA && (j >= nP || a <= p)) {
                cnt += (j < nP && p == a) ? 0 : 1;
                i++;
            } else {
                cnt += (i > 0 && A[i - 1] == p) ? 0 : 1;
                j++;
            }
        }
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) scratch[wid] = incl;
    __syncthreads();
    int off = incl - cnt, total = 0;
    for (int q = 0; q < nw; q++) {
        const int c = scratch[q];
        if (q < wid) off += c;
        total += c;
    }
    {
        int i = i0, j = j0;
        for (int d = d0; d < d1; d++) {
            const int a = i < nA ? A[i] : 0x7fffffff, p = j < nP ? P[j] : 0x7fffffff;
            if (i < nA && (j >= nP || a <= p)) {
                if (!(j < nP && p == a)) B[off++] = a;
                i++;
            } else {
                if (!(i > 0 && A[i - 1] == p)) B[off++] = p;
                j++;
            }
        }
    }
    __syncthreads();
    return total;
}

// Block copy of n ints (all threads of the CTA).
__device__ __forceinline__ void block_copy(int *dst, const int *src, int n) {
    if ((((uintptr_t)dst | (uintptr_t)src) & 15) == 0) {
        const int n4 = n >> 2;
        const int4 *s4 = reinterpret_cast<const int4 *>(src);
        int4 *d4 = reinterpret_cast<int4 *>(dst);
        for (int q = threadIdx.x; q < n4; q += blockDim.x) d4[q] = s4[q];
        for (int q = (n4 << 2) + threadIdx.x; q < n; q += blockDim.x) dst[q] = src[q];
    } else {
        for (int q = threadIdx.x; q < n; q += blockDim.x) dst[q] = src[q];
    }
    __syncthreads();
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
