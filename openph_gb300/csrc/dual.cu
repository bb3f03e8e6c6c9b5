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
//
// The transpose is built straight into the column store of D', without a
// general sort (the reference's analogue is the slot-store build create_rows_mp,
// src/cuda/kernels.cu:25-38):
//   count    cnt[c] = entries of D' column c (the entries of D in row m-1-c)
//   scan     the column offsets of D', an exclusive prefix sum of cnt (tile
//            sums, their scan, then the tiles)
//   scatter  every entry (r, j) of D writes row m-1-j of D' column m-1-r
//            into a slot taken from a per-column cursor counting down from
//            cnt[c]; D's columns are visited in roughly ascending j, so the
//            slots fill from the top down and the rows land nearly ascending
//   finish   a thread per column of D': the segment header, the bucket of
//            D's column in the reversed position, and for a column of at
//            most 8 rows its rows sorted in registers and its low; then a
//            warp per longer column of at most 1024 rows (a bitonic network
//            over the warp's registers, up to 8 values a lane, or over its
//            slice of shared memory; longer ones are queued)
//   long     a CTA per queued column: LSD radix sort, 8-bit digits, through
//            a scratch range at the column's own offsets
//   records  per row of D': its pivot record reset with left[] (row m-1-j of
//            D' first appears in column m-1-low_D(j)) and beta by atomicMax
#include <climits>

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
    // per-thread tallies, merged once per block (no shared atomic per
    // column): bucket counts, and the row bucket seen for each column bucket
    // (TAB_NONE or a bucket; a second, different one marks the input mixed)
    unsigned long long cnt[MAXC];
    int tabv[MAXC];
#pragma unroll
    for (int b = 0; b < MAXC; b++) {
        cnt[b] = 0;
        tabv[b] = TAB_NONE;
    }
    bool mixed_t = false, bad_t = false;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t lo = colptr[j], hi = colptr[j + 1];
        if (lo < 0 || hi < lo || hi > nnz) {  // bounds first: nothing is read past rows[nnz)
            bad_t = true;
            continue;
        }
        const int b = bucket_of(hi - lo);
        if (b + 1 >= MAXC) {  // a bucket the Phase I scan does not keep
            mixed_t = true;
            continue;
        }
        int rb = TAB_NONE, prev = -1;
        for (int64_t k = lo; k < hi; k++) {
            const int r = rows[k];
            if (r <= prev || r >= m) {
                bad_t = true;
                break;
            }
            prev = r;
            const int br = bucket[r];
            if (k == lo) rb = br;
            else if (br != rb) mixed_t = true;
        }
#pragma unroll
        for (int d = 0; d < MAXC; d++)
            if (d == b + 1) {
                cnt[d]++;
                if (rb != TAB_NONE) {
                    if (tabv[d] == TAB_NONE) tabv[d] = rb;
                    else if (tabv[d] != rb) mixed_t = true;
                }
            }
    }
#pragma unroll
    for (int d = 0; d < MAXC; d++) {
        unsigned long long c = cnt[d];
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_count[d], c);
        if (tabv[d] != TAB_NONE) {
            const int old = atomicCAS(&s_tab[d], TAB_NONE, tabv[d]);
            if (old != TAB_NONE && old != tabv[d]) mixed_t = true;
        }
    }
    if (mixed_t) s_flags[0] = 1;
    if (bad_t) s_flags[1] = 1;
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

// ------------------------------------------------------------- transpose
constexpr int SCAN_THREADS = 1024, SCAN_ITEMS = 4, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Sum of v over the block (every thread gets it); red holds 33 partials.
__device__ __forceinline__ long long block_sum(long long v, long long *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        long long t = lane < nw ? red[lane] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    const long long total = red[32];
    __syncthreads();
    return total;
}

// Exclusive prefix of v over the block; red holds 33 partials.
__device__ __forceinline__ long long block_exclusive(long long v, long long *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) red[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const long long t = lane < nw ? red[lane] : 0;
        long long ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long u = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= o) ti += u;
        }
        if (lane < nw) red[lane] = ti - t;  // exclusive prefix of the warp totals
    }
    __syncthreads();
    const long long out = red[wid] + incl - v;
    __syncthreads();
    return out;
}

__device__ __forceinline__ void load_items(const int *__restrict__ cnt, int64_t n, int64_t base, int *v) {
    if (base + SCAN_ITEMS <= n) {
        const int4 q = *reinterpret_cast<const int4 *>(cnt + base);
        v[0] = q.x;
        v[1] = q.y;
        v[2] = q.z;
        v[3] = q.w;
    } else {
#pragma unroll
        for (int t = 0; t < SCAN_ITEMS; t++) v[t] = base + t < n ? cnt[base + t] : 0;
    }
}

// (scan 1) the sum of every tile of SCAN_TILE counts
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(const int *__restrict__ cnt, int64_t n,
                                                            long long *__restrict__ tsum) {
    __shared__ long long red[33];
    for (int64_t t = blockIdx.x; t * SCAN_TILE < n; t += gridDim.x) {
        int v[SCAN_ITEMS];
        load_items(cnt, n, t * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS, v);
        const long long total = block_sum((long long)v[0] + v[1] + v[2] + v[3], red);
        if (threadIdx.x == 0) tsum[t] = total;
    }
}

// (scan 2) exclusive prefix of the tile sums in place (one block); the grand
// total into *total
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tsums(long long *__restrict__ tsum, int64_t ntiles,
                                                             int64_t *__restrict__ total) {
    __shared__ long long red[33];
    long long carry = 0;
    for (int64_t b0 = 0; b0 < ntiles; b0 += SCAN_THREADS) {
        const int64_t t = b0 + threadIdx.x;
        const long long v = t < ntiles ? tsum[t] : 0;
        const long long ex = block_exclusive(v, red);
        if (t < ntiles) tsum[t] = carry + ex;
        carry += block_sum(v, red);
    }
    if (threadIdx.x == 0) *total = carry;
}

// Segment of column c of a store whose column offsets are `off` (the layout
// of k_setup_columns: room for the header, capacities in 16-byte units).
__device__ __forceinline__ int64_t seg_start(int64_t c, int64_t off) { return 8 * c + 4 * ((off + 3) >> 2); }

// (scan 3) the offsets: out[i] = sum of cnt[0 .. i); with `cur`, also each
// column's scatter cursor: the pool index just past its last row slot
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const int *__restrict__ cnt, int64_t n,
                                                             const long long *__restrict__ tsum,
                                                             int64_t *__restrict__ out,
                                                             unsigned long long *__restrict__ cur) {
    __shared__ long long red[33];
    for (int64_t t = blockIdx.x; t * SCAN_TILE < n; t += gridDim.x) {
        const int64_t base = t * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
        int v[SCAN_ITEMS];
        load_items(cnt, n, base, v);
        long long run = tsum[t] + block_exclusive((long long)v[0] + v[1] + v[2] + v[3], red);
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS; q++) {
            if (base + q < n) {
                out[base + q] = run;
                if (cur) cur[base + q] = (unsigned long long)(seg_start(base + q, run) + SEG_HDR + v[q]);
            }
            run += v[q];
        }
    }
}

// In the count and the scatter the warp's threads walk their columns of D
// entry by entry in step, so equal targets in D' meet in one instruction and
// share one atomic (__match_any_sync): consecutive Rips triangles mostly
// share their longest edge, hence their last row.

// entries of every column of D' (= entries of D in each row)
__global__ void k_dual_count(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                             int *__restrict__ cnt) {
    const int lane = threadIdx.x & 31;
    for (int64_t j0 = blockIdx.x * (int64_t)blockDim.x; j0 < m; j0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = j0 + threadIdx.x;
        const int64_t lo = j < m ? colptr[j] : 0, hi = j < m ? colptr[j + 1] : 0;
        const int n = (int)(hi - lo);
        const int nmax = __reduce_max_sync(0xffffffffu, n);
        for (int t = 0; t < nmax; t++) {
            const int c = t < n ? (int)(m - 1 - rows[lo + t]) : -1;
            const unsigned peers = __match_any_sync(0xffffffffu, c);
            if (c >= 0 && lane == __ffs(peers) - 1) atomicAdd(&cnt[c], __popc(peers));
        }
    }
}


// every entry of D into its column of D' (row m-1-j), slots from the top;
// equal targets within the warp take their slots with one atomic on the
// column's cursor, which holds the pool index itself (no offset lookup)
__global__ void k_dual_scatter(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                               unsigned long long *__restrict__ cursor, int *__restrict__ pool, int roff) {
    const int lane = threadIdx.x & 31;
    for (int64_t j0 = blockIdx.x * (int64_t)blockDim.x; j0 < m; j0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = j0 + threadIdx.x;
        const int64_t lo = j < m ? colptr[j] : 0, hi = j < m ? colptr[j + 1] : 0;
        const int n = (int)(hi - lo);
        const int val = roff + (int)(m - 1 - j);
        const int nmax = __reduce_max_sync(0xffffffffu, n);
        for (int t = 0; t < nmax; t++) {
            const int c = t < n ? (int)(m - 1 - rows[lo + t]) : -1;
            const unsigned peers = __match_any_sync(0xffffffffu, c);
            const int leader = __ffs(peers) - 1;
            unsigned long long top = 0;
            if (c >= 0 && lane == leader) top = atomicAdd(&cursor[c], 0ull - (unsigned long long)__popc(peers));
            top = __shfl_sync(0xffffffffu, top, leader);
            if (c >= 0) {
                // the lower lane (the smaller column of D) takes the higher slot
                pool[(int64_t)top - 1 - __popc(peers & ((1u << lane) - 1u))] = val;
            }
        }
    }
}

constexpr int FIN_WARPS = 8, SHORT_COL = 8, WIDE_COL = 256, LONG_COL = 1024;

// a thread per column of D': the segment header, the bucket of D's column in
// the reversed position, and for a column of at most SHORT_COL rows its rows
// sorted (in registers) and its low; longer columns are queued for warps
__global__ void k_dual_finish(const int64_t *__restrict__ dcolptr, const int64_t *__restrict__ colptr, int64_t m,
                              int *__restrict__ pool, int64_t *__restrict__ seg, int32_t *__restrict__ low,
                              int8_t *__restrict__ dim, int *__restrict__ mid_list, int *mid_count,
                              int64_t seg_base) {
    for (int64_t c0 = blockIdx.x * (int64_t)blockDim.x; c0 < m; c0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = c0 + threadIdx.x;
        bool queue = false;
        if (c < m) {
            const int64_t a = dcolptr[c], b = dcolptr[c + 1];
            const int n = (int)(b - a);
            const int64_t s = seg_start(c, a), e = seg_start(c + 1, b);
            int *R = pool + s + SEG_HDR;
            *reinterpret_cast<int4 *>(pool + s) = make_int4(n, (int)(e - s - SEG_HDR), 0, 0);
            seg[c] = seg_base + s;
            const int64_t i = m - 1 - c;
            const int64_t nd = colptr[i + 1] - colptr[i];
            dim[c] = (int8_t)(nd - 1 > 126 ? 126 : nd - 1);
            if (n <= SHORT_COL) {
                int v[SHORT_COL];
#pragma unroll
                for (int k = 0; k < SHORT_COL; k++) v[k] = k < n ? R[k] : INT_MAX;
                // insertion sort (the rows arrive nearly ascending)
#pragma unroll
                for (int k = 1; k < SHORT_COL; k++)
#pragma unroll
                    for (int q = k; q > 0; q--) {
                        const int lo = min(v[q - 1], v[q]), hi = max(v[q - 1], v[q]);
                        v[q - 1] = lo;
                        v[q] = hi;
                    }
                int top = -1;
#pragma unroll
                for (int k = 0; k < SHORT_COL; k++)
                    if (k < n) {
                        R[k] = v[k];
                        top = v[k];
                    }
                low[c] = top;
            } else {
                queue = true;
            }
        }
        warp_append(queue, (int)c, mid_list, mid_count);
    }
}

// One stage of the network (SIZE, STRIDE as template arguments, so that
// every index into v is a constant and v stays in registers), then the next.
template <int K, int SIZE, int STRIDE>
__device__ __forceinline__ void warp_sort_stage(int (&v)[K], int lane) {
    if constexpr (STRIDE > 0) {
        if constexpr (STRIDE < K) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                const int q = k ^ STRIDE;
                if (q > k) {
                    const bool up = ((lane * K + k) & SIZE) == 0;
                    const int x = v[k], y = v[q];
                    v[k] = up ? min(x, y) : max(x, y);
                    v[q] = up ? max(x, y) : min(x, y);
                }
            }
        } else {
            constexpr int LS = STRIDE / K;
            const bool lower = (lane & LS) == 0;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const bool up = ((lane * K + k) & SIZE) == 0;
                const int o = __shfl_xor_sync(0xffffffffu, v[k], LS);
                v[k] = (lower == up) ? min(v[k], o) : max(v[k], o);
            }
        }
        warp_sort_stage<K, SIZE, STRIDE / 2>(v, lane);
    }
}
template <int K, int SIZE>
__device__ __forceinline__ void warp_sort_sizes(int (&v)[K], int lane) {
    if constexpr (SIZE <= 32 * K) {
        warp_sort_stage<K, SIZE, SIZE / 2>(v, lane);
        warp_sort_sizes<K, SIZE * 2>(v, lane);
    }
}

// Ascending order of the warp's 32 K values, lane l holding elements
// l K .. l K + K - 1: a bitonic network, in registers within a lane and by
// shuffles across lanes (K a power of two).
template <int K>
__device__ __forceinline__ void warp_sort_reg(int (&v)[K]) {
    warp_sort_sizes<K, 2>(v, threadIdx.x & 31);
}

// A column of n <= 32 K rows at R sorted by the warp; returns the low.
template <int K>
__device__ __forceinline__ int warp_sort_column(int *R, int n) {
    const int lane = threadIdx.x & 31;
    int v[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int e = lane * K + k;
        v[k] = e < n ? R[e] : INT_MAX;
    }
    // already ascending (each lane's run and its boundary with the next)?
    bool asc = true;
#pragma unroll
    for (int k = 0; k + 1 < K; k++) asc &= v[k] <= v[k + 1];
    const int next_first = __shfl_down_sync(0xffffffffu, v[0], 1);
    if (lane < 31) asc &= v[K - 1] <= next_first;
    if (__all_sync(0xffffffffu, asc)) {
        // the last element: lane (n-1)/K, slot (n-1)%K (selected with
        // constant indices, so that v stays in registers)
        int last = INT_MIN;
#pragma unroll
        for (int k = 0; k < K; k++)
            if (k == (n - 1) % K) last = v[k];
        return __shfl_sync(0xffffffffu, last, (n - 1) / K);
    }
    warp_sort_reg<K>(v);
    int top = INT_MIN;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int e = lane * K + k;
        if (e < n) {
            R[e] = v[k];
            top = v[k];
        }
    }
    return __reduce_max_sync(0xffffffffu, top);
}

// a warp per queued column (more than SHORT_COL rows): its rows sorted in
// registers and its low, for columns of at most MID_COL rows (a few values a
// lane keeps the kernel's registers, hence its occupancy, low); longer
// columns are queued for k_dual_finish_wide (<= LONG_COL) or a CTA
constexpr int MID_COL = 128;
__global__ void __launch_bounds__(FIN_WARPS * 32) k_dual_finish_warp(const int64_t *__restrict__ dcolptr,
                                                                     int *__restrict__ pool,
                                                                     int32_t *__restrict__ low,
                                                                     const int *__restrict__ mid_list,
                                                                     const int *mid_count,
                                                                     int *__restrict__ wide_list, int *wide_count,
                                                                     int *__restrict__ long_list, int *long_count) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * FIN_WARPS;
    const int count = *mid_count;
    for (int64_t idx = blockIdx.x * (int64_t)FIN_WARPS + wid; idx < count; idx += nwarps) {
        const int64_t c = mid_list[idx];
        const int64_t a = dcolptr[c];
        const int n = (int)(dcolptr[c + 1] - a);
        if (n > MID_COL) {
            if (lane == 0) {
                if (n <= LONG_COL) wide_list[atomicAdd(wide_count, 1)] = (int)c;
                else long_list[atomicAdd(long_count, 1)] = (int)c;
            }
            continue;
        }
        int *R = pool + seg_start(c, a) + SEG_HDR;
        const int top = n <= 32 ? warp_sort_column<1>(R, n) : warp_sort_column<4>(R, n);
        if (lane == 0) low[c] = top;
    }
}

// the same for the queued columns of MID_COL < n <= LONG_COL rows: eight
// values a lane up to WIDE_COL rows, sixteen up to twice that, else a
// bitonic network over the warp's slice of shared memory
__global__ void __launch_bounds__(FIN_WARPS * 32) k_dual_finish_wide(const int64_t *__restrict__ dcolptr,
                                                                     int *__restrict__ pool,
                                                                     int32_t *__restrict__ low,
                                                                     const int *__restrict__ wide_list,
                                                                     const int *wide_count) {
    __shared__ int sbuf[FIN_WARPS][LONG_COL];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * FIN_WARPS;
    const int count = *wide_count;
    int *B = sbuf[wid];
    for (int64_t idx = blockIdx.x * (int64_t)FIN_WARPS + wid; idx < count; idx += nwarps) {
        const int64_t c = wide_list[idx];
        const int64_t a = dcolptr[c];
        const int n = (int)(dcolptr[c + 1] - a);
        int *R = pool + seg_start(c, a) + SEG_HDR;
        if (n <= WIDE_COL) {
            const int top = warp_sort_column<8>(R, n);
            if (lane == 0) low[c] = top;
            continue;
        }
        if (n <= 2 * WIDE_COL) {  // sixteen values a lane: in registers, no warp barriers
            const int top = warp_sort_column<16>(R, n);
            if (lane == 0) low[c] = top;
            continue;
        }
        bool sorted = true;
        for (int k = lane; k + 1 < n; k += 32) sorted &= R[k] < R[k + 1];
        if (__all_sync(0xffffffffu, sorted)) {
            if (lane == 0) low[c] = R[n - 1];
            continue;
        }
        int N = 2 * WIDE_COL;
        while (N < n) N <<= 1;
        for (int k = lane; k < N; k += 32) B[k] = k < n ? R[k] : INT_MAX;
        __syncwarp();
        for (int size = 2; size <= N; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = lane; i < N; i += 32) {
                    const int l = i ^ stride;
                    if (l > i) {
                        const bool up = (i & size) == 0;
                        const int x = B[i], y = B[l];
                        if ((x > y) == up) {
                            B[i] = y;
                            B[l] = x;
                        }
                    }
                }
                __syncwarp();
            }
        for (int k = lane; k < n; k += 32) R[k] = B[k];
        if (lane == 0) low[c] = B[n - 1];
        __syncwarp();  // B is reused by the warp's next column
    }
}

// a CTA per column of more than LONG_COL rows: LSD radix sort, 8-bit digits,
// between the column's rows and scratch[dcolptr[c] ..] (four passes, so the
// result ends where it began); then its low
constexpr int LS_THREADS = 1024;
__global__ void __launch_bounds__(LS_THREADS) k_dual_sort_long(const int64_t *__restrict__ dcolptr,
                                                               int *__restrict__ pool, int32_t *__restrict__ low,
                                                               const int *__restrict__ long_list,
                                                               const int *long_count, int *long_cursor,
                                                               int *__restrict__ scratch) {
    __shared__ int base[256], tot[256];
    __shared__ int wcnt[LS_THREADS / 32][256];
    __shared__ int s_idx;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (;;) {
        if (tid == 0) s_idx = atomicAdd(long_cursor, 1);
        __syncthreads();
        const int idx = s_idx;
        __syncthreads();
        if (idx >= *long_count) break;
        const int64_t c = long_list[idx];
        const int64_t a = dcolptr[c];
        const int n = (int)(dcolptr[c + 1] - a);
        int *R = pool + seg_start(c, a) + SEG_HDR;
        int *src = R, *dst = scratch + a;
        for (int shift = 0; shift < 32; shift += 8) {
            if (tid < 256) base[tid] = 0;
            __syncthreads();
            for (int k = tid; k < n; k += LS_THREADS) atomicAdd(&base[(src[k] >> shift) & 255], 1);
            __syncthreads();
            if (tid < 32) {  // exclusive prefix of the 256 digit counts, 8 per lane
                int v[8], sum = 0;
                for (int q = 0; q < 8; q++) {
                    v[q] = base[8 * tid + q];
                    sum += v[q];
                }
                int incl = sum;
                for (int o = 1; o < 32; o <<= 1) {
                    const int u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += u;
                }
                int run = incl - sum;
                for (int q = 0; q < 8; q++) {
                    base[8 * tid + q] = run;
                    run += v[q];
                }
            }
            __syncthreads();
            // stable scatter, LS_THREADS elements at a time: the rank among
            // the warp's equal digits, then among earlier warps' (counts)
            for (int t0 = 0; t0 < n; t0 += LS_THREADS) {
                const int k = t0 + tid;
                const bool act = k < n;
                const int v = act ? src[k] : 0;
                const int d = act ? (v >> shift) & 255 : 256;
                for (int q = tid; q < (LS_THREADS / 32) * 256; q += LS_THREADS) (&wcnt[0][0])[q] = 0;
                __syncthreads();
                const unsigned peers = __match_any_sync(0xffffffffu, d);
                const int rank = __popc(peers & ((1u << lane) - 1u));
                if (act && rank == 0) wcnt[wid][d] = __popc(peers);
                __syncthreads();
                if (tid < 256) {
                    int run = 0;
                    for (int w = 0; w < LS_THREADS / 32; w++) {
                        const int x = wcnt[w][tid];
                        wcnt[w][tid] = run;
                        run += x;
                    }
                    tot[tid] = run;
                }
                __syncthreads();
                if (act) dst[base[d] + wcnt[wid][d] + rank] = v;
                __syncthreads();
                if (tid < 256) base[tid] += tot[tid];
                __syncthreads();
            }
            int *t = src;
            src = dst;
            dst = t;
        }
        if (tid == 0) low[c] = R[n - 1];
        __syncthreads();
    }
}

// ------------------------------------------- the transpose of a batch
// A block-diagonal matrix (instance b in columns, and rows, [off[b],
// off[b+1])) whose instances have at most IT_COLS columns, at most IT_ROWS
// distinct rows and D' columns of at most IT_MAXCOL rows (batches of small
// complexes) is transposed per instance with every count and cursor in
// shared memory, where the general transpose above takes a global atomic
// per entry and a sort per column after its scatter.  An instance's D'
// columns are contiguous and so are their entries, which start after the
// entries of every later instance (nnz - colptr[off[b+1]]): no global scan.
// k_dual_inst_a, a CTA per instance:
//   rows      the instance's rows marked in a bitmap of its columns, ranked
//             by popcount: each distinct row q gets a dense index d(q)
//             (a Rips filtration interleaves its triangles, never rows, with
//             its edges, so rows are few but spread over the columns);
//   count     entries per dense row (shared atomics), their exclusive prefix
//             in D' order (descending q): off[d];
//   headers   every D' column of the instance: segment, header, bucket of
//             D's column in the reversed position, low -1 if empty;
//   chunks    whole columns of at most IT_CAP entries (chunk k: the columns
//             whose entries start in [k IT_SPAN, (k+1) IT_SPAN)), each
//             described in a global list;
//   partition every entry (d, q, column) into its chunk's range of a
//             scratch array (shared cursors).
// k_dual_inst_b, a CTA per chunk (of every instance at once): its entries
// into shared memory, counted and placed per column (the chunk's columns
// are contiguous: its count prefix in D' order gives their starts), every
// column sorted by a warp there, then written out with its low.
// An instance outside those bounds sets *fail and the caller builds the
// whole store with the general transpose instead.
constexpr int IT_COLS = 1 << 19, IT_WORDS = IT_COLS / 32, IT_ROWS = 8192, IT_CAP = 3072, IT_MAXCOL = 512,
              IT_CHUNKS = 512;
constexpr int IT_SPAN = IT_CAP - IT_MAXCOL;
constexpr int ITA_THREADS = 1024, ITB_THREADS = 256;
constexpr size_t ITA_SMEM = sizeof(uint32_t) * IT_WORDS + sizeof(uint16_t) * IT_WORDS + sizeof(int) * IT_ROWS +
                            sizeof(int) * 5 * IT_CHUNKS;
constexpr size_t ITB_SMEM = sizeof(unsigned long long) * IT_CAP + sizeof(int) * (3 * IT_CAP + 1);
struct ItChunk {
    int b, lo, hi, dmin, dmax, pad[3];
};
// a scratch entry: dense row (13 bits) | q (19 bits) | column of the instance (32 bits)
__device__ __forceinline__ unsigned long long it_pack(int d, int q, int jl) {
    return ((unsigned long long)(((unsigned)d << 19) | (unsigned)q) << 32) | (unsigned)jl;
}

__global__ void __launch_bounds__(ITA_THREADS, 1)
    k_dual_inst_a(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m, int64_t nnz,
                  const int64_t *__restrict__ inst_off, int count, int *__restrict__ pool, int64_t *__restrict__ seg,
                  int32_t *__restrict__ low, int8_t *__restrict__ dim, unsigned long long *__restrict__ scratch,
                  ItChunk *__restrict__ chunks, int *nchunks, int *fail) {
    extern __shared__ __align__(16) unsigned char ita_smem[];  // ITA_SMEM bytes
    uint32_t *bits = reinterpret_cast<uint32_t *>(ita_smem);             // IT_WORDS
    uint16_t *wrank = reinterpret_cast<uint16_t *>(bits + IT_WORDS);     // IT_WORDS: set bits in earlier words
    int *off = reinterpret_cast<int *>(wrank + IT_WORDS);                // IT_ROWS: counts, then prefixes
    int *c_lo = off + IT_ROWS, *c_hi = c_lo + IT_CHUNKS, *c_dmin = c_hi + IT_CHUNKS, *c_dmax = c_dmin + IT_CHUNKS,
        *c_cur = c_dmax + IT_CHUNKS;
    __shared__ long long red[33];
    __shared__ int s_bad, s_base, s_rows;
    const int tid = threadIdx.x;
    constexpr int T = ITA_THREADS;
    for (int b = blockIdx.x; b < count; b += gridDim.x) {
        const int64_t o0 = inst_off[b], o1 = inst_off[b + 1], mb = o1 - o0;
        const int64_t e0 = colptr[o0], e1 = colptr[o1];
        const int total = (int)(e1 - e0);
        const int64_t A = nnz - e1;
        if (tid == 0) s_bad = (mb > IT_COLS || (e1 - e0) >= (1ll << 30)) ? 1 : 0;
        for (int w = tid; w < IT_WORDS; w += T) bits[w] = 0;
        for (int d = tid; d < IT_ROWS; d += T) off[d] = 0;
        __syncthreads();
        if (s_bad) {
            if (tid == 0) atomicExch(fail, 1);
            __syncthreads();
            continue;  // the whole store is rebuilt by the general transpose
        }
        // the rows that occur, four loads in flight per thread
        for (int64_t e = e0 + tid; e < e1; e += 4 * T) {
            int64_t q[4];
#pragma unroll
            for (int u = 0; u < 4; u++) q[u] = e + u * T < e1 ? (int64_t)rows[e + u * T] - o0 : -2;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (q[u] == -2) continue;
                if (q[u] < 0 || q[u] >= mb) s_bad = 1;
                else atomicOr(&bits[q[u] >> 5], 1u << (q[u] & 31));
            }
        }
        __syncthreads();
        {  // exclusive popcount prefix over the words: thread t holds words [PER t, PER (t+1))
            constexpr int PER = IT_WORDS / T;
            int v[PER], sum = 0;
#pragma unroll
            for (int k = 0; k < PER; k++) {
                v[k] = __popc(bits[PER * tid + k]);
                sum += v[k];
            }
            int run = (int)block_exclusive(sum, red);
            if (tid == T - 1) s_rows = run + sum;
#pragma unroll
            for (int k = 0; k < PER; k++) {
                wrank[PER * tid + k] = (uint16_t)min(run, 65535);
                run += v[k];
            }
        }
        __syncthreads();
        const int D = s_rows;
        if (s_bad || D > IT_ROWS) {
            if (tid == 0) atomicExch(fail, 1);
            __syncthreads();
            continue;
        }
        // the dense index of row q: its rank among the rows that occur
        auto dense = [&](int64_t q) -> int {
            return wrank[q >> 5] + __popc(bits[q >> 5] & ((1u << (q & 31)) - 1u));
        };
        for (int64_t e = e0 + tid; e < e1; e += 4 * T) {
            int d[4];
#pragma unroll
            for (int u = 0; u < 4; u++) d[u] = e + u * T < e1 ? dense((int64_t)rows[e + u * T] - o0) : -1;
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (d[u] >= 0) atomicAdd(&off[d[u]], 1);
        }
        __syncthreads();
        {  // exclusive prefix in D' order (descending d): thread t holds d in [IT_ROWS - PER (t+1), IT_ROWS - PER t)
            constexpr int PER = IT_ROWS / T;
            const int dtop = IT_ROWS - PER * tid;
            int v[PER], sum = 0;
#pragma unroll
            for (int k = 0; k < PER; k++) {
                v[k] = off[dtop - 1 - k];
                sum += v[k];
                if (v[k] > IT_MAXCOL) s_bad = 1;
            }
            int run = (int)block_exclusive(sum, red);
#pragma unroll
            for (int k = 0; k < PER; k++) {
                off[dtop - 1 - k] = run;
                run += v[k];
            }
        }
        __syncthreads();
        const int K = total / IT_SPAN + 1;
        if (s_bad || K > IT_CHUNKS) {
            if (tid == 0) atomicExch(fail, 1);
            __syncthreads();
            continue;
        }
        // entries of the columns of dense rows >= d: off[d - 1] (total for d = 0)
        auto above = [&](int d) -> int { return d == 0 ? total : off[d - 1]; };
        for (int64_t q = tid; q < mb; q += T) {
            const int64_t c = m - 1 - (o0 + q);
            const int d = dense(q);
            const bool occ = (bits[q >> 5] >> (q & 31)) & 1u;
            // a row that occurs: its own prefix; one that does not: the
            // entries of the rows above it, those of dense index >= d
            // (above(D) = 0: the prefix past the last row that occurs)
            const int rel = occ ? off[d] : above(d);
            const int n = occ ? above(d) - off[d] : 0;
            const int64_t a = A + rel;
            const int64_t s = seg_start(c, a), e = seg_start(c + 1, a + n);
            *reinterpret_cast<int4 *>(pool + s) = make_int4(n, (int)(e - s - SEG_HDR), 0, 0);
            seg[c] = s;
            const int64_t nd = colptr[o0 + q + 1] - colptr[o0 + q];
            dim[c] = (int8_t)(nd - 1 > 126 ? 126 : nd - 1);
            if (n == 0) low[c] = -1;
        }
        for (int k = tid; k < K; k += T) {
            c_lo[k] = INT_MAX;
            c_hi[k] = -1;
            c_dmin[k] = INT_MAX;
            c_dmax[k] = -1;
            c_cur[k] = 0;
        }
        __syncthreads();
        for (int d = tid; d < D; d += T) {
            const int k = off[d] / IT_SPAN;
            atomicMin(&c_lo[k], off[d]);
            atomicMax(&c_hi[k], above(d));
            atomicMin(&c_dmin[k], d);
            atomicMax(&c_dmax[k], d);
        }
        if (tid == 0) s_base = atomicAdd(nchunks, K);
        __syncthreads();
        for (int k = tid; k < K; k += T) {
            ItChunk ch;
            ch.b = b;
            ch.lo = c_hi[k] < 0 ? -1 : c_lo[k];  // -1: no column starts in this span
            ch.hi = c_hi[k];
            ch.dmin = c_dmin[k];
            ch.dmax = c_dmax[k];
            ch.pad[0] = ch.pad[1] = ch.pad[2] = 0;
            chunks[s_base + k] = ch;
        }
        // partition: every entry into its chunk's range of the scratch, four
        // columns a thread at a time (their offsets, then their rows, in flight)
        for (int64_t j0 = tid; j0 < mb; j0 += 4 * T) {
            int64_t lo[4], hi[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int64_t jl = j0 + u * T;
                lo[u] = jl < mb ? colptr[o0 + jl] : 0;
                hi[u] = jl < mb ? colptr[o0 + jl + 1] : 0;
            }
            int qs[4][MAXC - 1];
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int t = 0; t < MAXC - 1; t++)
                    qs[u][t] = lo[u] + t < hi[u] ? (int)((int64_t)rows[lo[u] + t] - o0) : -1;
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int t = 0; t < MAXC - 1; t++) {
                    if (qs[u][t] < 0) continue;
                    const int d = dense(qs[u][t]);
                    const int k = off[d] / IT_SPAN;
                    const int slot = atomicAdd(&c_cur[k], 1);
                    scratch[A + c_lo[k] + slot] = it_pack(d, qs[u][t], (int)(j0 + u * T));
                }
        }
        __syncthreads();  // the shared arrays are reset for the next instance
    }
}

__global__ void __launch_bounds__(ITB_THREADS, 3)
    k_dual_inst_b(int64_t m, int64_t nnz, const int64_t *__restrict__ colptr, const int64_t *__restrict__ inst_off,
                  int *__restrict__ pool, int32_t *__restrict__ low, const unsigned long long *__restrict__ scratch,
                  const ItChunk *__restrict__ chunks, const int *nchunks, int roff) {
    extern __shared__ __align__(16) unsigned char itb_smem[];  // ITB_SMEM bytes
    unsigned long long *pairs = reinterpret_cast<unsigned long long *>(itb_smem);  // IT_CAP
    int *placed = reinterpret_cast<int *>(pairs + IT_CAP);                       // IT_CAP
    int *start = placed + IT_CAP;                                                // IT_CAP + 1
    int *qof = start + IT_CAP + 1;                                               // IT_CAP
    __shared__ long long red[33];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    constexpr int T = ITB_THREADS;
    const int nch = *nchunks;
    for (int idx = blockIdx.x; idx < nch; idx += gridDim.x) {
        const ItChunk ch = chunks[idx];
        if (ch.lo < 0) continue;  // uniform: every thread read the same descriptor
        const int64_t o0 = inst_off[ch.b];
        const int64_t A = nnz - colptr[inst_off[ch.b + 1]];
        const int len = ch.hi - ch.lo, span = ch.dmax - ch.dmin + 1;
        if (len > IT_CAP || span > IT_CAP) continue;  // not reached: each column of the chunk holds a row
        for (int i = tid; i <= span; i += T) start[i] = 0;
        __syncthreads();
        for (int i = tid; i < len; i += T) {
            const unsigned long long pr = scratch[A + ch.lo + i];
            pairs[i] = pr;
            const int x = (int)(pr >> 51) - ch.dmin;
            atomicAdd(&start[x], 1);
            qof[x] = (int)((pr >> 32) & ((1u << 19) - 1u));
        }
        __syncthreads();
        {  // exclusive prefix in D' order (descending d): slot i holds d = dmax - i
            constexpr int PER = IT_CAP / T;
            int v[PER], sum = 0;
#pragma unroll
            for (int k = 0; k < PER; k++) {
                const int i = tid * PER + k;
                v[k] = i < span ? start[span - 1 - i] : 0;
                sum += v[k];
            }
            int run = (int)block_exclusive(sum, red);
#pragma unroll
            for (int k = 0; k < PER; k++) {
                const int i = tid * PER + k;
                if (i < span) start[span - 1 - i] = run;
                run += v[k];
            }
        }
        __syncthreads();
        // each entry into its column's slots (start[] moves to each column's end)
        for (int i = tid; i < len; i += T) {
            const unsigned long long pr = pairs[i];
            const int x = (int)(pr >> 51) - ch.dmin, jl = (int)(pr & 0xffffffffu);
            const int slot = atomicAdd(&start[x], 1);
            placed[slot] = roff + (int)(m - 1 - (o0 + jl));
        }
        __syncthreads();
        // a warp per column: its slots [end of the column before it in D' order, its end)
        for (int x = span - 1 - wid; x >= 0; x -= T / 32) {
            const int s0 = x == span - 1 ? 0 : start[x + 1];
            const int n = start[x] - s0;
            if (n == 0) continue;
            int *R = placed + s0;
            const int top = n <= 32 ? warp_sort_column<1>(R, n)
                                    : n <= 128 ? warp_sort_column<4>(R, n) : warp_sort_column<16>(R, n);
            __syncwarp();
            const int64_t c = m - 1 - (o0 + qof[x]);
            int *dst = pool + seg_start(c, A + ch.lo + s0) + SEG_HDR;
            for (int t = lane; t < n; t += 32) dst[t] = R[t];
            if (lane == 0) low[c] = top;
        }
        __syncthreads();
    }
}

// per row i of D' (column j = m-1-i of D): the pivot record reset, left[i] =
// m-1-low_D(j) (or -1 for an empty column), beta[left] = the largest row
__global__ void k_dual_rec(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                           PivRec *__restrict__ rec, int32_t *__restrict__ beta, int roff) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = m - 1 - i;
        const int64_t lo = colptr[j], hi = colptr[j + 1];
        const int l = hi > lo ? (int)(m - 1 - rows[hi - 1]) : -1;
        int4 *r = reinterpret_cast<int4 *>(rec + i);
        r[0] = make_int4(-1, 0, l >= 0 ? roff + l : -1, (int)SEG4_NONE);
        r[1] = make_int4(-1, -1, -1, -1);
        if (l >= 0) atomicMax(&beta[l], roff + (int)i);
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

// ----------------------------------------------------- blocks on D or D'
// The blocks of D (a bucket's columns with the rows they hold, all from one
// other bucket) reduce independently: a column only ever adds columns whose
// low lies in its own row bucket, all of them in its own bucket.  So each
// block may be reduced on D or on D' and the low pairs put together.

// D' columns pre-cleared for the D' reduction: the rows (reversed) of every
// column of a block reduced on D.  A simplex's cofaces all lie in one
// bucket, so a D' column is either all D-block or all D'-block.
__global__ void k_split_clear_dual(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                                   const int8_t *__restrict__ bucket, const uint8_t *__restrict__ split,
                                   uint8_t *__restrict__ clear) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        if (split[bucket[j] + 1]) continue;
        for (int64_t k = colptr[j]; k < colptr[j + 1]; k++) clear[m - 1 - rows[k]] = 1;
    }
}

// D's columns pre-cleared for the D reduction: those of the blocks reduced
// on D', and every row D' paired (low_D(j) = i makes column i positive: the
// twist clearing, across blocks).
__global__ void k_split_clear_primal(const int8_t *__restrict__ bucket, const uint8_t *__restrict__ split,
                                     const int32_t *__restrict__ low_dual, int64_t m, uint8_t *__restrict__ clear) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        if (split[bucket[j] + 1]) clear[j] = 1;
        const int i = low_dual[j];
        if (i >= 0) clear[i] = 1;
    }
}

// The D'-block columns take their lows from the D' reduction.
__global__ void k_split_merge(int32_t *__restrict__ low, const int32_t *__restrict__ low_dual,
                              const int8_t *__restrict__ bucket, const uint8_t *__restrict__ split, int64_t m) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        if (split[bucket[j] + 1]) low[j] = low_dual[j];
}

static int grid_of(int sm_count, int64_t n) {
    int64_t g = (n + 255) / 256, cap = (int64_t)sm_count * 16;
    return (int)std::max<int64_t>(1, std::min(g, cap));
}
static int grid_of(Context *ctx, int64_t n) { return grid_of(ctx->sm_count, n); }

struct Grade {
    unsigned long long count[MAXC];
    int tab[MAXC];
    int mixed, bad;
};

// The grading's temporaries: its tallies, each column's bucket (one byte)
// and the per-block choice (MAXC bytes, by column bucket + 1).
static size_t r256(size_t b) { return (b + 255) & ~(size_t)255; }
size_t dual_grade_tmp_bytes(int64_t m) { return r256(sizeof(Grade)) + r256((size_t)(m > 0 ? m : 1)) + 256; }
void dual_split_arrays(void *tmp, int64_t m, const int8_t **bucket, const uint8_t **split) {
    char *base = (char *)tmp + r256(sizeof(Grade));
    *bucket = (const int8_t *)base;
    *split = (const uint8_t *)(base + r256((size_t)(m > 0 ? m : 1)));
}

int dual_grade(cudaStream_t s, int sm_count, const int64_t *colptr, const int32_t *rows, int64_t m, int64_t nnz,
               int mode, void *tmp, int *choice, bool *bad_input, int *launches) {
    *choice = DUAL_CHOICE_D;
    *bad_input = false;
    if (mode == OPH_DUAL_NEVER || m == 0) return OPH_OK;
    Grade *d = (Grade *)tmp;
    int8_t *bucket = (int8_t *)tmp + r256(sizeof(Grade));
    uint8_t *split_d = (uint8_t *)bucket + r256((size_t)m);
    Grade init{};
    for (int b = 0; b < MAXC; b++) init.tab[b] = TAB_NONE;
    OPH_CUDA_TRY(cudaMemcpyAsync(d, &init, sizeof(Grade), cudaMemcpyHostToDevice, s));
    k_dual_buckets<<<grid_of(sm_count, m), 256, 0, s>>>(colptr, m, bucket);
    k_dual_grade<<<grid_of(sm_count, m), 256, 0, s>>>(colptr, rows, m, nnz, bucket, d->count, d->tab, &d->mixed,
                                                       &d->bad);
    if (launches) *launches += 2;
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
    if (mode == OPH_DUAL_ALWAYS ||
        (mode == OPH_DUAL_AUTO && m >= DUAL_MIN_M && lo >= 0 && hi > lo && g.count[lo] * DUAL_RATIO <= g.count[hi])) {
        *choice = DUAL_CHOICE_DUAL;
        return OPH_OK;
    }
    if (mode != OPH_DUAL_BLOCKS && !(mode == OPH_DUAL_AUTO && m >= DUAL_MIN_M)) return OPH_OK;
    // per block (the columns of bucket b with their rows, bucket tab[b]):
    // D' when its row simplices have at most two cofaces on average, as in
    // a triangulated surface, where every column of D' holds at most two
    // rows and so does every sum of them (a union-find walk), while D's
    // columns grow into the boundaries of ever larger regions
    uint8_t split[MAXC] = {};
    bool any_split = false, any_d = false;
    for (int b = 1; b < MAXC; b++) {
        if (!g.count[b] || g.tab[b] == TAB_NONE) continue;
        const int r = g.tab[b] + 1;
        split[b] = r >= 0 && r < MAXC && (unsigned long long)b * g.count[b] <= 2ull * g.count[r];
        if (split[b]) any_split = true;
        else any_d = true;
    }
    if (!any_split) return OPH_OK;
    if (!any_d) {
        *choice = DUAL_CHOICE_DUAL;
        return OPH_OK;
    }
    OPH_CUDA_TRY(cudaMemcpyAsync(split_d, split, MAXC, cudaMemcpyHostToDevice, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    *choice = DUAL_CHOICE_SPLIT;
    return OPH_OK;
}

int dual_choose(Context *ctx, const Work &w, int mode, int *choice, bool *bad_input) {
    *choice = DUAL_CHOICE_D;
    *bad_input = false;
    if (mode == OPH_DUAL_NEVER || w.m == 0) return OPH_OK;
    void *tmp = ctx_alloc(ctx, S_DGRADE, dual_grade_tmp_bytes(w.m));
    if (!tmp) return OPH_ERR_OOM;
    return dual_grade(ctx->stream, ctx->sm_count, w.colptr, w.rows, w.m, w.nnz, mode, tmp, choice, bad_input,
                      &ctx->launches);
}

bool host_prefers_dual(int64_t m, const int64_t *colptr, const int32_t *rows) {
    if (m < DUAL_MIN_M) return false;
    unsigned long long count[MAXC] = {};
    int tab[MAXC];
    for (int b = 0; b < MAXC; b++) tab[b] = TAB_NONE;
    auto bucket = [&](int64_t c) { return (int)std::min<int64_t>(colptr[c + 1] - colptr[c] - 1, 126); };
    for (int64_t j = 0; j < m; j++) {
        const int b = bucket(j);
        if (b + 1 >= MAXC) return false;
        count[b + 1]++;
        if (colptr[j + 1] == colptr[j]) continue;
        const int rb = bucket(rows[colptr[j]]);
        for (int64_t k = colptr[j] + 1; k < colptr[j + 1]; k++)
            if (bucket(rows[k]) != rb) return false;
        if (tab[b + 1] == TAB_NONE) tab[b + 1] = rb;
        else if (tab[b + 1] != rb) return false;
    }
    for (int a = 0; a < MAXC; a++)
        for (int b = a + 1; b < MAXC; b++)
            if (tab[a] != TAB_NONE && tab[a] == tab[b]) return false;
    int lo = -1, hi = -1;
    for (int b = 0; b < MAXC; b++)
        if (count[b]) {
            if (lo < 0) lo = b;
            hi = b;
        }
    return lo >= 0 && hi > lo && count[lo] * DUAL_RATIO <= count[hi];
}

// Layout of the transpose's temporaries: the column offsets of D', the
// counts, the scatter's cursors, the three queues of longer columns, the
// radix sort's scratch, four counters and the scan's tile sums.
struct DualTmp {
    int64_t o_dcolptr, o_cnt, o_cur, o_long, o_mid, o_wide, o_scr, o_ctr, o_tsum, bytes;
    DualTmp(int64_t m, int64_t nnz) {
        auto r256 = [](int64_t b) { return (b + 255) & ~255ll; };
        const int64_t ntiles = (m + SCAN_TILE - 1) / SCAN_TILE;
        o_dcolptr = 0;
        o_cnt = r256(8 * (m + 1));
        o_cur = o_cnt + r256(4 * m);
        o_long = o_cur + r256(8 * m);
        o_mid = o_long + r256(4 * m);
        o_wide = o_mid + r256(4 * m);
        o_scr = o_wide + r256(4 * m);
        o_ctr = o_scr + r256(4 * (nnz > 0 ? nnz : 1));
        o_tsum = o_ctr + 256;
        bytes = o_tsum + 8 * (ntiles + 1);
    }
};

size_t dual_tmp_bytes(int64_t m, int64_t nnz) { return (size_t)DualTmp(m, nnz).bytes; }

int dual_build_store(cudaStream_t s, int sm_count, const int64_t *colptr, const int32_t *rows, int64_t m,
                     int64_t nnz, int *pool, int64_t seg_base, int roff, int64_t *seg, int32_t *low, int8_t *dim,
                     PivRec *rec, int32_t *beta, void *tmp, int *launches) {
    if (m == 0) return OPH_OK;
    const DualTmp L(m, nnz);
    char *buf = (char *)tmp;
    int64_t *dcolptr = (int64_t *)(buf + L.o_dcolptr);
    int *cnt = (int *)(buf + L.o_cnt), *long_list = (int *)(buf + L.o_long), *mid_list = (int *)(buf + L.o_mid);
    unsigned long long *cur = (unsigned long long *)(buf + L.o_cur);
    int *wide_list = (int *)(buf + L.o_wide), *scratch = (int *)(buf + L.o_scr), *ctr = (int *)(buf + L.o_ctr);
    long long *tsum = (long long *)(buf + L.o_tsum);
    const int64_t ntiles = (m + SCAN_TILE - 1) / SCAN_TILE;
    OPH_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * m, s));
    OPH_CUDA_TRY(cudaMemsetAsync(ctr, 0, 256, s));
    OPH_CUDA_TRY(cudaMemsetAsync(beta, 0xff, sizeof(int32_t) * m, s));
    const int gm = grid_of(sm_count, m);
    const int gs = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)sm_count * 2));
    k_dual_count<<<gm, 256, 0, s>>>(colptr, rows, m, cnt);
    k_scan_sums<<<gs, SCAN_THREADS, 0, s>>>(cnt, m, tsum);
    k_scan_tsums<<<1, SCAN_THREADS, 0, s>>>(tsum, ntiles, dcolptr + m);
    k_scan_apply<<<gs, SCAN_THREADS, 0, s>>>(cnt, m, tsum, dcolptr, cur);
    k_dual_scatter<<<gm, 256, 0, s>>>(colptr, rows, m, cur, pool, roff);
    k_dual_finish<<<gm, 256, 0, s>>>(dcolptr, colptr, m, pool, seg, low, dim, mid_list, &ctr[2], seg_base);
    k_dual_finish_warp<<<sm_count * 8, FIN_WARPS * 32, 0, s>>>(dcolptr, pool, low, mid_list, &ctr[2], wide_list,
                                                             &ctr[3], long_list, &ctr[0]);
    k_dual_finish_wide<<<sm_count * 4, FIN_WARPS * 32, 0, s>>>(dcolptr, pool, low, wide_list, &ctr[3]);
    k_dual_sort_long<<<sm_count, LS_THREADS, 0, s>>>(dcolptr, pool, low, long_list, &ctr[0], &ctr[1], scratch);
    k_dual_rec<<<gm, 256, 0, s>>>(colptr, rows, m, rec, beta, roff);
    if (launches) *launches += 10;
    OPH_CUDA_TRY(cudaGetLastError());
    return OPH_OK;
}

// The transpose of a batch's instances (k_dual_inst_a, k_dual_inst_b) into
// wd's store, then the records; *done false when an instance is out of
// bounds (the caller then runs dual_build_store, which rewrites everything).
static int dual_build_store_inst(Context *ctx, const Work &w, Work &wd, bool *done) {
    cudaStream_t s = ctx->stream;
    *done = false;
    const int64_t max_chunks = w.nnz / IT_SPAN + w.inst_count + 1;
    unsigned long long *scratch =
        (unsigned long long *)ctx_alloc(ctx, S_DTEMP, sizeof(unsigned long long) * (w.nnz > 0 ? w.nnz : 1));
    char *meta = scratch ? (char *)ctx_alloc(ctx, S_DCOLPTR, 256 + sizeof(ItChunk) * max_chunks) : nullptr;
    if (!scratch || !meta) return OPH_OK;  // no room for its scratch: the general transpose
    int *fail = (int *)meta, *nchunks = fail + 1;
    ItChunk *chunks = reinterpret_cast<ItChunk *>(meta + 256);
    if (cudaFuncSetAttribute(k_dual_inst_a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ITA_SMEM) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_dual_inst_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ITB_SMEM) !=
            cudaSuccess) {
        cudaGetLastError();
        return OPH_OK;
    }
    OPH_CUDA_TRY(cudaMemsetAsync(meta, 0, 8, s));
    const int ga = std::max(1, std::min(w.inst_count, ctx->sm_count));
    k_dual_inst_a<<<ga, ITA_THREADS, ITA_SMEM, s>>>(w.colptr, w.rows, w.m, w.nnz, w.inst_off, w.inst_count, wd.pool, wd.seg,
                                             wd.low, wd.dim, scratch, chunks, nchunks, fail);
    k_dual_inst_b<<<4 * ctx->sm_count, ITB_THREADS, ITB_SMEM, s>>>(w.m, w.nnz, w.colptr, w.inst_off, wd.pool, wd.low,
                                                             scratch, chunks, nchunks, 0);
    ctx->launches += 2;
    OPH_CUDA_TRY(cudaGetLastError());
    int h_fail = 0;
    OPH_CUDA_TRY(cudaMemcpyAsync(&h_fail, fail, sizeof(int), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    if (h_fail) return OPH_OK;
    OPH_CUDA_TRY(cudaMemsetAsync(wd.beta, 0xff, sizeof(int32_t) * w.m, s));
    k_dual_rec<<<grid_of(ctx, w.m), 256, 0, s>>>(w.colptr, w.rows, w.m, wd.rec, wd.beta, 0);
    ctx->launches++;
    OPH_CUDA_TRY(cudaGetLastError());
    *done = true;
    return OPH_OK;
}

int dual_setup(Context *ctx, const Work &w, Work &wd) {
    wd = w;
    wd.ascending = true;
    wd.checked = true;
    wd.rows = nullptr;
    wd.colptr = nullptr;
    int rc = init_store(ctx, wd);
    if (rc) return rc;
    if (w.m == 0) return OPH_OK;
    if (w.inst_off && w.inst_count > 0 && !getenv("OPH_NO_INST_TRANSPOSE")) {
        bool done = false;
        if ((rc = dual_build_store_inst(ctx, w, wd, &done))) return rc;
        if (done) return OPH_OK;
    }
    void *tmp = ctx_alloc(ctx, S_DSORT, dual_tmp_bytes(w.m, w.nnz));
    if (!tmp) return OPH_ERR_OOM;
    return dual_build_store(ctx->stream, ctx->sm_count, w.colptr, w.rows, w.m, w.nnz, wd.pool, 0, 0, wd.seg, wd.low,
                            wd.dim, wd.rec, wd.beta, tmp, &ctx->launches);
}

void split_clear_dual(cudaStream_t s, int sm_count, const void *grade_tmp, const int64_t *colptr,
                      const int32_t *rows, int64_t m, uint8_t *clear) {
    const int8_t *bucket;
    const uint8_t *split;
    dual_split_arrays(const_cast<void *>(grade_tmp), m, &bucket, &split);
    k_split_clear_dual<<<grid_of(sm_count, m), 256, 0, s>>>(colptr, rows, m, bucket, split, clear);
}

void split_clear_primal(cudaStream_t s, int sm_count, const void *grade_tmp, int64_t m, const int32_t *low_dual,
                        uint8_t *clear) {
    const int8_t *bucket;
    const uint8_t *split;
    dual_split_arrays(const_cast<void *>(grade_tmp), m, &bucket, &split);
    k_split_clear_primal<<<grid_of(sm_count, m), 256, 0, s>>>(bucket, split, low_dual, m, clear);
}

int split_preclear_dual(Context *ctx, const Work &w, uint8_t *clear) {
    OPH_CUDA_TRY(cudaMemsetAsync(clear, 0, w.m, ctx->stream));
    split_clear_dual(ctx->stream, ctx->sm_count, ctx->bufs[S_DGRADE].ptr, w.colptr, w.rows, w.m, clear);
    ctx->launches++;
    OPH_CUDA_TRY(cudaGetLastError());
    return OPH_OK;
}

int split_preclear_primal(Context *ctx, int64_t m, const int32_t *low_dual, uint8_t *clear) {
    OPH_CUDA_TRY(cudaMemsetAsync(clear, 0, m, ctx->stream));
    split_clear_primal(ctx->stream, ctx->sm_count, ctx->bufs[S_DGRADE].ptr, m, low_dual, clear);
    ctx->launches++;
    OPH_CUDA_TRY(cudaGetLastError());
    return OPH_OK;
}

int split_merge(Context *ctx, int32_t *low, const int32_t *low_dual, int64_t m) {
    const int8_t *bucket;
    const uint8_t *split;
    dual_split_arrays(ctx->bufs[S_DGRADE].ptr, m, &bucket, &split);
    k_split_merge<<<grid_of(ctx, m), 256, 0, ctx->stream>>>(low, low_dual, bucket, split, m);
    ctx->launches++;
    OPH_CUDA_TRY(cudaGetLastError());
    return OPH_OK;
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
