// The standard, twist and row reductions as GPU kernels.
//
// These algorithms are sequential by definition (column by column, or row by
// row), and their results — low, and the ess estimate — follow from that
// order.  The reference runs them either on the host (standard.cu:1-57,
// twist.cu:10-87, ph_row.cu:38-121) or as one to five full-grid kernel
// launches per column/row with a single working thread
// (standard_parallel.cu:1-51, twist_parallel.cu:13-96,
// ph_row_parallel.cu:20-89).  Here each is ONE persistent launch:
//   * standard / twist: a single warp walks the columns in the algorithm's
//     order.  A 32-column window is inspected at once (lows, pivot-table
//     hits, repeated lows, twist clears landing inside the window) so that
//     columns needing no addition are retired 32 at a time; a column that
//     needs additions is reduced by the whole warp with the column kept in
//     shared memory across its chain of additions.
//   * row: one CTA walks the rows from the bottom; a warp finds the next row
//     with two or more columns on it (per-row buckets), and the CTA's 32
//     warps add the row's pivot into all of that row's other columns in
//     parallel (mark_neighbours / left_to_right_neighbours,
//     ph_row_parallel.cu:3-18).
// Column additions use the same group merge as pms; columns too wide for the
// shared buffers continue in pool-allocated global buffers.
#include <algorithm>

#include "oph_host.h"

namespace oph {

struct SeqArgs {
    int64_t m;
    int32_t *low;
    int32_t *arglow;   // standard/twist pivot table; row: pivots[] (first column ever holding each low)
    const int8_t *dim;
    int64_t *seg;
    int *pool;
    DevStatus *st;
    int32_t *ess;      // row (reference CPU form): the running essential estimate
    int32_t *bhead;    // row: bucket heads (columns whose low is the row)
    int32_t *bnext;    // row: bucket links
    int32_t *bcnt;     // row: bucket sizes
    int32_t *blist;    // row: the current row's bucket, gathered
    int start_dim;
    long long start_pos;
    int max_dim;
    int twist;         // standard (0) or twist (1)
    int row_quirk;     // row: keep the reference CPU form's running ess estimate
    long long *it_ns;  // standard / twist with trackers: end of every iteration (globaltimer), or nullptr
    long long it_base; //   the iteration this launch starts at (1, or where an interrupted walk stopped)
    // row with trackers: a log of the rows that had additions, each as
    // {row, pivot, neighbours k, end time (ns, two ints)} then k pairs
    // {column, its new low}; ev_cap ints, the length in ev[-2..-1] (int64),
    // nullptr without trackers
    int *ev;
    long long ev_cap;
};

__device__ __forceinline__ long long global_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Chain of additions into column j by one warp, `next(low)` giving the column
// to add next (or -1 to stop).  The column stays in shared memory (sA/sB/sC,
// `cap` ints each) while it fits and moves to pool-allocated buffers when it
// does not.  j is written back once.  Returns the new low of j, or -2 when
// the pool is exhausted (j unchanged).
template <class Tile, class Next>
__device__ int chain(const Tile &tile, const SeqArgs &a, int j, int *sA, int *sB, int *sC, int cap, Next next,
                     long long &adds, long long &slots) {
    const int lane = tile.thread_rank();
    int lj = a.low[j];
    int p = next(lj);
    if (p < 0) return lj;
    const long long sj = a.seg[j];
    int n = a.pool[sj];
    const int capj = a.pool[sj + 1];
    int *A, *X = nullptr, *Y = nullptr;
    int bcap;
    bool smem_mode = n <= cap;
    if (smem_mode) {
        group_copy<32>(tile, sA, a.pool + sj + SEG_HDR, n);
        A = sA;
        bcap = cap;
    } else {
        bcap = round4(max(2 * n, 1024));
        long long off = 0;
        if (lane == 0) off = pool_alloc(a.st, 2ll * bcap);
        off = tile.shfl(off, 0);
        if (off < 0) return -2;
        X = a.pool + off; Y = X + bcap;
        group_copy<32>(tile, X, a.pool + sj + SEG_HDR, n);
        A = X;
    }
    while (p >= 0) {
        const long long sp = a.seg[p];
        const int np = a.pool[sp];
        if (n + np > bcap) {
            int ncap = round4(max(2 * (n + np), 1024));
            long long off = 0;
            if (lane == 0) off = pool_alloc(a.st, 2ll * ncap);
            off = tile.shfl(off, 0);
            if (off < 0) return -2;
            int *NX = a.pool + off;
            group_copy<32>(tile, NX, A, n);
            A = NX; X = NX; Y = NX + ncap; bcap = ncap; smem_mode = false;
        }
        const int *P = a.pool + sp + SEG_HDR;
        int *out;
        if (smem_mode) {
            group_copy<32>(tile, sC, P, np);
            P = sC;
            out = (A == sA) ? sB : sA;
        } else {
            out = (A == X) ? Y : X;
        }
        const int nn = merge_xor<32>(tile, A, n, P, np, out);
        slots += n + np + nn;
        adds++;
        n = nn;
        A = out;
        lj = n ? A[n - 1] : -1;
        p = next(lj);
    }
    long long dst = sj;
    int dcap = capj;
    if (n > capj) {
        dcap = round4(max(2 * n, 16));
        long long off = 0;
        if (lane == 0) off = pool_alloc(a.st, SEG_HDR + dcap);
        off = tile.shfl(off, 0);
        if (off < 0) return -2;
        dst = off;
    }
    group_copy<32>(tile, a.pool + dst + SEG_HDR, A, n);
    if (lane == 0) {
        a.pool[dst] = n;
        a.pool[dst + 1] = dcap;
        a.seg[j] = dst;
        a.low[j] = lj;
    }
    tile.sync();
    return lj;
}

constexpr int SEQ_CAP = 4096;

// standard (reduce_col_host, kernels_host.cu:62-75, for j = 0..m-1) and
// twist (the same per dimension from the top down, dimensions >= 1 only,
// then low[low_j] := -1; twist.cu:10-87).
__global__ void __launch_bounds__(32) k_seq_walk(SeqArgs a) {
    extern __shared__ int smem[];
    int *sA = smem, *sB = smem + SEQ_CAP, *sC = smem + 2 * SEQ_CAP;
    auto tile = cg::tiled_partition<32>(cg::this_thread_block());
    const int lane = tile.thread_rank();
    long long adds = 0, slots = 0;
    // iterations (the reference's, one per visited column) and their end
    // times, when trackers are kept: columns retired together in a window
    // share its time evenly
    long long it = a.it_base;
    long long tprev = global_ns();
    if (a.it_ns && it == 1 && lane == 0) a.it_ns[0] = tprev;
    const int d_end = a.twist ? 1 : a.start_dim;
    for (int d = a.start_dim; d >= d_end; d--) {
        long long j0 = (d == a.start_dim) ? a.start_pos : 0;
        while (j0 < a.m) {
            const long long j = j0 + lane;
            const bool in = j < a.m && (!a.twist || a.dim[j] == d);
            const int lj = in ? a.low[j] : -1;
            const int pj = lj >= 0 ? a.arglow[lj] : -1;
            bool dup = false, hit = false;
            for (int q = 0; q < 31; q++) {
                int lq = tile.shfl(lj, q);
                if (q < lane && lq >= 0) {
                    if (lq == lj) dup = true;
                    if (a.twist && lq == (int)j) hit = true;
                }
            }
            const bool stop = (in && ((lj >= 0 && pj != -1) || dup)) || (j < a.m && hit);
            const unsigned sb = tile.ballot(stop);
            const int fs = sb ? __ffs(sb) - 1 : 32;
            if (lane < fs && in && lj >= 0) {
                a.arglow[lj] = (int)j;
                if (a.twist) a.low[lj] = -1;
            }
            {
                const unsigned retired = tile.ballot(in) & (fs == 32 ? 0xffffffffu : (1u << fs) - 1u);
                const int cnt = __popc(retired);
                if (a.it_ns && lane == 0 && cnt) {
                    const long long t = global_ns();
                    for (int q = 0; q < cnt; q++) a.it_ns[it + q] = tprev + (t - tprev) * (q + 1) / cnt;
                    tprev = t;
                }
                it += cnt;
            }
            tile.sync();
            if (fs == 32) { j0 += 32; continue; }
            const long long jj = j0 + fs;
            const bool jj_hit = tile.shfl(hit, fs);
            if (jj_hit) { j0 = jj; continue; }  // its low was just cleared: look at it again
            auto next = [&](int l) { return l >= 0 ? a.arglow[l] : -1; };
            const int nl = chain(tile, a, (int)jj, sA, sB, sC, SEQ_CAP, next, adds, slots);
            if (nl == -2) {
                if (lane == 0) { a.st->resume_dim = d; a.st->resume_pos = jj; a.st->resume_iter = it; }
                goto out;
            }
            if (nl >= 0 && lane == 0) {
                a.arglow[nl] = (int)jj;
                if (a.twist) a.low[nl] = -1;
            }
            if (a.it_ns && lane == 0) a.it_ns[it] = tprev = global_ns();
            it++;
            tile.sync();
            j0 = jj + 1;
        }
    }
    if (lane == 0) a.st->resume_pos = -1;
out:
    if (lane == 0) {
        a.st->additions += adds;
        a.st->slots += slots;
    }
}

// Row buckets: every column with a low joins the bucket of that row;
// pivots[r] = the first column holding low r (ph_row.cu:56-59).
__global__ void k_row_buckets(SeqArgs a) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < a.m; j += (int64_t)gridDim.x * blockDim.x) {
        int lj = a.low[j];
        if (lj >= 0) {
            a.bnext[j] = atomicExch(&a.bhead[lj], (int)j);
            atomicAdd(&a.bcnt[lj], 1);
            atomicMin(&a.arglow[lj], (int)j);
        }
    }
}

constexpr int ROW_THREADS = 1024;
constexpr int ROW_CAP = 512;

// The row algorithm (ph_row.cu:38-121 / ph_row_parallel.cu:20-89): for rows
// i = m-1 .. 0, the first column with low i is added into every other column
// with low i; those move to the buckets of their new lows.  With row_quirk
// the running ess estimate of the reference CPU form is kept: before each
// addition the row and the pivot pair are marked non-essential, and after it
// a column that is now the first ever to hold its new low is marked
// non-essential together with that low (ph_row.cu:2-31).
__global__ void __launch_bounds__(ROW_THREADS) k_row_walk(SeqArgs a) {
    extern __shared__ int smem[];
    __shared__ long long s_row;
    __shared__ int s_n, s_piv;
    const int wid = threadIdx.x >> 5;
    auto tile = cg::tiled_partition<32>(cg::this_thread_block());
    const int lane = tile.thread_rank();
    int *sA = smem + (size_t)wid * 3 * ROW_CAP, *sB = sA + ROW_CAP, *sC = sB + ROW_CAP;
    long long adds = 0, slots = 0;
    long long i = a.start_pos;
    __shared__ int s_fail;
    if (threadIdx.x == 0) s_fail = 0;
    if (a.ev && threadIdx.x == 0) {
        long long *t0 = reinterpret_cast<long long *>(a.ev) - 2;
        if (*t0 == 0) *t0 = global_ns();  // the first launch of the walk
    }
    while (i >= 0) {
        if (wid == 0) {
            long long r = i, found = -1;
            while (r >= 0) {
                long long rr = r - lane;
                int c = rr >= 0 ? a.bcnt[rr] : 0;
                unsigned b = tile.ballot(c >= 2);
                if (b) { found = r - (__ffs(b) - 1); break; }
                r -= 32;
            }
            if (lane == 0) {
                s_row = found;
                if (found >= 0) {
                    int n = 0, piv = 0x7fffffff;
                    for (int c = a.bhead[found]; c != -1; c = a.bnext[c]) {
                        a.blist[n++] = c;
                        piv = min(piv, c);
                    }
                    s_n = n;
                    s_piv = piv;
                    a.bhead[found] = -1;
                    a.bcnt[found] = 0;
                    if (a.row_quirk) { a.ess[found] = 0; a.ess[piv] = 0; }
                }
            }
        }
        __syncthreads();
        i = s_row;
        if (i < 0) break;
        const int n = s_n, piv = s_piv;
        for (int k = wid; k < n; k += ROW_THREADS / 32) {
            const int j = a.blist[k];
            if (j == piv) continue;
            bool once = true;
            auto next = [&](int) { int p = once ? piv : -1; once = false; return p; };
            const int nl = chain(tile, a, j, sA, sB, sC, ROW_CAP, next, adds, slots);
            if (nl == -2) {
                if (lane == 0) s_fail = 1;
                continue;
            }
            if (nl >= 0 && lane == 0) {
                a.bnext[j] = atomicExch(&a.bhead[nl], j);
                atomicAdd(&a.bcnt[nl], 1);
                atomicMin(&a.arglow[nl], j);
            }
        }
        __syncthreads();
        if (s_fail) break;
        if (a.ev && threadIdx.x == 0) {
            // the row's additions, for the host's tracker replay (a row that
            // failed is walked again after the regrow, and logged then)
            long long *len = reinterpret_cast<long long *>(a.ev) - 1;
            const long long at = *len, need = 5 + 2ll * (n - 1);
            if (at >= 0 && at + need <= a.ev_cap) {
                int *e = a.ev + at;
                const long long t = global_ns();
                e[0] = (int)i;
                e[1] = piv;
                e[2] = n - 1;
                e[3] = (int)(t & 0xffffffffll);
                e[4] = (int)(t >> 32);
                int q = 5;
                for (int k = 0; k < n; k++) {
                    const int j = a.blist[k];
                    if (j == piv) continue;
                    e[q++] = j;
                    e[q++] = a.low[j];
                }
                *len = at + need;
            } else {
                *len = -1;  // out of room: the host keeps the final entry only
            }
        }
        if (a.row_quirk) {
            for (int k = threadIdx.x; k < n; k += ROW_THREADS) {
                const int j = a.blist[k];
                if (j == piv) continue;
                const int nl = a.low[j];
                if (nl >= 0 && a.arglow[nl] == j) { a.ess[j] = 0; a.ess[nl] = 0; }
            }
        }
        __syncthreads();
        i--;
    }
    if (threadIdx.x == 0) {
        // a failed addition leaves its column unchanged but the row's bucket
        // was consumed; report the row so the host restarts the whole walk
        a.st->resume_pos = s_fail ? i : -1;
    }
    if (lane == 0 && adds) {
        atomicAdd(&a.st->additions, (unsigned long long)adds);
        atomicAdd(&a.st->slots, (unsigned long long)slots);
    }
}

// out[0] = largest dimension, out[1] = columns of dimension >= 1.
__global__ void k_dim_stats(const int8_t *dim, int64_t m, int *out) {
    int mx = -1, cnt = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        mx = max(mx, (int)dim[j]);
        cnt += dim[j] >= 1;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out[0], mx);
        atomicAdd(&out[1], cnt);
    }
}

int run_sequential(Context *ctx, Work &w, int algo, int32_t *d_ess, oph_info *info) {
    cudaStream_t s = ctx->stream;
    const int64_t m = w.m;
    SeqArgs a{};
    a.m = m; a.low = w.low; a.dim = w.dim; a.seg = w.seg; a.pool = w.pool; a.st = w.st;
    a.arglow = w.first;  // reuse: int32[m]
    const bool row = algo == OPH_ALGO_PH_ROW || algo == OPH_ALGO_PH_ROW_PARALLEL;
    const int grid_m = (int)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, (int64_t)ctx->sm_count * 16));
    cudaEventRecord(ctx->ev[0], s);
    int regrows = 0;
    long long iters = m + 1;
    if (!row) {
        a.twist = (algo == OPH_ALGO_TWIST || algo == OPH_ALGO_TWIST_PARALLEL);
        int *d_stats = (int *)w.agg;
        int hstats[2] = {-1, 0};
        OPH_CUDA_TRY(cudaMemcpyAsync(d_stats, hstats, sizeof(hstats), cudaMemcpyHostToDevice, s));
        k_dim_stats<<<grid_m, 256, 0, s>>>(w.dim, m, d_stats);
        ctx->launches++;
        OPH_CUDA_TRY(cudaMemcpyAsync(hstats, d_stats, sizeof(hstats), cudaMemcpyDeviceToHost, s));
        OPH_CUDA_TRY(cudaMemsetAsync(a.arglow, 0xff, sizeof(int32_t) * m, s));
        OPH_CUDA_TRY(cudaStreamSynchronize(s));
        const int maxdim = hstats[0];
        a.max_dim = maxdim;
        a.start_dim = a.twist ? maxdim : 0;
        a.start_pos = 0;
        if (a.twist && maxdim < 1) a.start_dim = 0;  // nothing to reduce: the loop below runs no dimension
        // the reference counts one iteration per column visited
        // (twist.cu:36-86 visits the columns of dimension >= 1)
        if (a.twist) iters = 1 + (long long)hstats[1];
        SeqTracking *tk = ctx->seq_track;
        a.it_base = 1;
        if (tk) {
            // the state the host replays from, and a stamp per iteration
            tk->iters = iters;
            tk->low0.resize(m);
            tk->dim.resize(m);
            a.it_ns = (long long *)ctx_alloc(ctx, S_SEQNS, sizeof(long long) * (size_t)(iters + 1));
            if (!a.it_ns) return OPH_ERR_OOM;
            OPH_CUDA_TRY(cudaMemsetAsync(a.it_ns, 0, sizeof(long long) * (size_t)(iters + 1), s));
            OPH_CUDA_TRY(cudaMemcpyAsync(tk->low0.data(), w.low, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
            OPH_CUDA_TRY(cudaMemcpyAsync(tk->dim.data(), w.dim, (size_t)m, cudaMemcpyDeviceToHost, s));
            OPH_CUDA_TRY(cudaStreamSynchronize(s));
        }
        static bool attr = false;
        const size_t smem = 3 * SEQ_CAP * sizeof(int);
        if (!attr) {
            OPH_CUDA_TRY(cudaFuncSetAttribute(k_seq_walk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            attr = true;
        }
        if (!(a.twist && maxdim < 1)) {
            for (;;) {
                k_seq_walk<<<1, 32, smem, s>>>(a);
                ctx->launches++;
                OPH_CUDA_TRY(cudaGetLastError());
                OPH_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, w.st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
                OPH_CUDA_TRY(cudaStreamSynchronize(s));
                if (ctx->h_status->resume_pos < 0) break;
                int g = grow_pool(ctx, w);
                if (g != OPH_OK) return g;
                a.pool = w.pool;
                a.start_dim = ctx->h_status->resume_dim;
                a.start_pos = ctx->h_status->resume_pos;
                a.it_base = ctx->h_status->resume_iter;
                regrows++;
            }
        }
        if (tk) {
            tk->ns.resize(iters);
            if (a.twist && maxdim < 1) {
                std::fill(tk->ns.begin(), tk->ns.end(), 0ll);
            } else {
                OPH_CUDA_TRY(cudaMemcpyAsync(tk->ns.data(), a.it_ns, sizeof(long long) * iters, cudaMemcpyDeviceToHost, s));
                OPH_CUDA_TRY(cudaStreamSynchronize(s));
            }
        }
    } else {
        a.bhead = (int32_t *)ctx_alloc(ctx, S_TMP, sizeof(int32_t) * (3 * m + 1));
        if (!a.bhead) return OPH_ERR_OOM;
        a.bnext = a.bhead + m; a.bcnt = a.bnext + m;
        a.blist = w.worklist;
        a.ess = d_ess;
        a.row_quirk = (algo == OPH_ALGO_PH_ROW) && d_ess != nullptr;
        SeqTracking *tk = ctx->seq_track;
        long long *ev_base = nullptr;
        if (tk) {
            // the initial lows and a log of the walk's additions for the
            // host's replay: {start ns, length} then the records
            tk->iters = iters;
            tk->low0.resize(m);
            OPH_CUDA_TRY(cudaMemcpyAsync(tk->low0.data(), w.low, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
            a.ev_cap = 8 * (long long)m + (1 << 20);
            ev_base = (long long *)ctx_alloc(ctx, S_SEQNS, 16 + sizeof(int) * (size_t)a.ev_cap);
            if (!ev_base) return OPH_ERR_OOM;
            OPH_CUDA_TRY(cudaMemsetAsync(ev_base, 0, 16, s));
            a.ev = reinterpret_cast<int *>(ev_base + 2);
        }
        static bool attr = false;
        const size_t smem = (size_t)(ROW_THREADS / 32) * 3 * ROW_CAP * sizeof(int);
        if (!attr) {
            OPH_CUDA_TRY(cudaFuncSetAttribute(k_row_walk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            attr = true;
        }
        for (;;) {
            OPH_CUDA_TRY(cudaMemsetAsync(a.bhead, 0xff, sizeof(int32_t) * m, s));
            OPH_CUDA_TRY(cudaMemsetAsync(a.bcnt, 0, sizeof(int32_t) * m, s));
            OPH_CUDA_TRY(cudaMemsetAsync(a.arglow, 0x7f, sizeof(int32_t) * m, s));
            k_row_buckets<<<grid_m, 256, 0, s>>>(a);
            a.start_pos = m - 1;
            k_row_walk<<<1, ROW_THREADS, smem, s>>>(a);
            ctx->launches += 2;
            OPH_CUDA_TRY(cudaGetLastError());
            OPH_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, w.st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
            OPH_CUDA_TRY(cudaStreamSynchronize(s));
            if (ctx->h_status->resume_pos < 0) break;
            // rows are consumed as they are walked, so an interrupted walk
            // restarts from the (consistent) column state with rebuilt buckets
            int g = grow_pool(ctx, w);
            if (g != OPH_OK) return g;
            a.pool = w.pool;
            regrows++;
        }
        if (tk) {
            long long hdr[2] = {0, 0};
            OPH_CUDA_TRY(cudaMemcpyAsync(hdr, ev_base, 16, cudaMemcpyDeviceToHost, s));
            OPH_CUDA_TRY(cudaStreamSynchronize(s));
            tk->ev_t0 = hdr[0];
            tk->rows_ok = hdr[1] >= 0;
            tk->ev.resize(hdr[1] > 0 ? (size_t)hdr[1] : 0);
            if (!tk->ev.empty()) {
                OPH_CUDA_TRY(cudaMemcpyAsync(tk->ev.data(), a.ev, sizeof(int) * tk->ev.size(), cudaMemcpyDeviceToHost, s));
                OPH_CUDA_TRY(cudaStreamSynchronize(s));
            }
        }
    }
    cudaEventRecord(ctx->ev[1], s);
    OPH_CUDA_TRY(cudaEventSynchronize(ctx->ev[1]));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    DevStatus hs = *ctx->h_status;
    if (info) {
        info->sweeps = 0;
        info->num_iters = (int32_t)iters;
        info->additions = (int64_t)hs.additions;
        info->slots_moved = (int64_t)hs.slots;
        info->pool_bytes = (int64_t)hs.pool_used * 4;
        info->regrows = regrows;
        info->device_ms = ms;
    }
    return OPH_OK;
}

}  // namespace oph
