// Reduction server with continuous batching.
//
// Requests (boundary matrices) are queued by oph_server_submit and reduced by
// one worker thread that owns a CUDA stream and a fixed device arena (the
// HBM budget).  All active requests live in ONE block-diagonal column space:
// request r holds columns [c0, c0 + m) and its rows are shifted by c0, so one
// pms sweep (pms.cu: Phase I + the Phase II tiers) advances every active
// request at once.  Between sweeps the worker
//   * retires every request whose last Phase I found no repeated low (its
//     lows are final): its lows and ess are copied out and its columns and
//     pool region are freed;
//   * admits queued requests, first come first served, while a column range
//     and a pool region fit in the arena; a request whose column range starts
//     before another's is still independent (rows of distinct requests are
//     disjoint and earlier ranges only hold smaller rows);
//   * regrows the pool region of any request whose column store overflowed
//     (copy, then rebase its segments and its pivot records).
// A request therefore joins the running batch at the next sweep boundary and
// leaves it as soon as it converges.
//
// Each request is reduced on the matrix plain pms would choose for it alone
// (the automatic rule of dual.cu, decided at submission): a Rips-like
// request goes through its anti-transpose, built at admission straight into
// its own column range and pool region, with its dimension buckets in
// ascending order (per instance: iasc / ibucket / iopen); a request split
// by dimension block (a lower-star image) as two instances side by side,
// its D' part first and its D part from the D' part's second sweep on, the
// lows merged when both have converged; the others on D.
// Phase I visits only the unresolved columns: a list in column order,
// compacted by every sweep, into which each admitted request's column range
// is merged (k_srv_merge).  A retired request's columns leave the list in
// the next sweep, and only then is its column range handed out again.  The
// bitmap tiers' chains stop after SERVE_CHAIN_CAP additions a sweep, so no
// sweep of every request waits on one long chain.  The reduction of a
// request is the same whether it runs alone or in the mix: block-diagonal
// columns never add into each other, and the lows of a reduced matrix are
// unique.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "pms.cuh"

namespace oph {

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over [0, cap) with coalescing.
struct RangeAlloc {
    std::map<int64_t, int64_t> free;  // start -> length
    int64_t cap = 0, used = 0;
    void init(int64_t c) {
        cap = c;
        used = 0;
        free.clear();
        if (c > 0) free[0] = c;
    }
    int64_t alloc(int64_t len, int64_t align) {
        for (auto it = free.begin(); it != free.end(); ++it) {
            const int64_t s = (it->first + align - 1) / align * align;
            const int64_t e = it->first + it->second;
            if (s + len <= e) {
                const int64_t fs = it->first;
                free.erase(it);
                if (s > fs) free[fs] = s - fs;
                if (s + len < e) free[s + len] = e - (s + len);
                used += len;
                return s;
            }
        }
        return -1;
    }
    void release(int64_t s, int64_t len) {
        used -= len;
        auto it = free.emplace(s, len).first;
        auto nx = std::next(it);
        if (nx != free.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free.erase(nx);
        }
        if (it != free.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free.erase(it);
            }
        }
    }
};

}  // namespace

struct Request {
    int64_t ticket = 0, m = 0, nnz = 0;
    // the server's own device copy of the CSC (colptr then rows), made at
    // submission and read in place at admission
    void *d_buf = nullptr;
    std::vector<int32_t> low, ess;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int sweeps = 0, status = OPH_OK, slot = -1;
    bool done = false;
    bool dual = false;  // reduced through its anti-transpose
    // some dimension blocks on D', the others on D: the request itself is
    // the D' part (dual set); after its first sweep an internal request for
    // the D part (user set) joins the head of the queue, its columns of the
    // D'-reduced blocks and of the rows the D' part has paired by then
    // cleared.  The grading (buckets, per-block choice), the D' part's lows
    // (mapped to D, then a scratch ess) and the D part's lows stay on the
    // device until both parts have converged.
    bool split = false;
    Request *user = nullptr;      // a D part: the request it belongs to
    Request *part = nullptr;      // a split request: its D part, once made
    int parts_left = 0;           // a split request: parts not yet converged
    bool part_done = false;       // a split request: its D' part converged
    int64_t sweep0 = 0;           // the server's sweep count at admission
    void *d_grade = nullptr;
    int32_t *d_mapped = nullptr;  // 3m ints: D' part's lows (mapped), ess scratch, D part's lows
    int64_t c0 = -1, reg = -1, reg_ints = 0;
    int64_t ring_off = -1;  // low then ess in the pinned result ring (ints), or -1
    bool listed = false;    // in the Phase I list: its sweeps have begun
};

// ------------------------------------------------------------------ kernels
// The structural checks of oph_server_submit on a CSC in device memory:
// columns of at most MAXC - 1 rows, rows strictly ascending and < m.
__global__ void k_srv_check(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                            int64_t nnz, int *bad) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t lo = colptr[j], hi = colptr[j + 1];
        // the bounds first: no row is read outside [0, nnz)
        bool ok = lo >= 0 && hi >= lo && hi <= nnz && hi - lo <= MAXC - 1;
        for (int64_t k = lo; ok && k < hi; k++) ok = rows[k] >= 0 && rows[k] < m && (k == lo || rows[k] > rows[k - 1]);
        if (!ok) atomicExch(bad, 1);
    }
}

// Admission: columns [c0, c0+m) of request slot `b`, input staged at
// colptr/rows (local), segments packed from pool offset `base`.
__global__ void k_srv_init(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                           int64_t c0, int b, int64_t base, PmsArgs a) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = c0 + jj;
        const int64_t lo = colptr[jj], hi = colptr[jj + 1];
        const int64_t s = base + 8 * jj + 4 * ((lo + 3) >> 2);
        const int64_t e = base + 8 * (jj + 1) + 4 * ((hi + 3) >> 2);
        const int n = (int)(hi - lo);
        a.seg[j] = s;
        a.pool[s] = n;
        a.pool[s + 1] = (int)(e - s - SEG_HDR);
        for (int64_t k = lo; k < hi; k++) a.pool[s + SEG_HDR + (k - lo)] = rows[k] + (int32_t)c0;
        a.low[j] = n > 0 ? rows[hi - 1] + (int32_t)c0 : -1;
        const_cast<int8_t *>(a.dim)[j] = (int8_t)(n - 1 > 126 ? 126 : n - 1);
        a.inst[j] = b;
        a.classes[j] = 0;
        a.clear[j] = 0;
        a.first[j] = FIRST_NONE;
        const_cast<int32_t *>(a.beta)[j] = -1;
        int4 *r = reinterpret_cast<int4 *>(a.rec + j);
        r[0] = make_int4(-1, 0, FIRST_NONE, (int)SEG4_NONE);
        r[1] = make_int4(-1, -1, -1, -1);
    }
}

// Admission of a request reduced through its anti-transpose: the per-column
// state that dual_build_store does not write.
__global__ void k_srv_init_cols(int64_t m, int64_t c0, int b, PmsArgs a) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = c0 + jj;
        a.inst[j] = b;
        a.classes[j] = 0;
        a.clear[j] = 0;
        a.first[j] = FIRST_NONE;
    }
}

// The Phase I list with the column ranges admitted since the last sweep merged in: the
// sorted list `in` (*in_count columns) and the ranges [r0[q], r0[q] + len of
// q) (ascending, disjoint from every listed column; pre[q] = columns of the
// ranges before q, pre[K] = all of them) into the sorted list `out`.
__global__ void k_srv_merge(const int32_t *__restrict__ in, const int *in_count, const int64_t *__restrict__ r0,
                            const int64_t *__restrict__ pre, int K, int32_t *__restrict__ out, int *out_count) {
    const int64_t n_in = *in_count, total = pre[K], N = n_in + total;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < N; x += (int64_t)gridDim.x * blockDim.x) {
        if (x < n_in) {
            const int v = in[x];
            int lo = 0, hi = K;  // ranges starting below v
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (r0[mid] < v) lo = mid + 1; else hi = mid;
            }
            out[x + pre[lo]] = v;
        } else {
            const int64_t y = x - n_in;
            int lo = 0, hi = K - 1;  // the range holding admitted column y
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (pre[mid] <= y) lo = mid; else hi = mid - 1;
            }
            const int64_t c = r0[lo] + (y - pre[lo]);
            int64_t a = 0, z = n_in;  // listed columns below the range
            while (a < z) {
                const int64_t mid = (a + z) >> 1;
                if (in[mid] < r0[lo]) a = mid + 1; else z = mid;
            }
            out[a + y] = (int32_t)c;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *out_count = (int)N;
}

__global__ void k_srv_left(const int64_t *__restrict__ colptr, const int32_t *__restrict__ rows, int64_t m,
                           int64_t c0, PmsArgs a) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x)
        for (int64_t k = colptr[jj]; k < colptr[jj + 1]; k++) atomicMin(&a.rec[rows[k] + c0].left, (int)(c0 + jj));
}

__global__ void k_srv_beta(int64_t m, int64_t c0, PmsArgs a) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = c0 + jj;
        const int l = a.rec[i].left;
        if (l == FIRST_NONE) a.rec[i].left = -1;
        else atomicMax(const_cast<int32_t *>(a.beta) + l, (int)i);
    }
}

// Retirement: local lows and ess of columns [c0, c0+m) into out (2m ints).
__global__ void k_srv_out1(int64_t m, int64_t c0, PmsArgs a, int32_t *out) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int l = a.low[c0 + jj];
        out[jj] = l >= 0 ? (int32_t)(l - c0) : -1;
        out[m + jj] = l >= 0 ? 0 : 1;
    }
}
__global__ void k_srv_out2(int64_t m, int64_t c0, PmsArgs a, int32_t *out) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int l = a.low[c0 + jj];
        if (l >= 0) out[m + (l - c0)] = 0;
    }
}
// The same for a request reduced through its anti-transpose: every pair
// (column c, low r) of D' (local indices) is the pair (column m-1-r, low
// m-1-c) of D; both ends of a pair are not essential.
__global__ void k_srv_out_dual1(int64_t m, int32_t *out) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        out[jj] = -1;
        out[m + jj] = 1;
    }
}
__global__ void k_srv_out_dual2(int64_t m, int64_t c0, PmsArgs a, int32_t *out) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < m; c += (int64_t)gridDim.x * blockDim.x) {
        const int l = a.low[c0 + c];
        if (l < 0) continue;
        const int64_t r = l - c0;
        out[m - 1 - r] = (int32_t)(m - 1 - c);
        out[m + (m - 1 - r)] = 0;
        out[m + (m - 1 - c)] = 0;
    }
}
// A split request's D part converged: its local lows, kept until the D'
// part has converged too.
__global__ void k_srv_save_local(int64_t m, int64_t c0, PmsArgs a, int32_t *__restrict__ out) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int l = a.low[c0 + jj];
        out[jj] = l >= 0 ? (int32_t)(l - c0) : -1;
    }
}
// Both parts converged: the columns of the D'-reduced blocks take the lows
// the D' part found (mapped), the others the D part's; then the ess pass
// runs over the merged lows.
__global__ void k_srv_out_split1(int64_t m, const int8_t *__restrict__ bucket, const uint8_t *__restrict__ split,
                                 const int32_t *__restrict__ mapped, const int32_t *__restrict__ lowd, int32_t *out) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = split[bucket[jj] + 1] ? mapped[jj] : lowd[jj];
        out[jj] = v;
        out[m + jj] = v >= 0 ? 0 : 1;
    }
}
// The D part's clears when its D' part is still being reduced: the columns
// of the D'-reduced blocks, and the D column m-1-c of every D' column c the
// D' part has made a pivot so far (its pair makes that column positive; a
// pivot's class is final, so a concurrent sweep can only add to the set).
__global__ void k_srv_split_clear_live(int64_t m, int64_t c0_dual, int64_t c0, PmsArgs a,
                                       const int8_t *__restrict__ bucket, const uint8_t *__restrict__ split) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        if (split[bucket[jj] + 1]) a.clear[c0 + jj] = 1;
        if (a.classes[c0_dual + jj] == -1) a.clear[c0 + (m - 1 - jj)] = 1;
    }
}
__global__ void k_srv_out_split2(int64_t m, int32_t *out) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int v = out[jj];
        if (v >= 0) out[m + v] = 0;
    }
}
// ... then the columns become inert (no low, cleared, no instance).
__global__ void k_srv_inert(int64_t m, int64_t c0, PmsArgs a) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = c0 + jj;
        a.low[j] = -1;
        a.classes[j] = 1;
        a.clear[j] = 0;
        a.inst[j] = -1;
        a.first[j] = FIRST_NONE;
        int4 *r = reinterpret_cast<int4 *>(a.rec + j);
        r[0] = make_int4(-1, 0, -1, (int)SEG4_NONE);
        r[1] = make_int4(-1, -1, -1, -1);
    }
}

// Regrow: shift the segments of columns [c0, c0+m) and the segment fields of
// their rows' pivot records by `delta` ints.
__global__ void k_srv_rebase(int64_t m, int64_t c0, int64_t delta, PmsArgs a) {
    for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < m; jj += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = c0 + jj;
        a.seg[j] += delta;
        if (a.rec[j].col >= 0) a.rec[j].seg4 = (unsigned)((((long long)a.rec[j].seg4) * 4 + delta) >> 2);
    }
}

__global__ void k_srv_set_region(unsigned long long *ipool, int *ireps, int *iover, int b, unsigned long long used,
                                 unsigned long long end) {
    ipool[2 * b] = used;
    ipool[2 * b + 1] = end;
    ireps[b] = 0;
    iover[b] = 0;
}

__global__ void k_srv_sweep_reset(DevStatus *st) {
    st->converged = 0;
    st->overflow = 0;
}

// ------------------------------------------------------------------ server
// The bitmap tiers' additions per column and sweep: a long chain goes on in
// the next sweep instead of holding every active request's sweep.
constexpr int SERVE_CHAIN_CAP = 128;

struct Server {
    Context *ctx = nullptr;  // owns the stream and the device buffers
    cudaStream_t sub_stream = nullptr;  // submissions: copy, check, grade
    cudaStream_t adm_stream = nullptr;  // admissions overlapping a sweep
    cudaEvent_t adm_done = nullptr;     //   and their completion
    int64_t budget = 0, mcap = 0, pool_ints = 0;
    int max_slots = 0;
    PmsArgs a{};
    SweepGrids g{};
    int *h_ireps = nullptr, *h_iover = nullptr;
    // the Phase I list: lp = which of its two arrays is current; the ranges
    // admitted since the last sweep (for k_srv_merge), their device copy; the column
    // ranges of retired requests, free once a sweep has dropped them
    int lp = 0;
    std::vector<std::pair<int64_t, int64_t>> admitted_rng;
    int64_t *d_rng = nullptr, *h_rng = nullptr;
    std::vector<std::pair<int64_t, int64_t>> retired_cols;
    // results of retired requests wait for their caller in a pinned ring (a
    // real asynchronous copy: the worker never blocks on a large result);
    // oph_server_wait copies them out and frees their space.  A result that
    // does not fit goes to the request's own host arrays.
    int32_t *h_ring = nullptr;
    RangeAlloc ring;
    RangeAlloc cols, pool;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending;
    std::map<int64_t, Request *> all;
    std::vector<Request *> slots;
    std::vector<Request *> all_split;  // split requests admitted without their D part yet (worker only)
    std::thread worker;
    bool stop = false;
    int64_t next_ticket = 1;
    // statistics
    int64_t completed = 0, sweeps = 0, admitted = 0, regrows = 0, dual_admitted = 0;
    int error = OPH_OK;

    int64_t packed_ints(int64_t m, int64_t nnz) const { return 8 * (m + 1) + 4 * ((nnz + 3) / 4) + 64; }
    int64_t region_ints(int64_t m, int64_t nnz) const { return packed_ints(m, nnz) * 4 + 4096; }
    // staging regions of admitted requests, released after the next sync
    std::vector<std::pair<int64_t, int64_t>> staged;

    int grid(int64_t n) const {
        int64_t gsz = (n + 255) / 256, cap = (int64_t)ctx->sm_count * 16;
        return (int)std::max<int64_t>(1, std::min(gsz, cap));
    }

    // Admission of one request into slot b; called by the worker only.
    int admit(Request *r, int b, cudaStream_t s) {
        // the request's CSC is the device copy made at submission; staging
        // holds the anti-transpose's temporaries
        const int64_t stage_ints = r->dual ? (int64_t)((dual_tmp_bytes(r->m, r->nnz) + 255) / 4) + 64 : 0;
        const int64_t reg_ints = region_ints(r->m, r->nnz);
        const int64_t c0 = cols.alloc(std::max<int64_t>(r->m, 1), 1);
        if (c0 < 0) return 1;
        const int64_t reg = pool.alloc(reg_ints, 64);
        if (reg < 0) { cols.release(c0, std::max<int64_t>(r->m, 1)); return 1; }
        const int64_t stg = stage_ints ? pool.alloc(stage_ints, 64) : 0;
        if (stg < 0) {
            cols.release(c0, std::max<int64_t>(r->m, 1));
            pool.release(reg, reg_ints);
            return 1;
        }
        r->c0 = c0; r->reg = reg; r->reg_ints = reg_ints; r->slot = b;
        const int64_t *d_colptr = static_cast<const int64_t *>(r->d_buf);
        const int32_t *d_rows = reinterpret_cast<const int32_t *>(d_colptr + r->m + 1);
        const int8_t asc = r->dual ? 1 : 0;
        cudaMemcpyAsync(const_cast<int8_t *>(a.iasc) + b, &asc, 1, cudaMemcpyHostToDevice, s);
        if (r->m > 0 && r->dual) {
            // the anti-transpose, straight into the request's columns and
            // region (rows shifted into its column range)
            k_srv_init_cols<<<grid(r->m), 256, 0, s>>>(r->m, c0, b, a);
            void *tmp = a.pool + stg;
            dual_build_store(s, ctx->sm_count, d_colptr, d_rows, r->m, r->nnz, a.pool + reg, reg, (int)c0,
                             a.seg + c0, a.low + c0, const_cast<int8_t *>(a.dim) + c0, a.rec + c0,
                             const_cast<int32_t *>(a.beta) + c0, tmp, nullptr);
            // a split request's D' part: its columns of the D-reduced blocks
            // pre-cleared (Phase 0 skips them, Phase I zeroes them)
            if (r->split) split_clear_dual(s, ctx->sm_count, r->d_grade, d_colptr, d_rows, r->m, a.clear + c0);
        } else if (r->m > 0) {
            k_srv_init<<<grid(r->m), 256, 0, s>>>(d_colptr, d_rows, r->m, c0, b, reg, a);
            k_srv_left<<<grid(r->m), 256, 0, s>>>(d_colptr, d_rows, r->m, c0, a);
            k_srv_beta<<<grid(r->m), 256, 0, s>>>(r->m, c0, a);
            // a split request's D part: the D'-reduced blocks' columns and
            // the rows its D' part has paired pre-cleared (from the D' part's
            // pivots while it runs, else from its lows)
            if (r->user) {
                Request *u = r->user;
                if (!u->part_done) {
                    const int8_t *bucket;
                    const uint8_t *split;
                    dual_split_arrays(u->d_grade, r->m, &bucket, &split);
                    k_srv_split_clear_live<<<grid(r->m), 256, 0, s>>>(r->m, u->c0, c0, a, bucket, split);
                } else {
                    split_clear_primal(s, ctx->sm_count, u->d_grade, r->m, u->d_mapped, a.clear + c0);
                }
            }
        }
        if (r->m > 0) admitted_rng.emplace_back(c0, r->m);
        dual_admitted += r->dual ? 1 : 0;
        k_srv_set_region<<<1, 1, 0, s>>>(a.ipool, a.ireps, a.iover, b,
                                         (unsigned long long)(reg + packed_ints(r->m, r->nnz)),
                                         (unsigned long long)(reg + reg_ints));
        if (r->m > 0) launch_phase0(a, c0, c0 + r->m, grid(r->m), s);
        if (stage_ints) {
            // the temporaries are used by the kernels above: their region is
            // released after the sweep's synchronisation
            staged.emplace_back(stg, stage_ints);
        }
        // the device copy is freed in stream order after those kernels (a
        // split request's D part reads it again)
        if (!(r->split && !r->user)) {
            cudaFreeAsync(r->d_buf, s);
            r->d_buf = nullptr;
        }
        if (r->t_admit == 0) r->t_admit = now_ms();
        r->sweep0 = sweeps;
        if (r->split && !r->user) all_split.push_back(r);
        slots[b] = r;
        admitted++;
        return 0;
    }

    // Retires every converged request: output kernels for all of them, then
    // the copies to the host, one synchronisation, then the notifications.
    // A part of a split request keeps its lows on the device; the request is
    // finished by the later of its two parts.
    void retire_all(const std::vector<Request *> &done) {
        if (done.empty()) return;
        cudaStream_t s = ctx->stream;
        std::vector<Request *> users;  // requests whose results go out now
        for (Request *r : done) {
            if (!r->split) {
                users.push_back(r);
                continue;
            }
            Request *u = r->user ? r->user : r;
            const int64_t m = r->m;
            if (r->user) {
                k_srv_save_local<<<grid(m), 256, 0, s>>>(m, r->c0, a, u->d_mapped + 2 * m);
            } else {
                k_srv_out_dual1<<<grid(m), 256, 0, s>>>(m, u->d_mapped);
                k_srv_out_dual2<<<grid(m), 256, 0, s>>>(m, r->c0, a, u->d_mapped);
            }
            k_srv_inert<<<grid(m), 256, 0, s>>>(m, r->c0, a);
            if (--u->parts_left == 0) users.push_back(u);
        }
        std::vector<std::pair<int64_t, int64_t>> outs;
        std::vector<int32_t *> dptr(users.size(), nullptr);
        for (size_t k = 0; k < users.size(); k++) {
            Request *r = users[k];
            const int64_t m = r->m;
            if (m == 0) continue;
            const int64_t out = pool.alloc(2 * m + 4, 64);
            if (out >= 0) {
                outs.emplace_back(out, 2 * m + 4);
                dptr[k] = a.pool + out;
            } else {
                // the request's own region is no longer read; a split
                // request's results go over its D' part's lows (each thread
                // reads its own element first) and the ess scratch after them
                dptr[k] = r->split ? r->d_mapped : a.pool + r->reg;
            }
            if (r->split) {
                const int8_t *bucket;
                const uint8_t *split;
                dual_split_arrays(r->d_grade, m, &bucket, &split);
                k_srv_out_split1<<<grid(m), 256, 0, s>>>(m, bucket, split, r->d_mapped, r->d_mapped + 2 * m,
                                                         dptr[k]);
                k_srv_out_split2<<<grid(m), 256, 0, s>>>(m, dptr[k]);
            } else if (r->dual) {
                k_srv_out_dual1<<<grid(m), 256, 0, s>>>(m, dptr[k]);
                k_srv_out_dual2<<<grid(m), 256, 0, s>>>(m, r->c0, a, dptr[k]);
            } else {
                k_srv_out1<<<grid(m), 256, 0, s>>>(m, r->c0, a, dptr[k]);
                k_srv_out2<<<grid(m), 256, 0, s>>>(m, r->c0, a, dptr[k]);
            }
        }
        for (size_t k = 0; k < users.size(); k++) {
            Request *r = users[k];
            if (r->m == 0) continue;
            if (h_ring) {
                std::lock_guard<std::mutex> lk(mu);
                r->ring_off = ring.alloc(2 * r->m, 16);
            }
            if (r->ring_off >= 0) {
                cudaMemcpyAsync(h_ring + r->ring_off, dptr[k], sizeof(int32_t) * 2 * r->m, cudaMemcpyDeviceToHost, s);
            } else {
                r->low.resize(r->m);
                r->ess.resize(r->m);
                cudaMemcpyAsync(r->low.data(), dptr[k], sizeof(int32_t) * r->m, cudaMemcpyDeviceToHost, s);
                cudaMemcpyAsync(r->ess.data(), dptr[k] + r->m, sizeof(int32_t) * r->m, cudaMemcpyDeviceToHost, s);
            }
            if (!r->split) k_srv_inert<<<grid(r->m), 256, 0, s>>>(r->m, r->c0, a);
        }
        for (Request *r : users)
            if (r->split) {
                cudaFreeAsync(r->d_grade, s);
                cudaFreeAsync(r->d_mapped, s);
                r->d_grade = nullptr;
                r->d_mapped = nullptr;
            }
        cudaStreamSynchronize(s);
        for (auto &o : outs) pool.release(o.first, o.second);
        const double t = now_ms();
        {
            std::lock_guard<std::mutex> lk(mu);
            for (Request *r : done) {
                // its columns leave the Phase I list in the next sweep; the
                // range is handed out again only after that
                retired_cols.emplace_back(r->c0, std::max<int64_t>(r->m, 1));
                pool.release(r->reg, r->reg_ints);
                slots[r->slot] = nullptr;
                r->slot = -1;
                if (r->split && !r->user) r->part_done = true;
            }
            for (Request *r : users) {
                if (r->part) {
                    delete r->part;
                    r->part = nullptr;
                }
                r->t_done = t;
                if (r->split) r->sweeps = (int)(sweeps - r->sweep0);
                r->done = true;
                completed++;
            }
        }
        cv_done.notify_all();
    }

    // After a sweep: the D part of every split request whose D' part has
    // been swept once (or has converged already, in that sweep), at the
    // head of the queue.
    void spawn_parts() {
        std::lock_guard<std::mutex> lk(mu);
        for (Request *u : all_split)
            if (!u->part && (u->part_done || (u->slot >= 0 && slots[u->slot] == u && u->listed))) {
                Request *b = new Request();
                b->m = u->m;
                b->nnz = u->nnz;
                b->d_buf = u->d_buf;  // freed by the D part's admission
                u->d_buf = nullptr;
                b->split = true;
                b->user = u;
                b->ticket = -1;
                b->t_submit = u->t_submit;
                u->part = b;
                pending.push_front(b);
            }
        all_split.erase(std::remove_if(all_split.begin(), all_split.end(), [](Request *u) { return u->part != nullptr; }),
                        all_split.end());
    }

    // Moves the pool region of request r to one twice as large.
    int regrow(Request *r) {
        cudaStream_t s = ctx->stream;
        unsigned long long reg[2];
        cudaMemcpy(reg, a.ipool + 2 * r->slot, sizeof(reg), cudaMemcpyDeviceToHost);
        const int64_t used = std::min<int64_t>((int64_t)reg[0], r->reg + r->reg_ints) - r->reg;
        const int64_t nints = r->reg_ints * 2;
        const int64_t nreg = pool.alloc(nints, 64);
        if (nreg < 0) return OPH_ERR_OOM;
        cudaMemcpyAsync(a.pool + nreg, a.pool + r->reg, sizeof(int) * used, cudaMemcpyDeviceToDevice, s);
        if (r->m > 0) k_srv_rebase<<<grid(r->m), 256, 0, s>>>(r->m, r->c0, nreg - r->reg, a);
        k_srv_set_region<<<1, 1, 0, s>>>(a.ipool, a.ireps, a.iover, r->slot, (unsigned long long)(nreg + used),
                                         (unsigned long long)(nreg + nints));
        cudaStreamSynchronize(s);
        pool.release(r->reg, r->reg_ints);
        r->reg = nreg;
        r->reg_ints = nints;
        regrows++;
        return OPH_OK;
    }

    void fail_all(int rc) {
        std::lock_guard<std::mutex> lk(mu);
        error = rc;
        for (auto &kv : all)
            if (!kv.second->done) {
                kv.second->status = rc;
                kv.second->done = true;
            }
        cv_done.notify_all();
    }

    // Admits queued requests, first come first served, on `s` while they
    // fit (slots, columns, pool); returns how many.
    int admit_pending(cudaStream_t s, int &active, bool wait_for_work) {
        int n = 0;
        for (;;) {
            Request *r = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu);
                if (wait_for_work && active == 0) cv_work.wait(lk, [&] { return stop || !pending.empty(); });
                if (pending.empty()) break;
                r = pending.front();
            }
            int b = -1;
            for (int k = 0; k < max_slots; k++)
                if (!slots[k]) { b = k; break; }
            if (b < 0 || admit(r, b, s) != 0) break;  // no room now: retry after the next sweep
            {
                std::lock_guard<std::mutex> lk(mu);
                pending.pop_front();
            }
            active++;
            n++;
        }
        return n;
    }

    void run() {
        cudaSetDevice(ctx->device);
        cudaStream_t s = ctx->stream;
        // OPH_TRACE=1: one line per sweep on stderr; OPH_TRACE=2 adds the
        // device time of the merge and of each phase (diagnostics only)
        const int trace = getenv("OPH_TRACE") ? atoi(getenv("OPH_TRACE")) : 0;
        cudaEvent_t tev[8] = {};
        if (trace > 1)
            for (auto &e : tev) cudaEventCreate(&e);
        for (;;) {
            const double t_round = now_ms();
            const int64_t admitted_before = admitted;
            int active = 0;
            for (auto *r : slots) active += r != nullptr;
            if (active == 0) {
                // nothing on the device: the list starts empty (retired
                // columns left in it go too), every range is free, and the
                // first requests are admitted here, before the sweep
                cudaMemsetAsync(&a.st->ucount[lp], 0, sizeof(int), s);
                {
                    std::lock_guard<std::mutex> lk(mu);
                    for (auto &rc : retired_cols) cols.release(rc.first, rc.second);
                    retired_cols.clear();
                    if (stop && pending.empty()) return;
                }
                admit_pending(s, active, true);
                {
                    std::lock_guard<std::mutex> lk(mu);
                    if (stop && pending.empty() && active == 0) return;
                }
                if (active == 0) {
                    if (!pending.empty()) {
                        // the head request cannot fit even in an empty arena
                        std::lock_guard<std::mutex> lk(mu);
                        Request *r = pending.front();
                        pending.pop_front();
                        if (r->user) {  // a split request's D part: the request fails
                            Request *u = r->user;
                            if (r->d_buf) cudaFree(r->d_buf);
                            u->part = nullptr;
                            delete r;
                            r = u;
                        }
                        r->status = OPH_ERR_OOM;
                        r->done = true;
                        cv_done.notify_all();
                    }
                    continue;
                }
            }
            if (trace > 1) cudaEventRecord(tev[6], s);
            // the ranges admitted since the last sweep into the Phase I list
            // (column order), after their set-up on the admission stream
            if (!admitted_rng.empty()) {
                cudaStreamWaitEvent(s, adm_done, 0);
                std::sort(admitted_rng.begin(), admitted_rng.end());
                const int K = (int)admitted_rng.size();
                int64_t acc = 0;
                for (int q = 0; q < K; q++) {
                    h_rng[q] = admitted_rng[q].first;
                    h_rng[K + q] = acc;
                    acc += admitted_rng[q].second;
                }
                h_rng[2 * K] = acc;
                cudaMemcpyAsync(d_rng, h_rng, sizeof(int64_t) * (2 * K + 1), cudaMemcpyHostToDevice, s);
                int32_t *L[2] = {a.ulist, a.ulist_next};
                k_srv_merge<<<grid(acc + 4096), 256, 0, s>>>(L[lp], &a.st->ucount[lp], d_rng, d_rng + K, K,
                                                             L[lp ^ 1], &a.st->ucount[lp ^ 1]);
                lp ^= 1;
                admitted_rng.clear();
            }
            for (auto *r : slots)
                if (r) r->listed = true;
            const size_t retired_before = retired_cols.size();
            // one sweep over every listed request
            int64_t hi = 0;
            for (auto *r : slots)
                if (r) hi = std::max(hi, r->c0 + std::max<int64_t>(r->m, 1));
            PmsArgs sa = a;
            sa.m = hi;
            sa.ntiles = (hi + 2047) / 2048;
            SweepGrids gg = g;
            gg.m = grid(hi);
            gg.t = (int)std::max<int64_t>(1, std::min<int64_t>(sa.ntiles, (int64_t)ctx->sm_count * 8));
            cudaMemsetAsync(a.ireps, 0, sizeof(int) * max_slots, s);
            k_srv_sweep_reset<<<1, 1, 0, s>>>(a.st);
            launch_sweep(sa, gg, s, lp, trace > 1 ? tev : nullptr);  // compacts list lp into the other one
            lp ^= 1;
            cudaMemcpyAsync(h_ireps, a.ireps, sizeof(int) * max_slots, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(h_iover, a.iover, sizeof(int) * max_slots, cudaMemcpyDeviceToHost, s);
            // while the sweep runs: the requests that arrived meanwhile are set
            // up on the admission stream (their columns, records and pool
            // regions are disjoint from every listed request's); they join
            // the list before the next sweep
            admit_pending(adm_stream, active, false);
            cudaEventRecord(adm_done, adm_stream);
            if (cudaStreamSynchronize(s) != cudaSuccess || cudaStreamSynchronize(adm_stream) != cudaSuccess) {
                fail_all(OPH_ERR_CUDA);
                return;
            }
            for (auto &st : staged) pool.release(st.first, st.second);
            staged.clear();
            {
                // columns retired before this sweep have left the list
                std::lock_guard<std::mutex> lk(mu);
                for (size_t q = 0; q < retired_before; q++) cols.release(retired_cols[q].first, retired_cols[q].second);
                retired_cols.erase(retired_cols.begin(), retired_cols.begin() + retired_before);
            }
            sweeps++;
            for (auto *r : slots)
                if (r && r->listed) r->sweeps++;
            // regrow first: an overflowed request is not converged
            for (int b = 0; b < max_slots; b++)
                if (slots[b] && slots[b]->listed && h_iover[b]) {
                    if (regrow(slots[b]) != OPH_OK) {
                        fail_all(OPH_ERR_OOM);
                        return;
                    }
                }
            std::vector<Request *> done;
            for (int b = 0; b < max_slots; b++)
                if (slots[b] && slots[b]->listed && h_ireps[b] == 0 && !h_iover[b]) done.push_back(slots[b]);
            const double t_swept = now_ms();
            retire_all(done);
            spawn_parts();
            if (trace)
                fprintf(stderr, "server sweep %lld: span %lld cols, %d active, %lld admitted, %zu retired | "
                                "round %.3f ms (sweep+admit %.3f, retire %.3f)\n",
                        (long long)sweeps, (long long)hi, active, (long long)(admitted - admitted_before),
                        done.size(), now_ms() - t_round, t_swept - t_round, now_ms() - t_swept);
            if (trace > 1) {
                float t[6] = {0, 0, 0, 0, 0, 0};
                cudaEventElapsedTime(&t[0], tev[6], tev[0]);
                for (int q = 0; q < 5; q++) cudaEventElapsedTime(&t[q + 1], tev[q], tev[q + 1]);
                fprintf(stderr, "  device ms: admit+merge %.3f p1 %.3f narrow %.3f t1 %.3f t2 %.3f t3 %.3f\n", t[0],
                        t[1], t[2], t[3], t[4], t[5]);
            }
        }
    }
};

}  // namespace oph

using namespace oph;

struct oph_server : public oph::Server {};

extern "C" {

__attribute__((visibility("default"))) int oph_server_create(int device, int64_t budget_bytes, int32_t max_active,
                                                             oph_server **out) {
    if (!out || budget_bytes < (int64_t)(64 << 20) || max_active < 1 || max_active > 65536) return OPH_ERR_BAD_INPUT;
    *out = nullptr;
    oph_server *sv = new oph_server();
    oph_context *raw = nullptr;
    int rc = oph_context_create(device, &raw);
    if (rc) {
        delete sv;
        return rc;
    }
    sv->ctx = reinterpret_cast<Context *>(raw);
    Context *ctx = sv->ctx;
    sv->budget = budget_bytes;
    sv->max_slots = max_active;
    // the arena: per-column arrays for mcap columns (a tenth of the budget)
    // and a segment pool for the rest (at most what 32-bit segment fields
    // address)
    const int64_t per_col = 4 + 1 + 1 + 1 + 4 + 4 + 4 + 4 + 4 + 8 + (int64_t)sizeof(PivRec) + 4 + 8 + 1;
    sv->mcap = std::min<int64_t>(budget_bytes / 10 / per_col, (1ll << 29) - 1);
    int64_t pool_bytes = budget_bytes - sv->mcap * per_col - budget_bytes / 16;
    sv->pool_ints = std::min<int64_t>(pool_bytes / 4 - POOL_PAD, MAX_POOL_INTS - 1);
    const int64_t mc = sv->mcap;
    PmsArgs &a = sv->a;
    a.low = (int32_t *)ctx_alloc(ctx, S_LOW, 4 * mc);
    a.classes = (int8_t *)ctx_alloc(ctx, S_CLASSES, mc);
    a.clear = (uint8_t *)ctx_alloc(ctx, S_CLEAR, mc);
    a.dim = (int8_t *)ctx_alloc(ctx, S_DIM, mc);
    a.first = (int32_t *)ctx_alloc(ctx, S_FIRST, 4 * mc);
    a.beta = (int32_t *)ctx_alloc(ctx, S_BETA, 4 * mc);
    a.worklist = (int32_t *)ctx_alloc(ctx, S_WORK, 4 * mc);
    a.widelist = (int32_t *)ctx_alloc(ctx, S_WIDE, 4 * mc);
    a.slist = (int32_t *)ctx_alloc(ctx, S_SLIST, 4 * mc);
    a.seg = (int64_t *)ctx_alloc(ctx, S_SEG, 8 * mc);
    a.rec = (PivRec *)ctx_alloc(ctx, S_ROWPIV, sizeof(PivRec) * mc);
    a.inst = (int *)ctx_alloc(ctx, S_LOWTRUE, 4 * mc);
    a.agg = (int32_t *)ctx_alloc(ctx, S_AGG, sizeof(int32_t) * MAXC * ((mc + 2047) / 2048 + 1));
    a.ipool = (unsigned long long *)ctx_alloc(ctx, S_INSTOFF, 16 * (size_t)max_active);
    a.ireps = (int *)ctx_alloc(ctx, S_TRACK, 4 * (size_t)max_active);
    a.iover = (int *)ctx_alloc(ctx, S_TMP, 4 * (size_t)max_active);
    a.st = (DevStatus *)ctx_alloc(ctx, S_STATUS, sizeof(DevStatus));
    a.pool = (int *)ctx_alloc(ctx, S_POOL, sizeof(int) * (sv->pool_ints + POOL_PAD));
    // the Phase I list (two arrays) and its per-tile counts
    a.ulist = (int32_t *)ctx_alloc(ctx, S_ULIST, sizeof(int32_t) * 2 * mc);
    a.ulist_next = a.ulist ? a.ulist + mc : nullptr;
    a.kagg = (int32_t *)ctx_alloc(ctx, S_KAGG, sizeof(int32_t) * ((mc + 2047) / 2048 + 2));
    // per-instance bucket order
    a.iasc = (const int8_t *)ctx_alloc(ctx, S_IASC, (size_t)max_active);
    a.ibucket = (int *)ctx_alloc(ctx, S_IBUCKET, sizeof(int) * MAXC * (size_t)max_active);
    a.iopen = (int *)ctx_alloc(ctx, S_IOPEN, sizeof(int) * (size_t)max_active);
    a.nslots = max_active;
    sv->d_rng = (int64_t *)ctx_alloc(ctx, S_RANGES, sizeof(int64_t) * (2 * (size_t)max_active + 1));
    // tier 3's bitmaps (one per CTA of its grid, a window of up to 2^23 rows)
    a.bm_words = std::min<int64_t>(((mc + 32) / 32 + 3) & ~3ll, 1 << 18);
    a.bm = (uint32_t *)ctx_alloc(ctx, S_BITMAP, sizeof(uint32_t) * (size_t)a.bm_words * ctx->sm_count);
    bool ok = a.ulist && a.kagg && a.iasc && a.ibucket && a.iopen && sv->d_rng && a.bm && a.low && a.classes &&
              a.clear && a.dim && a.first && a.beta && a.worklist && a.widelist &&
              a.slist && a.seg && a.rec && a.inst && a.agg && a.ipool && a.ireps && a.iover && a.st && a.pool;
    if (ok) ok = cudaMallocHost((void **)&sv->h_ireps, 4 * (size_t)max_active) == cudaSuccess &&
                 cudaMallocHost((void **)&sv->h_iover, 4 * (size_t)max_active) == cudaSuccess &&
                 cudaMallocHost((void **)&sv->h_rng, sizeof(int64_t) * (2 * (size_t)max_active + 1)) == cudaSuccess;
    // the result ring: 1/256 of the budget, 32 MB .. 512 MB (without it,
    // results are copied to pageable host arrays)
    const int64_t ring_ints = std::min<int64_t>(std::max<int64_t>(budget_bytes / 256, 32ll << 20), 512ll << 20) / 4;
    if (ok && cudaMallocHost((void **)&sv->h_ring, sizeof(int32_t) * ring_ints) == cudaSuccess) {
        sv->ring.init(ring_ints);
    } else {
        sv->h_ring = nullptr;
        cudaGetLastError();
    }
    if (ok) ok = sweep_grids(ctx, mc, (mc + 2047) / 2048, &sv->g) == OPH_OK;
    // columns wider than a CTA's shared window go to the cluster tier
    a.cluster_tier = ok && sv->g.g4 > 0;
    // no sweep waits on one long chain of the bitmap tiers
    a.chain_cap = getenv("OPH_SERVE_CHAIN_CAP") ? atoi(getenv("OPH_SERVE_CHAIN_CAP")) : SERVE_CHAIN_CAP;
    if (ok) ok = cudaStreamCreateWithFlags(&sv->sub_stream, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) ok = cudaStreamCreateWithFlags(&sv->adm_stream, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) ok = cudaEventCreateWithFlags(&sv->adm_done, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        if (sv->h_ireps) cudaFreeHost(sv->h_ireps);
        if (sv->h_iover) cudaFreeHost(sv->h_iover);
        if (sv->h_rng) cudaFreeHost(sv->h_rng);
        if (sv->h_ring) cudaFreeHost(sv->h_ring);
        if (sv->sub_stream) cudaStreamDestroy(sv->sub_stream);
        if (sv->adm_stream) cudaStreamDestroy(sv->adm_stream);
        if (sv->adm_done) cudaEventDestroy(sv->adm_done);
        oph_context_destroy(raw);
        delete sv;
        return OPH_ERR_OOM;
    }
    cudaStream_t s = ctx->stream;
    // every column starts inert
    cudaMemsetAsync(a.low, 0xff, 4 * mc, s);
    cudaMemsetAsync(a.classes, 1, mc, s);
    cudaMemsetAsync(a.clear, 0, mc, s);
    cudaMemsetAsync(a.inst, 0xff, 4 * mc, s);
    cudaMemsetAsync(a.first, 0x7f, 4 * mc, s);
    cudaMemsetAsync(a.iover, 0, 4 * (size_t)max_active, s);
    cudaMemsetAsync(a.ibucket, 0, sizeof(int) * MAXC * (size_t)max_active, s);
    cudaMemsetAsync(const_cast<int8_t *>(a.iasc), 0, (size_t)max_active, s);
    cudaMemsetAsync(a.bm, 0, sizeof(uint32_t) * (size_t)a.bm_words * ctx->sm_count, s);
    k_srv_inert<<<sv->grid(mc), 256, 0, s>>>(mc, 0, a);
    DevStatus init{};
    init.pool_used = 0;
    init.pool_size = (unsigned long long)sv->pool_ints;
    cudaMemcpyAsync(a.st, &init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        oph_context_destroy(raw);
        delete sv;
        return OPH_ERR_CUDA;
    }
    sv->cols.init(mc);
    sv->pool.init(sv->pool_ints);
    sv->slots.assign(max_active, nullptr);
    sv->worker = std::thread([sv] { sv->run(); });
    *out = sv;
    return OPH_OK;
}

}  // extern "C"

namespace {

// The server's own device copy of a submitted CSC (from host or device
// memory; the caller may free its buffers on return), its structural checks
// and its grading on the device (the matrix a single-matrix pms reduction
// would choose), then the request queued.  The submitting thread does no
// O(nnz) host work beyond the copy; the work runs on the submission stream,
// beside the worker's sweeps.
int submit_copy(oph_server *sv, int64_t m, int64_t nnz, const int64_t *colptr, const int32_t *rows,
                cudaMemcpyKind kind, int64_t *ticket) {
    // the request's region and, at admission, its anti-transpose's
    // temporaries must fit the arena's pool
    const int64_t tmp_ints = (int64_t)((dual_tmp_bytes(m, nnz) + 255) / 4) + 64;
    if (m > sv->mcap || sv->region_ints(m, nnz) + tmp_ints > sv->pool_ints) return OPH_ERR_OOM;
    cudaStream_t s = sv->sub_stream;
    const size_t bytes = sizeof(int64_t) * (m + 1) + sizeof(int32_t) * nnz + sizeof(int);
    void *buf = nullptr;
    if (cudaMallocAsync(&buf, bytes, s) != cudaSuccess) {
        cudaGetLastError();
        return OPH_ERR_OOM;
    }
    int64_t *cp = static_cast<int64_t *>(buf);
    int32_t *rw = reinterpret_cast<int32_t *>(cp + m + 1);
    int *bad = reinterpret_cast<int *>(rw + nnz);
    int h_bad = 0;
    cudaMemcpyAsync(cp, colptr, sizeof(int64_t) * (m + 1), kind, s);
    if (nnz) cudaMemcpyAsync(rw, rows, sizeof(int32_t) * nnz, kind, s);
    cudaMemsetAsync(bad, 0, sizeof(int), s);
    if (m > 0) k_srv_check<<<sv->grid(m), 256, 0, s>>>(cp, rw, m, nnz, bad);
    cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess || h_bad) {
        cudaFreeAsync(buf, s);
        cudaStreamSynchronize(s);
        return e != cudaSuccess ? OPH_ERR_CUDA : OPH_ERR_BAD_INPUT;
    }
    int choice = DUAL_CHOICE_D;
    bool bad_g = false;
    void *gtmp = nullptr;
    int32_t *mapped = nullptr;
    if (m >= DUAL_MIN_M && cudaMallocAsync(&gtmp, dual_grade_tmp_bytes(m), s) == cudaSuccess) {
        if (dual_grade(s, sv->ctx->sm_count, cp, rw, m, nnz, OPH_DUAL_AUTO, gtmp, &choice, &bad_g, nullptr) != OPH_OK ||
            bad_g)
            choice = DUAL_CHOICE_D;
        // a split request keeps its grading, and room for its parts' lows
        if (choice == DUAL_CHOICE_SPLIT && cudaMallocAsync(&mapped, sizeof(int32_t) * 3 * m, s) != cudaSuccess) {
            cudaGetLastError();
            choice = DUAL_CHOICE_D;
        }
        if (choice != DUAL_CHOICE_SPLIT) {
            cudaFreeAsync(gtmp, s);
            gtmp = nullptr;
        }
        // the worker uses both on its own streams
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            cudaFreeAsync(buf, s);
            if (gtmp) cudaFreeAsync(gtmp, s);
            if (mapped) cudaFreeAsync(mapped, s);
            cudaStreamSynchronize(s);
            return OPH_ERR_CUDA;
        }
    } else {
        cudaGetLastError();
    }
    Request *r = new Request();
    r->m = m;
    r->nnz = nnz;
    r->d_buf = buf;
    r->dual = choice != DUAL_CHOICE_D;
    r->split = choice == DUAL_CHOICE_SPLIT;
    r->parts_left = r->split ? 2 : 0;
    r->d_grade = gtmp;
    r->d_mapped = mapped;
    r->t_submit = now_ms();
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->error) {
            cudaFreeAsync(buf, s);
            if (gtmp) cudaFreeAsync(gtmp, s);
            if (mapped) cudaFreeAsync(mapped, s);
            delete r;
            return sv->error;
        }
        r->ticket = sv->next_ticket++;
        sv->all[r->ticket] = r;
        sv->pending.push_back(r);
        *ticket = r->ticket;
    }
    sv->cv_work.notify_one();
    return OPH_OK;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) int oph_server_submit(oph_server *sv, int64_t m, const int64_t *colptr,
                                                             const int32_t *rows, int64_t *ticket) {
    if (!sv || m < 0 || !colptr || !ticket || colptr[0] != 0) return OPH_ERR_BAD_INPUT;
    const int64_t nnz = colptr[m];
    if (nnz < 0 || (nnz > 0 && !rows)) return OPH_ERR_BAD_INPUT;
    OPH_CUDA_TRY(cudaSetDevice(sv->ctx->device));
    return submit_copy(sv, m, nnz, colptr, rows, cudaMemcpyHostToDevice, ticket);
}

__attribute__((visibility("default"))) int oph_server_submit_device(oph_server *sv, int64_t m,
                                                                    const int64_t *d_colptr, const int32_t *d_rows,
                                                                    int64_t *ticket) {
    if (!sv || m < 0 || !d_colptr || !ticket) return OPH_ERR_BAD_INPUT;
    OPH_CUDA_TRY(cudaSetDevice(sv->ctx->device));
    cudaStream_t s = sv->sub_stream;
    int64_t ends[2] = {0, 0};
    OPH_CUDA_TRY(cudaMemcpyAsync(&ends[0], d_colptr, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaMemcpyAsync(&ends[1], d_colptr + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    OPH_CUDA_TRY(cudaStreamSynchronize(s));
    const int64_t nnz = ends[1];
    if (ends[0] != 0 || nnz < 0 || (nnz > 0 && !d_rows)) return OPH_ERR_BAD_INPUT;
    return submit_copy(sv, m, nnz, d_colptr, d_rows, cudaMemcpyDeviceToDevice, ticket);
}

__attribute__((visibility("default"))) int oph_server_wait(oph_server *sv, int64_t ticket, int32_t *low,
                                                           int32_t *ess, oph_request_info *info, int64_t timeout_ms) {
    if (!sv) return OPH_ERR_BAD_INPUT;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->all.find(ticket);
    if (it == sv->all.end()) return OPH_ERR_BAD_INPUT;
    Request *r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) sv->cv_done.wait(lk, ready);
    else if (!sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return OPH_ERR_TIMEOUT;
    sv->all.erase(it);
    lk.unlock();
    const int rc = r->status;
    if (rc == OPH_OK && r->m > 0) {
        const int32_t *src = r->ring_off >= 0 ? sv->h_ring + r->ring_off : nullptr;
        if (low) memcpy(low, src ? src : r->low.data(), sizeof(int32_t) * r->m);
        if (ess) memcpy(ess, src ? src + r->m : r->ess.data(), sizeof(int32_t) * r->m);
    }
    if (r->ring_off >= 0) {
        std::lock_guard<std::mutex> lk2(sv->mu);
        sv->ring.release(r->ring_off, 2 * r->m);
    }
    if (info) {
        info->latency_ms = r->t_done - r->t_submit;
        info->queue_ms = r->t_admit > 0 ? r->t_admit - r->t_submit : 0;
        info->sweeps = r->sweeps;
        info->status = rc;
        info->m = r->m;
        info->submit_ms = r->t_submit;
        info->done_ms = r->t_done;
    }
    // device buffers a failed request still holds
    for (void *p : {r->d_buf, r->d_grade, static_cast<void *>(r->d_mapped)})
        if (p) cudaFree(p);
    delete r;
    return rc;
}

__attribute__((visibility("default"))) int oph_server_stats(oph_server *sv, oph_server_counters *out) {
    if (!sv || !out) return OPH_ERR_BAD_INPUT;
    std::lock_guard<std::mutex> lk(sv->mu);
    // requests as submitted: a split request counts once, by its D' part
    // while that is on the device, else by its D part
    int64_t active = 0, pending = 0;
    for (auto *r : sv->slots) active += r != nullptr && (!r->user || r->user->slot < 0);
    for (auto *r : sv->pending) pending += !r->user;
    out->completed = sv->completed;
    out->pending = pending;
    out->active = active;
    out->sweeps = sv->sweeps;
    out->regrows = sv->regrows;
    out->pool_bytes_in_use = sv->pool.used * 4;
    out->columns_in_use = sv->cols.used;
    out->arena_bytes = sv->budget;
    out->dual_admitted = sv->dual_admitted;
    return OPH_OK;
}

__attribute__((visibility("default"))) int oph_server_destroy(oph_server *sv) {
    if (!sv) return OPH_OK;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    cudaSetDevice(sv->ctx->device);
    // internal D parts of split requests left by a failure
    for (Request *r : sv->slots)
        if (r && r->user) {
            if (r->d_buf) cudaFree(r->d_buf);
            delete r;
        }
    for (Request *r : sv->pending)
        if (r->user) {
            if (r->d_buf) cudaFree(r->d_buf);
            delete r;
        }
    for (auto &kv : sv->all) {
        for (void *p : {kv.second->d_buf, kv.second->d_grade, static_cast<void *>(kv.second->d_mapped)})
            if (p) cudaFree(p);
        delete kv.second;
    }
    if (sv->sub_stream) cudaStreamDestroy(sv->sub_stream);
    if (sv->adm_stream) cudaStreamDestroy(sv->adm_stream);
    if (sv->adm_done) cudaEventDestroy(sv->adm_done);
    if (sv->h_ireps) cudaFreeHost(sv->h_ireps);
    if (sv->h_iover) cudaFreeHost(sv->h_iover);
    if (sv->h_rng) cudaFreeHost(sv->h_rng);
    if (sv->h_ring) cudaFreeHost(sv->h_ring);
    oph_context_destroy(reinterpret_cast<oph_context *>(sv->ctx));
    delete sv;
    return OPH_OK;
}

}  // extern "C"
