/*
 * ORACLE — test infrastructure only.  Nothing in the product path links,
 * loads or calls this file: only tests/, the smoke check and bench.py's CPU
 * baseline leg do, and only as the checker.
 *
 * A plain-C restatement of OpenPH's CPU reduction algorithms, over Z/2, on a
 * 0-based CSC boundary matrix (int64 colptr, int32 rows ascending in each
 * column).  Outputs are 0-based: low[j] = -1 for a zero or cleared column;
 * ess[j] = 1 for a column estimated essential.
 *
 *   oracle_twist      src/cuda/algorithms/twist/twist.cu:10-87
 *                     + algorithms/kernels_host.cu:62-75 (reduce_col_host)
 *                     + src/cuda/dimensions.cu:54-104 (dimension buckets)
 *   oracle_standard   src/cuda/algorithms/standard/standard.cu:1-57
 *   oracle_ph_row     src/cuda/algorithms/ph_row/ph_row.cu:2-121
 *   oracle_pms        src/cuda/algorithms/pms/pms.cu:1-118 with
 *                     pms_functions.cu:6-140 and beta.cu:2-15, one thread at a
 *                     time in column order (one legal interleaving of the
 *                     reference's racy sweep kernels)
 *   oracle_transverse pms_functions.cu:55-85, the serial walk, on a given state
 *   oracle_twist_fixed_p
 *                     twist with the reference's own memory layout: an m x p
 *                     int32 slot store padded with -1 plus an m x p aux store,
 *                     p = col_width * max column nnz (src/cuda/openph.cu:41),
 *                     column addition as kernels_host.cu:2-52.  Used as the
 *                     timed CPU baseline; overflow returns an error instead of
 *                     exiting the process (kernels_host.cu:21-24).
 *
 * Column storage in the adaptive variants is a bump-allocated pool with a
 * per-column (offset, length, capacity) triple; a column that outgrows its
 * capacity moves to the end of the pool with double the room.
 *
 * Statistics: every column addition T <- T xor P counts |P| + |T| slots read
 * and |T xor P| written, the per-addition term of the algorithmic byte count.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define ORACLE_API __attribute__((visibility("default")))

enum { ORC_OK = 0, ORC_NOMEM = 2, ORC_OVERFLOW = 3, ORC_BADINPUT = 1 };

typedef struct {
    int64_t additions;     /* column additions performed */
    int64_t slots_read;    /* sum |P| + |T| over additions */
    int64_t slots_written; /* sum |T xor P| over additions */
    int64_t max_len;       /* largest column length seen */
    int64_t iters;         /* algorithm-specific iteration count (num_iters) */
    int64_t columns_done;  /* columns fully processed (bounded runs) */
    double seconds;        /* wall time of the reduction loop */
} oracle_stats_t;

static double now_s(void) {
    struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ----------------------------------------------------------- column pool */
typedef struct {
    int32_t *pool; int64_t used, size;
    int64_t *off; int32_t *len, *cap;
    int32_t *tmp; int64_t tmp_size;
    oracle_stats_t *st;
} store_t;

static void store_free(store_t *s) { free(s->pool); free(s->off); free(s->len); free(s->cap); free(s->tmp); }

static int store_init(store_t *s, int64_t m, const int64_t *colptr, const int32_t *rows, oracle_stats_t *st) {
    memset(s, 0, sizeof(*s));
    s->st = st;
    int64_t nnz = colptr[m];
    s->size = nnz * 2 + 16;
    s->pool = (int32_t *)malloc(sizeof(int32_t) * s->size);
    s->off = (int64_t *)malloc(sizeof(int64_t) * (m ? m : 1));
    s->len = (int32_t *)malloc(sizeof(int32_t) * (m ? m : 1));
    s->cap = (int32_t *)malloc(sizeof(int32_t) * (m ? m : 1));
    s->tmp_size = 1024;
    s->tmp = (int32_t *)malloc(sizeof(int32_t) * s->tmp_size);
    if (!s->pool || !s->off || !s->len || !s->cap || !s->tmp) { store_free(s); return ORC_NOMEM; }
    for (int64_t j = 0; j < m; j++) {
        int64_t a = colptr[j], b = colptr[j + 1];
        s->off[j] = s->used; s->len[j] = (int32_t)(b - a); s->cap[j] = (int32_t)(b - a);
        memcpy(s->pool + s->used, rows + a, sizeof(int32_t) * (b - a));
        s->used += b - a;
    }
    return ORC_OK;
}

static inline int32_t store_low(const store_t *s, int64_t j) {
    return s->len[j] ? s->pool[s->off[j] + s->len[j] - 1] : -1;
}

/* col[t] <- col[t] xor col[p]; returns the new low of t (or -2 on OOM). */
static int32_t store_add(store_t *s, int64_t p, int64_t t) {
    int32_t lp = s->len[p], lt = s->len[t];
    if ((int64_t)lp + lt > s->tmp_size) {
        int64_t ns = ((int64_t)lp + lt) * 2;
        int32_t *nt = (int32_t *)realloc(s->tmp, sizeof(int32_t) * ns);
        if (!nt) return -2;
        s->tmp = nt; s->tmp_size = ns;
    }
    const int32_t *P = s->pool + s->off[p], *T = s->pool + s->off[t];
    int32_t *o = s->tmp;
    int32_t i = 0, k = 0, n = 0;
    while (i < lp && k < lt) {
        int32_t a = P[i], b = T[k];
        if (a < b) { o[n++] = a; i++; }
        else if (b < a) { o[n++] = b; k++; }
        else { i++; k++; }
    }
    while (i < lp) o[n++] = P[i++];
    while (k < lt) o[n++] = T[k++];
    if (s->st) {
        s->st->additions++; s->st->slots_read += lp + lt; s->st->slots_written += n;
        if (n > s->st->max_len) s->st->max_len = n;
    }
    if (n > s->cap[t]) {
        int32_t nc = n * 2;
        if (s->used + nc > s->size) {
            int64_t ns = (s->used + nc) * 2;
            int32_t *np = (int32_t *)realloc(s->pool, sizeof(int32_t) * ns);
            if (!np) return -2;
            s->pool = np; s->size = ns;
        }
        s->off[t] = s->used; s->cap[t] = nc; s->used += nc;
    }
    memcpy(s->pool + s->off[t], o, sizeof(int32_t) * n);
    s->len[t] = n;
    return n ? o[n - 1] : -1;
}

/* ----------------------------------------------------------- dimensions */
/* dim[j] = nnz(col j) - 1 (so a column with no entries is "-1"), buckets in
 * column order, as src/cuda/dimensions.cu:54-104 builds them. */
typedef struct { int32_t *dim; int32_t complex_dim; int32_t cdim; int32_t *start; int32_t *next; } dims_t;

static void dims_free(dims_t *d) { free(d->dim); free(d->start); free(d->next); }

static int dims_init(dims_t *d, int64_t m, const int64_t *colptr) {
    memset(d, 0, sizeof(*d));
    d->dim = (int32_t *)malloc(sizeof(int32_t) * (m ? m : 1));
    d->next = (int32_t *)malloc(sizeof(int32_t) * (m ? m : 1));
    if (!d->dim || !d->next) { dims_free(d); return ORC_NOMEM; }
    d->complex_dim = -1;
    for (int64_t j = 0; j < m; j++) {
        d->dim[j] = (int32_t)(colptr[j + 1] - colptr[j]) - 1;
        if (d->dim[j] > d->complex_dim) d->complex_dim = d->dim[j];
    }
    d->cdim = d->complex_dim + 2;
    d->start = (int32_t *)malloc(sizeof(int32_t) * d->cdim);
    int32_t *last = (int32_t *)malloc(sizeof(int32_t) * d->cdim);
    if (!d->start || !last) { free(last); dims_free(d); return ORC_NOMEM; }
    for (int c = 0; c < d->cdim; c++) { d->start[c] = -1; last[c] = -1; }
    for (int64_t j = 0; j < m; j++) {
        int c = d->dim[j] + 1;
        d->next[j] = -1;
        if (last[c] >= 0) d->next[last[c]] = (int32_t)j; else d->start[c] = (int32_t)j;
        last[c] = (int32_t)j;
    }
    free(last);
    return ORC_OK;
}

static int alloc_vecs(int64_t m, int32_t **arglow, int32_t **classes) {
    *arglow = (int32_t *)malloc(sizeof(int32_t) * (m ? m : 1));
    *classes = (int32_t *)calloc(m ? m : 1, sizeof(int32_t));
    if (!*arglow || !*classes) { free(*arglow); free(*classes); return ORC_NOMEM; }
    for (int64_t i = 0; i < m; i++) (*arglow)[i] = -1;
    return ORC_OK;
}

/* reduce_col_host (kernels_host.cu:62-75) */
static int reduce_col(store_t *s, int64_t j, int32_t *low, int32_t *arglow, int32_t *ess) {
    int32_t lj = low[j];
    while (lj > -1 && arglow[lj] != -1) {
        ess[lj] = 0;
        int32_t nl = store_add(s, arglow[lj], j);
        if (nl == -2) return ORC_NOMEM;
        low[j] = nl; lj = nl;
    }
    if (lj > -1) arglow[lj] = (int32_t)j;
    return ORC_OK;
}

/* ------------------------------------------------------------------ twist */
ORACLE_API int oracle_twist(int64_t m, const int64_t *colptr, const int32_t *rows,
                            int32_t *low, int32_t *ess, oracle_stats_t *st) {
    oracle_stats_t dummy; if (!st) st = &dummy;
    memset(st, 0, sizeof(*st));
    store_t s; dims_t d; int32_t *arglow, *classes;
    if (store_init(&s, m, colptr, rows, st)) return ORC_NOMEM;
    if (dims_init(&d, m, colptr)) { store_free(&s); return ORC_NOMEM; }
    if (alloc_vecs(m, &arglow, &classes)) { store_free(&s); dims_free(&d); return ORC_NOMEM; }
    for (int64_t j = 0; j < m; j++) { low[j] = store_low(&s, j); ess[j] = 1; }
    double t0 = now_s();
    int rc = ORC_OK; int64_t iter = 1;
    for (int dim = d.complex_dim; dim > 0 && rc == ORC_OK; dim--) {
        for (int32_t j = d.start[dim + 1]; j > -1; j = d.next[j]) {
            if ((rc = reduce_col(&s, j, low, arglow, ess))) break;
            if (low[j] > -1) low[low[j]] = -1; /* twist_step_host */
            if (low[j] > -1) { classes[j] = -1; classes[low[j]] = 1; ess[j] = 0; ess[low[j]] = 0; }
            else classes[j] = 1;
            iter++; st->columns_done++;
        }
    }
    st->seconds = now_s() - t0; st->iters = iter;
    free(arglow); free(classes); dims_free(&d); store_free(&s);
    return rc;
}

/* --------------------------------------------------------------- standard */
ORACLE_API int oracle_standard(int64_t m, const int64_t *colptr, const int32_t *rows,
                               int32_t *low, int32_t *ess, oracle_stats_t *st) {
    oracle_stats_t dummy; if (!st) st = &dummy;
    memset(st, 0, sizeof(*st));
    store_t s; int32_t *arglow, *classes;
    if (store_init(&s, m, colptr, rows, st)) return ORC_NOMEM;
    if (alloc_vecs(m, &arglow, &classes)) { store_free(&s); return ORC_NOMEM; }
    for (int64_t j = 0; j < m; j++) { low[j] = store_low(&s, j); ess[j] = 1; }
    double t0 = now_s();
    int rc = ORC_OK;
    for (int64_t j = 0; j < m; j++) {
        if ((rc = reduce_col(&s, j, low, arglow, ess))) break;
        if (low[j] > -1) { classes[j] = -1; classes[low[j]] = 1; ess[j] = 0; ess[low[j]] = 0; }
        else classes[j] = 1;
        st->columns_done++;
    }
    st->seconds = now_s() - t0; st->iters = m + 1;
    free(arglow); free(classes); store_free(&s);
    return rc;
}

/* ----------------------------------------------------------------- ph_row */
ORACLE_API int oracle_ph_row(int64_t m, const int64_t *colptr, const int32_t *rows,
                             int32_t *low, int32_t *ess, oracle_stats_t *st) {
    oracle_stats_t dummy; if (!st) st = &dummy;
    memset(st, 0, sizeof(*st));
    store_t s; dims_t d; int32_t *pivots, *classes;
    if (store_init(&s, m, colptr, rows, st)) return ORC_NOMEM;
    if (dims_init(&d, m, colptr)) { store_free(&s); return ORC_NOMEM; }
    if (alloc_vecs(m, &pivots, &classes)) { store_free(&s); dims_free(&d); return ORC_NOMEM; }
    int32_t *nb = (int32_t *)malloc(sizeof(int32_t) * (m ? m : 1));
    if (!nb) { free(pivots); free(classes); dims_free(&d); store_free(&s); return ORC_NOMEM; }
    for (int64_t j = 0; j < m; j++) { low[j] = store_low(&s, j); ess[j] = 1; }
    for (int64_t j = 0; j < m; j++)
        if (low[j] != -1 && (pivots[low[j]] == -1 || j < pivots[low[j]])) pivots[low[j]] = (int32_t)j;
    double t0 = now_s();
    int rc = ORC_OK;
    for (int64_t i = m - 1; i > -1 && rc == ORC_OK; i--) {
        int32_t pivot = pivots[i];
        if (pivot != -1) {
            /* get_neighbours_position_host: later columns of the pivot's
             * dimension list whose low equals the pivot's, in column order */
            int64_t nn = 0;
            for (int32_t c = d.next[pivot]; c != -1; c = d.next[c])
                if (low[c] == low[pivot]) nb[nn++] = c;
            /* left_to_right_neighbours_host */
            for (int64_t l = 0; l < nn; l++) {
                int32_t j = nb[l];
                if (low[j] > -1) ess[low[j]] = 0;
                ess[pivot] = 0; ess[low[pivot]] = 0;
                int32_t nl = store_add(&s, pivot, j);
                if (nl == -2) { rc = ORC_NOMEM; break; }
                low[j] = nl;
                if (nl != -1 && (pivots[nl] == -1 || j < pivots[nl])) pivots[nl] = j;
                /* the reference reads pivots[low[j]] even when low[j] == -1
                 * (an out-of-bounds read); a zero column is never a pivot */
                if (nl != -1 && pivots[nl] == j) { classes[j] = -1; classes[nl] = 1; ess[j] = 0; ess[nl] = 0; }
            }
        }
        if (i == 0) {
            for (int64_t jj = 0; jj < m; jj++)
                if (low[jj] > -1) { ess[jj] = 0; ess[low[jj]] = 0; classes[jj] = -1; classes[low[jj]] = 1; }
            for (int64_t jj = 0; jj < m; jj++)
                if (ess[jj] == 1 && classes[jj] == 0) classes[jj] = 2;
        }
        st->columns_done++;
    }
    st->seconds = now_s() - t0; st->iters = m + 1;
    free(nb); free(pivots); free(classes); dims_free(&d); store_free(&s);
    return rc;
}

/* -------------------------------------------------------------------- pms */
/* beta.cu:2-15: left[i] = first column holding row i; beta[j] = the largest
 * row whose first column is j. */
static void create_beta(int64_t m, const int64_t *colptr, const int32_t *rows, int32_t *beta, int32_t *left) {
    for (int64_t i = 0; i < m; i++) { left[i] = -1; beta[i] = -1; }
    for (int64_t j = 0; j < m; j++)
        for (int64_t k = colptr[j]; k < colptr[j + 1]; k++) {
            int32_t r = rows[k];
            if (left[r] == -1) { left[r] = (int32_t)j; if (r > beta[j]) beta[j] = r; }
        }
}

/* transverse_dimensions (pms_functions.cu:55-85): per dimension bucket, in
 * column order, a column whose low is seen for the first time this sweep,
 * which is still unclassified and whose low exceeds the running ceiling of
 * repeated lows is a pivot.  visited[] (size m) and ceil[] (size cdim) are
 * reset by the caller; clear[] marks rows to clear. */
ORACLE_API void oracle_transverse(int64_t m, int32_t cdim, const int32_t *dim, const int32_t *start,
                                  const int32_t *next, int32_t *low, int32_t *arglow, int32_t *classes,
                                  int32_t *clear, int32_t *visited, int32_t *ess, int32_t *ceil) {
    (void)m;
    for (int c = 0; c < cdim; c++)
        for (int32_t j = start[c]; j > -1; j = next[j]) {
            int32_t lj = low[j];
            if (lj > -1) {
                int pos = dim[j] + 1;
                int32_t dc = ceil[pos];
                if (visited[lj] == 0) {
                    if (classes[j] == 0 && lj > dc) {
                        arglow[lj] = j; classes[j] = -1; clear[lj] = 1; ess[lj] = 0; ess[j] = 0;
                    }
                } else {
                    ceil[pos] = lj > dc ? lj : dc;
                }
                visited[lj] = 1;
            }
        }
}

ORACLE_API int oracle_pms(int64_t m, const int64_t *colptr, const int32_t *rows,
                          int32_t *low, int32_t *ess, oracle_stats_t *st) {
    oracle_stats_t dummy; if (!st) st = &dummy;
    memset(st, 0, sizeof(*st));
    store_t s; dims_t d; int32_t *arglow, *classes;
    if (store_init(&s, m, colptr, rows, st)) return ORC_NOMEM;
    if (dims_init(&d, m, colptr)) { store_free(&s); return ORC_NOMEM; }
    if (alloc_vecs(m, &arglow, &classes)) { store_free(&s); dims_free(&d); return ORC_NOMEM; }
    int64_t mm = m ? m : 1;
    int32_t *beta = (int32_t *)malloc(sizeof(int32_t) * mm), *left = (int32_t *)malloc(sizeof(int32_t) * mm);
    int32_t *aux = (int32_t *)malloc(sizeof(int32_t) * mm), *clear = (int32_t *)malloc(sizeof(int32_t) * mm);
    int32_t *ceil = (int32_t *)malloc(sizeof(int32_t) * (d.cdim + 1));
    int rc = ORC_OK;
    if (!beta || !left || !aux || !clear || !ceil) { rc = ORC_NOMEM; goto done; }
    for (int64_t j = 0; j < m; j++) { low[j] = store_low(&s, j); ess[j] = 1; }
    create_beta(m, colptr, rows, beta, left);
    double t0 = now_s();
    /* Phase 0: mark_pivots_and_clear (pms_functions.cu:33-53) */
    for (int64_t j = 0; j < m; j++) {
        int32_t lj = low[j], bj = beta[j];
        if (lj == bj && bj > -1) {
            classes[j] = -1; low[lj] = -1; classes[lj] = 1; arglow[lj] = (int32_t)j; ess[lj] = 0; ess[j] = 0;
        }
    }
    int converged = 0; int64_t iter = 1;
    while (!converged) {
        /* Phase I */
        memset(aux, 0, sizeof(int32_t) * mm);
        for (int c = 0; c < d.cdim; c++) ceil[c] = -1;
        memset(clear, 0, sizeof(int32_t) * mm);
        oracle_transverse(m, d.cdim, d.dim, d.start, d.next, low, arglow, classes, clear, aux, ess, ceil);
        for (int64_t i = 0; i < m; i++) if (clear[i] == 1) { low[i] = -1; classes[i] = 1; }
        /* Phase II (pms_functions.cu:87-112), columns in order */
        memset(clear, 0, sizeof(int32_t) * mm);
        for (int64_t j = 0; j < m; j++) {
            int32_t lj = low[j];
            int32_t pivot = lj > -1 ? arglow[lj] : -1;
            while (-1 < pivot && pivot < j && classes[j] == 0) {
                if (low[j] > -1) ess[low[j]] = 0;
                int32_t nl = store_add(&s, pivot, j);
                if (nl == -2) { rc = ORC_NOMEM; goto done; }
                low[j] = nl; lj = nl;
                if (lj > -1) {
                    if (left[lj] == j) { arglow[lj] = (int32_t)j; classes[j] = -1; }
                    clear[lj] = 1;
                    pivot = arglow[lj];
                } else pivot = -1;
            }
        }
        for (int64_t i = 0; i < m; i++) if (clear[i] == 1) { low[i] = -1; classes[i] = 1; }
        /* ess_hat, update_classes (algorithms/kernels.cu:93-124) */
        for (int64_t j = 0; j < m; j++) {
            if (low[j] > -1) ess[low[j]] = 0;
            if (arglow[j] > -1) { ess[arglow[j]] = 0; ess[j] = 0; }
        }
        for (int64_t i = 0; i < m; i++) if (arglow[i] > -1) { classes[arglow[i]] = -1; classes[i] = 1; }
        /* is_reduced (pms_functions.cu:6-27): all lows distinct */
        memset(aux, 0, sizeof(int32_t) * mm);
        converged = 1;
        for (int64_t j = 0; j < m; j++) if (low[j] > -1 && ++aux[low[j]] > 1) converged = 0;
        if (converged) {
            for (int64_t j = 0; j < m; j++) if (low[j] > -1) { ess[j] = 0; ess[low[j]] = 0; }
        }
        iter++;
        if (iter > 4 * m + 16) { rc = ORC_OVERFLOW; break; } /* cannot happen on a boundary matrix */
    }
    st->seconds = now_s() - t0; st->iters = iter;
done:
    free(beta); free(left); free(aux); free(clear); free(ceil);
    free(arglow); free(classes); dims_free(&d); store_free(&s);
    return rc;
}

/* ------------------------------------------------ fixed-slot twist (port) */
/* left_to_right_host (kernels_host.cu:2-52) on the m x p layout. */
static int ltr_fixed(int64_t j0, int64_t j1, int32_t *rmp, int32_t *amp, int32_t *low, int64_t p) {
    int64_t i0 = j0 * p, i1 = j1 * p, e0 = (j0 + 1) * p, e1 = (j1 + 1) * p, o = i1;
    int ok0 = i0 < e0 && rmp[i0] != -1, ok1 = i1 < e1 && rmp[i1] != -1;
    while (ok0 || ok1) {
        if (ok0 && ok1) {
            if (rmp[i0] < rmp[i1]) { if (o >= e1) return ORC_OVERFLOW; amp[o++] = rmp[i0++]; }
            else if (rmp[i1] < rmp[i0]) { if (o >= e1) return ORC_OVERFLOW; amp[o++] = rmp[i1++]; }
            else { i0++; i1++; }
        } else {
            if (ok0) { if (o >= e1) return ORC_OVERFLOW; amp[o++] = rmp[i0++]; }
            if (ok1) { if (o >= e1) return ORC_OVERFLOW; amp[o++] = rmp[i1++]; }
        }
        ok0 = i0 < e0 && rmp[i0] != -1;
        ok1 = i1 < e1 && rmp[i1] != -1;
    }
    int32_t l = -1;
    i1 = j1 * p;
    while (i1 < e1 && amp[i1] != -1) { rmp[i1] = amp[i1]; amp[i1] = -1; l = rmp[i1]; i1++; }
    while (i1 < e1 && rmp[i1] != -1) { rmp[i1] = -1; i1++; }
    low[j1] = l;
    return ORC_OK;
}

/* Twist on the reference layout.  max_columns > 0 stops after that many
 * columns of the reduction order (a bounded sample of the same run) and
 * max_seconds > 0 after that much wall time; stats report what was done. */
ORACLE_API int oracle_twist_fixed_p(int64_t m, const int64_t *colptr, const int32_t *rows, int col_width,
                                    int64_t max_columns, double max_seconds,
                                    int32_t *low, int32_t *ess, oracle_stats_t *st) {
    oracle_stats_t dummy; if (!st) st = &dummy;
    memset(st, 0, sizeof(*st));
    int64_t maxnnz = 0;
    for (int64_t j = 0; j < m; j++) if (colptr[j + 1] - colptr[j] > maxnnz) maxnnz = colptr[j + 1] - colptr[j];
    int64_t p = (int64_t)col_width * maxnnz;
    if (p <= 0) p = 1;
    int32_t *rmp = (int32_t *)malloc(sizeof(int32_t) * m * p), *amp = (int32_t *)malloc(sizeof(int32_t) * m * p);
    dims_t d; int32_t *arglow, *classes;
    if (!rmp || !amp) { free(rmp); free(amp); return ORC_NOMEM; }
    if (dims_init(&d, m, colptr)) { free(rmp); free(amp); return ORC_NOMEM; }
    if (alloc_vecs(m, &arglow, &classes)) { free(rmp); free(amp); dims_free(&d); return ORC_NOMEM; }
    for (int64_t i = 0; i < m * p; i++) { rmp[i] = -1; amp[i] = -1; }
    for (int64_t j = 0; j < m; j++) {
        int64_t n = colptr[j + 1] - colptr[j];
        memcpy(rmp + j * p, rows + colptr[j], sizeof(int32_t) * n);
        low[j] = n ? rows[colptr[j + 1] - 1] : -1;
        ess[j] = 1;
    }
    double t0 = now_s();
    int rc = ORC_OK, stop = 0; int64_t iter = 1;
    for (int dim = d.complex_dim; dim > 0 && !stop; dim--) {
        for (int32_t j = d.start[dim + 1]; j > -1; j = d.next[j]) {
            int32_t lj = low[j];
            while (lj > -1 && arglow[lj] != -1) {
                ess[lj] = 0;
                int64_t j0 = arglow[lj];
                st->additions++;
                if ((rc = ltr_fixed(j0, j, rmp, amp, low, p))) { stop = 1; break; }
                lj = low[j];
            }
            if (stop) break;
            if (lj > -1) arglow[lj] = j;
            if (low[j] > -1) low[low[j]] = -1;
            if (low[j] > -1) { classes[j] = -1; classes[low[j]] = 1; ess[j] = 0; ess[low[j]] = 0; }
            else classes[j] = 1;
            iter++; st->columns_done++;
            if (max_columns > 0 && st->columns_done >= max_columns) { stop = 1; break; }
            if (max_seconds > 0 && (st->columns_done & 1023) == 0 && now_s() - t0 > max_seconds) { stop = 1; break; }
        }
    }
    st->seconds = now_s() - t0; st->iters = iter;
    free(rmp); free(amp); free(arglow); free(classes); dims_free(&d);
    return rc;
}

/* Reference-style initial setup, exposed for tests of the device setup
 * kernels: low from the last entry, beta/left as beta.cu:2-15, dims. */
ORACLE_API int oracle_setup(int64_t m, const int64_t *colptr, const int32_t *rows, int32_t *low,
                            int32_t *beta, int32_t *left, int32_t *dim, int32_t *complex_dim) {
    for (int64_t j = 0; j < m; j++) {
        low[j] = colptr[j + 1] > colptr[j] ? rows[colptr[j + 1] - 1] : -1;
        dim[j] = (int32_t)(colptr[j + 1] - colptr[j]) - 1;
    }
    int32_t cd = -1;
    for (int64_t j = 0; j < m; j++) if (dim[j] > cd) cd = dim[j];
    *complex_dim = cd;
    create_beta(m, colptr, rows, beta, left);
    return ORC_OK;
}
