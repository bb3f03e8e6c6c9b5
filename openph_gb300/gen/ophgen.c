/*
 * ophgen — seeded generators of filtered simplicial complexes and their Z/2
 * boundary matrices, in the canonical column order (value, dimension,
 * lexicographic vertex tuple).
 *
 * These replace the Javaplex streams the reference feeds to `ph`
 * (numerics/utils/example_factory.m:17-114, numerics/utils/stream2cmo.m:1-26):
 * a column per simplex, rows = filtration positions of its facets, rows
 * ascending inside each column.  Output is 0-based CSC (int64 colptr, int32
 * rows); the 1-based COO the `openph()` entry point takes is a view of it.
 *
 * Host code only.  Built with -ffp-contract=off so that the FP64 distances
 * (and therefore the column order) are the same on x86-64 and aarch64; the
 * only libm calls are log/sqrt/cos/sin in the point samplers.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OPHGEN_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ RNG */
/* xoshiro256** seeded by splitmix64; uniform doubles on [0,1) from the top
 * 53 bits; normals by the Marsaglia polar method.                         */
typedef struct { uint64_t s[4]; int has_spare; double spare; } oph_rng;

static uint64_t splitmix64(uint64_t *x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static void rng_seed(oph_rng *r, uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) r->s[i] = splitmix64(&x);
    r->has_spare = 0;
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t rng_next(oph_rng *r) {
    uint64_t *s = r->s;
    uint64_t res = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return res;
}
static double rng_uniform(oph_rng *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static double rng_normal(oph_rng *r) {
    if (r->has_spare) { r->has_spare = 0; return r->spare; }
    double u, v, s;
    do {
        u = 2.0 * rng_uniform(r) - 1.0;
        v = 2.0 * rng_uniform(r) - 1.0;
        s = u * u + v * v;
    } while (s >= 1.0 || s == 0.0);
    double f = sqrt(-2.0 * log(s) / s);
    r->spare = v * f; r->has_spare = 1;
    return u * f;
}

OPHGEN_API uint64_t oph_rng_u64(uint64_t seed, int64_t n, uint64_t *out) {
    oph_rng r; rng_seed(&r, seed);
    for (int64_t i = 0; i < n; i++) out[i] = rng_next(&r);
    return 0;
}

/* --------------------------------------------------------- point clouds */
OPHGEN_API void oph_points_cube(int n, int d, uint64_t seed, double *out) {
    oph_rng r; rng_seed(&r, seed);
    for (int i = 0; i < n * d; i++) out[i] = rng_uniform(&r);
}

/* Torus in R^3 with tube radius r around a circle of radius R in the xy
 * plane, angles uniform, plus isotropic Gaussian noise of std sigma. */
OPHGEN_API void oph_points_torus(int n, double R, double rr, double sigma, uint64_t seed, double *out) {
    oph_rng g; rng_seed(&g, seed);
    const double two_pi = 6.283185307179586476925286766559;
    for (int i = 0; i < n; i++) {
        double th = two_pi * rng_uniform(&g), ph = two_pi * rng_uniform(&g);
        double x = (R + rr * cos(ph)) * cos(th);
        double y = (R + rr * cos(ph)) * sin(th);
        double z = rr * sin(ph);
        out[3 * i + 0] = x + sigma * rng_normal(&g);
        out[3 * i + 1] = y + sigma * rng_normal(&g);
        out[3 * i + 2] = z + sigma * rng_normal(&g);
    }
}

/* Unit circle in the xy plane of R^3 plus isotropic Gaussian noise. */
OPHGEN_API void oph_points_circle(int n, double sigma, uint64_t seed, double *out) {
    oph_rng g; rng_seed(&g, seed);
    const double two_pi = 6.283185307179586476925286766559;
    for (int i = 0; i < n; i++) {
        double th = two_pi * rng_uniform(&g);
        out[3 * i + 0] = cos(th) + sigma * rng_normal(&g);
        out[3 * i + 1] = sin(th) + sigma * rng_normal(&g);
        out[3 * i + 2] = sigma * rng_normal(&g);
    }
}

/* Mirror an index about the border pixels (period 2n - 2), for any offset. */
static int reflect_index(int i, int n) {
    if (n == 1) return 0;
    int p = 2 * n - 2;
    i %= p;
    if (i < 0) i += p;
    return i < n ? i : p - i;
}

/* i.i.d. N(0,1) noise smoothed by a separable Gaussian of std sigma pixels
 * (kernel radius ceil(4 sigma), edges handled by reflection about the border
 * pixel), accumulated in FP64 and stored as FP32. */
OPHGEN_API int oph_image_smoothed(int h, int w, double sigma, uint64_t seed, float *out) {
    oph_rng g; rng_seed(&g, seed);
    double *a = (double *)malloc(sizeof(double) * (size_t)h * w);
    double *b = (double *)malloc(sizeof(double) * (size_t)h * w);
    if (!a || !b) { free(a); free(b); return -1; }
    for (int64_t i = 0; i < (int64_t)h * w; i++) a[i] = rng_normal(&g);
    int rad = sigma > 0 ? (int)ceil(4.0 * sigma) : 0;
    double *k = (double *)malloc(sizeof(double) * (2 * rad + 1));
    double ks = 0;
    for (int t = -rad; t <= rad; t++) { k[t + rad] = sigma > 0 ? exp(-0.5 * t * t / (sigma * sigma)) : 1.0; ks += k[t + rad]; }
    for (int t = 0; t <= 2 * rad; t++) k[t] /= ks;
#define REFL(i, n) reflect_index((i), (n))
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            double s = 0;
            for (int t = -rad; t <= rad; t++) { int xx = REFL(x + t, w); s += k[t + rad] * a[(int64_t)y * w + xx]; }
            b[(int64_t)y * w + x] = s;
        }
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            double s = 0;
            for (int t = -rad; t <= rad; t++) { int yy = REFL(y + t, h); s += k[t + rad] * b[(int64_t)yy * w + x]; }
            out[(int64_t)y * w + x] = (float)s;
        }
#undef REFL
    free(k); free(a); free(b);
    return 0;
}

/* ------------------------------------------------------------ complexes */
typedef struct {
    int64_t m, nnz;
    int64_t *colptr; /* m+1 */
    int32_t *rows;   /* nnz, 0-based, ascending within a column */
    double *value;   /* m, filtration value */
    int8_t *dim;     /* m, simplex dimension (0 vertex, 1 edge, 2 triangle) */
} oph_complex_t;

OPHGEN_API void oph_complex_free(oph_complex_t *c) {
    if (!c) return;
    free(c->colptr); free(c->rows); free(c->value); free(c->dim);
    memset(c, 0, sizeof(*c));
}

/* A simplex record before sorting: key = (value bits, dim/lex word). */
typedef struct { uint64_t vbits; uint64_t lex; int64_t id; } rec_t;

static inline uint64_t dbits(double v) {
    /* value >= 0 (distances, or values shifted by the caller) -> IEEE bits are
     * monotone; map negatives too so the order is total. */
    uint64_t u; memcpy(&u, &v, 8);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
static int rec_cmp(const void *pa, const void *pb) {
    const rec_t *a = (const rec_t *)pa, *b = (const rec_t *)pb;
    if (a->vbits != b->vbits) return a->vbits < b->vbits ? -1 : 1;
    if (a->lex != b->lex) return a->lex < b->lex ? -1 : 1;
    return (a->id > b->id) - (a->id < b->id);
}
/* dim in the top bits, then up to three 20-bit vertex ids (n <= 2^20). */
static inline uint64_t lexkey(int dim, uint32_t a, uint32_t b, uint32_t c) {
    return ((uint64_t)dim << 60) | ((uint64_t)a << 40) | ((uint64_t)b << 20) | (uint64_t)c;
}

/* Sort the records, then emit the boundary matrix.  facets[f*3 + k] holds
 * the pre-sort ids of the facets of pre-sort simplex f (-1 = none). */
static int emit_sorted(int64_t m, rec_t *recs, const int64_t *facets, const double *val,
                       const int8_t *dims, oph_complex_t *out) {
    qsort(recs, (size_t)m, sizeof(rec_t), rec_cmp);
    int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * m);
    if (!pos) return -1;
    for (int64_t r = 0; r < m; r++) pos[recs[r].id] = r;
    int64_t nnz = 0;
    for (int64_t r = 0; r < m; r++) nnz += dims[recs[r].id] > 0 ? dims[recs[r].id] + 1 : 0;
    out->m = m; out->nnz = nnz;
    out->colptr = (int64_t *)malloc(sizeof(int64_t) * (m + 1));
    out->rows = (int32_t *)malloc(sizeof(int32_t) * (nnz ? nnz : 1));
    out->value = (double *)malloc(sizeof(double) * m);
    out->dim = (int8_t *)malloc(m);
    if (!out->colptr || !out->rows || !out->value || !out->dim) { free(pos); oph_complex_free(out); return -1; }
    int64_t k = 0;
    for (int64_t r = 0; r < m; r++) {
        int64_t id = recs[r].id;
        out->colptr[r] = k;
        out->value[r] = val[id];
        out->dim[r] = dims[id];
        int d = dims[id];
        if (d > 0) {
            int32_t f[3]; int nf = d + 1;
            for (int t = 0; t < nf; t++) f[t] = (int32_t)pos[facets[id * 3 + t]];
            for (int a = 1; a < nf; a++) { int32_t x = f[a]; int b = a - 1; while (b >= 0 && f[b] > x) { f[b + 1] = f[b]; b--; } f[b + 1] = x; }
            for (int t = 0; t < nf; t++) out->rows[k++] = f[t];
        }
    }
    out->colptr[m] = k;
    free(pos);
    return 0;
}

static inline double dist(const double *p, int d, int a, int b) {
    double s = 0;
    for (int t = 0; t < d; t++) { double x = p[a * d + t] - p[b * d + t]; s += x * x; }
    return sqrt(s);
}

/* Vietoris–Rips complex of dimension <= 2 with edges of length <= thr
 * (thr = +inf gives the full 2-skeleton).  Value of a simplex = its largest
 * pairwise FP64 Euclidean distance; vertices have value 0. */
OPHGEN_API int oph_rips(const double *pts, int n, int d, double thr, oph_complex_t *out) {
    memset(out, 0, sizeof(*out));
    if (n <= 0 || n >= (1 << 20)) return -1;
    double *D = (double *)malloc(sizeof(double) * (size_t)n * n);
    int64_t *eid = (int64_t *)malloc(sizeof(int64_t) * (size_t)n * n);
    if (!D || !eid) { free(D); free(eid); return -1; }
    int64_t E = 0, T = 0;
    for (int a = 0; a < n; a++)
        for (int b = a + 1; b < n; b++) {
            double x = dist(pts, d, a, b);
            D[(size_t)a * n + b] = D[(size_t)b * n + a] = x;
            eid[(size_t)a * n + b] = eid[(size_t)b * n + a] = (x <= thr) ? E++ : -1;
        }
    for (int a = 0; a < n; a++)
        for (int b = a + 1; b < n; b++) {
            if (eid[(size_t)a * n + b] < 0) continue;
            for (int c = b + 1; c < n; c++)
                if (eid[(size_t)a * n + c] >= 0 && eid[(size_t)b * n + c] >= 0) T++;
        }
    int64_t m = n + E + T;
    rec_t *recs = (rec_t *)malloc(sizeof(rec_t) * m);
    int64_t *fac = (int64_t *)malloc(sizeof(int64_t) * 3 * m);
    double *val = (double *)malloc(sizeof(double) * m);
    int8_t *dims = (int8_t *)malloc(m);
    if (!recs || !fac || !val || !dims) { free(D); free(eid); free(recs); free(fac); free(val); free(dims); return -1; }
    for (int a = 0; a < n; a++) {
        val[a] = 0.0; dims[a] = 0; fac[a * 3] = fac[a * 3 + 1] = fac[a * 3 + 2] = -1;
        recs[a].vbits = dbits(0.0); recs[a].lex = lexkey(0, a, 0, 0); recs[a].id = a;
    }
    for (int a = 0; a < n; a++)
        for (int b = a + 1; b < n; b++) {
            int64_t e = eid[(size_t)a * n + b];
            if (e < 0) continue;
            int64_t id = n + e;
            double v = D[(size_t)a * n + b];
            val[id] = v; dims[id] = 1;
            fac[id * 3] = a; fac[id * 3 + 1] = b; fac[id * 3 + 2] = -1;
            recs[id].vbits = dbits(v); recs[id].lex = lexkey(1, a, b, 0); recs[id].id = id;
        }
    int64_t t = n + E;
    for (int a = 0; a < n; a++)
        for (int b = a + 1; b < n; b++) {
            int64_t eab = eid[(size_t)a * n + b];
            if (eab < 0) continue;
            for (int c = b + 1; c < n; c++) {
                int64_t eac = eid[(size_t)a * n + c], ebc = eid[(size_t)b * n + c];
                if (eac < 0 || ebc < 0) continue;
                double v = D[(size_t)a * n + b];
                if (D[(size_t)a * n + c] > v) v = D[(size_t)a * n + c];
                if (D[(size_t)b * n + c] > v) v = D[(size_t)b * n + c];
                val[t] = v; dims[t] = 2;
                fac[t * 3] = n + eab; fac[t * 3 + 1] = n + eac; fac[t * 3 + 2] = n + ebc;
                recs[t].vbits = dbits(v); recs[t].lex = lexkey(2, a, b, c); recs[t].id = t;
                t++;
            }
        }
    free(D); free(eid);
    int rc = emit_sorted(m, recs, fac, val, dims, out);
    free(recs); free(fac); free(val); free(dims);
    return rc;
}

/* k-th smallest (0-based) of x[0..n) by quickselect; x is permuted. */
static double kth_smallest(double *x, int64_t n, int64_t k) {
    int64_t lo = 0, hi = n - 1;
    uint64_t st = 0x1234567ull;
    while (lo < hi) {
        int64_t p = lo + (int64_t)(splitmix64(&st) % (uint64_t)(hi - lo + 1));
        double piv = x[p];
        int64_t i = lo, j = hi;
        while (i <= j) {
            while (x[i] < piv) i++;
            while (x[j] > piv) j--;
            if (i <= j) { double tmp = x[i]; x[i] = x[j]; x[j] = tmp; i++; j--; }
        }
        if (k <= j) hi = j; else if (k >= i) lo = i; else return x[k];
    }
    return x[k];
}

/* Edge-length threshold t such that the Rips complex of dimension <= 2 with
 * edges <= t has about target_m simplices: the (target_m - n)-th smallest of
 * all edge lengths and triangle diameters together. */
OPHGEN_API double oph_rips_threshold(const double *pts, int n, int d, int64_t target_m) {
    int64_t E = (int64_t)n * (n - 1) / 2, T = (int64_t)n * (n - 1) * (n - 2) / 6;
    int64_t tot = E + T, k = target_m - n - 1;
    if (k < 0) return 0.0;
    if (k >= tot) return INFINITY;
    double *D = (double *)malloc(sizeof(double) * (size_t)n * n);
    double *all = (double *)malloc(sizeof(double) * tot);
    if (!D || !all) { free(D); free(all); return NAN; }
    int64_t q = 0;
    for (int a = 0; a < n; a++)
        for (int b = a + 1; b < n; b++) { double x = dist(pts, d, a, b); D[(size_t)a * n + b] = x; all[q++] = x; }
    for (int a = 0; a < n; a++)
        for (int b = a + 1; b < n; b++)
            for (int c = b + 1; c < n; c++) {
                double v = D[(size_t)a * n + b];
                if (D[(size_t)a * n + c] > v) v = D[(size_t)a * n + c];
                if (D[(size_t)b * n + c] > v) v = D[(size_t)b * n + c];
                all[q++] = v;
            }
    double t = kth_smallest(all, tot, k);
    free(D); free(all);
    return t;
}

/* Lower-star filtration of an h x w FP32 image on the Freudenthal
 * triangulation (diagonals (y,x)-(y+1,x+1)).  Vertex id = y*w + x; the value
 * of a simplex is the max of its vertex values (compared in FP64 after the
 * exact FP32->FP64 widening). */
OPHGEN_API int oph_lower_star(const float *img, int h, int w, oph_complex_t *out) {
    memset(out, 0, sizeof(*out));
    if (h < 2 || w < 2 || (int64_t)h * w >= (1 << 20)) return -1;
    int64_t V = (int64_t)h * w;
    int64_t EH = (int64_t)h * (w - 1), EV = (int64_t)(h - 1) * w, ED = (int64_t)(h - 1) * (w - 1);
    int64_t E = EH + EV + ED, T = 2 * ED, m = V + E + T;
    rec_t *recs = (rec_t *)malloc(sizeof(rec_t) * m);
    int64_t *fac = (int64_t *)malloc(sizeof(int64_t) * 3 * m);
    double *val = (double *)malloc(sizeof(double) * m);
    int8_t *dims = (int8_t *)malloc(m);
    if (!recs || !fac || !val || !dims) { free(recs); free(fac); free(val); free(dims); return -1; }
#define VID(y, x) ((int64_t)(y) * w + (x))
#define EHID(y, x) (V + (int64_t)(y) * (w - 1) + (x))
#define EVID(y, x) (V + EH + (int64_t)(y) * w + (x))
#define EDID(y, x) (V + EH + EV + (int64_t)(y) * (w - 1) + (x))
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int64_t id = VID(y, x);
            val[id] = (double)img[id]; dims[id] = 0; fac[id * 3] = fac[id * 3 + 1] = fac[id * 3 + 2] = -1;
            recs[id].vbits = dbits(val[id]); recs[id].lex = lexkey(0, (uint32_t)id, 0, 0); recs[id].id = id;
        }
#define SET_EDGE(ID, A, B) do { int64_t _id = (ID); uint32_t _a = (uint32_t)(A), _b = (uint32_t)(B); \
        if (_a > _b) { uint32_t _t = _a; _a = _b; _b = _t; } \
        double _v = val[_a] > val[_b] ? val[_a] : val[_b]; \
        val[_id] = _v; dims[_id] = 1; fac[_id * 3] = _a; fac[_id * 3 + 1] = _b; fac[_id * 3 + 2] = -1; \
        recs[_id].vbits = dbits(_v); recs[_id].lex = lexkey(1, _a, _b, 0); recs[_id].id = _id; } while (0)
    for (int y = 0; y < h; y++)
        for (int x = 0; x + 1 < w; x++) SET_EDGE(EHID(y, x), VID(y, x), VID(y, x + 1));
    for (int y = 0; y + 1 < h; y++)
        for (int x = 0; x < w; x++) SET_EDGE(EVID(y, x), VID(y, x), VID(y + 1, x));
    for (int y = 0; y + 1 < h; y++)
        for (int x = 0; x + 1 < w; x++) SET_EDGE(EDID(y, x), VID(y, x), VID(y + 1, x + 1));
#undef SET_EDGE
    int64_t t = V + E;
    for (int y = 0; y + 1 < h; y++)
        for (int x = 0; x + 1 < w; x++) {
            /* upper: (y,x),(y,x+1),(y+1,x+1): edges H(y,x), V(y,x+1), D(y,x)
             * lower: (y,x),(y+1,x),(y+1,x+1): edges V(y,x), H(y+1,x), D(y,x) */
            for (int up = 1; up >= 0; up--) {
                uint32_t a = (uint32_t)VID(y, x);
                uint32_t b = up ? (uint32_t)VID(y, x + 1) : (uint32_t)VID(y + 1, x);
                uint32_t c = (uint32_t)VID(y + 1, x + 1);
                double v = val[a]; if (val[b] > v) v = val[b]; if (val[c] > v) v = val[c];
                val[t] = v; dims[t] = 2;
                if (up) { fac[t * 3] = EHID(y, x); fac[t * 3 + 1] = EVID(y, x + 1); }
                else { fac[t * 3] = EVID(y, x); fac[t * 3 + 1] = EHID(y + 1, x); }
                fac[t * 3 + 2] = EDID(y, x);
                /* a < b < c holds for both triangles in row-major ids */
                recs[t].vbits = dbits(v); recs[t].lex = lexkey(2, a, b, c); recs[t].id = t;
                t++;
            }
        }
#undef VID
#undef EHID
#undef EVID
#undef EDID
    int rc = emit_sorted(m, recs, fac, val, dims, out);
    free(recs); free(fac); free(val); free(dims);
    return rc;
}

/* ------------------------------------------------------------- batches */
/* One instance of the mixed batch: n points uniform in [0,1]^3 (even seed) or
 * on a noisy unit circle in R^3 (odd seed, sigma = 0.05), full 2-skeleton. */
static int mixed_instance(int n, uint64_t seed, oph_complex_t *out) {
    double *pts = (double *)malloc(sizeof(double) * 3 * n);
    if (!pts) return -1;
    if (seed % 2 == 0) oph_points_cube(n, 3, seed, pts);
    else oph_points_circle(n, 0.05, seed, pts);
    int rc = oph_rips(pts, n, 3, INFINITY, out);
    free(pts);
    return rc;
}

#include <pthread.h>

typedef struct {
    int count, nthreads, tid;
    const int *npts;
    const uint64_t *seeds;
    oph_complex_t *inst;
    int rc;
} batch_job_t;

static void *batch_worker(void *p) {
    batch_job_t *j = (batch_job_t *)p;
    for (int b = j->tid; b < j->count; b += j->nthreads)
        if (mixed_instance(j->npts[b], j->seeds[b], &j->inst[b]) != 0) j->rc = -1;
    return NULL;
}

typedef struct {
    int count, nthreads, tid;
    oph_complex_t *inst;
    const int64_t *col_off, *nnz_off;
    int64_t *colptr;
    int32_t *rows;
} cat_job_t;

static void *cat_worker(void *p) {
    cat_job_t *j = (cat_job_t *)p;
    for (int b = j->tid; b < j->count; b += j->nthreads) {
        oph_complex_t *c = &j->inst[b];
        for (int64_t k = 0; k < c->m; k++) j->colptr[j->col_off[b] + k] = j->nnz_off[b] + c->colptr[k];
        memcpy(j->rows + j->nnz_off[b], c->rows, sizeof(int32_t) * c->nnz);
        oph_complex_free(c);
    }
    return NULL;
}

/* `count` instances of the mixed batch generated on `nthreads` threads and
 * concatenated: col_off[count+1] column offsets, out->colptr (global, m+1)
 * and out->rows holding each instance's LOCAL row ids.  out->value and
 * out->dim are not filled (NULL). */
OPHGEN_API int oph_rips_mixed_batch(int count, const int *npts, const uint64_t *seeds, int nthreads,
                                    int64_t *col_off, oph_complex_t *out) {
    memset(out, 0, sizeof(*out));
    if (count <= 0) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    oph_complex_t *inst = (oph_complex_t *)calloc(count, sizeof(oph_complex_t));
    int64_t *nnz_off = (int64_t *)malloc(sizeof(int64_t) * (count + 1));
    pthread_t th[256];
    batch_job_t bj[256];
    if (!inst || !nnz_off) { free(inst); free(nnz_off); return -1; }
    for (int t = 0; t < nthreads; t++) {
        bj[t] = (batch_job_t){count, nthreads, t, npts, seeds, inst, 0};
        pthread_create(&th[t], NULL, batch_worker, &bj[t]);
    }
    int rc = 0;
    for (int t = 0; t < nthreads; t++) { pthread_join(th[t], NULL); rc |= bj[t].rc; }
    if (rc) {
        for (int b = 0; b < count; b++) oph_complex_free(&inst[b]);
        free(inst); free(nnz_off);
        return -1;
    }
    col_off[0] = 0; nnz_off[0] = 0;
    for (int b = 0; b < count; b++) { col_off[b + 1] = col_off[b] + inst[b].m; nnz_off[b + 1] = nnz_off[b] + inst[b].nnz; }
    out->m = col_off[count]; out->nnz = nnz_off[count];
    out->colptr = (int64_t *)malloc(sizeof(int64_t) * (out->m + 1));
    out->rows = (int32_t *)malloc(sizeof(int32_t) * (out->nnz ? out->nnz : 1));
    if (!out->colptr || !out->rows) {
        for (int b = 0; b < count; b++) oph_complex_free(&inst[b]);
        free(inst); free(nnz_off); oph_complex_free(out);
        return -1;
    }
    cat_job_t cj[256];
    for (int t = 0; t < nthreads; t++) {
        cj[t] = (cat_job_t){count, nthreads, t, inst, col_off, nnz_off, out->colptr, out->rows};
        pthread_create(&th[t], NULL, cat_worker, &cj[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    out->colptr[out->m] = out->nnz;
    free(inst); free(nnz_off);
    return 0;
}
