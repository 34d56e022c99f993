/*
 * fair_oracle.c -- CPU oracle for the AIR reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see fair_oracle.h): a serial FP64 restatement of
 * the reference Fortran, line by line, used to check the GPU library. Build
 * with -O2 -ffp-contract=off so that no multiply-add is fused: the reference
 * built with the default x86-64 gfortran flags rounds every product and sum.
 *
 * Parity status: UNPINNED by the reference (no golden vectors exist and the
 * Fortran cannot be compiled here); pinned by analytic known-answer tests.
 *
 * Citations are file:line in the reference project.
 */
#include "fair_oracle.h"

#include <math.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double PI = 3.141592653589793; /* = 4*atan(1d0), system_generation.f90:4 */

/* gfortran MAX/MIN: the result is the non-NaN argument when one is NaN. */
static inline double fmax_f(double a, double b) { return (b > a || a != a) ? b : a; }
static inline double fmin_f(double a, double b) { return (b < a || a != a) ? b : a; }

/* ------------------------------------------------------------------------- */
/* Project PRNG: SplitMix64 (Steele, Lea & Flood 2014), one global stream.    */
/* It stands in for the unseeded Fortran random_number stream; every consumer */
/* draws from it in the same order as the reference draws from random_number. */
/* ------------------------------------------------------------------------- */
static uint64_t g_seed = 0, g_ctr = 0;

void or_random_seed(uint64_t seed) { g_seed = seed; g_ctr = 0; }
uint64_t or_random_counter(void) { return g_ctr; }

static uint64_t sm64(uint64_t seed, uint64_t k) {
    uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double or_random_number(void) {
    uint64_t z = sm64(g_seed, g_ctr++);
    return (double)(z >> 11) * 0x1.0p-53; /* uniform on [0,1) */
}

/* ------------------------------------------------------------------------- */
/* system_generation.f90                                                     */
/* ------------------------------------------------------------------------- */

/* linspace, system_generation.f90:17-35: x(i) = c*i + d with d = a - c. */
void or_linspace(double a, double b, int n, double *x) {
    double c = (b - a) / (n - 1);
    double d = a - c;
    for (int i = 1; i <= n; ++i) x[i - 1] = c * i + d;
}

/* quicksort, system_generation.f90:37-77 (Hoare partition, middle pivot,
 * carrying the index permutation). Arrays are addressed 1-based here. */
static void quicksort1(double *a, int32_t *ind, int f, int l) {
    double x = a[(f + l) / 2], t;
    int i = f, j = l, m;
    for (;;) {
        while (a[i] < x) i++;
        while (x < a[j]) j--;
        if (i >= j) break;
        t = a[i]; a[i] = a[j]; a[j] = t;
        m = ind[i]; ind[i] = ind[j]; ind[j] = m;
        i++;
        j--;
    }
    if (f < i - 1) quicksort1(a, ind, f, i - 1);
    if (j + 1 < l) quicksort1(a, ind, j + 1, l);
}

void or_csr_free(or_csr *A) {
    free(A->IA); free(A->JA); free(A->vA);
    A->IA = NULL; A->JA = NULL; A->vA = NULL;
}

/* Work arrays for one ray (sizes n+1 and 2n+2, 1-based addressing). */
typedef struct {
    int n;
    double *x, *y, *tx, *yx, *ty, *xy, *t, *xxy, *yxy, *pxx, *pyy, *txx, *tyy;
    int32_t *ind;
} ray_work;

static int ray_work_alloc(ray_work *w, int n) {
    w->n = n;
    size_t a1 = (size_t)(n + 2), a2 = (size_t)(2 * n + 3);
    w->x = calloc(a1, 8); w->y = calloc(a1, 8); w->tx = calloc(a1, 8);
    w->yx = calloc(a1, 8); w->ty = calloc(a1, 8); w->xy = calloc(a1, 8);
    w->t = calloc(a2, 8); w->xxy = calloc(a2, 8); w->yxy = calloc(a2, 8);
    w->pxx = calloc(a2, 8); w->pyy = calloc(a2, 8);
    w->txx = calloc(a2, 8); w->tyy = calloc(a2, 8);
    w->ind = calloc(a2, 4);
    return (w->x && w->y && w->tx && w->yx && w->ty && w->xy && w->t && w->xxy &&
            w->yxy && w->pxx && w->pyy && w->txx && w->tyy && w->ind) ? 0 : -1;
}

static void ray_work_free(ray_work *w) {
    free(w->x); free(w->y); free(w->tx); free(w->yx); free(w->ty); free(w->xy);
    free(w->t); free(w->xxy); free(w->yxy); free(w->pxx); free(w->pyy);
    free(w->txx); free(w->tyy); free(w->ind);
}

/*
 * One ray of paralleltomo/fanlineartomo: intersections, sort, in-box filter.
 * system_generation.f90:163-193 (fan) and :357-387 (parallel), identical code.
 * Returns n_int, the number of in-box points left in txx/tyy (1-based).
 */
static int ray_points(ray_work *w, double a, double b, double x0th, double y0th) {
    const int n = w->n, np = n + 1, nt = 2 * n + 2;
    for (int k = 1; k <= np; ++k) {
        w->tx[k] = (w->x[k] - x0th) / a;
        w->yx[k] = b * w->tx[k] + y0th;
        w->ty[k] = (w->y[k] - y0th) / b;
        w->xy[k] = a * w->ty[k] + x0th;
    }
    for (int k = 1; k <= np; ++k) {
        w->t[k] = w->tx[k];       w->t[np + k] = w->ty[k];
        w->xxy[k] = w->x[k];      w->xxy[np + k] = w->xy[k];
        w->yxy[k] = w->yx[k];     w->yxy[np + k] = w->y[k];
    }
    for (int k = 1; k <= nt; ++k) w->ind[k] = k;
    quicksort1(w->t, w->ind, 1, nt);
    for (int k = 1; k <= nt; ++k) {
        w->pxx[k] = w->xxy[w->ind[k]];
        w->pyy[k] = w->yxy[w->ind[k]];
    }
    const double lo = -.5 * n, hi = .5 * n;
    int n_int = 0;
    for (int k = 1; k <= nt; ++k) {
        if (w->pxx[k] >= lo && w->pxx[k] <= hi && w->pyy[k] >= lo && w->pyy[k] <= hi) {
            n_int++;
            w->txx[n_int] = w->pxx[k];
            w->tyy[n_int] = w->pyy[k];
        }
    }
    return n_int;
}

/*
 * Segments of one ray: the "remove double points" loop and the column rule,
 * system_generation.f90:196-203/:279-297 (fan) and :390-397/:463-482
 * (parallel). `excluded` is the parallel-beam boundary rule of :393-394.
 * With vA == NULL only counts. Returns the count, or -1 when a column index
 * outside 1..n^2 appears. The reference stops for index 0 ("++ Something went
 * wrong", :293/:478); an index above n^2 (a ray lying on the right or top edge
 * whose direction component is a rounding residue rather than exactly 0, so
 * the boundary rule does not drop it) would be written out of range and read
 * out of bounds by every later product, so it is refused the same way.
 */
static int64_t ray_segments(const ray_work *w, int n_int, int excluded,
                            int32_t *JA, double *vA) {
    const int n = w->n;
    int64_t m = 0;
    for (int k = 1; k <= n_int - 1; ++k) {
        double dx = w->txx[k] - w->txx[k + 1];
        double dy = w->tyy[k] - w->tyy[k + 1];
        double test_val = sqrt(dx * dx + dy * dy);
        if (test_val > 1e-10 && !excluded) {
            if (vA) {
                vA[m] = test_val;
                double xm = .5 * (w->txx[k] + w->txx[k + 1] + n);
                double ym = .5 * (w->tyy[k] + w->tyy[k + 1] + n);
                int32_t ja = (int32_t)floor(xm) * n + (n - (int32_t)floor(ym));
                if (ja < 1 || ja > n * n) return -1;
                JA[m] = ja;
            }
            m++;
        }
    }
    return m;
}

/* Shared two-pass CSR build: count pass, then fill pass (:143-212/:221-302). */
typedef void (*ray_param_fn)(void *ctx, int i, int j, double *a, double *b,
                             double *x0th, double *y0th, int *excluded);

static int build_two_pass(int n, int nth, int p, ray_work *w, ray_param_fn fn,
                          void *ctx, or_csr *A) {
    int64_t m = (int64_t)nth * p;
    A->IA = calloc((size_t)m + 1, sizeof(int64_t));
    if (!A->IA) return OR_ERR_ALLOC;
    A->IA[0] = 0;
    int64_t nnz = 0;
    for (int i = 1; i <= nth; ++i) {
        for (int j = 1; j <= p; ++j) {
            double a, b, x0th, y0th;
            int excl;
            fn(ctx, i, j, &a, &b, &x0th, &y0th, &excl);
            int n_int = ray_points(w, a, b, x0th, y0th);
            int64_t c = ray_segments(w, n_int, excl, NULL, NULL);
            nnz += c;
            int64_t r = (int64_t)(i - 1) * p + j;
            A->IA[r] = A->IA[r - 1] + c;
        }
    }
    A->m = (int32_t)m;
    A->n = n * n;
    A->nnz = nnz;
    A->vA = malloc((size_t)(nnz ? nnz : 1) * sizeof(double));
    A->JA = malloc((size_t)(nnz ? nnz : 1) * sizeof(int32_t));
    if (!A->vA || !A->JA) return OR_ERR_ALLOC;
    int64_t count = 0;
    for (int i = 1; i <= nth; ++i) {
        for (int j = 1; j <= p; ++j) {
            double a, b, x0th, y0th;
            int excl;
            fn(ctx, i, j, &a, &b, &x0th, &y0th, &excl);
            int n_int = ray_points(w, a, b, x0th, y0th);
            int64_t c = ray_segments(w, n_int, excl, A->JA + count, A->vA + count);
            if (c < 0) return OR_ERR_GEOMETRY;
            count += c;
        }
    }
    if (count < nnz) return OR_ERR_GEOMETRY; /* "Didn't hit all elements" */
    return OR_OK;
}

/* paralleltomo per-ray parameters, system_generation.f90:328-363. */
typedef struct { int n, p; const double *theta; double *x0, *y0; } par_ctx;

static void par_params(void *vctx, int i, int j, double *a, double *b,
                       double *x0th, double *y0th, int *excluded) {
    par_ctx *c = (par_ctx *)vctx;
    double th = c->theta[i - 1];
    double ct = cos(th), st = sin(th);
    *x0th = ct * c->x0[j - 1] - st * c->y0[j - 1];
    *y0th = st * c->x0[j - 1] + ct * c->y0[j - 1];
    *a = -st;
    *b = ct;
    *excluded = ((*b == 0.0 && fabs(*y0th - .5 * c->n) < 1e-15) ||
                 (*a == 0.0 && fabs(*x0th - .5 * c->n) < 1e-15));
}

int or_paralleltomo(int n, int nth, int p, const double *theta, or_csr *A) {
    memset(A, 0, sizeof(*A));
    ray_work w;
    if (ray_work_alloc(&w, n)) return OR_ERR_ALLOC;
    double *x0 = malloc(sizeof(double) * p), *y0 = malloc(sizeof(double) * p);
    double d = p - 1;
    or_linspace(-.5 * d, .5 * d, p, x0);
    for (int j = 0; j < p; ++j) y0[j] = 0 * x0[j];
    or_linspace(-.5 * n, .5 * n, n + 1, w.x + 1);
    for (int k = 1; k <= n + 1; ++k) w.y[k] = w.x[k];
    par_ctx ctx = {n, p, theta, x0, y0};
    int st = build_two_pass(n, nth, p, &w, par_params, &ctx, A);
    free(x0); free(y0);
    ray_work_free(&w);
    return st;
}

/* The two-pass build of build_two_pass with the rays split over threads
 * (OpenMP): the same per-ray code, so the result is identical; used to build
 * the large parity and timing inputs. grid holds the n+1 grid lines (the same
 * for x and y). */
static int build_two_pass_mt(int n, int nth, int p, const double *grid, ray_param_fn fn,
                             void *ctx, int nthreads, or_csr *A) {
    int64_t m = (int64_t)nth * p;
    A->IA = calloc((size_t)m + 1, sizeof(int64_t));
    int64_t *cnt = calloc((size_t)(m ? m : 1), sizeof(int64_t));
    if (!A->IA || !cnt) { free(cnt); return OR_ERR_ALLOC; }
    int st = OR_OK;
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
    {
        ray_work w;
        int ok = ray_work_alloc(&w, n) == 0;
        if (!ok) {
#pragma omp atomic write
            st = OR_ERR_ALLOC;
        } else {
            memcpy(w.x + 1, grid, sizeof(double) * (n + 1));
            memcpy(w.y + 1, grid, sizeof(double) * (n + 1));
        }
#pragma omp for schedule(dynamic, 64)
        for (int64_t r = 0; r < m; ++r) {
            if (!ok) continue;
            double a, b, x0th, y0th;
            int excl;
            fn(ctx, (int)(r / p) + 1, (int)(r % p) + 1, &a, &b, &x0th, &y0th, &excl);
            int n_int = ray_points(&w, a, b, x0th, y0th);
            cnt[r] = ray_segments(&w, n_int, excl, NULL, NULL);
        }
#pragma omp single
        {
            for (int64_t r = 0; r < m; ++r) A->IA[r + 1] = A->IA[r] + cnt[r];
            A->nnz = A->IA[m];
            A->vA = malloc(sizeof(double) * (size_t)(A->nnz ? A->nnz : 1));
            A->JA = malloc(sizeof(int32_t) * (size_t)(A->nnz ? A->nnz : 1));
            if (!A->vA || !A->JA) st = OR_ERR_ALLOC;
        }
#pragma omp for schedule(dynamic, 64)
        for (int64_t r = 0; r < m; ++r) {
            if (!ok || st == OR_ERR_ALLOC) continue;
            double a, b, x0th, y0th;
            int excl;
            fn(ctx, (int)(r / p) + 1, (int)(r % p) + 1, &a, &b, &x0th, &y0th, &excl);
            int n_int = ray_points(&w, a, b, x0th, y0th);
            int64_t c = ray_segments(&w, n_int, excl, A->JA + A->IA[r], A->vA + A->IA[r]);
            if (c < 0) {
#pragma omp atomic write
                st = OR_ERR_GEOMETRY;
            }
        }
        if (ok) ray_work_free(&w);
    }
    A->m = (int32_t)m;
    A->n = n * n;
    free(cnt);
    return st;
}

/* paralleltomo with the rays split over threads (identical result). */
int or_paralleltomo_mt(int n, int nth, int p, const double *theta, int nthreads, or_csr *A) {
    memset(A, 0, sizeof(*A));
    double *x0 = malloc(sizeof(double) * p), *y0 = malloc(sizeof(double) * p);
    double *grid = malloc(sizeof(double) * (n + 1));
    if (!x0 || !y0 || !grid) { free(x0); free(y0); free(grid); return OR_ERR_ALLOC; }
    double d = p - 1;
    or_linspace(-.5 * d, .5 * d, p, x0);
    for (int j = 0; j < p; ++j) y0[j] = 0 * x0[j];
    or_linspace(-.5 * n, .5 * n, n + 1, grid);
    par_ctx ctx = {n, p, theta, x0, y0};
    int st = build_two_pass_mt(n, nth, p, grid, par_params, &ctx, nthreads, A);
    free(x0); free(y0); free(grid);
    return st;
}

/* fanlineartomo per-ray parameters, system_generation.f90:98-157. */
typedef struct { double R, x0, y0; const double *theta; double *omega; } fan_ctx;

static void fan_params(void *vctx, int i, int j, double *a, double *b,
                       double *x0th, double *y0th, int *excluded) {
    fan_ctx *c = (fan_ctx *)vctx;
    double th = c->theta[i - 1];
    double ct = cos(th), st = sin(th);
    *x0th = ct * c->x0 - st * c->y0;
    *y0th = st * c->x0 + ct * c->y0;
    double ath = -*x0th / c->R;
    double bth = -*y0th / c->R;
    double om = c->omega[j - 1];
    *a = cos(om) * ath - sin(om) * bth;
    *b = sin(om) * ath + cos(om) * bth;
    *excluded = 0;
}

/* Per-bin ray angles of fanlineartomo, system_generation.f90:114-130.
 * geometry_fix = 0 reproduces the odd-p ray angles of :122 (offset .5 where
 * the even branch at :129 has .5*pi); geometry_fix = 1 uses .5*pi for both. */
static void fan_omega(int p, double dew, double sdn, int geometry_fix, double *omega) {
    if (p % 2 == 1) {
        int h = (p - 1) / 2;
        for (int i = 1; i <= h; ++i) {
            double dep = i * dew;
            omega[h - i] = atan(sdn / dep) - (geometry_fix ? .5 * PI : .5);
            omega[h + i] = .5 * PI - atan(sdn / dep);
        }
        omega[h] = 0.0;
    } else {
        int h = p / 2;
        for (int i = 1; i <= h; ++i) {
            double dep = (i - .5) * dew;
            omega[h - i] = atan(sdn / dep) - .5 * PI;
            omega[h + i - 1] = .5 * PI - atan(sdn / dep);
        }
    }
}

/* fanlineartomo, system_generation.f90:79-307 (grid lines i - n/2 - 1,
 * :104-108; source at (0, R) rotated by theta, :146-157). */
int or_fanlineartomo(int n, int nth, int p, double r, double dw, double sd,
                     const double *theta, int geometry_fix, or_csr *A) {
    memset(A, 0, sizeof(*A));
    ray_work w;
    if (ray_work_alloc(&w, n)) return OR_ERR_ALLOC;
    double R = r * n, dwn = dw * n, sdn = sd * n;
    double dew = dwn / p;
    for (int i = 1; i <= n + 1; ++i) {
        w.x[i] = i - .5 * n - 1.0;
        w.y[i] = i - .5 * n - 1.0;
    }
    double *omega = malloc(sizeof(double) * p);
    if (!omega) { ray_work_free(&w); return OR_ERR_ALLOC; }
    fan_omega(p, dew, sdn, geometry_fix, omega);
    fan_ctx ctx = {R, 0.0, R, theta, omega};
    int st = build_two_pass(n, nth, p, &w, fan_params, &ctx, A);
    free(omega);
    ray_work_free(&w);
    return st;
}

/* fanlineartomo with the rays split over threads (identical result). */
int or_fanlineartomo_mt(int n, int nth, int p, double r, double dw, double sd,
                        const double *theta, int geometry_fix, int nthreads, or_csr *A) {
    memset(A, 0, sizeof(*A));
    double R = r * n, dwn = dw * n, sdn = sd * n;
    double dew = dwn / p;
    double *grid = malloc(sizeof(double) * (n + 1)), *omega = malloc(sizeof(double) * p);
    if (!grid || !omega) { free(grid); free(omega); return OR_ERR_ALLOC; }
    for (int i = 1; i <= n + 1; ++i) grid[i - 1] = i - .5 * n - 1.0;
    fan_omega(p, dew, sdn, geometry_fix, omega);
    fan_ctx ctx = {R, 0.0, R, theta, omega};
    int st = build_two_pass_mt(n, nth, p, grid, fan_params, &ctx, nthreads, A);
    free(grid); free(omega);
    return st;
}

/* add_white_noise, system_generation.f90:709-745 (Newton inverse normal CDF
 * on uniforms drawn from the project stream). */
int or_add_white_noise(int64_t m, const double *b, double eta, double *bt, double *e) {
    const double tol = 1e-14;
    for (int64_t k = 0; k < m; ++k) {
        double u = or_random_number();
        double x = 0.0;
        for (int i = 1; i <= 100; ++i) {
            double f = .5 * (1 + erf(x / sqrt(2.0))) - u;
            double df = sqrt(2.0 / PI) * exp(-.5 * (x * x));
            if (fabs(f / df) < tol) break;
            if (i == 100 && fabs(f / df) > tol) return OR_ERR_NEWTON;
            x = x - f / df;
        }
        e[k] = x;
    }
    double nb = 0, ne = 0;
    for (int64_t k = 0; k < m; ++k) nb += b[k] * b[k];
    for (int64_t k = 0; k < m; ++k) ne += e[k] * e[k];
    nb = sqrt(nb);
    ne = sqrt(ne);
    double s = eta * nb;
    for (int64_t k = 0; k < m; ++k) {
        e[k] = s * e[k] / ne;
        bt[k] = b[k] + e[k];
    }
    return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* sparse_matrices.f90                                                       */
/* ------------------------------------------------------------------------- */

/* csr_matrowvec, sparse_matrices.f90:252-270 (k is 1-based). */
double or_rowvecmult(const or_csr *A, int k, const double *v) {
    double f = 0.0;
    for (int64_t i = A->IA[k - 1]; i < A->IA[k]; ++i) f = f + v[A->JA[i] - 1] * A->vA[i];
    return f;
}

/* MMRS, sparse_matrices.f90:349-368 (row-parallel, each row serial). */
void or_matvecmul(const or_csr *A, const double *v, double *w, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 1) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int k = 1; k <= A->m; ++k) w[k - 1] = or_rowvecmult(A, k, v);
        return;
    }
#endif
    (void)nthreads;
    for (int k = 1; k <= A->m; ++k) w[k - 1] = or_rowvecmult(A, k, v);
}

/* MMCS via sparsetransmul, sparse_matrices.f90:300-347/:370-393, with the
 * serial scatter order (the shipped OpenMP version of this loop races). */
void or_transvecmul(const or_csr *A, const double *v, double *w) {
    memset(w, 0, sizeof(double) * (size_t)A->n);
    for (int k = 1; k <= A->m; ++k) {
        for (int64_t i = A->IA[k - 1]; i < A->IA[k]; ++i) {
            int32_t c = A->JA[i] - 1;
            w[c] = w[c] + v[k - 1] * A->vA[i];
        }
    }
}

/* The shipped OpenMP form of MMCS (sparse_matrices.f90:382-392): rows split
 * statically over the threads, every thread scattering into the one shared w
 * with no atomics, so concurrent updates of a column can be lost. The loads
 * and stores are relaxed atomics: on the CPU they are the plain moves of the
 * reference's loop and lose updates the same way, without making the program
 * undefined. For timing the reference as shipped; its result differs from
 * run to run. */
void or_transvecmul_racy(const or_csr *A, const double *v, double *w, int nthreads) {
    _Atomic double *aw = (_Atomic double *)w;
    const int64_t n = A->n;
    for (int64_t j = 0; j < n; ++j) atomic_store_explicit(&aw[j], 0.0, memory_order_relaxed);
#pragma omp parallel for num_threads(nthreads > 1 ? nthreads : 1) schedule(static)
    for (int64_t k = 0; k < (int64_t)A->m; ++k)
        for (int64_t i = A->IA[k]; i < A->IA[k + 1]; ++i) {
            int32_t c = A->JA[i] - 1;
            double cur = atomic_load_explicit(&aw[c], memory_order_relaxed);
            atomic_store_explicit(&aw[c], cur + v[k] * A->vA[i], memory_order_relaxed);
        }
}

/* How or_sirt forms A'r when nthreads > 1: 0 race-free per-thread copies
 * (default), 1 the shipped racy scatter. Serial when nthreads <= 1. */
static int g_mmcs_mode = 0;
void or_set_mmcs_mode(int mode) { g_mmcs_mode = mode; }

/* The same product on nthreads threads, for timing the reference's CPU path:
 * the reference runs this scatter under OpenMP into one shared vector (a data
 * race, sparse_matrices.f90:382-392); here each thread scatters a static
 * range of rows into its own copy of w and the copies are added in thread
 * order, so the result is deterministic for a given thread count (it differs
 * from the serial order only by rounding). */
int or_transvecmul_mt(const or_csr *A, const double *v, double *w, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 1) {
        const int64_t n = A->n;
        double *part = calloc((size_t)nthreads * (size_t)(n ? n : 1), sizeof(double));
        if (!part) return OR_ERR_ALLOC;
#pragma omp parallel num_threads(nthreads)
        {
            const int t = omp_get_thread_num(), nt = omp_get_num_threads();
            double *wt = part + (size_t)t * (size_t)n;
            const int64_t k0 = (int64_t)A->m * t / nt, k1 = (int64_t)A->m * (t + 1) / nt;
            for (int64_t k = k0; k < k1; ++k)
                for (int64_t i = A->IA[k]; i < A->IA[k + 1]; ++i) {
                    int32_t c = A->JA[i] - 1;
                    wt[c] = wt[c] + v[k] * A->vA[i];
                }
#pragma omp barrier
#pragma omp for schedule(static)
            for (int64_t c = 0; c < n; ++c) {
                double s = 0.0;
                for (int u = 0; u < nt; ++u) s = s + part[(size_t)u * (size_t)n + (size_t)c];
                w[c] = s;
            }
        }
        free(part);
        return OR_OK;
    }
#endif
    (void)nthreads;
    or_transvecmul(A, v, w);
    return OR_OK;
}

/* reorder, sparse_matrices.f90:492-570: stable counting sort; B is the CSR
 * form of A^T (B.m = A.n, B.JA holds 1-based row indices of A). */
int or_reorder(const or_csr *A, or_csr *B) {
    memset(B, 0, sizeof(*B));
    int nc = A->n;
    B->m = A->n;
    B->n = A->m;
    B->nnz = A->nnz;
    B->IA = calloc((size_t)nc + 1, sizeof(int64_t));
    B->JA = malloc(sizeof(int32_t) * (size_t)(A->nnz ? A->nnz : 1));
    B->vA = malloc(sizeof(double) * (size_t)(A->nnz ? A->nnz : 1));
    if (!B->IA || !B->JA || !B->vA) return OR_ERR_ALLOC;
    for (int64_t i = 0; i < A->nnz; ++i) B->IA[A->JA[i]] += 1;
    int64_t cumsum = 0;
    for (int i = 0; i <= nc; ++i) { cumsum += B->IA[i]; B->IA[i] = cumsum; }
    for (int i = 1; i <= A->m; ++i) {
        for (int64_t j = A->IA[i - 1]; j < A->IA[i]; ++j) {
            int col = A->JA[j] - 1;
            int64_t dest = B->IA[col];
            B->JA[dest] = i;
            B->vA[dest] = A->vA[j];
            B->IA[col] += 1;
        }
    }
    int64_t last = 0;
    for (int col = 0; col <= nc - 1; ++col) { int64_t t = B->IA[col]; B->IA[col] = last; last = t; }
    return OR_OK;
}

/* compute_row_norms, sparse_matrices.f90:740-780. */
void or_row_norms(const or_csr *A, int p, double *nrA, int nthreads) {
    (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads > 1 ? nthreads : 1) schedule(static)
#endif
    for (int k = 1; k <= A->m; ++k) {
        double s = 0.0;
        for (int64_t i = A->IA[k - 1]; i < A->IA[k]; ++i) {
            double av = fabs(A->vA[i]);
            double pw = av;
            for (int q = 1; q < p; ++q) pw *= av;
            s = s + pw;
        }
        nrA[k - 1] = pow(s, 1.0 / p);
    }
}

/* compute_column_norms, sparse_matrices.f90:782-793 (= row norms of A^T). */
int or_column_norms(const or_csr *A, int p, double *ncA) {
    or_csr B;
    int st = or_reorder(A, &B);
    if (st) return st;
    or_row_norms(&B, p, ncA, 1);
    or_csr_free(&B);
    return OR_OK;
}

/* add_mult_row, sparse_matrices.f90:795-822: bound only the touched entries,
 * lower bound first, then upper bound. */
void or_add_mult_row(const or_csr *A, int k, double c, double *w,
                     const double *lwrb, const double *upb) {
    for (int64_t i = A->IA[k - 1]; i < A->IA[k]; ++i) {
        int32_t j = A->JA[i] - 1;
        w[j] = w[j] + c * A->vA[i];
        if (lwrb) w[j] = fmax_f(w[j], *lwrb);
        if (upb) w[j] = fmin_f(w[j], *upb);
    }
}

/* scalar_mult, sparse_matrices.f90:824-831. */
void or_scalar_mult(or_csr *A, double c) {
    for (int64_t i = 0; i < A->nnz; ++i) A->vA[i] = c * A->vA[i];
}

/* ------------------------------------------------------------------------- */
/* AIRMs.f90                                                                 */
/* ------------------------------------------------------------------------- */

/* initialise_options, AIRMs.f90:17-37 */
void or_initialise_options(or_opts *o) {
    o->upb = 0; o->lwrb = 0; o->ubound = 0.0; o->lbound = 1.0;
    o->damp = 0.0; o->relaxpar = 1.0; o->verbose = 0; o->rowprobability = 0;
}

static double norm2v(const double *v, int64_t n) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += v[i] * v[i];
    return sqrt(s);
}

static double dotv(const double *a, const double *b, int64_t n) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

static void apply_box(double *x, int64_t n, int upb, int lwrb, double ub, double lb) {
    /* AIRMs.f90:1093-1100 / :963-970: upper bound first, then lower bound */
    if (upb && !lwrb) { for (int64_t j = 0; j < n; ++j) x[j] = fmin_f(x[j], ub); }
    else if (!upb && lwrb) { for (int64_t j = 0; j < n; ++j) x[j] = fmax_f(x[j], lb); }
    else if (upb && lwrb) {
        for (int64_t j = 0; j < n; ++j) { x[j] = fmin_f(x[j], ub); x[j] = fmax_f(x[j], lb); }
    }
}

/* sirt, AIRMs.f90:997-1127 */
int or_sirt(const char *method, const or_csr *A, const double *b, int maxits,
            const double *x0, const or_opts *o, double *xout, int nthreads) {
    int upb = 0, lwrb = 0;
    double ub = 0.0, lb = 1.0, omg = 1.0;
    if (o) { upb = o->upb; lwrb = o->lwrb; ub = o->ubound; lb = o->lbound; omg = o->relaxpar; }
    const int64_t m = A->m, n = A->n;
    double *x = malloc(sizeof(double) * n), *xn = malloc(sizeof(double) * n);
    double *D = malloc(sizeof(double) * n), *M = malloc(sizeof(double) * m);
    double *r = malloc(sizeof(double) * m), *g = malloc(sizeof(double) * n);
    if (!x || !xn || !D || !M || !r || !g) return OR_ERR_ALLOC;
    for (int64_t j = 0; j < n; ++j) x[j] = x0 ? x0[j] : 0.0;
    if (!strcmp(method, "cimmino")) {
        or_row_norms(A, 2, M, nthreads);
        for (int64_t i = 0; i < m; ++i) M[i] = (double)A->m * (M[i] * M[i]);
        for (int64_t j = 0; j < n; ++j) D[j] = 1.0;
    } else if (!strcmp(method, "sart")) {
        or_row_norms(A, 1, M, nthreads);
        int st = or_column_norms(A, 1, D);
        if (st) return st;
    } else {
        free(x); free(xn); free(D); free(M); free(r); free(g);
        return OR_ERR_METHOD; /* "Not a recognised SIRT method." */
    }
    for (int it = 1; it <= maxits; ++it) {
        or_matvecmul(A, x, r, nthreads);
        for (int64_t i = 0; i < m; ++i) r[i] = (b[i] - r[i]) / M[i];
        if (nthreads > 1 && g_mmcs_mode == 1) {
            or_transvecmul_racy(A, r, g, nthreads);
        } else if (nthreads > 1) {
            int st = or_transvecmul_mt(A, r, g, nthreads);
            if (st) { free(x); free(xn); free(D); free(M); free(r); free(g); return st; }
        } else {
            or_transvecmul(A, r, g);
        }
        for (int64_t j = 0; j < n; ++j) xn[j] = x[j] + omg * g[j] / D[j];
        apply_box(xn, n, upb, lwrb, ub, lb);
        memcpy(x, xn, sizeof(double) * n);
    }
    memcpy(xout, x, sizeof(double) * n);
    free(x); free(xn); free(D); free(M); free(r); free(g);
    return OR_OK;
}

/* FP64 adjoint of K unrolled SIRT steps (the iteration of sirt, AIRMs.f90:
 * 1089-1110, with x_{k+1} = P(x_k + lam * D^-1 A' M^-1 (b - A x_k))): stores
 * every iterate, then runs the reverse recursion
 *   gz = gx * [P does not clamp z_k]; glam += <gz, D^-1 g_k>;
 *   w = M^-1 A D^-1 gz (0 on empty rows); gb += lam w; gx = gz - lam A' w.
 * Returns x_K, dL/db, dL/dx0 and dL/dlam for gx = dL/dx_K. */
int or_sirt_adjoint(const char *method, const or_csr *A, const double *b, const double *x0,
                    int K, double lam, const or_opts *o, const double *gxK, double *xK,
                    double *gb, double *gx0, double *glam) {
    int upb = 0, lwrb = 0;
    double ub = 0.0, lb = 1.0;
    if (o) { upb = o->upb; lwrb = o->lwrb; ub = o->ubound; lb = o->lbound; }
    const int64_t m = A->m, n = A->n;
    int sart = !strcmp(method, "sart");
    if (!sart && strcmp(method, "cimmino")) return OR_ERR_METHOD;
    double *M = malloc(8 * m), *D = malloc(8 * n), *r = malloc(8 * m), *w = malloc(8 * m);
    double *X = malloc(8 * n * (size_t)(K + 1)), *Gk = malloc(8 * n * (size_t)(K > 0 ? K : 1));
    double *gx = malloc(8 * n), *gz = malloc(8 * n), *t = malloc(8 * n), *h = malloc(8 * n);
    if (sart) {
        or_row_norms(A, 1, M, 1);
        int st = or_column_norms(A, 1, D);
        if (st) return st;
    } else {
        or_row_norms(A, 2, M, 1);
        for (int64_t i = 0; i < m; ++i) M[i] = (double)A->m * (M[i] * M[i]);
        for (int64_t j = 0; j < n; ++j) D[j] = 1.0;
    }
    for (int64_t j = 0; j < n; ++j) X[j] = x0 ? x0[j] : 0.0;
    for (int k = 0; k < K; ++k) {
        double *xk = X + (size_t)k * n, *x1 = X + (size_t)(k + 1) * n, *g = Gk + (size_t)k * n;
        or_matvecmul(A, xk, r, 1);
        for (int64_t i = 0; i < m; ++i) r[i] = (b[i] - r[i]) / M[i];
        or_transvecmul(A, r, g);
        for (int64_t j = 0; j < n; ++j) {
            double z = xk[j] + lam * g[j] / D[j];
            if (upb) z = fmin_f(z, ub);
            if (lwrb) z = fmax_f(z, lb);
            x1[j] = z;
        }
    }
    memcpy(xK, X + (size_t)K * n, 8 * n);
    memcpy(gx, gxK, 8 * n);
    memset(gb, 0, 8 * m);
    double gl = 0.0;
    for (int k = K - 1; k >= 0; --k) {
        double *xk = X + (size_t)k * n, *g = Gk + (size_t)k * n;
        for (int64_t j = 0; j < n; ++j) {
            double z = xk[j] + lam * g[j] / D[j];
            int pass = 1;
            double zc = z;
            if (upb) { pass = pass && z < ub; zc = z < ub ? z : ub; }
            if (lwrb) pass = pass && zc > lb;
            gz[j] = pass ? gx[j] : 0.0;
            gl += gz[j] * (g[j] / D[j]);
            t[j] = gz[j] / D[j];
        }
        or_matvecmul(A, t, w, 1);
        for (int64_t i = 0; i < m; ++i) {
            w[i] = M[i] != 0.0 ? w[i] / M[i] : 0.0;
            gb[i] += lam * w[i];
        }
        or_transvecmul(A, w, h);
        for (int64_t j = 0; j < n; ++j) gx[j] = gz[j] - lam * h[j];
    }
    memcpy(gx0, gx, 8 * n);
    *glam = gl;
    free(M); free(D); free(r); free(w); free(X); free(Gk); free(gx); free(gz); free(t); free(h);
    return OR_OK;
}

/* normest, AIRMs.f90:1129-1173, with the start vector v0 given (the
 * reference draws it with random_number). */
double or_normest(const or_csr *A, double tol, int maxit, const double *v0, int nthreads) {
    const int64_t m = A->m, n = A->n;
    double *v = malloc(sizeof(double) * n), *vn = malloc(sizeof(double) * n);
    double *w = malloc(sizeof(double) * m), *d = malloc(sizeof(double) * n);
    memcpy(v, v0, sizeof(double) * n);
    for (int i = 1; i <= maxit; ++i) {
        or_matvecmul(A, v, w, nthreads);
        or_transvecmul(A, w, vn);
        double s = norm2v(vn, n);
        for (int64_t j = 0; j < n; ++j) vn[j] = vn[j] / s;
        for (int64_t j = 0; j < n; ++j) d[j] = vn[j] - v[j];
        if (norm2v(d, n) < tol) break;
        memcpy(v, vn, sizeof(double) * n);
    }
    or_matvecmul(A, v, w, nthreads);
    double sigma = sqrt(dotv(w, w, m) / dotv(v, v, n));
    free(v); free(vn); free(w); free(d);
    return sigma;
}

/* gradient_descent, AIRMs.f90:860-995. v0 is normest's start vector, drawn
 * from the project stream when NULL. */
int or_gradient_descent(const or_csr *A, const double *b, int max_iter,
                        const double *x0, double rho, double tol,
                        const or_opts *o, const double *v0, double *xout,
                        int *iters_done, int nthreads) {
    int upb = 0, lwrb = 0;
    double ub = 0.0, lb = 1.0;
    if (o) { upb = o->upb; lwrb = o->lwrb; ub = o->ubound; lb = o->lbound; }
    if (tol < 0.0) return OR_ERR_ARG; /* "Must use positive tolerance." */
    const int64_t m = A->m, n = A->n;
    for (int64_t j = 0; j < n; ++j) xout[j] = x0 ? x0[j] : 0.0;
    double *vs = NULL;
    if (!v0) {
        vs = malloc(sizeof(double) * n);
        for (int64_t j = 0; j < n; ++j) vs[j] = or_random_number();
        v0 = vs;
    }
    double sigma = or_normest(A, 1e-5, 100, v0, nthreads);
    free(vs);
    sigma = sigma * sigma;
    double *r = malloc(sizeof(double) * m), *g = malloc(sizeof(double) * n);
    double *xn = malloc(sizeof(double) * n), *d = malloc(sizeof(double) * n);
    for (int64_t i = 0; i < m; ++i) r[i] = -b[i];
    int it, done = 0;
    for (it = 1; it <= max_iter; ++it) {
        or_transvecmul(A, r, g);
        double s = rho / sigma;
        for (int64_t j = 0; j < n; ++j) xn[j] = xout[j] - s * g[j];
        apply_box(xn, n, upb, lwrb, ub, lb);
        for (int64_t j = 0; j < n; ++j) d[j] = xn[j] - xout[j];
        if (norm2v(d, n) < tol) break;
        memcpy(xout, xn, sizeof(double) * n);
        or_matvecmul(A, xout, r, nthreads);
        for (int64_t i = 0; i < m; ++i) r[i] = r[i] - b[i];
        done = it;
    }
    if (iters_done) *iters_done = done;
    free(r); free(g); free(xn); free(d);
    return OR_OK;
}

/* scramble, AIRMs.f90:1175-1212: two passes of random swaps over 1..n. */
void or_scramble(int n, int32_t *arr) {
    for (int i = 1; i <= n; ++i) arr[i - 1] = i;
    for (int k = 1; k <= 2; ++k) {
        for (int i = 1; i <= n; ++i) {
            double u = or_random_number();
            int j = 1 + (int)floor(n * u);
            int32_t t = arr[j - 1];
            arr[j - 1] = arr[i - 1];
            arr[i - 1] = t;
        }
    }
}

typedef struct {
    const or_csr *A;
    const double *b, *nrA, *cumul;
    int isrand, rowprob, upb, lwrb;
    double omg, ub, lb;
} sweep_ctx;

/* basic_sweep, AIRMs.f90:813-858. ord is 1-based rows; dir = -1 walks it
 * reversed (the ord(nord:1:-1) actual argument). */
static void basic_sweep(const sweep_ctx *c, double *x, const int32_t *ord, int nord, int dir) {
    for (int ii = 1; ii <= nord; ++ii) {
        int i = dir > 0 ? ord[ii - 1] : ord[nord - ii];
        int ri;
        if (c->isrand && c->rowprob) {
            double u = or_random_number();
            ri = 1;
            while (ri < c->A->m && c->cumul[ri - 1] < u) ri++;
        } else {
            ri = i;
        }
        double inp = or_rowvecmult(c->A, ri, x);
        double coeff = (c->omg * (c->b[ri - 1] - inp) / c->nrA[ri - 1]);
        or_add_mult_row(c->A, ri, coeff, x, c->lwrb ? &c->lb : NULL, c->upb ? &c->ub : NULL);
    }
}

/* Shared set-up of art and twin_art: AIRMs.f90:217-312 / :525-628. */
static int art_setup(const char *method, const or_csr *A, const int *Kin, int nK,
                     const int32_t *order, int nord_in, double dmp, int rowprob,
                     int *Kuse, int32_t *ord, int *nord_out, double *nrA,
                     double *cumul, int *isrand, int *issym) {
    const int m = A->m;
    int nord;
    *isrand = 0;
    *issym = 0;
    for (int l = 0; l < nK; ++l) Kuse[l] = Kin[l];
    if (!strcmp(method, "kaczmarz") || !strcmp(method, "symkaczmarz") ||
        !strcmp(method, "randkaczmarz")) {
        if (!strcmp(method, "symkaczmarz")) {
            for (int l = 0; l < nK; ++l) if (Kin[l] % 2 == 1) return OR_ERR_ARG;
            for (int l = 0; l < nK; ++l) Kuse[l] = Kuse[l] / 2;
            *issym = 1;
        }
        if (!strcmp(method, "randkaczmarz")) *isrand = 1;
        if (order) { nord = nord_in; for (int i = 0; i < nord; ++i) ord[i] = order[i]; }
        else { nord = m; for (int i = 0; i < m; ++i) ord[i] = i + 1; }
    } else {
        return OR_ERR_METHOD;
    }
    or_row_norms(A, 2, nrA, 1);
    double mx = -INFINITY;
    for (int i = 0; i < m; ++i) { nrA[i] = nrA[i] * nrA[i]; if (nrA[i] > mx) mx = nrA[i]; }
    for (int i = 0; i < m; ++i) nrA[i] = nrA[i] + dmp * mx;
    int l = nord, k = 0;
    for (int i = 0; i < l; ++i) if (nrA[ord[i] - 1] > 0) ord[k++] = ord[i];
    nord = k;
    if (*isrand) {
        or_scramble(nord, ord);
        if (rowprob) {
            double cs = 0;
            for (int i = 0; i < nord; ++i) { cs = cs + nrA[i]; cumul[i] = cs; }
            double s = 0;
            for (int i = 0; i < m; ++i) s += nrA[i];
            for (int i = 0; i < nord; ++i) cumul[i] = cumul[i] / s;
            for (int i = nord; i < m; ++i) cumul[i] = 1.0;
        }
    }
    *nord_out = nord;
    return OR_OK;
}

/* art, AIRMs.f90:59-369. Xout is n x nK, column-major. */
int or_art(const char *method, const or_csr *A, const double *b, const int *Kin,
           int nK, const double *x0, const double *xref, const int32_t *order,
           int nord_in, const or_opts *o, double *Xout) {
    const int64_t m = A->m, n = A->n;
    int upb = 0, lwrb = 0, rowprob = 0;
    double ub = 0.0, lb = 1.0, dmp = 0.0, omg = 1.0;
    if (o) {
        upb = o->upb; lwrb = o->lwrb; ub = o->ubound; lb = o->lbound;
        dmp = o->damp; omg = o->relaxpar; rowprob = o->rowprobability;
    }
    for (int l = 1; l < nK; ++l) if (Kin[l] < Kin[l - 1]) return OR_ERR_ARG;
    int *Kuse = malloc(sizeof(int) * nK);
    int32_t *ord = malloc(sizeof(int32_t) * (m + 1));
    double *nrA = malloc(sizeof(double) * m), *cumul = calloc(m, sizeof(double));
    double *x = malloc(sizeof(double) * n), *xp = malloc(sizeof(double) * n);
    double *d = malloc(sizeof(double) * n);
    int nord, isrand, issym;
    int st = art_setup(method, A, Kin, nK, order, nord_in, dmp, rowprob, Kuse, ord,
                       &nord, nrA, cumul, &isrand, &issym);
    if (st) { free(Kuse); free(ord); free(nrA); free(cumul); free(x); free(xp); free(d); return st; }
    for (int64_t j = 0; j < n; ++j) x[j] = x0 ? x0[j] : 0.0;
    memset(Xout, 0, sizeof(double) * n * nK);
    sweep_ctx c = {A, b, nrA, cumul, isrand, rowprob, upb, lwrb, omg, ub, lb};
    int maxiter = 0;
    for (int l = 0; l < nK; ++l) if (Kuse[l] > maxiter) maxiter = Kuse[l];
    int l = 0;
    for (int iter = 1; iter <= maxiter; ++iter) {
        if (isrand) or_scramble(nord, ord);
        if (xref) memcpy(xp, x, sizeof(double) * n);
        basic_sweep(&c, x, ord, nord, +1);
        if (issym) basic_sweep(&c, x, ord, nord, -1);
        if (xref) {
            for (int64_t j = 0; j < n; ++j) d[j] = x[j] - xref[j];
            double e1 = norm2v(d, n);
            for (int64_t j = 0; j < n; ++j) d[j] = xp[j] - xref[j];
            double e0 = norm2v(d, n);
            if (e1 > e0) { memcpy(Xout + (size_t)n * (nK - 1), xp, sizeof(double) * n); break; }
        }
        if (l < nK && iter == Kuse[l]) { memcpy(Xout + (size_t)n * l, x, sizeof(double) * n); l++; }
    }
    free(Kuse); free(ord); free(nrA); free(cumul); free(x); free(xp); free(d);
    return OR_OK;
}

/* twin_art, AIRMs.f90:371-811. Xstore/Ystore are n x nK column-major; EG has
 * max(Kin) entries. slack < 0 selects the default of 7. */
int or_twin_art(const char *method, const char *stoprule, const or_csr *A,
                const double *b, const int *Kin, int nK, const double *x0,
                const double *y0, const int32_t *order, int nord_in, int slack,
                const or_opts *o, double *xout, int *final_it, double *Xstore,
                double *Ystore, double *EG) {
    const int64_t m = A->m, n = A->n;
    int slck = slack >= 0 ? slack : 7;
    int upb = 0, lwrb = 0, rowprob = 0;
    double ub = 0.0, lb = 1.0, dmp = 0.0, omg = 1.0;
    if (o) {
        upb = o->upb; lwrb = o->lwrb; ub = o->ubound; lb = o->lbound;
        dmp = o->damp; omg = o->relaxpar; rowprob = o->rowprobability;
    }
    int eg = !strcmp(stoprule, "errorgauge"), ms = !strcmp(stoprule, "mutualstep");
    for (int l = 1; l < nK; ++l) if (Kin[l] < Kin[l - 1]) return OR_ERR_ARG;
    int maxK = 0;
    for (int l = 0; l < nK; ++l) if (Kin[l] > maxK) maxK = Kin[l];
    int *Kuse = malloc(sizeof(int) * nK);
    int32_t *ord = malloc(sizeof(int32_t) * (m + 1));
    double *nrA = malloc(sizeof(double) * m), *cumul = calloc(m, sizeof(double));
    int nord, isrand, issym;
    int st = art_setup(method, A, Kin, nK, order, nord_in, dmp, rowprob, Kuse, ord,
                       &nord, nrA, cumul, &isrand, &issym);
    if (!st && !eg && !ms) st = OR_ERR_METHOD;
    if (st) { free(Kuse); free(ord); free(nrA); free(cumul); return st; }
    double *x = calloc(n, 8), *y = calloc(n, 8), *v = calloc(n, 8), *w = calloc(n, 8);
    double *d = calloc(n, 8);
    sweep_ctx c = {A, b, nrA, cumul, isrand, rowprob, upb, lwrb, omg, ub, lb};
    memset(Xstore, 0, sizeof(double) * n * nK);
    memset(Ystore, 0, sizeof(double) * n * nK);
    memset(EG, 0, sizeof(double) * (maxK > 0 ? maxK : 1));
    int startiter;
    if (x0 && y0) {
        memcpy(x, x0, 8 * n); memcpy(y, y0, 8 * n);
        for (int64_t j = 0; j < n; ++j) d[j] = x0[j] - y0[j];
        if (norm2v(d, n) < 1e-10) { st = OR_ERR_ARG; goto done; }
        startiter = 1;
    } else {
        const double *s0 = x0 ? x0 : y0;
        for (int64_t j = 0; j < n; ++j) { x[j] = s0 ? s0[j] : 0.0; y[j] = x[j]; }
        basic_sweep(&c, x, ord, nord, +1);
        if (issym) basic_sweep(&c, x, ord, nord, -1);
        basic_sweep(&c, y, ord, nord, -1);
        if (issym) basic_sweep(&c, y, ord, nord, +1);
        for (int64_t j = 0; j < n; ++j) d[j] = x[j] - y[j];
        EG[0] = norm2v(d, n);
        startiter = 2;
    }
    int maxiter = 0;
    for (int l = 0; l < nK; ++l) if (Kuse[l] > maxiter) maxiter = Kuse[l];
    int l = 0, trck = 0, iter;
    double minEG = 1.79769313486231570815e308; /* huge(minEG) */
    *final_it = 0;
    for (iter = startiter; iter <= maxiter; ++iter) {
        if (isrand) or_scramble(nord, ord);
        if (ms) memcpy(v, x, 8 * n);
        basic_sweep(&c, x, ord, nord, +1);
        if (issym) basic_sweep(&c, x, ord, nord, -1);
        if (ms) {
            for (int64_t j = 0; j < n; ++j) v[j] = x[j] - v[j];
            for (int64_t j = 0; j < n; ++j) x[j] = x[j] - v[j];
        }
        if (ms) memcpy(w, y, 8 * n);
        basic_sweep(&c, y, ord, nord, -1);
        if (issym) basic_sweep(&c, y, ord, nord, +1);
        if (ms) {
            for (int64_t j = 0; j < n; ++j) w[j] = y[j] - w[j];
            for (int64_t j = 0; j < n; ++j) y[j] = y[j] - w[j];
        }
        if (eg) {
            for (int64_t j = 0; j < n; ++j) d[j] = x[j] - y[j];
            EG[iter - 1] = norm2v(d, n);
            if (EG[iter - 1] < minEG) {
                minEG = EG[iter - 1];
                memcpy(v, x, 8 * n); memcpy(w, y, 8 * n);
                trck = 0;
                *final_it = iter;
            } else {
                trck = trck + 1;
                if (trck >= slck) break;
            }
        } else {
            double nw = norm2v(w, n), nv = norm2v(v, n);
            for (int64_t j = 0; j < n; ++j) w[j] = w[j] / nw;
            for (int64_t j = 0; j < n; ++j) v[j] = v[j] / nv;
            for (int64_t j = 0; j < n; ++j) d[j] = x[j] - y[j];
            double mat1 = dotv(v, v, n), mat2 = dotv(w, w, n), mat3 = -dotv(v, w, n);
            double rhs1 = -dotv(v, d, n), rhs2 = dotv(w, d, n);
            double det = mat1 * mat2 - mat3 * mat3;
            double alph = (rhs1 * mat2 - rhs2 * mat3) / det;
            double bet = (mat1 * rhs2 - mat3 * rhs1) / det;
            for (int64_t j = 0; j < n; ++j) x[j] = x[j] + alph * v[j];
            for (int64_t j = 0; j < n; ++j) y[j] = y[j] + bet * w[j];
            for (int64_t j = 0; j < n; ++j) d[j] = x[j] - y[j];
            EG[iter - 1] = norm2v(d, n);
            if (fabs(alph) + fabs(bet) < 1e-5) break;
        }
        if (l < nK && iter == Kuse[l]) {
            memcpy(Xstore + (size_t)n * l, x, 8 * n);
            memcpy(Ystore + (size_t)n * l, y, 8 * n);
            l++;
        }
    }
    if (eg) {
        for (int64_t j = 0; j < n; ++j) xout[j] = .5 * (v[j] + w[j]);
    } else {
        for (int64_t j = 0; j < n; ++j) xout[j] = .5 * (x[j] + y[j]);
        *final_it = iter;
    }
done:
    free(Kuse); free(ord); free(nrA); free(cumul);
    free(x); free(y); free(v); free(w); free(d);
    return st;
}

/* ------------------------------------------------------------------------- */
/* phantomgallery.f90                                                        */
/* ------------------------------------------------------------------------- */

/* shepplogan, phantomgallery.f90:116-164 on the meshgrid of :17-56, returned
 * already vectorised column by column (vectorise, :672-690). */
/* Max-normalise (x = x/maxval(x)). */
static void normalise_max(double *v, int64_t n) {
    double mx = v[0];
    for (int64_t k = 1; k < n; ++k) if (v[k] > mx) mx = v[k];
    for (int64_t k = 0; k < n; ++k) v[k] = v[k] / mx;
}

/* smooth, phantomgallery.f90:166-199 (p = 4). intmeshgrid: xc(i,j) = j+1,
 * yc(i,j) = i+1. Rows 2-4 of the centres are default-real (single
 * precision) literals times N, as written in the reference. */
void or_smooth(int N, double *v) {
    const double sigma = 0.25 * N;
    const double c1[4] = {0.6 * N, (double)(0.5f * (float)N), (double)(0.2f * (float)N),
                          (double)(0.8f * (float)N)};
    const double c2[4] = {0.6 * N, (double)(0.3f * (float)N), (double)(0.7f * (float)N),
                          (double)(0.2f * (float)N)};
    const double a[4] = {1.0, 0.5, 0.7, 0.9};
    const double sx = 1.2 * sigma, sx2 = sx * sx, sy2 = sigma * sigma;
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            double xc = j + 1, yc = i + 1, acc = 0.0;
            for (int k = 0; k < 4; ++k) {
                double dx = xc - c1[k], dy = yc - c2[k];
                acc = acc + a[k] * exp(-(dx * dx) / sx2 - (dy * dy) / sy2);
            }
            v[(int64_t)j * N + i] = acc;
        }
    normalise_max(v, (int64_t)N * N);
}

/* grains, phantomgallery.f90:529-600 ('uniform'): p = int(3 sqrt(N)) seeds
 * drawn into x0(2,p) in element order, then p values drawn (unused); image =
 * index of the nearest seed (first on ties), max-normalised. Distances are
 * sqrt(dx^2 + dy^2) (the reference's norm2 scales). */
void or_grains(int N, double *v) {
    const int p = (int)(3 * sqrt(N * 1.0));
    double *sx = malloc(sizeof(double) * p), *sy = malloc(sizeof(double) * p);
    for (int k = 0; k < p; ++k) {
        double ux = or_random_number(), uy = or_random_number();
        sx[k] = 1.5 * (2.0 * ux - 1.0);
        sy[k] = 1.5 * (2.0 * uy - 1.0);
    }
    for (int k = 0; k < p; ++k) (void)or_random_number();  /* vals */
    double *lx = malloc(sizeof(double) * N), *ly = malloc(sizeof(double) * N);
    or_linspace(-1.0, 1.0, N, lx);
    or_linspace(1.0, -1.0, N, ly);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            double dmin = 1.7976931348623157e308;
            int kmin = 0;
            for (int k = 0; k < p; ++k) {
                double dx = lx[j] - sx[k], dy = ly[i] - sy[k];
                double d = sqrt(dx * dx + dy * dy);
                if (d < dmin) { dmin = d; kmin = k + 1; }
            }
            v[(int64_t)j * N + i] = kmin;
        }
    normalise_max(v, (int64_t)N * N);
    free(sx); free(sy); free(lx); free(ly);
}

/* threephases, phantomgallery.f90:201-254 (p = 100): two sets of p random
 * centres (c(p,2) filled column by column, times N) on the mesh
 * linspace(1, N) in both directions; the second sum divides the cubes by a
 * square, as the reference does (:243). */
void or_threephases(int N, double *v) {
    const int p = 100;
    double *c1x = malloc(sizeof(double) * p), *c1y = malloc(sizeof(double) * p);
    double *c2x = malloc(sizeof(double) * p), *c2y = malloc(sizeof(double) * p);
    for (int k = 0; k < p; ++k) c1x[k] = or_random_number() * N;
    for (int k = 0; k < p; ++k) c1y[k] = or_random_number() * N;
    for (int k = 0; k < p; ++k) c2x[k] = or_random_number() * N;
    for (int k = 0; k < p; ++k) c2y[k] = or_random_number() * N;
    double *lx = malloc(sizeof(double) * N), *ly = malloc(sizeof(double) * N);
    or_linspace(1.0, (double)N, N, lx);
    or_linspace(1.0, (double)N, N, ly);
    const double s1 = 0.025 * N, s2 = 0.025 * N;
    const double s1c = (2.5 * s1) * (2.5 * s1) * (2.5 * s1), s2s = (2.5 * s2) * (2.5 * s2);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            double xc = lx[j], yc = ly[i], im1 = 0.0, im2 = 0.0;
            for (int k = 0; k < p; ++k) {
                double ax = fabs(xc - c1x[k]), ay = fabs(yc - c1y[k]);
                im1 = im1 + exp(-(ax * ax * ax) / s1c - (ay * ay * ay) / s1c);
            }
            for (int k = 0; k < p; ++k) {
                double ax = fabs(xc - c2x[k]), ay = fabs(yc - c2y[k]);
                im2 = im2 + exp(-(ax * ax * ax) / s2s - (ay * ay * ay) / s2s);
            }
            im1 = im1 < 0.35 ? 0.0 : 2.0;
            im2 = im2 < 0.55 ? 0.0 : 1.0;
            double t = im1 + im2;
            v[(int64_t)j * N + i] = t == 3.0 ? 1.0 : t;
        }
    normalise_max(v, (int64_t)N * N);
    free(c1x); free(c1y); free(c2x); free(c2y); free(lx); free(ly);
}

void or_shepplogan(int N, double *v) {
    static const double e[10][6] = {
        {1, .69, .92, 0, 0, 0},          {-.8, .6624, .874, 0, -.0184, 0},
        {-.2, .11, .31, .22, 0, -18},    {-.2, .16, .41, -.22, 0, 18},
        {.1, .21, .25, 0, .35, 0},       {.1, .046, .046, 0, .1, 0},
        {.1, .046, .046, 0, -.1, 0},     {.1, .046, .023, -.08, -.605, 0},
        {.1, .023, .023, 0, -.606, 0},   {.1, .023, .046, .06, -.605, 0}};
    double *lx = malloc(sizeof(double) * N), *ly = malloc(sizeof(double) * N);
    or_linspace(-1.0, 1.0, N, lx);  /* x(i,j) = lx(j) */
    or_linspace(1.0, -1.0, N, ly);  /* y(i,j) = ly(i) */
    for (int64_t k = 0; k < (int64_t)N * N; ++k) v[k] = 0.0;
    for (int q = 0; q < 10; ++q) {
        double A = e[q][0], a2 = e[q][1] * e[q][1], b2 = e[q][2] * e[q][2];
        double x0 = e[q][3], y0 = e[q][4], phi = e[q][5] * PI / 180.0;
        double c = cos(phi), s = sin(phi);
        for (int j = 0; j < N; ++j) {
            for (int i = 0; i < N; ++i) {
                double xc = lx[j], yc = ly[i];
                double u = (xc - x0) * c + (yc - y0) * s;
                double w = (yc - y0) * c - (xc - x0) * s;
                if (u * u / a2 + w * w / b2 <= 1.0) v[(int64_t)j * N + i] += A;
            }
        }
    }
    free(lx); free(ly);
}
