/*
 * fair_oracle.h -- CPU oracle for the AIR reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C, FP64, serial-semantics
 * restatement of the reference Fortran (BartvLith/fortran_AIRtools) used to
 * check the GPU library: only the tests, the smoke check and the CPU-baseline
 * leg of the benchmark may load it. Nothing in the product links it.
 *
 * Parity status: UNPINNED by the reference itself. The reference ships no
 * tests, fixtures or golden vectors, and it is Fortran with no Fortran
 * compiler available to build it. The oracle is pinned instead by analytic
 * known-answer tests (chord lengths, per-angle area sums, adjoint identities,
 * consistent-system convergence) in tests/test_oracle_kat.py.
 *
 * Conventions follow the reference's CSR type (sparse_matrices.f90:9-49):
 * IA has m+1 entries with IA[0] = 0 (cumulative counts), JA is 1-based.
 * IA is held as int64 so that sizes beyond 2^31-1 nonzeros stay representable.
 */
#ifndef FAIR_ORACLE_H
#define FAIR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t m, n;
    int64_t nnz;
    int64_t *IA; /* m+1 */
    int32_t *JA; /* nnz, 1-based */
    double *vA;  /* nnz */
} or_csr;

typedef struct {
    double relaxpar, ubound, lbound, damp;
    int32_t verbose, upb, lwrb, rowprobability;
} or_opts;

/* status codes shared with the GPU library's error codes */
enum {
    OR_OK = 0,
    OR_ERR_SIZE = 1,      /* "Vector input size incorrect." */
    OR_ERR_METHOD = 2,    /* unknown method / stopping rule */
    OR_ERR_GEOMETRY = 3,  /* "++ Something went wrong" */
    OR_ERR_ARG = 4,       /* other argument errors (e.g. odd K for symkaczmarz) */
    OR_ERR_NEWTON = 5,    /* "Newton method did not converge." */
    OR_ERR_ALLOC = 6
};

/* ---- project PRNG (stand-in for the Fortran random_number stream) ---- */
void or_random_seed(uint64_t seed);
double or_random_number(void);
uint64_t or_random_counter(void);

/* ---- system_generation.f90 ---- */
void or_linspace(double a, double b, int n, double *x);
int or_paralleltomo(int n, int nth, int p, const double *theta, or_csr *A);
int or_paralleltomo_mt(int n, int nth, int p, const double *theta, int nthreads, or_csr *A);
int or_fanlineartomo(int n, int nth, int p, double r, double dw, double sd,
                     const double *theta, int geometry_fix, or_csr *A);
/* The same with the rays split over nthreads threads (identical result). */
int or_fanlineartomo_mt(int n, int nth, int p, double r, double dw, double sd,
                        const double *theta, int geometry_fix, int nthreads, or_csr *A);
void or_csr_free(or_csr *A);
int or_add_white_noise(int64_t m, const double *b, double eta, double *bt, double *e);

/* ---- sparse_matrices.f90 ---- */
double or_rowvecmult(const or_csr *A, int k, const double *v);
void or_matvecmul(const or_csr *A, const double *v, double *w, int nthreads);
void or_transvecmul(const or_csr *A, const double *v, double *w);
/* The same on nthreads threads (per-thread copies added in thread order). */
int or_transvecmul_mt(const or_csr *A, const double *v, double *w, int nthreads);
/* The shipped OpenMP scatter into one shared vector (racy: updates can be
 * lost; for timing the reference as shipped). */
void or_transvecmul_racy(const or_csr *A, const double *v, double *w, int nthreads);
/* or_sirt's threaded transposed product: 0 race-free copies, 1 the racy scatter. */
void or_set_mmcs_mode(int mode);
int or_reorder(const or_csr *A, or_csr *B);
void or_row_norms(const or_csr *A, int p, double *nrA, int nthreads);
int or_column_norms(const or_csr *A, int p, double *ncA);
void or_add_mult_row(const or_csr *A, int k, double c, double *w,
                     const double *lwrb, const double *upb);
void or_scalar_mult(or_csr *A, double c);

/* ---- AIRMs.f90 ---- */
void or_initialise_options(or_opts *o);
int or_sirt(const char *method, const or_csr *A, const double *b, int maxits,
            const double *x0, const or_opts *o, double *xout, int nthreads);
int or_gradient_descent(const or_csr *A, const double *b, int max_iter,
                        const double *x0, double rho, double tol,
                        const or_opts *o, const double *v0, double *xout,
                        int *iters_done, int nthreads);
double or_normest(const or_csr *A, double tol, int maxit, const double *v0,
                  int nthreads);
int or_sirt_adjoint(const char *method, const or_csr *A, const double *b, const double *x0,
                    int K, double lam, const or_opts *o, const double *gxK, double *xK,
                    double *gb, double *gx0, double *glam);
void or_scramble(int n, int32_t *out);
int or_art(const char *method, const or_csr *A, const double *b, const int *Kin,
           int nK, const double *x0, const double *xref, const int32_t *order,
           int nord_in, const or_opts *o, double *Xout);
int or_twin_art(const char *method, const char *stoprule, const or_csr *A,
                const double *b, const int *Kin, int nK, const double *x0,
                const double *y0, const int32_t *order, int nord_in, int slack,
                const or_opts *o, double *xout, int *final_it, double *Xstore,
                double *Ystore, double *EG);

/* ---- phantomgallery.f90 ---- */
void or_shepplogan(int N, double *x_colmajor);
void or_smooth(int N, double *v);
void or_grains(int N, double *v);
void or_threephases(int N, double *v);

#ifdef __cplusplus
}
#endif
#endif
