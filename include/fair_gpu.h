/*
 * fair_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of the FAIR tools
 * reconstruction hot path: ray-traced system matrix, CSR operators and the
 * AIR iterations (Kaczmarz family, Cimmino/SART, gradient descent).
 *
 * Every entry point replaces one procedure of the reference Fortran modules
 * (BartvLith/fortran_AIRtools); the comment above each names the procedure
 * and its file:line. A Fortran program binds them with ISO_C_BINDING
 * interfaces (bind(C), scalars by value, arrays as assumed-size).
 *
 * Conventions (as the reference's CSR type, sparse_matrices.f90:9-49):
 *   - IA has m+1 entries, IA[0] = 0, IA[k] = nonzeros in rows 1..k;
 *   - JA holds 1-based column indices; `order` arrays hold 1-based rows;
 *   - images are column-major vectors of length N*N (phantomgallery.f90:672);
 *   - all host arrays belong to the caller and are only read/written during
 *     the call; the matrix itself lives on the GPU inside the opaque handle.
 *
 * Errors: every function returns 0 on success or a FAIR_ERR_* code; the text
 * the reference prints with `stop` is returned by fair_error_string().
 * Threading: a handle is not reentrant; one CUDA stream per handle.
 */
#ifndef FAIR_GPU_H
#define FAIR_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    FAIR_OK = 0,
    FAIR_ERR_SIZE = 1,     /* "Vector input size incorrect." (sparse_matrices.f90:287) */
    FAIR_ERR_METHOD = 2,   /* unknown method or stopping rule (AIRMs.f90:267, :584, :1082) */
    FAIR_ERR_GEOMETRY = 3, /* "++ Something went wrong" (system_generation.f90:293, :478) */
    FAIR_ERR_ARG = 4,      /* invalid argument (e.g. odd K for symkaczmarz, AIRMs.f90:233) */
    FAIR_ERR_NEWTON = 5,   /* "Newton method did not converge." (system_generation.f90:735) */
    FAIR_ERR_ALLOC = 6,    /* device or host allocation failed */
    FAIR_ERR_CUDA = 7,     /* a CUDA runtime call failed (detail in fair_last_error_detail) */
    FAIR_ERR_NULL = 8,     /* null handle or required pointer */
    FAIR_ERR_STATE = 9,    /* handle holds no matrix */
    FAIR_ERR_NOGPU = 10    /* no CUDA device / driver */
};

/* Reference text for a status code (static storage). */
const char *fair_error_string(int status);
/* Detail of the last failure on the calling thread (static storage). */
const char *fair_last_error_detail(void);

/* ---- value precision of the stored matrix ------------------------------ */
enum {
    FAIR_PREC_F64 = 0, /* FP64 values, FP64 accumulation (the reference's real(8)) */
    FAIR_PREC_F32 = 1, /* FP32 values and vectors, FP32 accumulation, FP64 weights */
    FAIR_PREC_F16 = 2, /* FP16-stored values, FP32 vectors/accumulation, FP64 weights */
    FAIR_PREC_Q16 = 3  /* 16-bit fixed-point values scaled by the largest |value|
                          (unsigned when no value is negative), FP32 vectors and
                          accumulation, FP64 weights and scale */
};

/* ---- opaque device matrix (type(csr_matrix), sparse_matrices.f90:157) --- */
typedef struct fair_csr_s *fair_csr;

/* Geometry record: type(data), system_generation.f90:6-12. `theta` holds nth
 * angles in radians; r, dw and sd are in units of n (the reference's scaling,
 * system_generation.f90:98-100). The transmission data T is not needed. */
typedef struct fair_data {
    int32_t n, p, nth;
    double r, dw, sd;
    const double *theta;
} fair_data;

/* Solver options: type(opts), AIRMs.f90:6-13, field for field. */
typedef struct fair_opts {
    double relaxpar, ubound, lbound, damp;
    int32_t verbose, upb, lwrb, rowprobability;
} fair_opts;

/* ---- handle lifetime ----------------------------------------------------- */
/* New empty matrix handle bound to the current CUDA device. */
int fair_csr_create(fair_csr *out);
int fair_csr_destroy(fair_csr h);
/* Use the caller's cudaStream_t for all work on this handle (NULL = own). */
int fair_csr_set_stream(fair_csr h, void *cuda_stream);
/* Shape: A%m, A%n, A%nnz (sparse_matrices.f90:47). */
int fair_csr_info(fair_csr h, int32_t *m, int32_t *n, int64_t *nnz);
/* Value precision used by matvecmul/transvecmul/sirt/gradient_descent. */
int fair_csr_set_precision(fair_csr h, int32_t prec);

/* construct_csr_matrix, sparse_matrices.f90:180-197: upload host CSR arrays
 * (IA int32 with m+1 entries, JA 1-based). */
int fair_construct_csr_matrix(int32_t m, int32_t n, const double *vA,
                              const int32_t *IA, const int32_t *JA, fair_csr h);
/* Same with 64-bit row offsets, for more than 2^31-1 nonzeros. */
int fair_construct_csr_matrix64(int32_t m, int32_t n, const double *vA,
                                const int64_t *IA, const int32_t *JA, fair_csr h);
/* Copy the matrix back to host arrays: vA (nnz), IA (m+1, int64), JA (nnz,
 * 1-based). Any pointer may be NULL to skip that array. */
int fair_csr_download(fair_csr h, double *vA, int64_t *IA, int32_t *JA);

/* ---- system_generation.f90 -------------------------------------------- */
/* linspace, system_generation.f90:17-35 (x(i) = c*i + d rounding). */
int fair_linspace(double a, double b, int32_t n, double *x);
/* paralleltomo, system_generation.f90:309-492: parallel-beam CSR build on
 * the GPU. Column indices and row lengths are bit-exact to the reference. */
int fair_paralleltomo(const fair_data *dat, fair_csr h);
/* fanlineartomo, system_generation.f90:79-307. geometry_fix = 0 keeps the
 * reference's odd-p ray angles (:122); 1 uses the even-p rule for odd p. */
int fair_fanlineartomo(const fair_data *dat, int32_t geometry_fix, fair_csr h);
/* add_white_noise, system_generation.f90:709-745 (host; draws from the
 * library's random stream, see fair_random_seed). */
int fair_add_white_noise(double *bt, double *e, const double *b, int64_t m, double eta);

/* ---- sparse_matrices.f90 (type-bound procedures) ----------------------- */
/* matvecmul -> sparsematmul/MMRS, :272-298/:349-368: w(m) = A*v(n). */
int fair_matvecmul(fair_csr h, const double *v, int64_t size_v, double *w);
/* transvecmul -> sparsetransmul/MMCS, :300-347/:370-393: w(n) = A'*v(m).
 * Deterministic (gather over the transposed CSR; no scatter race). */
int fair_transvecmul(fair_csr h, const double *v, int64_t size_v, double *w);
/* rowvecmult -> csr_matrowvec, :252-270: *f = row k (1-based) . v. */
int fair_rowvecmult(fair_csr h, int32_t k, const double *v, int64_t size_v, double *f);
/* add_scalar_mult_row -> add_mult_row, :795-822: w(JA) += c*vA on row k,
 * then max(lwrb), then min(upb) on the touched entries (NULL = absent). */
int fair_add_scalar_mult_row(fair_csr h, int32_t k, double c, double *w, int64_t size_w,
                             const double *lwrb, const double *upb);
/* row_norms -> compute_row_norms, :740-780: p-norm of every row (m). */
int fair_row_norms(fair_csr h, int32_t p, double *nrA);
/* column_norms -> compute_column_norms, :782-793: p-norm of every column (n). */
int fair_column_norms(fair_csr h, int32_t p, double *ncA);
/* transpose -> transposition/reorder, :395-411/:492-570: A becomes A' (stable
 * counting-sort order: entries of a column keep ascending row order). */
int fair_transpose(fair_csr h);
/* multiply_by_scalar -> scalar_mult, :824-831: vA = c*vA. */
int fair_multiply_by_scalar(fair_csr h, double c);

/* ---- AIRMs.f90 ---------------------------------------------------------- */
/* initialise_options / set_ubound / set_lbound, AIRMs.f90:17-57. */
int fair_opts_initialise(fair_opts *o);
int fair_opts_set_ubound(fair_opts *o, double ubound);
int fair_opts_set_lbound(fair_opts *o, double lbound);

/* sirt, AIRMs.f90:997-1127: 'cimmino' or 'sart', max(Kin) iterations from
 * x0 (NULL = 0), options may be NULL; xout has n entries. */
int fair_sirt(double *xout, const char *sirt_method, fair_csr h, const double *b,
              const int32_t *Kin, int32_t nK, const double *x0, const fair_opts *options);
/* gradient_descent, AIRMs.f90:860-995 (NULL optional arguments take the
 * reference defaults: 100 iterations, rho 1.5, tolerance 1e-6, x0 = 0).
 * iters_done (may be NULL) receives the number of accepted steps. */
int fair_gradient_descent(double *xout, fair_csr h, const double *b, const int32_t *max_iter,
                          const double *x0, const double *rho_in, const double *tolerance,
                          const fair_opts *options, int32_t *iters_done);
/* normest, AIRMs.f90:1129-1173 (start vector drawn from the library stream;
 * NULL tolerance/max_its take the defaults 1e-5 and 100). */
int fair_normest(fair_csr h, const double *tolerance, const int32_t *max_its, double *sigma);
/* art, AIRMs.f90:59-369: 'kaczmarz', 'symkaczmarz' or 'randkaczmarz'. Xout is
 * n x nK column-major. x0, xref (oracle stop), order (1-based, nord entries)
 * and options may be NULL/0. */
int fair_art(double *Xout, const char *art_method, fair_csr h, const double *b,
             const int32_t *Kin, int32_t nK, const double *x0, const double *xref,
             const int32_t *order, int32_t nord, const fair_opts *options);
/* twin_art, AIRMs.f90:371-811: stopping rules 'errorgauge' / 'mutualstep'.
 * Xstore, Ystore are n x nK; EG has max(Kin) entries; slack < 0 = 7. */
int fair_twin_art(double *xout, int32_t *final_it, double *Xstore, double *Ystore,
                  double *EG, const char *art_method, const char *stoprule, fair_csr h,
                  const double *b, const int32_t *Kin, int32_t nK, const double *x0,
                  const double *y0, const int32_t *order, int32_t nord, int32_t slack,
                  const fair_opts *options);
/* scramble, AIRMs.f90:1175-1212: the reference's two-pass swap recipe. */
int fair_scramble(int32_t n, int32_t *out);

/* ---- random stream (stands in for Fortran random_number) ---------------- */
/* The reference draws from the unseeded gfortran random_number stream; this
 * library draws every random number (scramble, row sampling, normest start
 * vector, noise) from one seeded SplitMix64 stream instead, in the same
 * order as the reference. */
int fair_random_seed(uint64_t seed);
int fair_random_number(double *u, int64_t k);

/* ---- phantomgallery.f90 (inputs) ---------------------------------------- */
/* shepplogan, phantomgallery.f90:116-164, vectorised (:672-690). */
int fair_shepplogan(int32_t N, double *x);

#ifdef __cplusplus
}
#endif
#endif /* FAIR_GPU_H */
