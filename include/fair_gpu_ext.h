/*
 * fair_gpu_ext.h -- device-resident entry points of the GB300 library.
 *
 * These have no counterpart in the reference (which has no device memory):
 * they run the same kernels as fair_sirt / fair_matvecmul on vectors that
 * already live in GPU memory, enqueued on the handle's stream without any
 * host synchronisation, so that callers which keep their data on the GPU
 * (and the benchmark) can time the iterations alone.
 */
#ifndef FAIR_GPU_EXT_H
#define FAIR_GPU_EXT_H

#include "fair_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Prepare SIRT on the handle: transpose, weights (FP64) and the value copies
 * of the handle's precision. method is 'cimmino' or 'sart' (AIRMs.f90:1070). */
int fair_sirt_prepare(fair_csr h, const char *sirt_method, const fair_opts *options);

/* Enqueue K SIRT iterations on device vectors (FP64 b of m entries, FP64 x of
 * n entries, updated in place). Asynchronous on the handle's stream. */
int fair_sirt_run_device(fair_csr h, const double *d_b, double *d_x, int32_t K);

/* Same, recording CUDA events around every kernel: on return (synchronised)
 * ms_pass1 / ms_pass2 hold the summed durations of the residual pass over A
 * and of the update pass over A'. */
int fair_sirt_run_device_timed(fair_csr h, const double *d_b, double *d_x, int32_t K,
                               float *ms_pass1, float *ms_pass2);

/* Kernel launches one fair_sirt_run_device(K) enqueues. */
int fair_sirt_launches(fair_csr h, int32_t K, int64_t *launches);

/* Enqueue one product y = A x (trans = 0) or y = A' x (trans = 1) on device
 * vectors: FP64 vectors for FAIR_PREC_F64, FP32 vectors otherwise. */
int fair_spmv_device(fair_csr h, int32_t trans, const void *d_x, void *d_y);

/* Reverse-mode adjoint of K unrolled SIRT steps with box projection (no
 * counterpart in the reference; it differentiates the iteration of sirt,
 * AIRMs.f90:1089-1110). For nrhs right-hand sides sharing the matrix:
 *   x_{k+1} = P(x_k + lambda_c D^-1 A' M^-1 (b_c - A x_k)),  P = bounds of options
 * ('cimmino' or 'sart' weights). Given gx = dL/dx_K (n x nrhs, column-major)
 * it returns gb = dL/db (m x nrhs), gx0 = dL/dx0 (n x nrhs) and glam = dL/dlambda
 * (nrhs); xK (may be NULL) receives x_K. x0 may be NULL (zeros). Checkpoints
 * every ceil(sqrt(K)) steps. FP64 for FAIR_PREC_F64, FP32 values and vectors
 * for FAIR_PREC_F32 (the lambda gradient is summed in FP64). */
int fair_sirt_adjoint(fair_csr h, const char *sirt_method, int32_t nrhs, const double *b,
                      const double *x0, int32_t K, const double *lambda, const fair_opts *options,
                      const double *gx, double *xK, double *gb, double *gx0, double *glam);

/* Autotuner of the SIRT passes (no reference counterpart): after
 * fair_sirt_prepare, times each pass over A and A' on every layout the
 * matrix has and every lanes-per-row choice (reps launches each, CUDA events
 * on the handle's stream), and keeps the fastest for the handle's current
 * precision. config (may be NULL) receives {lanes A, lanes A', layout A,
 * layout A'}. Layout codes:
 *   0     the CSR (int32 columns + values), 4, 8, 16 or 32 lanes per row;
 *   1, 2  the packed index stream with padded values, that many groups of 4
 *         entries per lane and step;
 *   3, 4  the fused 16-byte records {index word, 4 values} of the 2-byte
 *         forms (f16, q16), 1 or 2 records per lane and step;
 *   5, 6  the sliced copy of the packed stream (fused records for the 2-byte
 *         forms): slices of 32/G rows with G = 1, 2, 4 or 8 lanes per row,
 *         the groups of a slice interleaved by step, 2 or 4 steps of 32 slots
 *         in flight per warp; lanes per row 0 chooses G per chunk of 32 rows
 *         from the rows' column steps (8 when most steps are +-1, else 1);
 *   7, 8  as 5, 6 with the gathers of x issued one step ahead;
 *   9, 10 the tiled copy: pass 1 (A, whose n columns are an N x N image)
 *         cuts the rows by 96 x 96 tiles of the image and stages each tile
 *         of x in shared memory; pass 2 (A', whose rows are an N x N image
 *         and whose columns are rays of p bins per angle, p its stride hint)
 *         cuts the rows by 32 x 32 pixel tiles times blocks of angles and
 *         stages each tile's window of residual bins; 16-bit tile-local
 *         indices, one partial sum per segment added up per row in a second
 *         kernel; 2 slots in flight (9) or 4 (10);
 *   11-13 the delta copy: the sliced layout with one lane per row whose
 *         slots hold column steps from the row's previous entry instead of
 *         columns: four 7-bit steps beside 4 FP32/FP64 values, or one 16-byte
 *         record of six 5-bit steps and six 2-byte values (f16, q16); 11 with
 *         2 slots in flight, 12 with 4 and the gathers one slot ahead, 13
 *         with 2 and the gathers one slot ahead;
 *   14    (f16 and q16) the tiled copy with 16-byte records of six 5-bit
 *         steps of the tile-local index and six 2-byte values (else code 9).
 * A code whose layout the matrix lacks falls back to the nearest one it has.
 * d_b as in fair_sirt_run_device; d_x is scratch (overwritten). */
int fair_sirt_autotune(fair_csr h, const double *d_b, double *d_x, int32_t reps,
                       int32_t *config);

/* Sets {lanes A, lanes A', layout A, layout A'} of the SIRT passes for the
 * handle's current precision: layout codes 0-14 as listed at
 * fair_sirt_autotune, with 4, 8, 16 or 32 lanes per row for codes 0-4 and
 * 9-14 (unused by 9-14) and 0, 1, 2, 4 or 8 for codes 5-8 (else
 * FAIR_ERR_ARG). No reference counterpart. */
int fair_sirt_set_lanes(fair_csr h, const int32_t *config);

/* Packed index stream of A (which = 0) or A' (which = 1), built by the first
 * reduced-precision SIRT on the handle (no reference counterpart): has = 1
 * when built, the groups of 4 entries, the groups stored in the escape
 * table, and the step code's stride S and low-part width L. The packed
 * stream is used unless the environment sets FAIR_PACKED=0. */
int fair_csr_packed_info(fair_csr h, int32_t which, int32_t *has, int64_t *ngroups,
                         int64_t *nesc, int32_t *stride, int32_t *low_bits);

/* Sliced copy (SELL-32) of the packed stream of A (which = 0) or A' (1),
 * built when a SIRT pass is set to layout 5 or 6 or by the autotuner (no
 * reference counterpart): has = 1 when built, nslots = its slots (groups plus
 * the padding of each chunk of 32 rows to its longest row). */
int fair_csr_sliced_info(fair_csr h, int32_t which, int32_t *has, int64_t *nslots);

/* Tile shape of the tiled copies (layout codes 9, 10, 14; no reference
 * counterpart): shape = {side of A's T x T image tiles (16-128), side of A''s
 * pixel tiles (8-64), residual cells a tile of A' holds, i.e. angles per block
 * x bins per angle (1024-16384)}, 0 for the default of each (96, 32, 13000).
 * The copies are rebuilt with the new shape when a pass next reads them.
 * fair_sirt_autotune tries other shapes for a tiled pass unless one was set
 * here; fair_csr_tiled_info reports the shape in use. */
int fair_sirt_set_tiles(fair_csr h, const int32_t *shape);

/* Shape of the tiled copy of A (which = 0) or A' (which = 1), built when a
 * SIRT pass is set to layout 9, 10 or 14 or by the autotuner (no reference
 * counterpart). shape receives 8 values: {built (0/1), tile side T, tiles per
 * image side, angles per block NA, angle blocks, residual window W (bins per
 * angle; A' only), work units, kind (0: tiles of A's image columns, 1: pixel
 * tiles of A' times angle blocks)}; all zero when no copy is built. */
int fair_csr_tiled_info(fair_csr h, int32_t which, int32_t *shape);

/* paralleltomo (system_generation.f90:309-492) for the FP32 form only: the
 * same rays, columns and values (traced in FP64, stored rounded to FP32), with
 * A and A' held as FP32 values, int32 column indices and int64 row offsets
 * (8 bytes per nonzero each), built by blocks of block_angles angles (0: blocks
 * of about 2^28 nonzeros) so that the FP64 matrix is never held whole: the
 * N=2048, 1440-angle, 2896-bin problem (7.69e9 nonzeros) needs 123 GB instead
 * of the FP64 build's ~280 GB. The row and column 1- and 2-norms are kept from
 * the FP64 values (SIRT weights). The handle's precision becomes FAIR_PREC_F32
 * and stays so; fair_matvecmul, fair_transvecmul, the norms, fair_sirt and the
 * device-resident SIRT entry points work on it (FP32 products, any FP32
 * layout); entry points that read FP64 values (the Kaczmarz family, gradient
 * descent, normest, the adjoint, row edits, FP64 downloads of vA, batches)
 * return FAIR_ERR_STATE. No reference counterpart beyond paralleltomo. */
int fair_paralleltomo_f32(const fair_data *dat, int32_t block_angles, fair_csr h);

/* Capacity, in doubles, of the fixed device array behind
 * fair_matvecmul_noalloc (32 MiB): n + m of the matrix must fit in it. */
#define FAIR_NOALLOC_MAX_ENTRIES 4194304

/* w(m) = A*v(n) with host vectors, like fair_matvecmul, but without
 * allocating any GPU memory: for callers that cannot call cudaMalloc during
 * their run (a program that has reserved the GPU's memory for its own pool,
 * a real-time loop that cannot take cudaMalloc's device synchronisation, a
 * job held to a fixed memory budget on a shared GPU). No counterpart in the
 * reference. The vectors are staged in one fixed device array of
 * FAIR_NOALLOC_MAX_ENTRIES doubles that every GPU loading the library holds
 * until exit; larger problems fail with FAIR_ERR_ARG. Computed in FP64 for
 * any handle precision. Every call looks up the array's address with the
 * handle's device current; the first call on a device also loads it: make
 * that call before any stream capture.
 * Calls share the array, so calls that overlap on the GPU race. */
int fair_matvecmul_noalloc(fair_csr h, const double *v, int64_t size_v, double *w);

#ifdef __cplusplus
}
#endif
#endif /* FAIR_GPU_EXT_H */
