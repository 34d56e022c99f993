/* fair_batch.h -- many independent SIRT/SART problems advanced together on
 * one GPU (no counterpart in the reference, whose sirt (AIRMs.f90:997-1127)
 * solves one problem per call).
 *
 * A batch holds P problems, each with its own matrix (any sizes), and runs
 * the K iterations of AIRMs.f90:1089-1110 for all of them with one kernel
 * launch per pass and iteration covering every problem (warps claim chunks
 * of rows of any problem from one counter), the K iterations captured once
 * in a CUDA graph. Per problem it keeps only what the passes read: for the
 * reduced forms (FAIR_PREC_F32/F16/Q16) the packed index streams of A and A'
 * with their padded values plus the FP64 weights; for FAIR_PREC_F64 the CSR
 * of A and A' and the weights. Vectors are concatenated over the problems in
 * the order they were added (fair_batch_offsets).
 */
#ifndef FAIR_BATCH_H
#define FAIR_BATCH_H

#include "fair_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fair_batch_s *fair_batch;

/* New empty batch computing in `prec` (FAIR_PREC_*), on the current device
 * and on a stream of its own. */
int fair_batch_create(fair_batch *out, int32_t prec);
int fair_batch_destroy(fair_batch b);
/* Use the caller's stream (NULL: back to a stream of the batch's own). */
int fair_batch_set_stream(fair_batch b, void *cuda_stream);

/* Layout of the problems' passes, chosen before the first fair_batch_add:
 * 0 (default) the packed index streams (the CSR in FAIR_PREC_F64); 1 the
 * tiled copies of A (rays cut by 96 x 96 image tiles) and A' (pixels cut by
 * 32 x 32 tiles times angle blocks), the vector gathered into shared memory
 * per tile (the layout of fair_sirt_set_lanes code 9), for every problem
 * whose columns form an N x N image and whose rays are p bins per angle;
 * other problems keep the packed layout. A tiled pass is two launches
 * (partial sums per ray segment, then row sums in row order), each covering
 * every tiled problem; the results equal fair_sirt with layout code 9.
 * 2 chooses per class of problems (the same image side and bins per angle):
 * the first problem of a class is timed alone on the packed streams (the CSR
 * in FAIR_PREC_F64) and on its tiled copies with each candidate tile shape
 * (A's tiles 96, 64, 128; A''s pixel tiles x residual cells 32 x 13000,
 * 32 x 6500, 16 x 6500, 48 x 13000), and the class takes the faster layout
 * with the fastest shape per pass (fair_batch_problem_layout reports it);
 * the results equal fair_sirt on that layout and shape. */
int fair_batch_set_layout(fair_batch b, int32_t layout);

/* The layout problem p (0-based, in the order added) runs on: layout[0] = 1
 * for the tiled copies (0: packed streams / CSR), then A's tile side, A''s
 * pixel-tile side and residual cells per tile (0 when not tiled). */
int fair_batch_problem_layout(fair_batch b, int32_t p, int32_t *layout);

/* Appends the matrix of handle h as the next problem. take = 1 moves the
 * matrix out of h (h is left holding no matrix, as after fair_csr_create);
 * take = 0 copies it. The weights of both SIRT methods are computed in FP64
 * from the FP64 values before the batch drops what its passes do not read.
 * A reduced-precision batch needs a matrix whose packed index stream builds
 * (every ray matrix of fair_paralleltomo / fair_fanlineartomo does). */
int fair_batch_add(fair_batch b, fair_csr h, int32_t take);

/* Problems, total rows, total columns, total nonzeros and device bytes held. */
int fair_batch_info(fair_batch b, int32_t *nprob, int64_t *rows, int64_t *cols, int64_t *nnz,
                    int64_t *device_bytes);
/* row_off and col_off (nprob + 1 each): problem p's rows are
 * row_off[p]..row_off[p+1]-1 of the concatenated b, its columns
 * col_off[p]..col_off[p+1]-1 of the concatenated x. */
int fair_batch_offsets(fair_batch b, int64_t *row_off, int64_t *col_off);

/* Algorithmic bytes of one iteration's two passes: the matrix streams
 * (packed words, padded values and escape rows, or CSR), their offsets, and
 * each vector read or written once (the column weights D only for SART). */
int fair_batch_pass_bytes(fair_batch b, int32_t sart, int64_t *pass1, int64_t *pass2);

/* K iterations of sirt_method ('cimmino' or 'sart') on every problem with
 * the same options: host vectors b_all (rows) and x_all (columns), x0_all
 * (columns) or NULL for zeros. */
int fair_batch_sirt(fair_batch b, const char *sirt_method, const double *b_all, int32_t K,
                    const double *x0_all, const fair_opts *options, double *x_all);

/* Device-resident form: fair_batch_prepare once per method/options, then
 * fair_batch_run_device (device pointers, asynchronous on the batch's
 * stream; the first call with a given K captures the graph). */
int fair_batch_prepare(fair_batch b, const char *sirt_method, const fair_opts *options);
int fair_batch_run_device(fair_batch b, const double *d_b, double *d_x, int32_t K);
/* The same K iterations launched problem by problem (two launches per
 * problem and iteration, no graph): the unbatched comparison. */
int fair_batch_run_device_unbatched(fair_batch b, const double *d_b, double *d_x, int32_t K);
/* Kernel launches of one fair_batch_run_device call of K iterations. */
int fair_batch_launches(fair_batch b, int32_t K, int64_t *launches);

/* Autotuner: times each batched pass for 4/8/16/32 lanes per row and, in
 * the reduced forms, 1 or 2 groups per lane (d_x is scratch), keeps the
 * fastest; config (may be NULL) receives {lanes A, lanes A', groups A,
 * groups A'}. fair_batch_set_config sets them directly. */
int fair_batch_autotune(fair_batch b, const double *d_b, double *d_x, int32_t reps,
                        int32_t *config);
int fair_batch_set_config(fair_batch b, const int32_t *config);

#ifdef __cplusplus
}
#endif
#endif /* FAIR_BATCH_H */
