/* fair_mf.h -- matrix-free projector / backprojector pairs for the
 * parallel-beam geometry of paralleltomo (system_generation.f90:309-492) and
 * the fan-beam geometry of fanlineartomo (system_generation.f90:79-307), and
 * SIRT/SART on them (no counterpart in the reference, which always stores the
 * system matrix).
 *
 * Entry a_ij is the length of ray i inside pixel j, computed in closed form
 * from the signed distance between the pixel centre and the ray (the chord
 * of a unit square): the same segment lengths the ray tracer of
 * paralleltomo produces (to rounding, in FP64), with ties of axis-aligned
 * rays on a grid line going to the pixel on the positive side, as the
 * reference's floor-of-midpoint column rule does. The distance is evaluated
 * in 64-bit fixed point (46 fractional bits), so the projector (one thread
 * per ray) and the backprojector (one thread per pixel, gathering over the
 * rays of every angle) compute bit-identical entries: the pair is an exact
 * adjoint, deterministic, without atomics. Nothing of size nnz is stored.
 */
#ifndef FAIR_MF_H
#define FAIR_MF_H

#include "fair_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fair_mf_s *fair_mf;

/* Operator of the parallel-beam geometry in dat (n, p, nth, theta; r, dw, sd
 * unused, as in paralleltomo): m = nth*p rays, N*N pixels, column-major;
 * n <= 8192, 2 <= p <= 16384.
 * prec FAIR_PREC_F64 (FP64 entries, vectors and sums) or FAIR_PREC_F32
 * (FP32 entries, vectors and sums; SIRT keeps FP64 weights and iterate). */
int fair_mf_create_parallel(fair_mf *out, const fair_data *dat, int32_t prec);
/* Operator of the fan-beam geometry in dat (n, p, nth, r, dw, sd, theta) as
 * fanlineartomo builds it (system_generation.f90:79-307; geometry_fix as in
 * fair_fanlineartomo: 0 keeps the reference's odd-p bin angles of :122):
 * each ray's line from the same source position and direction values, one
 * record per ray (about 112 bytes: 58 MB for 720 angles x 725 bins). The
 * backprojector finds a pixel's rays per angle by the angle of the pixel
 * seen from the source. A ray that the reference's rounding tilts across a
 * grid line (odd p: the central ray at theta = pi/2, pi, 3pi/2, where the
 * residue of cos or sin moves it by ~1e-16) lies on one side here. */
int fair_mf_create_fan(fair_mf *out, const fair_data *dat, int32_t geometry_fix, int32_t prec);
int fair_mf_destroy(fair_mf A);
int fair_mf_set_stream(fair_mf A, void *cuda_stream);
int fair_mf_info(fair_mf A, int32_t *m, int32_t *n);

/* Number of (ray, pixel) pairs with a positive entry (the nonzeros the
 * stored matrix would hold), counted by one projector pass. */
int fair_mf_nnz(fair_mf A, int64_t *nnz);

/* y(m) = A x(n) and x(n) = A' y(m), host vectors (FP64 in and out). */
int fair_mf_project(fair_mf A, const double *x, double *y);
int fair_mf_backproject(fair_mf A, const double *y, double *x);

/* K iterations of sirt_method ('cimmino' or 'sart') with options, as
 * fair_sirt (AIRMs.f90:1089-1110): host vectors b (m), x0 (n, NULL: zeros),
 * x (n). The weights (row sums or squared row norms, column sums) come from
 * one FP64 pass each, computed once per method. */
int fair_mf_sirt(fair_mf A, const char *sirt_method, const double *b, int32_t K,
                 const double *x0, const fair_opts *options, double *x);

/* Device-resident form: prepare once, then run on device vectors (FP64 b
 * and x), asynchronous on the operator's stream. */
int fair_mf_sirt_prepare(fair_mf A, const char *sirt_method, const fair_opts *options);
int fair_mf_sirt_run_device(fair_mf A, const double *d_b, double *d_x, int32_t K);
/* Per-pass timing of K device iterations (ms summed over the iterations). */
int fair_mf_sirt_run_device_timed(fair_mf A, const double *d_b, double *d_x, int32_t K,
                                  float *ms_project, float *ms_backproject);

#ifdef __cplusplus
}
#endif
#endif /* FAIR_MF_H */
