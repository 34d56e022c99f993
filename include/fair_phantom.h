/* fair_phantom.h -- test phantoms and measurement noise generated on the GPU
 * (phantomgallery.f90, system_generation.f90:709-745), for large batches.
 *
 * Phantoms, vectorised column-major (phantomgallery.f90:672-690):
 *   'shepplogan'  (:116-164) -- the same image as fair_shepplogan, bit for bit;
 *   'smooth'      (:166-199) -- four Gaussians (the reference's centres,
 *                  including its single-precision literals), normalised;
 *   'grains'      (:529-600, uniform seeds) -- Voronoi cell index of the
 *                  nearest of p = int(3 sqrt(N)) seeds, normalised;
 *   '3phases'     (:201-254) -- two thresholded sums of 100 cubic bumps.
 * The random ones draw their seeds/centres from the library stream in the
 * reference's order (the reference's random_number stream is unseeded).
 * Distances use sqrt(dx^2 + dy^2) where the reference's norm2 scales
 * (same argmin up to ties); exp is CUDA's, so values agree with a host
 * evaluation to the last bits (thresholds can flip on exact borders).
 */
#ifndef FAIR_PHANTOM_H
#define FAIR_PHANTOM_H

#include "fair_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* N*N values into host memory x (computed on the GPU). An unknown name is
 * FAIR_ERR_ARG with "Not a recognised phantom." (phantomgallery.f90:111). */
int fair_phantom(const char *name, int32_t N, double *x);
/* The same into device memory, on cuda_stream (NULL: the legacy stream). */
int fair_phantom_device(const char *name, int32_t N, double *d_x, void *cuda_stream);

/* add_white_noise (system_generation.f90:709-745) on device vectors:
 * e_k = Phi^-1(u_k) by the reference's Newton iteration (tolerance 1e-14,
 * 100 iterations, FAIR_ERR_NEWTON when it does not converge), u_k the next m
 * draws of the library stream, then e = eta*|b|*e/|e| and bt = b + e. */
int fair_add_white_noise_device(double *d_bt, double *d_e, const double *d_b, int64_t m,
                                double eta, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* FAIR_PHANTOM_H */
