// sirt_epi.cuh -- the per-row epilogues of the two SIRT passes
// (AIRMs.f90:1089-1110), shared by the single-problem passes (solvers.cu)
// and the batched passes (batch.cu), so both compute the same numbers.
#pragma once

#include "fair_internal.cuh"

namespace fair {

__device__ __forceinline__ double sirt_box(double t, int bmode, double lb, double ub) {
    // AIRMs.f90:1093-1100: upper bound first, then lower bound
    if (bmode & 1) t = fmin_f(t, ub);
    if (bmode & 2) t = fmax_f(t, lb);
    return t;
}

// The weights arrive as reciprocals (sirt_weights_recip): a row costs one FP64
// multiply where the reference divides (an FP64 division is a sequence of
// FP64-pipe instructions, 64 cycles each on GB300); the result differs from
// the reference's quotient by at most about an ulp. 1/0 = Inf keeps the
// reference's Inf and 0/0 = NaN cases (x * Inf, 0 * Inf).
struct EpiResidF64 {  // r = (b - Ax) / M
    const double *b, *Mi;  // Mi = 1/M
    double *r;
    __device__ void operator()(int64_t i, double acc) const {
        r[i] = __dmul_rn(__dsub_rn(b[i], acc), Mi[i]);
    }
};
struct EpiResidLP {  // same, FP32 dot, FP64 weighting, FP32 residual
    const double *b, *Mi;
    float *r;
    double scale;  // 1, or the fixed-point scale of 16-bit codes
    __device__ void operator()(int64_t i, float acc) const {
        r[i] = (float)__dmul_rn(__dsub_rn(b[i], __dmul_rn((double)acc, scale)), Mi[i]);
    }
};
struct EpiUpdateF64 {  // x = P(x + omg * (A'r) / D)
    const double *Di;  // 1/D (null: D = 1)
    double *x;
    double omg, lb, ub;
    int bmode;
    __device__ void operator()(int64_t j, double acc) const {
        double g = __dmul_rn(omg, acc);
        if (Di) g = __dmul_rn(g, Di[j]);
        x[j] = sirt_box(__dadd_rn(x[j], g), bmode, lb, ub);
    }
};
struct EpiUpdateLP {
    const double *Di;
    double *x;
    float *x32;
    double omg, lb, ub;
    int bmode;
    double scale;  // 1, or the fixed-point scale of 16-bit codes
    __device__ void operator()(int64_t j, float acc) const {
        double g = __dmul_rn(omg, __dmul_rn((double)acc, scale));
        if (Di) g = __dmul_rn(g, Di[j]);
        double t = sirt_box(__dadd_rn(x[j], g), bmode, lb, ub);
        x[j] = t;
        x32[j] = (float)t;
    }
};

}  // namespace fair
