// solvers.cu -- the simultaneous AIR iterations of AIRMs.f90 as fused GPU
// kernels on the row-product engine of rows.cuh.
//
// SIRT (AIRMs.f90:1089-1110) is two passes per iteration:
//   pass 1 over A:  r_i = (b_i - a_i . x) / M_i            (residual + weighting)
//   pass 2 over A': x_j = P(x_j + omg * (a^j . r) / D_j)   (backprojection + bounded update)
// with P = min(ub) then max(lb) (:1093-1100). Each pass streams its matrix once
// and applies the vector work in the coalesced per-chunk epilogue. The
// FP32/FP16 forms read FP32/FP16 values and FP32 vectors and accumulate in
// FP32, while the weights M, D and the iterate x stay FP64.
//
// Gradient descent (:959-982) and the power method of normest (:1159-1171)
// use the same passes plus deterministic block reductions. Their early exits
// are evaluated on the GPU: a flag set by a one-block kernel gates the later
// kernels, so the host enqueues all iterations without synchronising.
#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "fair_internal.cuh"
#include "rows.cuh"
#include "sirt_epi.cuh"

namespace fair {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of one double per thread into partials[blockIdx.x] (fixed order).
__device__ __forceinline__ void block_partial(double v, double *partials) {
    __shared__ double sh[32];
    v = warp_sum(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
        partials[blockIdx.x] = s;
    }
}

// ---- epilogues (SIRT ones in sirt_epi.cuh) ----------------------------------------
struct EpiGdUpdate {  // xn = P(x - step * A'r), partial sum of (xn - x)^2
    const double *x;
    double *xn;
    double step, lb, ub;
    int bmode;
    double part = 0.0;
    __device__ void operator()(int64_t j, double acc) {
        double t = sirt_box(__dsub_rn(x[j], __dmul_rn(step, acc)), bmode, lb, ub);
        xn[j] = t;
        double d = t - x[j];
        part += d * d;
    }
};
struct EpiGdResid {  // r = A xn - b
    const double *b;
    double *r;
    __device__ void operator()(int64_t i, double acc) const { r[i] = __dsub_rn(acc, b[i]); }
};
struct EpiStoreSq {  // y = Ax, partial sum of y^2
    double *y;
    double part = 0.0;
    __device__ void operator()(int64_t i, double acc) {
        y[i] = acc;
        part += acc * acc;
    }
};

// ---- kernels --------------------------------------------------------------------
template <int G>
__global__ void __launch_bounds__(256) k_sirt_resid_f64(const int64_t *rowptr, int32_t m,
                                                        const int32_t *col, const double *v,
                                                        const double *x, EpiResidF64 epi,
                                                        unsigned *sched) {
    chunk_rows<double, double, double, G>(rowptr, m, col, v, x, epi, sched);
}
// Matrices with few rows: a group of 32/G rows per warp (rows_by_group, the
// same per-row arithmetic as the chunked kernels above).
template <int G, class Epi>
__global__ void __launch_bounds__(256) k_sirt_rows_f64(const int64_t *rowptr, int32_t m,
                                                       const int32_t *col, const double *v,
                                                       const double *x, Epi epi) {
    rows_by_group<double, double, double, G>(rowptr, m, col, v, x, epi);
}
template <typename VT, int G>
__global__ void __launch_bounds__(256) k_sirt_resid_lp(const int64_t *rowptr, int32_t m,
                                                       const int32_t *col, const VT *v,
                                                       const float *x, EpiResidLP epi,
                                                       unsigned *sched) {
    chunk_rows<VT, float, float, G>(rowptr, m, col, v, x, epi, sched);
}
// Packed index stream (rows.cuh) with padded values.
struct PkArgs {
    const int64_t *prow;
    const uint2 *gidx;
    const int4 *gside;
    int S, L;
};
template <typename VT, int G, int NG>
__global__ void __launch_bounds__(256) k_sirt_resid_pk(PkArgs P, int32_t m, const VT *v,
                                                       const float *x, EpiResidLP epi,
                                                       unsigned *sched) {
    chunk_rows_pk<VT, float, float, G, NG>(P.prow, m, P.gidx, P.gside, P.S, P.L, v, x, epi, sched);
}
template <typename VT, int G, int NG>
__global__ void __launch_bounds__(256) k_sirt_update_pk(PkArgs P, int32_t m, const VT *v,
                                                        const float *r, EpiUpdateLP epi,
                                                        unsigned *sched) {
    chunk_rows_pk<VT, float, float, G, NG>(P.prow, m, P.gidx, P.gside, P.S, P.L, v, r, epi, sched);
}
template <typename VT, int G, int NG>
__global__ void __launch_bounds__(256) k_sirt_resid_pkf(PkArgs P, int32_t m, const uint4 *rec,
                                                        const float *x, EpiResidLP epi,
                                                        unsigned *sched) {
    chunk_rows_pkf<VT, G, NG>(P.prow, m, rec, P.gside, P.S, P.L, x, epi, sched);
}
template <typename VT, int G, int NG>
__global__ void __launch_bounds__(256) k_sirt_update_pkf(PkArgs P, int32_t m, const uint4 *rec,
                                                         const float *r, EpiUpdateLP epi,
                                                         unsigned *sched) {
    chunk_rows_pkf<VT, G, NG>(P.prow, m, rec, P.gside, P.S, P.L, r, epi, sched);
}
template <int G, int NG>
__global__ void __launch_bounds__(256) k_sirt_resid_pk64(PkArgs P, int32_t m, const double *v,
                                                         const double *x, EpiResidF64 epi,
                                                         unsigned *sched) {
    chunk_rows_pk<double, double, double, G, NG>(P.prow, m, P.gidx, P.gside, P.S, P.L, v, x, epi,
                                                 sched);
}
template <int G, int NG>
__global__ void __launch_bounds__(256) k_sirt_update_pk64(PkArgs P, int32_t m, const double *v,
                                                          const double *r, EpiUpdateF64 epi,
                                                          unsigned *sched) {
    chunk_rows_pk<double, double, double, G, NG>(P.prow, m, P.gidx, P.gside, P.S, P.L, v, r, epi,
                                                 sched);
}
template <int G>
__global__ void __launch_bounds__(256) k_sirt_update_f64(const int64_t *rowptr, int32_t m,
                                                         const int32_t *col, const double *v,
                                                         const double *r, EpiUpdateF64 epi,
                                                         unsigned *sched) {
    chunk_rows<double, double, double, G>(rowptr, m, col, v, r, epi, sched);
}
template <typename VT, int G>
__global__ void __launch_bounds__(256) k_sirt_update_lp(const int64_t *rowptr, int32_t m,
                                                        const int32_t *col, const VT *v,
                                                        const float *r, EpiUpdateLP epi,
                                                        unsigned *sched) {
    chunk_rows<VT, float, float, G>(rowptr, m, col, v, r, epi, sched);
}
template <int G>
__global__ void __launch_bounds__(256) k_gd_update(const int64_t *rowptr, int32_t m,
                                                   const int32_t *col, const double *v,
                                                   const double *r, EpiGdUpdate epi,
                                                   const int *flag, double *partials) {
    if (flag[0]) return;
    chunk_rows<double, double, double, G>(rowptr, m, col, v, r, epi);
    block_partial(epi.part, partials);
}
template <int G>
__global__ void __launch_bounds__(256) k_gd_resid(const int64_t *rowptr, int32_t m,
                                                  const int32_t *col, const double *v,
                                                  const double *xn, EpiGdResid epi, double *x,
                                                  int32_t n, const int *flag) {
    if (flag[0]) return;
    chunk_rows<double, double, double, G>(rowptr, m, col, v, xn, epi);
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
         j += (int64_t)gridDim.x * blockDim.x)
        x[j] = xn[j];
}
template <int G>
__global__ void __launch_bounds__(256) k_pm_spmv(const int64_t *rowptr, int32_t m,
                                                 const int32_t *col, const double *v,
                                                 const double *x, EpiStoreSq epi, const int *flag,
                                                 double *partials) {
    if (flag && flag[0]) return;
    chunk_rows<double, double, double, G>(rowptr, m, col, v, x, epi);
    if (partials) block_partial(epi.part, partials);
}

__global__ void k_cimmino_M(double *M, int32_t m) {
    // AIRMs.f90:1072: Mdiag = m * row_norms(2)**2
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x)
        M[i] = __dmul_rn((double)m, __dmul_rn(M[i], M[i]));
}

__global__ void k_to_f32v(const double *a, int64_t n, float *o) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        o[i] = (float)a[i];
}

__global__ void k_f32_to_f64v(const float *a, int64_t n, double *o) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        o[i] = (double)a[i];
}

// ---- elementwise vector kernels (separately rounded, like the reference) ----
__global__ void k_vec_op(int op, double *out, const double *a, const double *b, double c,
                         int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        switch (op) {
            case VEC_SUB: out[i] = __dsub_rn(a[i], b[i]); break;
            case VEC_AXPY: out[i] = __dadd_rn(a[i], __dmul_rn(c, b[i])); break;
            case VEC_DIV: out[i] = __ddiv_rn(a[i], c); break;
            case VEC_MEAN: out[i] = __dmul_rn(0.5, __dadd_rn(a[i], b[i])); break;
            default: out[i] = a[i]; break;
        }
    }
}

// ---- reductions ---------------------------------------------------------------
__global__ void k_sumsq_diff(const double *a, const double *b, int64_t n, double *partials) {
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double d = b ? a[i] - b[i] : a[i];
        s += d * d;
    }
    block_partial(s, partials);
}

__global__ void k_dot(const double *a, const double *b, int64_t n, double *partials) {
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    block_partial(s, partials);
}

// One block: fixed-order sum of np partials. mode 0: out = sum; mode 1:
// out = sqrt(sum) (normest norm); mode 2: flag[0] = sqrt(sum) < tol, else
// flag[1]++ (gradient descent exit test, AIRMs.f90:972); mode 3: flag[0] =
// sqrt(sum) < tol (normest exit test, :1164). Modes 1-3 are skipped once
// flag[0] is set.
__global__ void k_finish(const double *partials, int np, double *out, int mode, double tol,
                         int *flag) {
    __shared__ double sh[32];
    if (mode > 0 && flag[0]) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        if (mode == 0) *out = t;
        else if (mode == 1) *out = sqrt(t);
        else if (mode == 2) { if (sqrt(t) < tol) flag[0] = 1; else flag[1] += 1; }
        else if (sqrt(t) < tol) flag[0] = 1;
    }
}

__global__ void k_neg(const double *b, int64_t m, double *r) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x)
        r[i] = -b[i];
}

// vn = vn / s; partial sums of (vn - v)^2
__global__ void k_pm_scale(double *vn, const double *v, int64_t n, const double *scal,
                           const int *flag, double *partials) {
    if (flag[0]) return;
    double s = scal[0], part = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double t = __ddiv_rn(vn[i], s);
        vn[i] = t;
        double d = t - v[i];
        part += d * d;
    }
    block_partial(part, partials);
}

__global__ void k_copy_gated(const double *src, double *dst, int64_t n, const int *flag) {
    if (flag[0]) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

__global__ void k_uniform(double *v, int64_t n, uint64_t seed, uint64_t ctr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        v[i] = uniform01(seed, ctr + (uint64_t)i);
}

int elem_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    int64_t cap = std::min<int64_t>((int64_t)sm_count() * 4, kReduceBlocks);
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}

#define FAIR_G_DISPATCH(G, CALL)                 \
    switch (G) {                                 \
        case 4: { constexpr int g_ = 4; CALL; } break;   \
        case 16: { constexpr int g_ = 16; CALL; } break; \
        case 32: { constexpr int g_ = 32; CALL; } break; \
        default: { constexpr int g_ = 8; CALL; } break;  \
    }

}  // namespace

// ------------------------------------------------------------------ host ----
int sirt_weights(const DevCSR &A, const DevCSR &AT, bool sart, double *d_M, double *d_D,
                 cudaStream_t s) {
    if (!sart) {
        FAIR_TRY(csr_row_norms(A, 2, d_M, s));
        if (A.m > 0) k_cimmino_M<<<elem_grid(A.m), 256, 0, s>>>(d_M, A.m);
        FAIR_CUDA(cudaGetLastError());
    } else {
        // AIRMs.f90:1076-1079: row 1-norms, column 1-norms (via the transpose)
        FAIR_TRY(csr_row_norms(A, 1, d_M, s));
        FAIR_TRY(csr_row_norms(AT, 1, d_D, s));
    }
    return FAIR_OK;
}

__global__ void k_reciprocal(double *v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        v[i] = __ddiv_rn(1.0, v[i]);
}

int vec_reciprocal(double *v, int64_t n, cudaStream_t s) {
    if (n <= 0) return FAIR_OK;
    k_reciprocal<<<elem_grid(n), 256, 0, s>>>(v, n);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int sirt_weights_recip(const DevCSR &A, const DevCSR &AT, bool sart, double *d_Mi, double *d_Di,
                       cudaStream_t s) {
    FAIR_TRY(sirt_weights(A, AT, sart, d_Mi, d_Di, s));
    FAIR_TRY(vec_reciprocal(d_Mi, A.m, s));
    if (sart) FAIR_TRY(vec_reciprocal(d_Di, A.n, s));
    return FAIR_OK;
}

int sirt_prepare_shadow(const SirtDev &S, cudaStream_t s) {
    if (S.prec != FAIR_PREC_F64 && S.n > 0) {
        k_to_f32v<<<elem_grid(S.n), 256, 0, s>>>(S.x, S.n, S.x32);
        FAIR_CUDA(cudaGetLastError());
    }
    return FAIR_OK;
}

// One reduced-precision pass on the layout `code` selects (0 the CSR; 1, 2
// the packed stream with that many groups per lane; 3, 4 the fused records),
// falling back to the layouts that exist: `pvals` (padded values) and
// `fused` may be null.
template <typename VT>
static void lp_pass(const SirtDev &S, const DevCSR &M, int pass, const VT *vals,
                    const VT *pvals, const uint4 *fused, double scale, int code,
                    cudaStream_t s) {
    const PkArgs P{M.prow.as<int64_t>(), M.gidx.as<uint2>(), M.gside.as<int4>(), M.pk_S, M.pk_L};
    const int G = M.sirt_lanes[S.prec];
    if (code == 14) {  // the tiled copy's step records (else its 4-entry slots)
        if (sirt_pass_tiled(S, M, pass, code, s)) return;
        code = 9;
    }
    if (code >= 11 && code <= 13) {
        if (sirt_pass_delta(S, M, pass, code, s)) return;
        code = code == 11 ? 5 : 8;  // no delta copy: the sliced copy
    }
    if (code == 9 || code == 10) {
        if (sirt_pass_tiled(S, M, pass, code, s)) return;
        code = 3;  // no tiled copy: the fused records (else the packed stream)
    }
    if (code >= 5) {
        if (sirt_pass_sliced(S, M, pass, code, s)) return;
        code = (code & 1) ? 1 : 2;  // no sliced copy: the packed stream's lane layout
    }
    if (code >= 3 && (!fused || sizeof(VT) != 2)) code -= 2;
    if (code >= 1 && !pvals) code = 0;
    if (pass == 1) {
        EpiResidLP e{S.b, S.Minv, (float *)S.r, scale};
        switch (code) {
            case 4:
                if constexpr (sizeof(VT) == 2)
                    FAIR_G_DISPATCH(G, (k_sirt_resid_pkf<VT, g_, 2><<<chunk_grid(k_sirt_resid_pkf<VT, g_, 2>, M.m), 256, 0, s>>>(
                                           P, M.m, fused, S.x32, e, S.sched)))
                break;
            case 3:
                if constexpr (sizeof(VT) == 2)
                    FAIR_G_DISPATCH(G, (k_sirt_resid_pkf<VT, g_, 1><<<chunk_grid(k_sirt_resid_pkf<VT, g_, 1>, M.m), 256, 0, s>>>(
                                           P, M.m, fused, S.x32, e, S.sched)))
                break;
            case 2: FAIR_G_DISPATCH(G, (k_sirt_resid_pk<VT, g_, 2><<<chunk_grid(k_sirt_resid_pk<VT, g_, 2>, M.m), 256, 0, s>>>(
                                           P, M.m, pvals, S.x32, e, S.sched))) break;
            case 1: FAIR_G_DISPATCH(G, (k_sirt_resid_pk<VT, g_, 1><<<chunk_grid(k_sirt_resid_pk<VT, g_, 1>, M.m), 256, 0, s>>>(
                                           P, M.m, pvals, S.x32, e, S.sched))) break;
            default: FAIR_G_DISPATCH(G, (k_sirt_resid_lp<VT, g_><<<chunk_grid(k_sirt_resid_lp<VT, g_>, M.m), 256, 0, s>>>(
                                            M.rowptr.as<int64_t>(), M.m, M.col.as<int32_t>(), vals, S.x32, e, S.sched))) break;
        }
    } else {
        EpiUpdateLP e{S.D, S.x, S.x32, S.omg, S.lb, S.ub, S.bmode, scale};
        const float *r = (const float *)S.r;
        switch (code) {
            case 4:
                if constexpr (sizeof(VT) == 2)
                    FAIR_G_DISPATCH(G, (k_sirt_update_pkf<VT, g_, 2><<<chunk_grid(k_sirt_update_pkf<VT, g_, 2>, M.m), 256, 0, s>>>(
                                           P, M.m, fused, r, e, S.sched)))
                break;
            case 3:
                if constexpr (sizeof(VT) == 2)
                    FAIR_G_DISPATCH(G, (k_sirt_update_pkf<VT, g_, 1><<<chunk_grid(k_sirt_update_pkf<VT, g_, 1>, M.m), 256, 0, s>>>(
                                           P, M.m, fused, r, e, S.sched)))
                break;
            case 2: FAIR_G_DISPATCH(G, (k_sirt_update_pk<VT, g_, 2><<<chunk_grid(k_sirt_update_pk<VT, g_, 2>, M.m), 256, 0, s>>>(
                                           P, M.m, pvals, r, e, S.sched))) break;
            case 1: FAIR_G_DISPATCH(G, (k_sirt_update_pk<VT, g_, 1><<<chunk_grid(k_sirt_update_pk<VT, g_, 1>, M.m), 256, 0, s>>>(
                                           P, M.m, pvals, r, e, S.sched))) break;
            default: FAIR_G_DISPATCH(G, (k_sirt_update_lp<VT, g_><<<chunk_grid(k_sirt_update_lp<VT, g_>, M.m), 256, 0, s>>>(
                                            M.rowptr.as<int64_t>(), M.m, M.col.as<int32_t>(), vals, r, e, S.sched))) break;
        }
    }
}

// One pass of a SIRT iteration: pass 1 = residual over A, pass 2 = update over A'.
void sirt_pass(const SirtDev &S, int pass, cudaStream_t s) {
    const DevCSR &M = pass == 1 ? *S.A : *S.AT;
    if (M.m == 0) return;
    if (S.prec == FAIR_PREC_F64) {
        const int G = M.sirt_lanes[FAIR_PREC_F64];
        int NG = M.sirt_groups[FAIR_PREC_F64];
        if (NG > 0 && M.haspk && M.hasp64 && packed_enabled()) {
            const PkArgs P{M.prow.as<int64_t>(), M.gidx.as<uint2>(), M.gside.as<int4>(), M.pk_S,
                           M.pk_L};
            const double *pv = M.pv64.as<double>();
            if (NG == 14) NG = 9;  // step records: 2-byte forms only
            if (NG >= 11 && NG <= 13 && sirt_pass_delta(S, M, pass, NG, s)) return;
            if ((NG == 9 || NG == 10) && sirt_pass_tiled(S, M, pass, NG, s)) return;
            if (NG >= 5 && NG <= 8 && sirt_pass_sliced(S, M, pass, NG, s)) return;
            if (NG >= 9) NG = 1;
            if (NG > 2) NG = 2 - (NG & 1);  // 3, 5 -> 1 group per lane; 4, 6 -> 2
            if (pass == 1) {
                EpiResidF64 e{S.b, S.Minv, (double *)S.r};
                if (NG == 2)
                    FAIR_G_DISPATCH(G, (k_sirt_resid_pk64<g_, 2><<<chunk_grid(k_sirt_resid_pk64<g_, 2>, M.m), 256, 0, s>>>(
                                           P, M.m, pv, S.x, e, S.sched)))
                else
                    FAIR_G_DISPATCH(G, (k_sirt_resid_pk64<g_, 1><<<chunk_grid(k_sirt_resid_pk64<g_, 1>, M.m), 256, 0, s>>>(
                                           P, M.m, pv, S.x, e, S.sched)))
            } else {
                EpiUpdateF64 e{S.D, S.x, S.omg, S.lb, S.ub, S.bmode};
                if (NG == 2)
                    FAIR_G_DISPATCH(G, (k_sirt_update_pk64<g_, 2><<<chunk_grid(k_sirt_update_pk64<g_, 2>, M.m), 256, 0, s>>>(
                                           P, M.m, pv, (const double *)S.r, e, S.sched)))
                else
                    FAIR_G_DISPATCH(G, (k_sirt_update_pk64<g_, 1><<<chunk_grid(k_sirt_update_pk64<g_, 1>, M.m), 256, 0, s>>>(
                                           P, M.m, pv, (const double *)S.r, e, S.sched)))
            }
            return;
        }
        const int64_t *rp = M.rowptr.as<int64_t>();
        const int32_t *cl = M.col.as<int32_t>();
        // fewer 32-row chunks than 16 warps per SM: a group of rows per warp
        // (FAIR_ROWS_BY_GROUP=0: the chunked engine for every matrix)
        const char *bg = getenv("FAIR_ROWS_BY_GROUP");
        if (!(bg && bg[0] == '0') && ((int64_t)M.m + 31) / 32 < (int64_t)sm_count() * 16) {
            auto go = [&](auto kern, const double *xv, const auto &e) {
                int occ = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 256, 0);
                const int64_t units = ((int64_t)M.m * G + 31) / 32;  // groups of 32/G rows
                const int64_t blocks = std::min<int64_t>((units + 7) / 8, (int64_t)sm_count() * std::max(occ, 1));
                kern<<<(int)std::max<int64_t>(blocks, 1), 256, 0, s>>>(rp, M.m, cl, M.v64.as<double>(), xv, e);
            };
            if (pass == 1) {
                const EpiResidF64 e{S.b, S.Minv, (double *)S.r};
                FAIR_G_DISPATCH(G, go(k_sirt_rows_f64<g_, EpiResidF64>, S.x, e));
            } else {
                const EpiUpdateF64 e{S.D, S.x, S.omg, S.lb, S.ub, S.bmode};
                FAIR_G_DISPATCH(G, go(k_sirt_rows_f64<g_, EpiUpdateF64>, (const double *)S.r, e));
            }
            return;
        }
        if (pass == 1) {
            EpiResidF64 e{S.b, S.Minv, (double *)S.r};
            FAIR_G_DISPATCH(G, (k_sirt_resid_f64<g_><<<chunk_grid(k_sirt_resid_f64<g_>, M.m), 256, 0, s>>>(
                                                  rp, M.m, cl, M.v64.as<double>(), S.x, e, S.sched)));
        } else {
            EpiUpdateF64 e{S.D, S.x, S.omg, S.lb, S.ub, S.bmode};
            FAIR_G_DISPATCH(G, (k_sirt_update_f64<g_><<<chunk_grid(k_sirt_update_f64<g_>, M.m), 256, 0, s>>>(
                                                  rp, M.m, cl, M.v64.as<double>(), (const double *)S.r, e, S.sched)));
        }
        return;
    }
    const bool pk = M.haspk && packed_enabled();
    const int code = M.sirt_groups[S.prec];
    const uint4 *f16 = pk && M.hasf16 ? M.pf16.as<uint4>() : nullptr;
    const uint4 *fq = pk && M.hasfq ? M.pfq.as<uint4>() : nullptr;
    if (S.prec == FAIR_PREC_F32) {
        lp_pass(S, M, pass, M.v32.as<float>(), pk && M.hasp32 ? M.pv32.as<float>() : nullptr,
                nullptr, 1.0, code, s);
    } else if (S.prec == FAIR_PREC_F16) {
        lp_pass(S, M, pass, M.v16.as<__half>(), pk && M.hasp16 ? M.pv16.as<__half>() : nullptr,
                f16, 1.0, code, s);
    } else if (M.qsigned) {
        lp_pass(S, M, pass, M.vq.as<int16_t>(), pk && M.haspq ? M.pvq.as<int16_t>() : nullptr,
                fq, M.qscale, code, s);
    } else {
        lp_pass(S, M, pass, M.vq.as<uint16_t>(), pk && M.haspq ? M.pvq.as<uint16_t>() : nullptr,
                fq, M.qscale, code, s);
    }
}

// The derived value copies (and packed index streams) a reduced-precision
// SIRT needs on A and A'. With `all` (the autotuner) the packed layouts of
// the form are built; otherwise the ones the passes are set to read. Sliced
// copies are built only for a pass set to read one (the autotuner builds its
// own candidates); `sliced` = false leaves them out.
int sirt_make_forms(DevCSR &A, DevCSR &AT, int prec, cudaStream_t s, bool all, bool sliced) {
    if (prec != FAIR_PREC_F64) {
        FAIR_TRY(csr_make_lowprec(A, prec, s));
        FAIR_TRY(csr_make_lowprec(AT, prec, s));
    }
    // FP64 reads the CSR unless tuned (or asked) to read the packed stream,
    // whose padded FP64 values cost 8 bytes per nonzero more
    const bool f64_pk = all || A.sirt_groups[FAIR_PREC_F64] > 0 ||
                        AT.sirt_groups[FAIR_PREC_F64] > 0;
    if (packed_enabled() && (prec != FAIR_PREC_F64 || f64_pk)) {
        FAIR_TRY(csr_make_packed(A, prec, s));
        FAIR_TRY(csr_make_packed(AT, prec, s));
        FAIR_TRY(csr_make_fused(A, prec, s));
        FAIR_TRY(csr_make_fused(AT, prec, s));
        if (sliced && A.sirt_groups[prec] >= 5 && A.sirt_groups[prec] <= 8)
            FAIR_TRY(csr_make_sliced(A, prec, A.sirt_lanes[prec], s));
        if (sliced && AT.sirt_groups[prec] >= 5 && AT.sirt_groups[prec] <= 8)
            FAIR_TRY(csr_make_sliced(AT, prec, AT.sirt_lanes[prec], s));
        auto tiled = [](int g) { return g == 9 || g == 10 || g == 14; };
        auto delta = [](int g) { return g >= 11 && g <= 13; };
        if (sliced && tiled(A.sirt_groups[prec])) FAIR_TRY(csr_make_tiled(A, prec, 1, s));
        if (sliced && tiled(AT.sirt_groups[prec])) FAIR_TRY(csr_make_tiled(AT, prec, 2, s));
        if (sliced && delta(A.sirt_groups[prec])) FAIR_TRY(csr_make_delta(A, prec, s));
        if (sliced && delta(AT.sirt_groups[prec])) FAIR_TRY(csr_make_delta(AT, prec, s));
    }
    return FAIR_OK;
}

int sirt_iterations(const SirtDev &S, int K, cudaStream_t s) {
    FAIR_TRY(sirt_make_forms(const_cast<DevCSR &>(*S.A), const_cast<DevCSR &>(*S.AT), S.prec, s));
    for (int it = 0; it < K; ++it) {
        sirt_pass(S, 1, s);
        sirt_pass(S, 2, s);
        FAIR_CUDA(cudaGetLastError());
    }
    return FAIR_OK;
}

// True when some form of M is set to read its sliced copy.
static bool uses_sliced(const DevCSR &M) {
    for (int g : M.sirt_groups)
        if (g >= 5 && g <= 8) return true;
    return false;
}
static bool uses_tiled(const DevCSR &M) {
    for (int g : M.sirt_groups)
        if (g == 9 || g == 10 || g == 14) return true;
    return false;
}
static bool uses_delta(const DevCSR &M) {
    for (int g : M.sirt_groups)
        if (g >= 11 && g <= 13) return true;
    return false;
}

int sirt_autotune(const SirtDev &S, DevCSR &A, DevCSR &AT, int reps, cudaStream_t s,
                  float *ms_best) {
    FAIR_TRY(sirt_make_forms(A, AT, S.prec, s, true));
    FAIR_TRY(sirt_prepare_shadow(S, s));
    cudaEvent_t ev[2];
    for (auto &e : ev) FAIR_CUDA(cudaEventCreate(&e));
    int st = FAIR_OK;
    for (int pass = 1; pass <= 2 && st == FAIR_OK; ++pass) {
        DevCSR &M = pass == 1 ? A : AT;
        const bool pk = M.haspk && packed_enabled() &&
                        (S.prec != FAIR_PREC_F64 || M.hasp64);
        const bool fu = pk && (S.prec == FAIR_PREC_F16 ? M.hasf16 : S.prec == FAIR_PREC_Q16 && M.hasfq);
        // candidates {layout code, lanes per row}: the CSR (0), the packed
        // stream (1, 2), the fused records (3, 4) with 4-32 lanes per row;
        // the sliced copy (5-8) with 1-8, or 0 (per chunk); the tiled copy (9, 10);
        // the delta copy (11-13)
        struct Cand { int code, lanes; };
        Cand cand[56];
        int nc = 0;
        for (int code = 0; code <= 4; ++code) {
            if ((code >= 1 && !pk) || (code >= 3 && !fu)) continue;
            for (int g : {4, 8, 16, 32}) cand[nc++] = {code, g};
        }
        if (pk && (S.prec == FAIR_PREC_F64 || S.prec == FAIR_PREC_F32 || fu))
            for (int g : {0, 1, 2, 4, 8})
                for (int code : {5, 6, 7, 8}) cand[nc++] = {code, g};
        // the delta copy (11-13)
        st = csr_make_delta(M, S.prec, s);
        if (st != FAIR_OK) break;
        if (M.dl[S.prec == FAIR_PREC_F16 || S.prec == FAIR_PREC_Q16].built)
            for (int code : {11, 12, 13}) cand[nc++] = {code, 8};
        // the tiled copy (9, 10; 14 its step records): image tiles of A's
        // columns for pass 1, pixel tiles x angle blocks of A' for pass 2
        st = csr_make_tiled(M, S.prec, pass, s);
        if (st != FAIR_OK) break;
        if (M.tl.built())
            for (int code : {9, 10}) cand[nc++] = {code, 8};
        if (M.tl.built6 && (S.prec == FAIR_PREC_F16 || S.prec == FAIR_PREC_Q16)) cand[nc++] = {14, 8};
        int best_g = M.sirt_lanes[S.prec], best_code = M.sirt_groups[S.prec];
        float best_ms = -1.f;
        float t[56];
        // two rounds over the candidates; each keeps its faster round
        for (int round = 0; round < 2 && st == FAIR_OK; ++round)
            for (int i = 0; i < nc && st == FAIR_OK; ++i) {
                const Cand c = cand[i];
                if (c.code >= 5 && c.code <= 8) {
                    st = csr_make_sliced(M, S.prec, c.lanes, s);
                    if (st != FAIR_OK) break;
                    if (!M.hassl) { t[i] = -1.f; continue; }  // no sliced copy for this matrix
                }
                M.sirt_lanes[S.prec] = c.lanes;
                M.sirt_groups[S.prec] = c.code;
                sirt_pass(S, pass, s);  // warm-up
                cudaEventRecord(ev[0], s);
                for (int r = 0; r < reps; ++r) sirt_pass(S, pass, s);
                cudaEventRecord(ev[1], s);
                cudaError_t e = cudaEventSynchronize(ev[1]);
                if (e == cudaSuccess) e = cudaGetLastError();  // a launch that failed times as nothing
                if (e != cudaSuccess) { st = cuda_fail(e, "autotune", __FILE__, __LINE__); break; }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev[0], ev[1]);
                ms /= reps;
                t[i] = round == 0 ? ms : std::min(t[i], ms);
                if (round == 1 && (best_ms < 0.f || t[i] < best_ms)) {
                    best_ms = t[i];
                    best_g = c.lanes;
                    best_code = c.code;
                }
            }
        M.sirt_lanes[S.prec] = best_g;
        M.sirt_groups[S.prec] = best_code;
        // a tiled pass: try other tile shapes (the copy is rebuilt for each)
        // unless the caller asked for one
        if (st == FAIR_OK && (best_code == 9 || best_code == 10 || best_code == 14) &&
            M.tile_req[0] == 0 && M.tile_req[1] == 0) {
            static const int shapes[2][4][2] = {{{96, 0}, {64, 0}, {128, 0}, {0, 0}},
                                                {{32, 13000}, {32, 6500}, {16, 6500}, {48, 13000}}};
            int best_shape = 0;
            float best_t = best_ms;
            for (int k = 1; k < 4 && st == FAIR_OK; ++k) {
                if (shapes[pass - 1][k][0] == 0) continue;
                M.tile_req[0] = shapes[pass - 1][k][0];
                M.tile_req[1] = shapes[pass - 1][k][1];
                st = csr_make_tiled(M, S.prec, pass, s);
                if (st != FAIR_OK) break;
                if (!M.tl.built() || (best_code == 14 && !M.tl.built6)) continue;
                float tk = -1.f;
                for (int round = 0; round < 2 && st == FAIR_OK; ++round) {
                    sirt_pass(S, pass, s);  // warm-up
                    cudaEventRecord(ev[0], s);
                    for (int r = 0; r < reps; ++r) sirt_pass(S, pass, s);
                    cudaEventRecord(ev[1], s);
                    cudaError_t e = cudaEventSynchronize(ev[1]);
                    if (e == cudaSuccess) e = cudaGetLastError();
                    if (e != cudaSuccess) { st = cuda_fail(e, "autotune", __FILE__, __LINE__); break; }
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, ev[0], ev[1]);
                    ms /= reps;
                    tk = round == 0 ? ms : std::min(tk, ms);
                }
                if (st == FAIR_OK && tk >= 0.f && tk < best_t) {
                    best_t = tk;
                    best_shape = k;
                }
            }
            // keep the best shape; the default is recorded as no request
            M.tile_req[0] = best_shape ? shapes[pass - 1][best_shape][0] : 0;
            M.tile_req[1] = best_shape ? shapes[pass - 1][best_shape][1] : 0;
            if (st == FAIR_OK) st = csr_make_tiled(M, S.prec, pass, s);
            best_ms = best_t;
        }
        if (st == FAIR_OK && best_code >= 5 && best_code <= 8) st = csr_make_sliced(M, S.prec, best_g, s);
        if (!uses_sliced(M)) M.drop_sliced();  // free the copies no pass reads
        if (!uses_tiled(M)) M.tl.release();
        if (!uses_delta(M)) {
            M.dl[0].release();
            M.dl[1].release();
        }
        if (ms_best) ms_best[pass - 1] = best_ms;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return st;
}

int sirt_iterations_timed(const SirtDev &S, int K, cudaStream_t s, float *ms1, float *ms2) {
    FAIR_TRY(sirt_make_forms(const_cast<DevCSR &>(*S.A), const_cast<DevCSR &>(*S.AT), S.prec, s));
    cudaEvent_t ev[3];
    for (auto &e : ev) FAIR_CUDA(cudaEventCreate(&e));
    float t1 = 0.f, t2 = 0.f;
    int st = FAIR_OK;
    for (int it = 0; it < K && st == FAIR_OK; ++it) {
        cudaEventRecord(ev[0], s);
        sirt_pass(S, 1, s);
        cudaEventRecord(ev[1], s);
        sirt_pass(S, 2, s);
        cudaEventRecord(ev[2], s);
        cudaError_t e = cudaEventSynchronize(ev[2]);
        if (e != cudaSuccess) { st = cuda_fail(e, "sirt pass", __FILE__, __LINE__); break; }
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        t1 += a;
        t2 += b;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    *ms1 = t1;
    *ms2 = t2;
    return st;
}

int vec_op(int op, double *out, const double *a, const double *b, double c, int64_t n,
           cudaStream_t s) {
    if (n > 0) k_vec_op<<<elem_grid(n), 256, 0, s>>>(op, out, a, b, c, n);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int vec_to_f32(const double *a, int64_t n, float *o, cudaStream_t s) {
    if (n > 0) k_to_f32v<<<elem_grid(n), 256, 0, s>>>(a, n, o);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int vec_to_f64(const float *a, int64_t n, double *o, cudaStream_t s) {
    if (n > 0) k_f32_to_f64v<<<elem_grid(n), 256, 0, s>>>(a, n, o);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int dev_sumsq_diff(const double *a, const double *b, int64_t n, double *d_partials,
                   double *d_out, cudaStream_t s) {
    int g = elem_grid(n);
    k_sumsq_diff<<<g, 256, 0, s>>>(a, b, n, d_partials);
    k_finish<<<1, 256, 0, s>>>(d_partials, g, d_out, 0, 0.0, nullptr);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int dev_dot(const double *a, const double *b, int64_t n, double *d_partials, double *d_out,
            cudaStream_t s) {
    int g = elem_grid(n);
    k_dot<<<g, 256, 0, s>>>(a, b, n, d_partials);
    k_finish<<<1, 256, 0, s>>>(d_partials, g, d_out, 0, 0.0, nullptr);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int fill_uniform(double *d_v, int64_t n, uint64_t seed, uint64_t ctr, cudaStream_t s) {
    if (n > 0) k_uniform<<<elem_grid(n), 256, 0, s>>>(d_v, n, seed, ctr);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int gd_run(const GdDev &G, int maxiter, cudaStream_t s) {
    const DevCSR &A = *G.A, &AT = *G.AT;
    FAIR_CUDA(cudaMemsetAsync(G.flag, 0, 2 * sizeof(int), s));
    if (A.m > 0) k_neg<<<elem_grid(A.m), 256, 0, s>>>(G.b, A.m, G.r);  // r = -b (:954)
    for (int it = 0; it < maxiter; ++it) {
        int gT = 1;
        EpiGdUpdate eu{G.x, G.xn, G.step, G.lb, G.ub, G.bmode};
        FAIR_G_DISPATCH(AT.lanes_per_row, (gT = chunk_grid(k_gd_update<g_>, AT.m),
                        k_gd_update<g_><<<gT, 256, 0, s>>>(AT.rowptr.as<int64_t>(), AT.m,
                                                           AT.col.as<int32_t>(), AT.v64.as<double>(),
                                                           G.r, eu, G.flag, G.partials)));
        k_finish<<<1, 256, 0, s>>>(G.partials, gT, nullptr, 2, G.tol, G.flag);
        EpiGdResid er{G.b, G.r};
        FAIR_G_DISPATCH(A.lanes_per_row, (k_gd_resid<g_><<<chunk_grid(k_gd_resid<g_>, A.m), 256, 0, s>>>(
                                              A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(),
                                              A.v64.as<double>(), G.xn, er, G.x, A.n, G.flag)));
        FAIR_CUDA(cudaGetLastError());
    }
    return FAIR_OK;
}

int normest_run(const DevCSR &A, const DevCSR &AT, double *d_v, double *d_vn, double *d_w,
                double *d_partials, int *d_flag, double tol, int maxit, double *sigma,
                cudaStream_t s) {
    const int gE = elem_grid(A.n);
    double *scal = d_partials + kReduceBlocks;  // [0] norm, [1] ww, [2] vv
    FAIR_CUDA(cudaMemsetAsync(d_flag, 0, 2 * sizeof(int), s));
    for (int i = 0; i < maxit; ++i) {
        EpiStoreSq ew{d_w};
        FAIR_G_DISPATCH(A.lanes_per_row, (k_pm_spmv<g_><<<chunk_grid(k_pm_spmv<g_>, A.m), 256, 0, s>>>(
                                              A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(),
                                              A.v64.as<double>(), d_v, ew, d_flag, nullptr)));
        int gT = 1;
        EpiStoreSq ev{d_vn};
        FAIR_G_DISPATCH(AT.lanes_per_row, (gT = chunk_grid(k_pm_spmv<g_>, AT.m),
                        k_pm_spmv<g_><<<gT, 256, 0, s>>>(AT.rowptr.as<int64_t>(), AT.m,
                                                         AT.col.as<int32_t>(), AT.v64.as<double>(),
                                                         d_w, ev, d_flag, d_partials)));
        k_finish<<<1, 256, 0, s>>>(d_partials, gT, scal, 1, 0.0, d_flag);
        k_pm_scale<<<gE, 256, 0, s>>>(d_vn, d_v, A.n, scal, d_flag, d_partials);
        k_finish<<<1, 256, 0, s>>>(d_partials, gE, nullptr, 3, tol, d_flag);
        k_copy_gated<<<gE, 256, 0, s>>>(d_vn, d_v, A.n, d_flag);
        FAIR_CUDA(cudaGetLastError());
    }
    EpiStoreSq ew{d_w};
    FAIR_G_DISPATCH(A.lanes_per_row, (k_pm_spmv<g_><<<chunk_grid(k_pm_spmv<g_>, A.m), 256, 0, s>>>(
                                          A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(),
                                          A.v64.as<double>(), d_v, ew, nullptr, nullptr)));
    FAIR_CUDA(cudaGetLastError());
    FAIR_TRY(dev_dot(d_w, d_w, A.m, d_partials, scal + 1, s));
    FAIR_TRY(dev_dot(d_v, d_v, A.n, d_partials, scal + 2, s));
    double h[2];
    FAIR_CUDA(cudaMemcpyAsync(h, scal + 1, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    *sigma = sqrt(h[0] / h[1]);
    return FAIR_OK;
}

}  // namespace fair
