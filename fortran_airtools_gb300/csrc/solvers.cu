// solvers.cu -- the simultaneous AIR iterations of AIRMs.f90 as fused GPU
// kernels.
//
// SIRT (AIRMs.f90:1089-1110) is two row-parallel passes per iteration:
//   pass 1 over A:  r_i = (b_i - a_i . x) / M_i            (residual + weighting)
//   pass 2 over A': x_j = P(x_j + omg * (a^j . r) / D_j)   (backprojection + bounded update)
// with P = min(ub) then max(lb) (:1093-1100). Each pass reads its matrix once;
// the vector work is done in the epilogue of the warp that produced the dot
// product. The FP32/FP16 forms read FP32/FP16 values and FP32 vectors and
// accumulate in FP32, while the weights M, D and the iterate x stay FP64.
//
// Gradient descent (:959-982) and the power method of normest (:1159-1171)
// use the same passes plus deterministic block reductions. Their early exits
// are evaluated on the GPU: a flag set by a one-block kernel gates the later
// kernels, so the host enqueues all iterations without synchronising.
#include <algorithm>

#include "fair_internal.cuh"

namespace fair {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename VT> __device__ __forceinline__ float ldv32(const VT *p);
template <> __device__ __forceinline__ float ldv32<float>(const float *p) { return __ldcs(p); }
template <> __device__ __forceinline__ float ldv32<__half>(const __half *p) {
    return __half2float(__ldcs(p));
}

// Dot product of row r with the gathered vector x, one warp, result in all lanes.
__device__ __forceinline__ double row_dot_f64(const int64_t *__restrict__ rowptr,
                                              const int32_t *__restrict__ col,
                                              const double *__restrict__ v,
                                              const double *__restrict__ x, int64_t r, int lane) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    double acc = 0.0;
    int64_t j = s + lane;
    for (; j + 96 < e; j += 128) {
        int32_t c0 = __ldcs(col + j), c1 = __ldcs(col + j + 32), c2 = __ldcs(col + j + 64),
                c3 = __ldcs(col + j + 96);
        double v0 = __ldcs(v + j), v1 = __ldcs(v + j + 32), v2 = __ldcs(v + j + 64),
               v3 = __ldcs(v + j + 96);
        acc += __ldg(x + c0) * v0;
        acc += __ldg(x + c1) * v1;
        acc += __ldg(x + c2) * v2;
        acc += __ldg(x + c3) * v3;
    }
    for (; j < e; j += 32) acc += __ldg(x + __ldcs(col + j)) * __ldcs(v + j);
    return warp_sum(acc);
}

template <typename VT>
__device__ __forceinline__ float row_dot_lp(const int64_t *__restrict__ rowptr,
                                            const int32_t *__restrict__ col,
                                            const VT *__restrict__ v,
                                            const float *__restrict__ x, int64_t r, int lane) {
    int64_t s = rowptr[r], e = rowptr[r + 1];
    float acc = 0.f;
    int64_t j = s + lane;
    for (; j + 96 < e; j += 128) {
        int32_t c0 = __ldcs(col + j), c1 = __ldcs(col + j + 32), c2 = __ldcs(col + j + 64),
                c3 = __ldcs(col + j + 96);
        float v0 = ldv32(v + j), v1 = ldv32(v + j + 32), v2 = ldv32(v + j + 64),
              v3 = ldv32(v + j + 96);
        acc += __ldg(x + c0) * v0;
        acc += __ldg(x + c1) * v1;
        acc += __ldg(x + c2) * v2;
        acc += __ldg(x + c3) * v3;
    }
    for (; j < e; j += 32) acc += __ldg(x + __ldcs(col + j)) * ldv32(v + j);
    return warp_sum(acc);
}

__device__ __forceinline__ double box(double t, int bmode, double lb, double ub) {
    // AIRMs.f90:1093-1100: upper bound first, then lower bound
    if (bmode & 1) t = fmin_f(t, ub);
    if (bmode & 2) t = fmax_f(t, lb);
    return t;
}

#define WARP_LOOP                                                               \
    int lane = threadIdx.x & 31;                                                \
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;      \
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;                       \
    for (int64_t r = warp; r < m; r += nw)

// ---- SIRT pass 1: r = (b - A x) ./ M -------------------------------------
__global__ void __launch_bounds__(256) k_sirt_resid_f64(const int64_t *rowptr, int32_t m,
                                                        const int32_t *col, const double *v,
                                                        const double *x, const double *b,
                                                        const double *M, double *res) {
    WARP_LOOP {
        double acc = row_dot_f64(rowptr, col, v, x, r, lane);
        if (lane == 0) res[r] = __ddiv_rn(__dsub_rn(b[r], acc), M[r]);
    }
}

template <typename VT>
__global__ void __launch_bounds__(256) k_sirt_resid_lp(const int64_t *rowptr, int32_t m,
                                                       const int32_t *col, const VT *v,
                                                       const float *x, const double *b,
                                                       const double *M, float *res) {
    WARP_LOOP {
        float acc = row_dot_lp(rowptr, col, v, x, r, lane);
        if (lane == 0) res[r] = (float)__ddiv_rn(__dsub_rn(b[r], (double)acc), M[r]);
    }
}

// ---- SIRT pass 2: x = P(x + omg * (A' r) ./ D) ----------------------------
__global__ void __launch_bounds__(256) k_sirt_update_f64(const int64_t *rowptr, int32_t m,
                                                         const int32_t *col, const double *v,
                                                         const double *res, const double *D,
                                                         double *x, double omg, int bmode,
                                                         double lb, double ub) {
    WARP_LOOP {
        double acc = row_dot_f64(rowptr, col, v, res, r, lane);
        if (lane == 0) {
            double g = __dmul_rn(omg, acc);
            if (D) g = __ddiv_rn(g, D[r]);
            x[r] = box(__dadd_rn(x[r], g), bmode, lb, ub);
        }
    }
}

template <typename VT>
__global__ void __launch_bounds__(256) k_sirt_update_lp(const int64_t *rowptr, int32_t m,
                                                        const int32_t *col, const VT *v,
                                                        const float *res, const double *D,
                                                        double *x, float *x32, double omg,
                                                        int bmode, double lb, double ub) {
    WARP_LOOP {
        float acc = row_dot_lp(rowptr, col, v, res, r, lane);
        if (lane == 0) {
            double g = __dmul_rn(omg, (double)acc);
            if (D) g = __ddiv_rn(g, D[r]);
            double t = box(__dadd_rn(x[r], g), bmode, lb, ub);
            x[r] = t;
            x32[r] = (float)t;
        }
    }
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

// ---- reductions ---------------------------------------------------------------
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

__global__ void k_finish_sum(const double *partials, int np, double *out) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        *out = t;
    }
}

// ---- gradient descent ---------------------------------------------------------
// pass A': xn = P(x - step * A' r), partial sums of (xn - x)^2
__global__ void __launch_bounds__(256) k_gd_update(const int64_t *rowptr, int32_t m,
                                                   const int32_t *col, const double *v,
                                                   const double *res, const double *x,
                                                   double *xn, double step, int bmode, double lb,
                                                   double ub, const int *flag, double *partials) {
    if (flag[0]) return;
    double part = 0.0;
    WARP_LOOP {
        double acc = row_dot_f64(rowptr, col, v, res, r, lane);
        if (lane == 0) {
            double t = box(__dsub_rn(x[r], __dmul_rn(step, acc)), bmode, lb, ub);
            xn[r] = t;
            double d = t - x[r];
            part += d * d;
        }
    }
    block_partial(part, partials);
}

// one block: exit test norm2(xn - x) < tol (AIRMs.f90:972)
__global__ void k_gd_check(const double *partials, int np, double tol, int *flag) {
    __shared__ double sh[32];
    if (flag[0]) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        if (sqrt(t) < tol) flag[0] = 1;
        else flag[1] += 1;
    }
}

// pass A: r = A xn - b and x = xn
__global__ void __launch_bounds__(256) k_gd_resid(const int64_t *rowptr, int32_t m,
                                                  const int32_t *col, const double *v,
                                                  const double *xn, const double *b, double *res,
                                                  double *x, int32_t n, const int *flag) {
    if (flag[0]) return;
    WARP_LOOP {
        double acc = row_dot_f64(rowptr, col, v, xn, r, lane);
        if (lane == 0) res[r] = __dsub_rn(acc, b[r]);
    }
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
         j += (int64_t)gridDim.x * blockDim.x)
        x[j] = xn[j];
}

__global__ void k_neg(const double *b, int64_t m, double *r) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x)
        r[i] = -b[i];
}

// ---- power method (normest) ---------------------------------------------------
__global__ void __launch_bounds__(256) k_pm_spmv(const int64_t *rowptr, int32_t m,
                                                 const int32_t *col, const double *v,
                                                 const double *x, double *y, const int *flag,
                                                 double *partials) {
    if (flag && flag[0]) return;
    double part = 0.0;
    WARP_LOOP {
        double acc = row_dot_f64(rowptr, col, v, x, r, lane);
        if (lane == 0) {
            y[r] = acc;
            part += acc * acc;
        }
    }
    if (partials) block_partial(part, partials);
}

__global__ void k_pm_norm(const double *partials, int np, double *scal, const int *flag) {
    __shared__ double sh[32];
    if (flag[0]) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        scal[0] = sqrt(t);
    }
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

__global__ void k_pm_check(const double *partials, int np, double tol, int *flag) {
    __shared__ double sh[32];
    if (flag[0]) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        if (sqrt(t) < tol) flag[0] = 1;
    }
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

// ---- elementwise vector kernels (separately rounded, like the reference) ----
__global__ void k_vec_op(int op, double *out, const double *a, const double *b, double c,
                         int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        switch (op) {
            case 0: out[i] = __dsub_rn(a[i], b[i]); break;                 // a - b
            case 1: out[i] = __dadd_rn(a[i], __dmul_rn(c, b[i])); break;   // a + c*b
            case 2: out[i] = __ddiv_rn(a[i], c); break;                    // a / c
            case 3: out[i] = __dmul_rn(0.5, __dadd_rn(a[i], b[i])); break; // .5*(a+b)
            default: out[i] = a[i]; break;
        }
    }
}

__global__ void k_f32_to_f64v(const float *a, int64_t n, double *o) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        o[i] = (double)a[i];
}

int rows_grid(int64_t m) {
    int64_t b = (m * 32 + 255) / 256;
    int64_t cap = std::min<int64_t>((int64_t)sm_count() * 8, kReduceBlocks);
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}
int elem_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    int64_t cap = std::min<int64_t>((int64_t)sm_count() * 4, kReduceBlocks);
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, cap));
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

int sirt_prepare_shadow(const SirtDev &S, cudaStream_t s) {
    if (S.prec != FAIR_PREC_F64 && S.n > 0) {
        k_to_f32v<<<elem_grid(S.n), 256, 0, s>>>(S.x, S.n, S.x32);
        FAIR_CUDA(cudaGetLastError());
    }
    return FAIR_OK;
}

// One pass of a SIRT iteration: pass 1 = residual over A, pass 2 = update over A'.
static void sirt_pass(const SirtDev &S, int pass, cudaStream_t s) {
    const DevCSR &A = *S.A, &AT = *S.AT;
    if (pass == 1) {
        if (A.m == 0) return;
        int g = rows_grid(A.m);
        if (S.prec == FAIR_PREC_F64)
            k_sirt_resid_f64<<<g, 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(),
                                              A.v64.as<double>(), S.x, S.b, S.Minv, (double *)S.r);
        else if (S.prec == FAIR_PREC_F32)
            k_sirt_resid_lp<float><<<g, 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m,
                                                    A.col.as<int32_t>(), A.v32.as<float>(), S.x32,
                                                    S.b, S.Minv, (float *)S.r);
        else
            k_sirt_resid_lp<__half><<<g, 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m,
                                                     A.col.as<int32_t>(), A.v16.as<__half>(),
                                                     S.x32, S.b, S.Minv, (float *)S.r);
    } else {
        if (AT.m == 0) return;
        int g = rows_grid(AT.m);
        if (S.prec == FAIR_PREC_F64)
            k_sirt_update_f64<<<g, 256, 0, s>>>(AT.rowptr.as<int64_t>(), AT.m,
                                               AT.col.as<int32_t>(), AT.v64.as<double>(),
                                               (const double *)S.r, S.D, S.x, S.omg, S.bmode,
                                               S.lb, S.ub);
        else if (S.prec == FAIR_PREC_F32)
            k_sirt_update_lp<float><<<g, 256, 0, s>>>(
                AT.rowptr.as<int64_t>(), AT.m, AT.col.as<int32_t>(), AT.v32.as<float>(),
                (const float *)S.r, S.D, S.x, S.x32, S.omg, S.bmode, S.lb, S.ub);
        else
            k_sirt_update_lp<__half><<<g, 256, 0, s>>>(
                AT.rowptr.as<int64_t>(), AT.m, AT.col.as<int32_t>(), AT.v16.as<__half>(),
                (const float *)S.r, S.D, S.x, S.x32, S.omg, S.bmode, S.lb, S.ub);
    }
}

int sirt_iterations(const SirtDev &S, int K, cudaStream_t s) {
    if (S.prec != FAIR_PREC_F64) {
        FAIR_TRY(csr_make_lowprec(const_cast<DevCSR &>(*S.A), S.prec, s));
        FAIR_TRY(csr_make_lowprec(const_cast<DevCSR &>(*S.AT), S.prec, s));
    }
    for (int it = 0; it < K; ++it) {
        sirt_pass(S, 1, s);
        sirt_pass(S, 2, s);
        FAIR_CUDA(cudaGetLastError());
    }
    return FAIR_OK;
}

int sirt_iterations_timed(const SirtDev &S, int K, cudaStream_t s, float *ms1, float *ms2) {
    if (S.prec != FAIR_PREC_F64) {
        FAIR_TRY(csr_make_lowprec(const_cast<DevCSR &>(*S.A), S.prec, s));
        FAIR_TRY(csr_make_lowprec(const_cast<DevCSR &>(*S.AT), S.prec, s));
    }
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

int dev_sumsq_diff(const double *a, const double *b, int64_t n, double *d_partials,
                   double *d_out, cudaStream_t s) {
    int g = elem_grid(n);
    k_sumsq_diff<<<g, 256, 0, s>>>(a, b, n, d_partials);
    k_finish_sum<<<1, 256, 0, s>>>(d_partials, g, d_out);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int dev_dot(const double *a, const double *b, int64_t n, double *d_partials, double *d_out,
            cudaStream_t s) {
    int g = elem_grid(n);
    k_dot<<<g, 256, 0, s>>>(a, b, n, d_partials);
    k_finish_sum<<<1, 256, 0, s>>>(d_partials, g, d_out);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
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

int fill_uniform(double *d_v, int64_t n, uint64_t seed, uint64_t ctr, cudaStream_t s) {
    if (n > 0) k_uniform<<<elem_grid(n), 256, 0, s>>>(d_v, n, seed, ctr);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int gd_run(const GdDev &G, int maxiter, cudaStream_t s) {
    const DevCSR &A = *G.A, &AT = *G.AT;
    int gA = rows_grid(A.m), gT = rows_grid(AT.m);
    FAIR_CUDA(cudaMemsetAsync(G.flag, 0, 2 * sizeof(int), s));
    if (A.m > 0) k_neg<<<elem_grid(A.m), 256, 0, s>>>(G.b, A.m, G.r);  // r = -b (:954)
    for (int it = 0; it < maxiter; ++it) {
        k_gd_update<<<gT, 256, 0, s>>>(AT.rowptr.as<int64_t>(), AT.m, AT.col.as<int32_t>(),
                                       AT.v64.as<double>(), G.r, G.x, G.xn, G.step, G.bmode, G.lb,
                                       G.ub, G.flag, G.partials);
        k_gd_check<<<1, 256, 0, s>>>(G.partials, gT, G.tol, G.flag);
        k_gd_resid<<<gA, 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(),
                                      A.v64.as<double>(), G.xn, G.b, G.r, G.x, A.n, G.flag);
        FAIR_CUDA(cudaGetLastError());
    }
    return FAIR_OK;
}

int normest_run(const DevCSR &A, const DevCSR &AT, double *d_v, double *d_vn, double *d_w,
                double *d_partials, int *d_flag, double tol, int maxit, double *sigma,
                cudaStream_t s) {
    int gA = rows_grid(A.m), gT = rows_grid(AT.m), gE = elem_grid(A.n);
    double *scal = d_partials + kReduceBlocks;  // [0] norm, [1] ww, [2] vv
    FAIR_CUDA(cudaMemsetAsync(d_flag, 0, 2 * sizeof(int), s));
    for (int i = 0; i < maxit; ++i) {
        k_pm_spmv<<<gA, 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(),
                                     A.v64.as<double>(), d_v, d_w, d_flag, nullptr);
        k_pm_spmv<<<gT, 256, 0, s>>>(AT.rowptr.as<int64_t>(), AT.m, AT.col.as<int32_t>(),
                                     AT.v64.as<double>(), d_w, d_vn, d_flag, d_partials);
        k_pm_norm<<<1, 256, 0, s>>>(d_partials, gT, scal, d_flag);
        k_pm_scale<<<gE, 256, 0, s>>>(d_vn, d_v, A.n, scal, d_flag, d_partials);
        k_pm_check<<<1, 256, 0, s>>>(d_partials, gE, tol, d_flag);
        k_copy_gated<<<gE, 256, 0, s>>>(d_vn, d_v, A.n, d_flag);
        FAIR_CUDA(cudaGetLastError());
    }
    k_pm_spmv<<<gA, 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(),
                                 A.v64.as<double>(), d_v, d_w, nullptr, nullptr);
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
