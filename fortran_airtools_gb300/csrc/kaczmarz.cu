// kaczmarz.cu -- the ordered row-action sweep of basic_sweep
// (AIRMs.f90:813-858) as one thread block that walks the rows strictly in the
// reference's order; the threads of the block share each row's dot product
// (csr_matrowvec, sparse_matrices.f90:252-270) and its bounded update
// (add_mult_row, :795-822). Row i+1 starts only after row i's update is
// visible to the whole block (one barrier per row), so the iterate follows the
// reference's sequence of projections; only the summation order inside a dot
// product differs (a tree instead of a left-to-right sum).
//
// When the iterate fits in shared memory it is kept there for the whole
// sweep; otherwise it stays in global memory (L2-resident at these sizes).
#include <algorithm>

#include "fair_internal.cuh"

namespace fair {

namespace {

constexpr int kSweepThreads = 256;
constexpr int kSweepWarps = kSweepThreads / 32;
constexpr int kCache = 8;  // row entries held in registers per thread

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// first index i in [0, m) with cumul[i] >= u (the linear scan of
// AIRMs.f90:831-835 finds the same row on the nondecreasing cumul); m-1 if none
__device__ __forceinline__ int32_t sample_row(const double *cumul, int32_t m, double u) {
    int32_t L = 0, R = m;
    while (L < R) {
        int32_t mid = (L + R) >> 1;
        if (__ldg(cumul + mid) >= u) R = mid; else L = mid + 1;
    }
    return L < m ? L : m - 1;
}

template <bool SMEM_X, bool ROWPROB>
__global__ void __launch_bounds__(kSweepThreads) k_sweep(
    const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
    const double *__restrict__ val, const double *__restrict__ b,
    const double *__restrict__ nrA, const double *__restrict__ cumul, int32_t m, int32_t n,
    double *xg, const int32_t *__restrict__ ord, int32_t nord, int dir, double omg, int bmode,
    double lb, double ub, uint64_t seed, uint64_t ctr) {
    extern __shared__ double xs[];
    __shared__ double red[kSweepWarps];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    double *x = SMEM_X ? xs : xg;
    if (SMEM_X) {
        for (int32_t j = tid; j < n; j += kSweepThreads) xs[j] = xg[j];
        __syncthreads();
    }
    for (int32_t ii = 0; ii < nord; ++ii) {
        int32_t ri;
        if (ROWPROB) ri = sample_row(cumul, m, uniform01(seed, ctr + (uint64_t)ii));
        else ri = __ldg(ord + (dir > 0 ? ii : nord - 1 - ii)) - 1;
        const int64_t s = __ldg(rowptr + ri), e = __ldg(rowptr + ri + 1);
        int32_t cc[kCache];
        double vv[kCache];
        double part = 0.0;
#pragma unroll
        for (int q = 0; q < kCache; ++q) {
            int64_t j = s + tid + (int64_t)q * kSweepThreads;
            if (j < e) {
                cc[q] = __ldg(col + j);
                vv[q] = __ldg(val + j);
                part += x[cc[q]] * vv[q];
            }
        }
        for (int64_t j = s + tid + (int64_t)kCache * kSweepThreads; j < e; j += kSweepThreads)
            part += x[__ldg(col + j)] * __ldg(val + j);
        part = warp_sum(part);
        if (lane == 0) red[wid] = part;
        __syncthreads();
        double inp = 0.0;
#pragma unroll
        for (int w = 0; w < kSweepWarps; ++w) inp += red[w];
        // coeff = omg*(b(ri) - inp)/nrA(ri), AIRMs.f90:842
        const double coeff = __ddiv_rn(__dmul_rn(omg, __dsub_rn(__ldg(b + ri), inp)), __ldg(nrA + ri));
#pragma unroll
        for (int q = 0; q < kCache; ++q) {
            int64_t j = s + tid + (int64_t)q * kSweepThreads;
            if (j < e) {
                double t = __dadd_rn(x[cc[q]], __dmul_rn(coeff, vv[q]));
                if (bmode & 2) t = fmax_f(t, lb);
                if (bmode & 1) t = fmin_f(t, ub);
                x[cc[q]] = t;
            }
        }
        for (int64_t j = s + tid + (int64_t)kCache * kSweepThreads; j < e; j += kSweepThreads) {
            int32_t c = __ldg(col + j);
            double t = __dadd_rn(x[c], __dmul_rn(coeff, __ldg(val + j)));
            if (bmode & 2) t = fmax_f(t, lb);
            if (bmode & 1) t = fmin_f(t, ub);
            x[c] = t;
        }
        __syncthreads();
    }
    if (SMEM_X) {
        for (int32_t j = tid; j < n; j += kSweepThreads) xg[j] = xs[j];
    }
}

template <bool SMEM_X, bool ROWPROB>
int launch_sweep(const SweepDev &S, int dir, size_t smem, cudaStream_t s) {
    auto kern = k_sweep<SMEM_X, ROWPROB>;
    if (SMEM_X) FAIR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem));
    const DevCSR &A = *S.A;
    kern<<<1, kSweepThreads, smem, s>>>(A.rowptr.as<int64_t>(), A.col.as<int32_t>(),
                                        A.v64.as<double>(), S.b, S.nrA, S.cumul, A.m, A.n, S.x,
                                        S.ord, S.nord, dir, S.omg, S.bmode, S.lb, S.ub, S.seed,
                                        S.ctr);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

}  // namespace

int kaczmarz_sweep(const SweepDev &S, int dir, cudaStream_t s) {
    if (S.nord <= 0) return FAIR_OK;
    int dev = 0, optin = 0;
    FAIR_CUDA(cudaGetDevice(&dev));
    FAIR_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    size_t need = sizeof(double) * (size_t)S.A->n;
    bool smem = need + 1024 <= (size_t)optin;
    if (smem) {
        return S.rand_rowprob ? launch_sweep<true, true>(S, dir, need, s)
                              : launch_sweep<true, false>(S, dir, need, s);
    }
    return S.rand_rowprob ? launch_sweep<false, true>(S, dir, 0, s)
                          : launch_sweep<false, false>(S, dir, 0, s);
}

}  // namespace fair
