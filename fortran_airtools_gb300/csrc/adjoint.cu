// adjoint.cu -- reverse-mode adjoint of K unrolled SIRT/SART steps with box
// projection, for up to 16 right-hand sides sharing one matrix.
//
// Forward (AIRMs.f90:1089-1110, per right-hand side c with relaxation lam_c):
//   r_k = M^-1 (b - A x_k),  g_k = A' r_k,  z_k = x_k + (lam_c g_k) / D,
//   x_{k+1} = P(z_k) = max(min(z_k, ub), lb)   (the bounds present in opts)
// Reverse, for k = K-1 .. 0, starting from gx = dL/dx_K:
//   gz = gx * [P does not clamp z_k]
//   glam_c += <gz, g_k / D>
//   w = M^-1 A (D^-1 gz)        (w_i = 0 on empty rows, which b does not reach)
//   gb += lam_c w
//   gx = gz - lam_c A' w
// and dL/dx0 = gx after the last step. Checkpoints of x every ceil(sqrt(K))
// steps; each segment is recomputed forward (keeping x_k and g_k) before it
// is reversed, so memory is O(sqrt(K)) vectors and work is three forward
// sweeps of products.
//
// Vectors of the batch are interleaved ([row][NR]) so that one gather loads
// every right-hand side of a column; the multi-vector row engine follows the
// chunk layout of rows.cuh (32 rows per warp chunk, G lanes per row, results
// moved to lane row mod 32 for a coalesced epilogue).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fair_gpu_ext.h"
#include "fair_internal.cuh"
#include "rows.cuh"

namespace fair {

namespace {

constexpr int kG = 8;        // lanes per row of the multi-vector engine (one right-hand side)
constexpr int kRhsRows = 8;  // rows per chunk of the engine with right-hand sides across lanes

template <typename T, int NR>
__device__ __forceinline__ void load_row_vec(const T *__restrict__ p, T (&o)[NR]) {
#pragma unroll
    for (int r = 0; r < NR; ++r) o[r] = __ldg(p + r);
}

template <typename T, int NR, class Epi>
__device__ __forceinline__ void chunk_rows_multi(const int64_t *__restrict__ rowptr, int32_t m,
                                                 const int32_t *__restrict__ col,
                                                 const T *__restrict__ val,
                                                 const T *__restrict__ x, Epi &epi,
                                                 unsigned *sched) {
    constexpr int G = kG, R = 32 / G;
    const int lane = threadIdx.x & 31, g = lane / G, gl = lane % G;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = ((int64_t)m + 31) >> 5;
    for (int64_t ch = next_chunk(sched, 0, nwarps, lane); ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int64_t base = ch << 5;
        T mine[NR];
#pragma unroll
        for (int r = 0; r < NR; ++r) mine[r] = 0;
#pragma unroll 1
        for (int sub = 0; sub < 32; sub += R) {
            const int64_t row = base + sub + g;
            int64_t s = 0, e = 0;
            if (row < m) {
                s = __ldg(rowptr + row);
                e = __ldg(rowptr + row + 1);
            }
            T acc[NR];
#pragma unroll
            for (int r = 0; r < NR; ++r) acc[r] = 0;
            for (int64_t k = s + gl; k < e; k += G) {
                const int32_t c = __ldcs(col + k);
                const T v = __ldcs(val + k);
                T xv[NR];
                load_row_vec<T, NR>(x + (size_t)c * NR, xv);
#pragma unroll
                for (int r = 0; r < NR; ++r) acc[r] += v * xv[r];
            }
#pragma unroll
            for (int r = 0; r < NR; ++r) {
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
                T t = __shfl_sync(0xffffffffu, acc[r], ((lane - sub) & (R - 1)) * G);
                if (lane >= sub && lane < sub + R) mine[r] = t;
            }
        }
        const int64_t row = base + lane;
        if (row < m) epi(row, mine);
    }
    finish_chunks(sched, nwarps, lane);
}

// The same products with the right-hand sides across the lanes (NR = 4 or
// 16): lane l handles right-hand side l % NR of entry slot l / NR, so a warp
// step covers E = 32 / NR entries of one row and each entry's NR values of x
// are one contiguous run of NR x sizeof(T) bytes. The warp reads a row's
// entries 32 at a time (lane l loads entry l of the block: one coalesced load
// of columns and one of values, the next block's issued before the current
// one is used), hands each entry to its slot's lanes by shuffles, and keeps
// the block's 32 / E gathers of x in flight. The E slots are added by
// shuffles at the row's end and lanes 0..NR-1 apply the epilogue to the row's
// NR sums (Epi::one). A warp walks the kRhsRows rows of a chunk in turn;
// small chunks keep every warp of a persistent grid busy.
template <typename T, int NR, class Epi>
__device__ __forceinline__ void chunk_rows_rhs(const int64_t *__restrict__ rowptr, int32_t m,
                                               const int32_t *__restrict__ col,
                                               const T *__restrict__ val, const T *__restrict__ x,
                                               const Epi &epi, unsigned *sched) {
    static_assert(NR == 4 || NR == 16, "4 or 16 right-hand sides");
    constexpr int E = 32 / NR, STEPS = 32 / E, NA = 4, CR = kRhsRows;
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, slot = lane / NR, c = lane % NR;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = ((int64_t)m + CR - 1) / CR;
    for (int64_t ch = next_chunk(sched, 0, nwarps, lane); ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int64_t base = ch * CR;
        const int rows = (int)((int64_t)m - base < CR ? (int64_t)m - base : CR);
        for (int rr = 0; rr < rows; ++rr) {
            const int64_t row = base + rr;
            const int64_t s = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
            T acc[NA];
#pragma unroll
            for (int a = 0; a < NA; ++a) acc[a] = 0;
            int64_t kk = s + lane;
            int32_t cl = kk < e ? __ldcs(col + kk) : 0;
            T vl = kk < e ? __ldcs(val + kk) : (T)0;
            for (int64_t kb = s; kb < e; kb += 32) {
                // the next block's entries, loaded while this one is used
                const int64_t kn = kb + 32 + lane;
                const int32_t cn = kn < e ? __ldcs(col + kn) : 0;
                const T vn = kn < e ? __ldcs(val + kn) : (T)0;
                const int nb = (int)(e - kb < 32 ? e - kb : 32);
#pragma unroll
                for (int t = 0; t < STEPS; ++t) {
                    // steps past the row's end stay predicated: leaving the loop there
                    // (a warp-uniform break) keeps the gathers from issuing ahead, and
                    // measured FP32 throughput fell from 25 to 11 batch gradients/s
                    const int src = t * E + slot;
                    const int32_t cj = __shfl_sync(FULL, cl, src);
                    const T vj = __shfl_sync(FULL, vl, src);
                    if (src < nb) acc[t % NA] += vj * __ldg(x + (size_t)cj * NR + c);
                }
                cl = cn;
                vl = vn;
            }
            T v = (acc[0] + acc[1]) + (acc[2] + acc[3]);
#pragma unroll
            for (int o = 16; o >= NR; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
            if (lane < NR) epi.one(row, c, v);
        }
    }
    finish_chunks(sched, nwarps, lane);
}

template <typename T>
__device__ __forceinline__ T boxT(T t, int bmode, T lb, T ub) {
    if (bmode & 1) t = t < ub || t != t ? t : ub;   // min(t, ub), the non-NaN wins
    if (bmode & 2) t = t > lb || t != t ? t : lb;   // max(t, lb)
    return t;
}

// forward pass 1: r = (b - A x) / M
template <typename T, int NR>
struct EpiFwdResid {
    const T *b, *M;
    T *r;
    __device__ void one(int64_t i, int c, T v) const { r[i * NR + c] = (b[i * NR + c] - v) / M[i]; }
    __device__ void operator()(int64_t i, const T (&acc)[NR]) const {
#pragma unroll
        for (int c = 0; c < NR; ++c) one(i, c, acc[c]);
    }
};
// forward pass 2: g = A' r (kept when recording), x = P(x + lam g / D)
template <typename T, int NR>
struct EpiFwdUpdate {
    const T *D, *lam;
    T *x, *gsave;
    T lb, ub;
    int bmode;
    __device__ void one(int64_t j, int c, T v) const {
        T u = lam[c] * v;
        if (D) u = u / D[j];
        if (gsave) gsave[j * NR + c] = v;
        x[j * NR + c] = boxT<T>(x[j * NR + c] + u, bmode, lb, ub);
    }
    __device__ void operator()(int64_t j, const T (&acc)[NR]) const {
#pragma unroll
        for (int c = 0; c < NR; ++c) one(j, c, acc[c]);
    }
};
// reverse, over A: w = (A t) / M (0 on empty rows), gb += lam w
template <typename T, int NR>
struct EpiAdjA {
    const T *M, *lam;
    T *w, *gb;
    __device__ void one(int64_t i, int c, T v) const {
        T wi = M[i] != (T)0 ? v / M[i] : (T)0;
        w[i * NR + c] = wi;
        gb[i * NR + c] += lam[c] * wi;
    }
    __device__ void operator()(int64_t i, const T (&acc)[NR]) const {
#pragma unroll
        for (int c = 0; c < NR; ++c) one(i, c, acc[c]);
    }
};
// reverse, over A': gx = gz - lam A' w
template <typename T, int NR>
struct EpiAdjAT {
    const T *gz, *lam;
    T *gx;
    __device__ void one(int64_t j, int c, T v) const { gx[j * NR + c] = gz[j * NR + c] - lam[c] * v; }
    __device__ void operator()(int64_t j, const T (&acc)[NR]) const {
#pragma unroll
        for (int c = 0; c < NR; ++c) one(j, c, acc[c]);
    }
};

// (256, 4): up to 64 registers, so the 16 gathers of a block stay in flight
// without spills (measured: FP32 39 ms per 16-problem adjoint against 58 ms
// when the compiler chose 32 registers).
template <typename T, int NR, class Epi>
__global__ void __launch_bounds__(256, 4) k_multi(const int64_t *rowptr, int32_t m, const int32_t *col,
                                               const T *val, const T *x, Epi epi, unsigned *sched) {
    if constexpr (NR == 1)
        chunk_rows_multi<T, NR>(rowptr, m, col, val, x, epi, sched);
    else
        chunk_rows_rhs<T, NR>(rowptr, m, col, val, x, epi, sched);
}

// Elementwise reverse step: gz = gx * [P does not clamp z], t = gz / D,
// per-block partial sums of gz * g / D for every column (FP64).
template <typename T, int NR>
__global__ void __launch_bounds__(256) k_adj_mask(int64_t n, const T *x, const T *gk, const T *D,
                                                  const T *lam, const T *gx, T *gz, T *t, int bmode,
                                                  T lb, T ub, double *partials) {
    __shared__ double sh[NR][8];
    double part = 0.0;
    const int64_t total = n * NR;
    // blockDim.x (256) and the grid stride are multiples of NR, so each thread
    // always handles the same column c = threadIdx.x % NR
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / NR;
        const int c = (int)(e % NR);
        T g = gk[e];
        T u = lam[c] * g;
        T d = D ? D[j] : (T)1;
        if (D) u = u / d;
        T z = x[e] + u;
        bool pass = true;
        T zc = z;
        if (bmode & 1) { pass = pass && (z < ub); zc = z < ub ? z : ub; }
        if (bmode & 2) pass = pass && (zc > lb);
        T gzv = pass ? gx[e] : (T)0;
        gz[e] = gzv;
        t[e] = D ? gzv / d : gzv;
        part += (double)gzv * (double)(D ? g / d : g);
    }
    // reduce over the threads sharing a column: lanes c, c+NR, ... then warps
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o >= NR; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane < NR) sh[lane][wid] = part;
    __syncthreads();
    if (threadIdx.x < NR) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[threadIdx.x][w];
        partials[(size_t)blockIdx.x * NR + threadIdx.x] = s;
    }
}

// x0 (column-major n x nrhs, or zeros) into the interleaved layout
template <typename T>
__global__ void k_interleave(const double *src, int64_t rows, int nrhs, int NRt, int c0, T *dst) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rows * NRt;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e / NRt;
        int c = (int)(e % NRt);
        dst[e] = (src && c0 + c < nrhs && c < NRt) ? (T)src[(size_t)(c0 + c) * rows + i] : (T)0;
    }
}

template <typename T>
__global__ void k_deinterleave(const T *src, int64_t rows, int nrhs, int NRt, int c0, int ncols,
                               double *dst) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rows * ncols;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e % rows;
        int c = (int)(e / rows);
        dst[(size_t)(c0 + c) * rows + i] = (double)src[i * NRt + c];
    }
}

template <typename T>
__global__ void k_cast(const double *a, int64_t n, T *o) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        o[i] = (T)a[i];
}

int egrid(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm_count() * 4));
}

// Blocks of 8 warps for the chunks of m rows (32 rows per chunk for one
// right-hand side, kRhsRows for more), at most the resident blocks.
template <class K>
int mgrid(K kernel, int64_t m, int nr) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, 0);
    if (occ < 1) occ = 1;
    const int64_t rpc = nr == 1 ? 32 : kRhsRows;
    int64_t need = (((int64_t)m + rpc - 1) / rpc + 7) / 8;
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sm_count() * occ, need));
}

struct AdjBufs {
    DevBuf b, x, r, gk_seg, x_seg, cp, gx, gz, t, w, gb, lam, M, D, part;
};

template <typename T, int NR>
int run_group(const DevCSR &A, const DevCSR &AT, const T *vA, const T *vAT, bool sart,
              const double *h_b, const double *h_x0, const double *h_gx, const double *h_lam,
              int nrhs, int c0, int ncols, int K, int bmode, double lb, double ub,
              const double *d_M64, const double *d_D64, unsigned *sched, cudaStream_t s,
              double *h_xK, double *h_gb, double *h_gx0, double *h_glam) {
    const int64_t m = A.m, n = A.n;
    const int C = K > 0 ? (int)std::ceil(std::sqrt((double)K)) : 1;
    const int nseg = K > 0 ? (K + C - 1) / C : 0;
    AdjBufs B;
    FAIR_TRY(B.b.grow(sizeof(T) * m * NR));
    FAIR_TRY(B.r.grow(sizeof(T) * m * NR));
    FAIR_TRY(B.w.grow(sizeof(T) * m * NR));
    FAIR_TRY(B.gb.grow(sizeof(T) * m * NR));
    FAIR_TRY(B.x.grow(sizeof(T) * n * NR));
    FAIR_TRY(B.gx.grow(sizeof(T) * n * NR));
    FAIR_TRY(B.gz.grow(sizeof(T) * n * NR));
    FAIR_TRY(B.t.grow(sizeof(T) * n * NR));
    FAIR_TRY(B.cp.grow(sizeof(T) * n * NR * (size_t)(nseg + 1)));
    FAIR_TRY(B.x_seg.grow(sizeof(T) * n * NR * (size_t)C));
    FAIR_TRY(B.gk_seg.grow(sizeof(T) * n * NR * (size_t)C));
    FAIR_TRY(B.lam.grow(sizeof(T) * NR));
    FAIR_TRY(B.M.grow(sizeof(T) * m));
    FAIR_TRY(B.D.grow(sizeof(T) * n));
    const int ge = egrid(n * NR);
    FAIR_TRY(B.part.grow(sizeof(double) * (size_t)ge * NR));
    // inputs
    DevBuf stage;
    FAIR_TRY(stage.grow(sizeof(double) * std::max<int64_t>(m, n) * ncols));
    FAIR_CUDA(cudaMemcpyAsync(stage.p, h_b + (size_t)c0 * m, sizeof(double) * m * ncols,
                              cudaMemcpyHostToDevice, s));
    k_interleave<T><<<egrid(m * NR), 256, 0, s>>>(stage.as<double>(), m, ncols, NR, 0, B.b.as<T>());
    if (h_x0) {
        FAIR_CUDA(cudaMemcpyAsync(stage.p, h_x0 + (size_t)c0 * n, sizeof(double) * n * ncols,
                                  cudaMemcpyHostToDevice, s));
        k_interleave<T><<<egrid(n * NR), 256, 0, s>>>(stage.as<double>(), n, ncols, NR, 0, B.x.as<T>());
    } else {
        k_interleave<T><<<egrid(n * NR), 256, 0, s>>>(nullptr, n, ncols, NR, 0, B.x.as<T>());
    }
    FAIR_CUDA(cudaStreamSynchronize(s));  // stage reused below
    FAIR_CUDA(cudaMemcpyAsync(stage.p, h_gx + (size_t)c0 * n, sizeof(double) * n * ncols,
                              cudaMemcpyHostToDevice, s));
    k_interleave<T><<<egrid(n * NR), 256, 0, s>>>(stage.as<double>(), n, ncols, NR, 0, B.gx.as<T>());
    T lamh[NR];
    for (int c = 0; c < NR; ++c) lamh[c] = (T)(c < ncols ? h_lam[c0 + c] : 0.0);
    FAIR_CUDA(cudaMemcpyAsync(B.lam.p, lamh, sizeof(lamh), cudaMemcpyHostToDevice, s));
    k_cast<T><<<egrid(m), 256, 0, s>>>(d_M64, m, B.M.as<T>());
    if (sart) k_cast<T><<<egrid(n), 256, 0, s>>>(d_D64, n, B.D.as<T>());
    FAIR_CUDA(cudaMemsetAsync(B.gb.p, 0, sizeof(T) * m * NR, s));
    FAIR_CUDA(cudaGetLastError());
    const T *D = sart ? B.D.as<T>() : nullptr;
    const T tlb = (T)lb, tub = (T)ub;
    auto fwd_step = [&](T *gsave) -> int {
        EpiFwdResid<T, NR> e1{B.b.as<T>(), B.M.as<T>(), B.r.as<T>()};
        auto k1 = k_multi<T, NR, EpiFwdResid<T, NR>>;
        k1<<<mgrid(k1, m, NR), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(), vA,
                                        B.x.as<T>(), e1, sched);
        EpiFwdUpdate<T, NR> e2{D, B.lam.as<T>(), B.x.as<T>(), gsave, tlb, tub, bmode};
        auto k2 = k_multi<T, NR, EpiFwdUpdate<T, NR>>;
        k2<<<mgrid(k2, n, NR), 256, 0, s>>>(AT.rowptr.as<int64_t>(), AT.m, AT.col.as<int32_t>(), vAT,
                                        B.r.as<T>(), e2, sched);
        FAIR_CUDA(cudaGetLastError());
        return FAIR_OK;
    };
    const size_t vecb = sizeof(T) * n * NR;
    // forward with checkpoints
    for (int k = 0; k < K; ++k) {
        if (k % C == 0)
            FAIR_CUDA(cudaMemcpyAsync(B.cp.as<char>() + vecb * (k / C), B.x.p, vecb,
                                      cudaMemcpyDeviceToDevice, s));
        FAIR_TRY(fwd_step(nullptr));
    }
    if (h_xK) {
        k_deinterleave<T><<<egrid(n * ncols), 256, 0, s>>>(B.x.as<T>(), n, nrhs, NR, 0, ncols,
                                                           stage.as<double>());
        FAIR_CUDA(cudaMemcpyAsync(h_xK + (size_t)c0 * n, stage.p, sizeof(double) * n * ncols,
                                  cudaMemcpyDeviceToHost, s));
        FAIR_CUDA(cudaStreamSynchronize(s));
    }
    // reverse, one segment at a time
    std::vector<double> glam_acc(NR, 0.0), hpart((size_t)ge * NR);
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int k0 = seg * C, k1 = std::min(K, k0 + C);
        FAIR_CUDA(cudaMemcpyAsync(B.x.p, B.cp.as<char>() + vecb * seg, vecb,
                                  cudaMemcpyDeviceToDevice, s));
        for (int k = k0; k < k1; ++k) {
            FAIR_CUDA(cudaMemcpyAsync(B.x_seg.as<char>() + vecb * (k - k0), B.x.p, vecb,
                                      cudaMemcpyDeviceToDevice, s));
            FAIR_TRY(fwd_step((T *)(B.gk_seg.as<char>() + vecb * (k - k0))));
        }
        for (int k = k1 - 1; k >= k0; --k) {
            const T *xk = (const T *)(B.x_seg.as<char>() + vecb * (k - k0));
            const T *gk = (const T *)(B.gk_seg.as<char>() + vecb * (k - k0));
            k_adj_mask<T, NR><<<ge, 256, 0, s>>>(n, xk, gk, D, B.lam.as<T>(), B.gx.as<T>(),
                                                 B.gz.as<T>(), B.t.as<T>(), bmode, tlb, tub,
                                                 B.part.as<double>());
            FAIR_CUDA(cudaGetLastError());
            FAIR_CUDA(cudaMemcpyAsync(hpart.data(), B.part.p, sizeof(double) * ge * NR,
                                      cudaMemcpyDeviceToHost, s));
            EpiAdjA<T, NR> ea{B.M.as<T>(), B.lam.as<T>(), B.w.as<T>(), B.gb.as<T>()};
            auto ka = k_multi<T, NR, EpiAdjA<T, NR>>;
            ka<<<mgrid(ka, m, NR), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(), vA,
                                            B.t.as<T>(), ea, sched);
            EpiAdjAT<T, NR> eb{B.gz.as<T>(), B.lam.as<T>(), B.gx.as<T>()};
            auto kb = k_multi<T, NR, EpiAdjAT<T, NR>>;
            kb<<<mgrid(kb, n, NR), 256, 0, s>>>(AT.rowptr.as<int64_t>(), AT.m, AT.col.as<int32_t>(),
                                            vAT, B.w.as<T>(), eb, sched);
            FAIR_CUDA(cudaGetLastError());
            FAIR_CUDA(cudaStreamSynchronize(s));
            for (int bl = 0; bl < ge; ++bl)
                for (int c = 0; c < NR; ++c) glam_acc[c] += hpart[(size_t)bl * NR + c];
        }
    }
    // outputs
    k_deinterleave<T><<<egrid(m * ncols), 256, 0, s>>>(B.gb.as<T>(), m, nrhs, NR, 0, ncols,
                                                       stage.as<double>());
    FAIR_CUDA(cudaMemcpyAsync(h_gb + (size_t)c0 * m, stage.p, sizeof(double) * m * ncols,
                              cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    k_deinterleave<T><<<egrid(n * ncols), 256, 0, s>>>(B.gx.as<T>(), n, nrhs, NR, 0, ncols,
                                                       stage.as<double>());
    FAIR_CUDA(cudaMemcpyAsync(h_gx0 + (size_t)c0 * n, stage.p, sizeof(double) * n * ncols,
                              cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    for (int c = 0; c < ncols; ++c) h_glam[c0 + c] = glam_acc[c];
    return FAIR_OK;
}

}  // namespace

int sirt_adjoint(fair_csr h, bool sart, int nrhs, const double *b, const double *x0, int K,
                 const double *lam, int bmode, double lb, double ub, const double *gx,
                 double *xK, double *gb, double *gx0, double *glam) {
    DevCSR &A = h->A, &AT = h->AT;
    cudaStream_t s = h->stream;
    FAIR_TRY(h->w_M.grow(sizeof(double) * ((size_t)A.m + 1)));
    FAIR_TRY(h->w_D.grow(sizeof(double) * ((size_t)A.n + 1)));
    FAIR_TRY(sirt_weights(A, AT, sart, h->w_M.as<double>(), h->w_D.as<double>(), s));
    const bool f32 = h->prec == FAIR_PREC_F32;
    if (f32) {
        FAIR_TRY(csr_make_lowprec(A, FAIR_PREC_F32, s));
        FAIR_TRY(csr_make_lowprec(AT, FAIR_PREC_F32, s));
    }
    unsigned *sched = h->w_sched.as<unsigned>();
    for (int c0 = 0; c0 < nrhs; c0 += 16) {
        const int nc = std::min(16, nrhs - c0);
        const int NRt = nc == 1 ? 1 : (nc <= 4 ? 4 : 16);
#define FAIR_ADJ_GROUP(T, NRC, VA, VAT)                                                          \
    run_group<T, NRC>(A, AT, VA, VAT, sart, b, x0, gx, lam, nrhs, c0, nc, K, bmode, lb, ub,      \
                      h->w_M.as<double>(), h->w_D.as<double>(), sched, s, xK, gb, gx0, glam)
        int st;
        if (f32) {
            const float *va = A.v32.as<float>(), *vt = AT.v32.as<float>();
            st = NRt == 1 ? FAIR_ADJ_GROUP(float, 1, va, vt)
                 : NRt == 4 ? FAIR_ADJ_GROUP(float, 4, va, vt) : FAIR_ADJ_GROUP(float, 16, va, vt);
        } else {
            const double *va = A.v64.as<double>(), *vt = AT.v64.as<double>();
            st = NRt == 1 ? FAIR_ADJ_GROUP(double, 1, va, vt)
                 : NRt == 4 ? FAIR_ADJ_GROUP(double, 4, va, vt) : FAIR_ADJ_GROUP(double, 16, va, vt);
        }
#undef FAIR_ADJ_GROUP
        if (st) return st;
    }
    return FAIR_OK;
}

}  // namespace fair
