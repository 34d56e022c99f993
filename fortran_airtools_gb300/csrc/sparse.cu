// sparse.cu -- CSR operators of sparse_matrices.f90 on the GPU.
//
//  * spmv: y = A x, one warp per row, grid-stride over rows (MMRS,
//    sparse_matrices.f90:349-368). The transposed product runs the same
//    kernel on the transposed CSR (deterministic gather instead of the
//    reference's racy scatter, :382-392).
//  * transpose: the reference's stable counting sort (reorder, :492-570):
//    column histogram, scan, slot claim, then each column's entries are put
//    back in source order (= ascending row) by a per-column sort on the
//    source position, which is unique, so the result equals the serial order.
//  * row norms (:740-780), row dot (:252-270), bounded row axpy (:795-822),
//    scaling (:824-831).
#include <algorithm>

#include "fair_internal.cuh"
#include "rows.cuh"

namespace fair {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------- scan ----
constexpr int kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

// Inclusive block scan of one int64 per thread; returns the block total.
__device__ int64_t block_incl_scan(int64_t v, int64_t *sh /*[32]*/, int64_t &total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    if (lane == 31) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int nw = blockDim.x >> 5;
        int64_t w = lane < nw ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t n = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += n;
        }
        if (lane < nw) sh[lane] = w;
    }
    __syncthreads();
    int64_t add = wid > 0 ? sh[wid - 1] : 0;
    total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return v + add;
}

__global__ void k_scan_tiles(const int32_t *in, int64_t m, int64_t *tile_sums) {
    __shared__ int64_t sh[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < m) s += in[base + k];
    int64_t total;
    block_incl_scan(s, sh, total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int64_t *sums, int64_t nt) {
    __shared__ int64_t sh[32];
    int64_t carry = 0;
    for (int64_t b0 = 0; b0 < nt; b0 += blockDim.x) {
        int64_t idx = b0 + threadIdx.x;
        int64_t v = idx < nt ? sums[idx] : 0;
        int64_t total;
        int64_t inc = block_incl_scan(v, sh, total);
        if (idx < nt) sums[idx] = carry + inc - v;  // exclusive
        carry += total;
    }
}

__global__ void k_scan_apply(const int32_t *in, int64_t m, const int64_t *tile_off, int64_t *out) {
    __shared__ int64_t sh[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < m ? in[base + k] : 0;
        s += v[k];
    }
    int64_t total;
    int64_t inc = block_incl_scan(s, sh, total);
    int64_t run = tile_off[blockIdx.x] + inc - s;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < m) out[base + k] = run;
        run += v[k];
    }
    // the thread holding element m-1 writes the grand total
    if (base <= m - 1 && m - 1 < base + kScanItems) out[m] = run;
}

__global__ void k_zero_total(int64_t *out) { out[0] = 0; }

// ------------------------------------------------------------ row stats ----
__global__ void k_max_row(const int64_t *rowptr, int32_t m, int32_t *out) {
    int32_t best = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
         r += (int64_t)gridDim.x * blockDim.x) {
        int32_t len = (int32_t)(rowptr[r + 1] - rowptr[r]);
        best = max(best, len);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

// ------------------------------------------------------------ transpose ----
__global__ void k_col_hist(const int32_t *col, int64_t nnz, int32_t *cnt) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
         e += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[col[e]], 1);
}

// Row index of every nonzero, then claim a slot in its column.
__global__ void k_col_scatter(const int64_t *rowptr, int32_t m, const int32_t *col,
                              const int64_t *colptr, int32_t *fill, int64_t *tsrc,
                              int32_t *trow) {
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < m; r += nw) {
        int64_t s = rowptr[r], e = rowptr[r + 1];
        for (int64_t j = s + lane; j < e; j += 32) {
            int32_t c = col[j];
            int64_t pos = colptr[c] + atomicAdd(&fill[c], 1);
            tsrc[pos] = j;
            trow[pos] = (int32_t)r;
        }
    }
}

// Sort each column's (src, row) pairs by src: bitonic sort in shared memory
// for columns up to kColCap entries, in global memory (scratch) above that.
constexpr int kColCap = 4096;

__global__ void __launch_bounds__(256) k_col_sort_smem(const int64_t *colptr, int32_t ncol,
                                                       int64_t *tsrc, int32_t *trow) {
    __shared__ int64_t ks[kColCap];
    __shared__ int32_t vs[kColCap];
    for (int32_t c = blockIdx.x; c < ncol; c += gridDim.x) {
        int64_t s = colptr[c];
        int len = (int)(colptr[c + 1] - s);
        if (len <= 1 || len > kColCap) continue;
        int P = 1;
        while (P < len) P <<= 1;
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            ks[i] = i < len ? tsrc[s + i] : INT64_MAX;
            vs[i] = i < len ? trow[s + i] : 0;
        }
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = threadIdx.x; i < P; i += blockDim.x) {
                    int ixj = i ^ j;
                    if (ixj > i) {
                        bool up = (i & k) == 0;
                        int64_t a = ks[i], b = ks[ixj];
                        if ((a > b) == up) {
                            ks[i] = b; ks[ixj] = a;
                            int32_t t = vs[i]; vs[i] = vs[ixj]; vs[ixj] = t;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            tsrc[s + i] = ks[i];
            trow[s + i] = vs[i];
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_col_sort_global(const int64_t *colptr,
                                                         const int32_t *long_cols, int32_t nlong,
                                                         int64_t *tsrc, int32_t *trow,
                                                         int64_t *ks, int32_t *vs, int P) {
    for (int32_t q = blockIdx.x; q < nlong; q += gridDim.x) {
        int32_t c = long_cols[q];
        int64_t s = colptr[c];
        int len = (int)(colptr[c + 1] - s);
        int64_t *K = ks + (size_t)blockIdx.x * P;
        int32_t *V = vs + (size_t)blockIdx.x * P;
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            K[i] = i < len ? tsrc[s + i] : INT64_MAX;
            V[i] = i < len ? trow[s + i] : 0;
        }
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = threadIdx.x; i < P; i += blockDim.x) {
                    int ixj = i ^ j;
                    if (ixj > i) {
                        bool up = (i & k) == 0;
                        int64_t a = K[i], b = K[ixj];
                        if ((a > b) == up) {
                            K[i] = b; K[ixj] = a;
                            int32_t t = V[i]; V[i] = V[ixj]; V[ixj] = t;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            tsrc[s + i] = K[i];
            trow[s + i] = V[i];
        }
        __syncthreads();
    }
}

__global__ void k_list_long_cols(const int64_t *colptr, int32_t ncol, int32_t *list,
                                 int32_t *nlist) {
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncol; c += gridDim.x * blockDim.x)
        if (colptr[c + 1] - colptr[c] > kColCap) list[atomicAdd(nlist, 1)] = c;
}

__global__ void k_gather_vals(const int64_t *tsrc, int64_t nnz, const double *v, double *tv) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
         e += (int64_t)gridDim.x * blockDim.x)
        tv[e] = v[tsrc[e]];
}

// -------------------------------------------------------- precision copies ----
__global__ void k_to_f32(const double *v, int64_t n, float *o) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x)
        o[e] = (float)v[e];
}
__global__ void k_to_f16(const double *v, int64_t n, __half *o) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x)
        o[e] = __double2half(v[e]);
}
// Largest |v| and smallest v of the array: per-block values, finished on the host.
__global__ void k_absmax_min(const double *v, int64_t n, double *bmax, double *bmin) {
    __shared__ double smax[32], smin[32];
    double mx = 0.0, mn = INFINITY;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        mx = fmax(mx, fabs(v[e]));
        mn = fmin(mn, v[e]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { smax[wid] = mx; smin[wid] = mn; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { mx = fmax(mx, smax[w]); mn = fmin(mn, smin[w]); }
        bmax[blockIdx.x] = fmax(smax[0], mx);
        bmin[blockIdx.x] = fmin(smin[0], mn);
    }
}

// 16-bit fixed point: q = round(v / scale), unsigned or signed codes.
template <typename Q>
__global__ void k_to_q16(const double *v, int64_t n, double inv_scale, Q *o) {
    const long long lo = (Q)-1 < 0 ? -32767 : 0, hi = (Q)-1 < 0 ? 32767 : 65535;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        long long q = llrint(v[e] * inv_scale);
        o[e] = (Q)(q < lo ? lo : (q > hi ? hi : q));
    }
}

__global__ void k_scale(double *v, int64_t n, double c) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x)
        v[e] = __dmul_rn(c, v[e]);
}

// 1-based JA to 0-based, flagging indices outside 1..n.
__global__ void k_fix_cols(int32_t *col, int64_t nnz, int32_t n, int *err) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
         e += (int64_t)gridDim.x * blockDim.x) {
        int32_t c = col[e] - 1;
        if (c < 0 || c >= n) {
            atomicOr(err, 1);
            c = 0;
        }
        col[e] = c;
    }
}

// Row offsets must start at 0 and never decrease.
__global__ void k_check_rowptr(const int64_t *rowptr, int32_t m, int *err) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
         r += (int64_t)gridDim.x * blockDim.x)
        if (rowptr[r + 1] < rowptr[r]) atomicOr(err, 2);
}

// ------------------------------------------------------------ row norms ----
// p-norm of every row (compute_row_norms, sparse_matrices.f90:740-780): a warp
// per row, four independent loads in flight per lane. P = 1 and 2 are
// compiled with one FP64 operation per entry (|a| added; a*a fused into the
// sum: on this part every FP64 warp instruction holds its pipe for 64
// cycles, so the entry count of FP64 operations bounds the kernel); P = 0
// takes p at run time.
template <int P>
__device__ __forceinline__ double norm_term(double acc, double a, int p) {
    if constexpr (P == 1) return acc + fabs(a);
    else if constexpr (P == 2) return fma(a, a, acc);
    else {
        a = fabs(a);
        double t = a;
        for (int q = 1; q < p; ++q) t *= a;
        return acc + t;
    }
}

template <int P>
__global__ void k_row_norms(const int64_t *rowptr, int32_t m, const double *v, int p,
                            double *out) {
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < m; r += nw) {
        const int64_t s = rowptr[r], e = rowptr[r + 1];
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        int64_t j = s + lane;
        for (; j + 96 < e; j += 128) {
            const double a[4] = {__ldcs(v + j), __ldcs(v + j + 32), __ldcs(v + j + 64),
                                 __ldcs(v + j + 96)};
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] = norm_term<P>(acc[u], a[u], p);
        }
        for (; j < e; j += 32) acc[0] = norm_term<P>(acc[0], __ldcs(v + j), p);
        double sum = warp_sum((acc[0] + acc[1]) + (acc[2] + acc[3]));
        if (lane == 0) out[r] = p == 1 ? sum : (p == 2 ? sqrt(sum) : pow(sum, 1.0 / p));
    }
}

__global__ void k_row_dot(const int64_t *rowptr, int32_t row, const int32_t *col,
                          const double *v, const double *x, double *out) {
    int64_t s = rowptr[row], e = rowptr[row + 1];
    double acc = 0.0;
    for (int64_t j = s + threadIdx.x; j < e; j += 32) acc += x[col[j]] * v[j];
    acc = warp_sum(acc);
    if (threadIdx.x == 0) *out = acc;
}

// Entries of one row touch distinct columns, so the lanes do not collide.
__global__ void k_add_mult_row(const int64_t *rowptr, int32_t row, const int32_t *col,
                               const double *v, double c, double *w, int bmode, double lb,
                               double ub) {
    int64_t s = rowptr[row], e = rowptr[row + 1];
    for (int64_t j = s + threadIdx.x; j < e; j += blockDim.x) {
        int32_t k = col[j];
        double t = __dadd_rn(w[k], __dmul_rn(c, v[j]));
        if (bmode & 2) t = fmax_f(t, lb);
        if (bmode & 1) t = fmin_f(t, ub);
        w[k] = t;
    }
}

// ----------------------------------------------------------------- SpMV ----
struct EpiStore64 {
    double *y;
    __device__ void operator()(int64_t i, double acc) const { y[i] = acc; }
};
struct EpiStore32 {
    float *y;
    float scale;  // 1 for FP32/FP16 values, the fixed-point scale for 16-bit codes
    __device__ void operator()(int64_t i, float acc) const { y[i] = acc * scale; }
};

template <int G>
__global__ void __launch_bounds__(256) k_spmv_f64(const int64_t *rowptr, int32_t m,
                                                  const int32_t *col, const double *v,
                                                  const double *x, EpiStore64 epi,
                                                  unsigned *sched) {
    chunk_rows<double, double, double, G>(rowptr, m, col, v, x, epi, sched);
}

template <typename VT, int G>
__global__ void __launch_bounds__(256) k_spmv_lp(const int64_t *rowptr, int32_t m,
                                                 const int32_t *col, const VT *v,
                                                 const float *x, EpiStore32 epi,
                                                 unsigned *sched) {
    chunk_rows<VT, float, float, G>(rowptr, m, col, v, x, epi, sched);
}

int grid_for(int threads, int64_t work_items, int per_sm = 8) {
    int64_t b = (work_items + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count() * per_sm;
    if (b < 1) b = 1;
    return (int)std::min<int64_t>(b, cap);
}

}  // namespace

// ------------------------------------------------------------------ host ----
int scan_counts(const int32_t *counts, int64_t m, int64_t *out, cudaStream_t s) {
    if (m == 0) {
        k_zero_total<<<1, 1, 0, s>>>(out);
        FAIR_CUDA(cudaGetLastError());
        return FAIR_OK;
    }
    int64_t ntiles = (m + kScanTile - 1) / kScanTile;
    DevBuf sums;
    FAIR_TRY(sums.grow(sizeof(int64_t) * ntiles));
    k_scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, s>>>(counts, m, sums.as<int64_t>());
    k_scan_sums<<<1, 1024, 0, s>>>(sums.as<int64_t>(), ntiles);
    k_scan_apply<<<(unsigned)ntiles, kScanThreads, 0, s>>>(counts, m, sums.as<int64_t>(), out);
    FAIR_CUDA(cudaGetLastError());
    FAIR_CUDA(cudaStreamSynchronize(s));
    sums.release();
    return FAIR_OK;
}

int csr_max_row(DevCSR &A, cudaStream_t s) {
    DevBuf d;
    FAIR_TRY(d.grow(sizeof(int32_t)));
    FAIR_CUDA(cudaMemsetAsync(d.p, 0, sizeof(int32_t), s));
    if (A.m > 0)
        k_max_row<<<grid_for(256, A.m), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, d.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    FAIR_CUDA(cudaMemcpyAsync(&A.max_row, d.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    d.release();
    return FAIR_OK;
}

int csr_build_transpose(const DevCSR &A, DevCSR &AT, cudaStream_t s) {
    AT.release();
    AT.m = A.n;
    AT.n = A.m;
    AT.nnz = A.nnz;
    AT.stride_hint = A.tstride_hint;
    AT.tstride_hint = A.stride_hint;
    const int64_t nnz = A.nnz;
    DevBuf cnt, fill, tsrc;
    FAIR_TRY(cnt.grow(sizeof(int32_t) * ((size_t)A.n + 1)));
    FAIR_TRY(fill.grow(sizeof(int32_t) * ((size_t)A.n + 1)));
    FAIR_TRY(tsrc.grow(sizeof(int64_t) * (nnz > 0 ? nnz : 1)));
    FAIR_TRY(AT.rowptr.grow(sizeof(int64_t) * ((size_t)A.n + 1)));
    FAIR_TRY(AT.alloc_entries(nnz, s));
    FAIR_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * ((size_t)A.n + 1), s));
    FAIR_CUDA(cudaMemsetAsync(fill.p, 0, sizeof(int32_t) * ((size_t)A.n + 1), s));
    if (nnz > 0)
        k_col_hist<<<grid_for(256, nnz), 256, 0, s>>>(A.col.as<int32_t>(), nnz, cnt.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    FAIR_TRY(scan_counts(cnt.as<int32_t>(), A.n, AT.rowptr.as<int64_t>(), s));
    if (A.m > 0)
        k_col_scatter<<<grid_for(256, (int64_t)A.m * 32), 256, 0, s>>>(
            A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(), AT.rowptr.as<int64_t>(),
            fill.as<int32_t>(), tsrc.as<int64_t>(), AT.col.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    if (A.n > 0)
        k_col_sort_smem<<<(unsigned)std::min<int64_t>(A.n, (int64_t)sm_count() * 16), 256, 0, s>>>(
            AT.rowptr.as<int64_t>(), A.n, tsrc.as<int64_t>(), AT.col.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    // columns longer than the shared-memory capacity
    DevBuf list, nlist;
    FAIR_TRY(list.grow(sizeof(int32_t) * ((size_t)A.n + 1)));
    FAIR_TRY(nlist.grow(sizeof(int32_t)));
    FAIR_CUDA(cudaMemsetAsync(nlist.p, 0, sizeof(int32_t), s));
    if (A.n > 0)
        k_list_long_cols<<<grid_for(256, A.n), 256, 0, s>>>(AT.rowptr.as<int64_t>(), A.n,
                                                          list.as<int32_t>(), nlist.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    int32_t h_nlong = 0;
    FAIR_CUDA(cudaMemcpyAsync(&h_nlong, nlist.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    if (h_nlong > 0) {
        FAIR_TRY(csr_max_row(AT, s));
        int P = 1;
        while (P < AT.max_row) P <<= 1;
        int nb = std::min<int>(h_nlong, 64);
        DevBuf ks, vs;
        FAIR_TRY(ks.grow(sizeof(int64_t) * (size_t)P * nb));
        FAIR_TRY(vs.grow(sizeof(int32_t) * (size_t)P * nb));
        k_col_sort_global<<<nb, 256, 0, s>>>(AT.rowptr.as<int64_t>(), list.as<int32_t>(), h_nlong,
                                             tsrc.as<int64_t>(), AT.col.as<int32_t>(),
                                             ks.as<int64_t>(), vs.as<int32_t>(), P);
        FAIR_CUDA(cudaGetLastError());
        FAIR_CUDA(cudaStreamSynchronize(s));
        ks.release();
        vs.release();
    }
    if (nnz > 0)
        k_gather_vals<<<grid_for(256, nnz), 256, 0, s>>>(tsrc.as<int64_t>(), nnz,
                                                        A.v64.as<double>(), AT.v64.as<double>());
    FAIR_CUDA(cudaGetLastError());
    FAIR_CUDA(cudaStreamSynchronize(s));
    cnt.release(); fill.release(); tsrc.release(); list.release(); nlist.release();
    FAIR_TRY(csr_max_row(AT, s));
    return FAIR_OK;
}

int csr_check_upload(DevCSR &A, cudaStream_t s) {
    DevBuf err;
    FAIR_TRY(err.grow(sizeof(int)));
    FAIR_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    if (A.nnz > 0)
        k_fix_cols<<<grid_for(256, A.nnz), 256, 0, s>>>(A.col.as<int32_t>(), A.nnz, A.n, err.as<int>());
    if (A.m > 0)
        k_check_rowptr<<<grid_for(256, A.m), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, err.as<int>());
    FAIR_CUDA(cudaGetLastError());
    int h = 0;
    FAIR_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    err.release();
    if (h & 1) { set_detail("JA holds a column index outside 1..n"); return FAIR_ERR_ARG; }
    if (h & 2) { set_detail("IA decreases"); return FAIR_ERR_ARG; }
    return csr_max_row(A, s);
}

int csr_make_lowprec(DevCSR &A, int prec, cudaStream_t s) {
    const int64_t n = A.nnz + kEntryPad;  // conversion covers the zeroed pad too
    if (prec == FAIR_PREC_F32 && !A.has32) {
        FAIR_TRY(A.v32.grow(sizeof(float) * n));
        k_to_f32<<<grid_for(256, n), 256, 0, s>>>(A.v64.as<double>(), n, A.v32.as<float>());
        FAIR_CUDA(cudaGetLastError());
        A.has32 = true;
    }
    if (prec == FAIR_PREC_F16 && !A.has16) {
        FAIR_TRY(A.v16.grow(sizeof(__half) * n));
        k_to_f16<<<grid_for(256, n), 256, 0, s>>>(A.v64.as<double>(), n, A.v16.as<__half>());
        FAIR_CUDA(cudaGetLastError());
        A.has16 = true;
    }
    if (prec == FAIR_PREC_Q16 && !A.hasq) {
        const int nb = 512;
        DevBuf ext;
        FAIR_TRY(ext.grow(sizeof(double) * 2 * nb));
        k_absmax_min<<<nb, 256, 0, s>>>(A.v64.as<double>(), A.nnz, ext.as<double>(),
                                        ext.as<double>() + nb);
        FAIR_CUDA(cudaGetLastError());
        double h[2 * nb];
        FAIR_CUDA(cudaMemcpyAsync(h, ext.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        FAIR_CUDA(cudaStreamSynchronize(s));
        ext.release();
        double mx = 0.0, mn = INFINITY;
        for (int b = 0; b < nb; ++b) { mx = std::max(mx, h[b]); mn = std::min(mn, h[nb + b]); }
        A.qsigned = mn < 0.0;
        const double top = A.qsigned ? 32767.0 : 65535.0;
        A.qscale = mx > 0.0 ? mx / top : 1.0;
        FAIR_TRY(A.vq.grow(sizeof(uint16_t) * n));  // the pad converts from zeros
        if (A.qsigned)
            k_to_q16<int16_t><<<grid_for(256, n), 256, 0, s>>>(A.v64.as<double>(), n, 1.0 / A.qscale,
                                                               A.vq.as<int16_t>());
        else
            k_to_q16<uint16_t><<<grid_for(256, n), 256, 0, s>>>(A.v64.as<double>(), n, 1.0 / A.qscale,
                                                                A.vq.as<uint16_t>());
        FAIR_CUDA(cudaGetLastError());
        A.hasq = true;
    }
    return FAIR_OK;
}

int csr_scale(DevCSR &A, double c, cudaStream_t s) {
    if (A.nnz > 0)  // the pad stays 0 (c * 0 = 0 for finite c; the pad is never used)
        k_scale<<<grid_for(256, A.nnz), 256, 0, s>>>(A.v64.as<double>(), A.nnz, c);
    FAIR_CUDA(cudaGetLastError());
    // derived copies are rebuilt from the scaled master values
    A.has32 = false;
    A.has16 = false;
    A.hasq = false;
    A.hasp64 = A.hasp32 = A.hasp16 = A.haspq = A.hasf16 = A.hasfq = false;
    A.hassv64 = A.hassv32 = A.hassf16 = A.hassfq = false;
    A.tl.has_v64 = A.tl.has_v32 = A.tl.has_r16 = A.tl.has_rq = false;
    A.tl.has6_16 = A.tl.has6_q = false;
    for (auto &d : A.dl) d.has_v64 = d.has_v32 = d.has_r16 = d.has_rq = false;
    return FAIR_OK;
}

int csr_row_norms(const DevCSR &A, int p, double *d_out, cudaStream_t s) {
    if (A.f32_only) {  // no FP64 values: the norms kept from the FP64 build
        if (p != 1 && p != 2) {
            set_detail("a matrix held in FP32 only keeps its row 1- and 2-norms, no other p");
            return FAIR_ERR_STATE;
        }
        if (A.m > 0)
            FAIR_CUDA(cudaMemcpyAsync(d_out, (p == 1 ? A.rn1 : A.rn2).p, sizeof(double) * (size_t)A.m,
                                      cudaMemcpyDeviceToDevice, s));
        return FAIR_OK;
    }
    if (A.m > 0) {
        const int g = grid_for(256, (int64_t)A.m * 32);
        const int64_t *rp = A.rowptr.as<int64_t>();
        const double *v = A.v64.as<double>();
        if (p == 1) k_row_norms<1><<<g, 256, 0, s>>>(rp, A.m, v, p, d_out);
        else if (p == 2) k_row_norms<2><<<g, 256, 0, s>>>(rp, A.m, v, p, d_out);
        else k_row_norms<0><<<g, 256, 0, s>>>(rp, A.m, v, p, d_out);
    }
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int csr_row_dot(const DevCSR &A, int32_t row, const double *d_x, double *d_out, cudaStream_t s) {
    k_row_dot<<<1, 32, 0, s>>>(A.rowptr.as<int64_t>(), row, A.col.as<int32_t>(),
                               A.v64.as<double>(), d_x, d_out);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int csr_add_mult_row(const DevCSR &A, int32_t row, double c, double *d_w, int bmode, double lb,
                     double ub, cudaStream_t s) {
    k_add_mult_row<<<1, 256, 0, s>>>(A.rowptr.as<int64_t>(), row, A.col.as<int32_t>(),
                                     A.v64.as<double>(), c, d_w, bmode, lb, ub);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int spmv(const DevCSR &A, int prec, const void *d_x, void *d_y, cudaStream_t s,
         unsigned *sched) {
    if (A.m == 0) return FAIR_OK;
    const int64_t *rp = A.rowptr.as<int64_t>();
    const int32_t *cl = A.col.as<int32_t>();
    const int G = A.lanes_per_row;
#define SPMV_G(CALL)                                          \
    switch (G) {                                              \
        case 4: { constexpr int g_ = 4; CALL; } break;        \
        case 16: { constexpr int g_ = 16; CALL; } break;      \
        case 32: { constexpr int g_ = 32; CALL; } break;      \
        default: { constexpr int g_ = 8; CALL; } break;       \
    }
    if (prec == FAIR_PREC_F64) {
        EpiStore64 e{(double *)d_y};
        SPMV_G((k_spmv_f64<g_><<<chunk_grid(k_spmv_f64<g_>, A.m), 256, 0, s>>>(
            rp, A.m, cl, A.v64.as<double>(), (const double *)d_x, e, sched)));
    } else if (prec == FAIR_PREC_F32) {
        FAIR_TRY(csr_make_lowprec(const_cast<DevCSR &>(A), prec, s));
        EpiStore32 e{(float *)d_y, 1.0f};
        SPMV_G((k_spmv_lp<float, g_><<<chunk_grid(k_spmv_lp<float, g_>, A.m), 256, 0, s>>>(
            rp, A.m, cl, A.v32.as<float>(), (const float *)d_x, e, sched)));
    } else if (prec == FAIR_PREC_F16) {
        FAIR_TRY(csr_make_lowprec(const_cast<DevCSR &>(A), prec, s));
        EpiStore32 e{(float *)d_y, 1.0f};
        SPMV_G((k_spmv_lp<__half, g_><<<chunk_grid(k_spmv_lp<__half, g_>, A.m), 256, 0, s>>>(
            rp, A.m, cl, A.v16.as<__half>(), (const float *)d_x, e, sched)));
    } else {
        FAIR_TRY(csr_make_lowprec(const_cast<DevCSR &>(A), prec, s));
        EpiStore32 e{(float *)d_y, (float)A.qscale};
        if (A.qsigned)
            SPMV_G((k_spmv_lp<int16_t, g_><<<chunk_grid(k_spmv_lp<int16_t, g_>, A.m), 256, 0, s>>>(
                rp, A.m, cl, A.vq.as<int16_t>(), (const float *)d_x, e, sched)))
        else
            SPMV_G((k_spmv_lp<uint16_t, g_><<<chunk_grid(k_spmv_lp<uint16_t, g_>, A.m), 256, 0, s>>>(
                rp, A.m, cl, A.vq.as<uint16_t>(), (const float *)d_x, e, sched)))
    }
#undef SPMV_G
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

}  // namespace fair
