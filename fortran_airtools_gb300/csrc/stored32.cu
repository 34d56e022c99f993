// stored32.cu -- paralleltomo (system_generation.f90:309-492) with the matrix
// and its transpose held in FP32 values only, built by blocks of angles.
//
// The FP64 build keeps the matrix's FP64 values (the master copy every form is
// derived from) and builds the transpose from them with a source index, so a
// problem needs about 36 bytes per nonzero on the GPU while it is built. At
// N=2048 with 1440 angles and 2896 bins (7.69e9 nonzeros) that is 280 GB, more
// than the GPU holds. The FP32 SIRT form only reads FP32 values, int32 column
// indices and int64 row offsets: 8 bytes per nonzero for A and 8 for A'
// (123 GB at that size). This builder produces exactly that:
//
//   * phase 0 counts the nonzeros of every block of angles (the count pass
//     of the ray tracer), so A's arrays are allocated once at their size;
//   * phase 1 traces each block of angles in FP64 (the same kernels as the
//     FP64 build, so columns and values are bit-identical), stores the
//     block's rows into A as FP32 values, keeps the rows' 1- and 2-norms from
//     the FP64 values (the SIRT weights) and counts the entries of every
//     column;
//   * phase 2 traces each block again, transposes it (the stable counting
//     sort of the FP64 transpose: a column's entries in ascending row
//     order) and appends every column's entries to its row of A' after those
//     of the earlier blocks, so A' equals the transpose of the whole matrix
//     entry for entry; the columns' 1-norms and squared 2-norms are summed in
//     FP64, block by block.
//
// Row offsets are 64-bit throughout (the reference's default-integer IA
// overflows past 2^31 - 1 nonzeros, sparse_matrices.f90:33-49 and
// system_generation.f90:404). The handle then holds A and A' for FP32 only:
// products and SIRT run in FP32 on any layout the FP32 form supports (CSR,
// packed stream, sliced, tiled, delta copies, all built from the FP32
// values); operations that need FP64 values return FAIR_ERR_STATE.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fair_gpu_ext.h"
#include "fair_internal.cuh"

namespace fair {
namespace {

// Releases a matrix or a table set when the scope ends (early returns included).
struct CsrScope {
    DevCSR &c;
    ~CsrScope() { c.release(); }
};
struct TablesScope {
    GeomTables &t;
    ~TablesScope() { t.release(); }
};

int s32_grid(int64_t items) {
    const int64_t b = (items + 255) / 256;
    const int64_t cap = (int64_t)sm_count() * 16;
    return (int)std::max<int64_t>(1, std::min(b, cap));
}

// Rows r0 .. r0 + bm of A from a block traced in FP64: row offsets (the block's
// offsets shifted by the entries of the earlier blocks) and the entries.
__global__ void k_s32_rows(const int64_t *__restrict__ brp, int32_t bm, int64_t base,
                           int64_t *__restrict__ rp) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + 1; i <= bm;
         i += (int64_t)gridDim.x * blockDim.x)
        rp[i] = base + brp[i];
}
__global__ void k_s32_entries(const int32_t *__restrict__ bcol, const double *__restrict__ bv,
                              int64_t bnnz, int32_t *__restrict__ col, float *__restrict__ v32,
                              int32_t *__restrict__ colcount) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < bnnz;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = bcol[k];
        col[k] = c;
        v32[k] = (float)bv[k];  // round to nearest, as the FP64 handle's FP32 copy
        atomicAdd(colcount + c, 1);
    }
}

// One warp per row j of the block's transpose (pixel j): its entries go to row
// j of A' after the entries the earlier blocks put there, their row indices
// shifted by the block's first row r0; the row's sums of |v| and v^2 (a fixed
// warp reduction order) are added to the column norms.
__global__ void k_s32_append(const int64_t *__restrict__ trp, int32_t n,
                             const int32_t *__restrict__ tcol, const double *__restrict__ tv,
                             int32_t r0, const int64_t *__restrict__ grp, int32_t *__restrict__ cursor,
                             int32_t *__restrict__ gcol, float *__restrict__ gv,
                             double *__restrict__ norm1, double *__restrict__ norm2sq) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = warp; j < n; j += nw) {
        const int64_t s = trp[j], e = trp[j + 1];
        if (s == e) continue;
        const int64_t dst = grp[j] + cursor[j] - s;
        double a1 = 0.0, a2 = 0.0;
        for (int64_t k = s + lane; k < e; k += 32) {
            const double v = tv[k];
            gcol[dst + k] = tcol[k] + r0;
            gv[dst + k] = (float)v;
            a1 += fabs(v);
            a2 = fma(v, v, a2);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
            a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        }
        __syncwarp();
        if (lane == 0) {
            cursor[j] += (int32_t)(e - s);
            norm1[j] += a1;
            norm2sq[j] += a2;
        }
    }
}

__global__ void k_s32_sqrt(double *a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        a[i] = sqrt(a[i]);
}

// Entries and FP32 values of an FP32-only matrix, the spare entries zeroed.
int alloc_f32(DevCSR &M, int64_t nnz, cudaStream_t s) {
    FAIR_TRY(M.col.grow(sizeof(int32_t) * (size_t)(nnz + kEntryPad)));
    FAIR_TRY(M.v32.grow(sizeof(float) * (size_t)(nnz + kEntryPad)));
    FAIR_CUDA(cudaMemsetAsync(M.col.as<int32_t>() + nnz, 0, sizeof(int32_t) * kEntryPad, s));
    FAIR_CUDA(cudaMemsetAsync(M.v32.as<float>() + nnz, 0, sizeof(float) * kEntryPad, s));
    M.nnz = nnz;
    M.has32 = true;
    M.f32_only = true;
    return FAIR_OK;
}

// Parallel-beam tables of angles a0 .. a1 (system_generation.f90:328-363,
// host libm for the angles as in the FP64 build).
struct ParTables {
    int N = 0, p = 0;
    std::vector<double> x0, y0, grid, ct, st;
    int make(const fair_data *dat, cudaStream_t s, int a0, int a1, GeomTables &T) const {
        T.release();
        T.kind = 0; T.N = N; T.nth = a1 - a0; T.p = p;
        auto up = [&](DevBuf &b, const double *src, size_t cnt) -> int {
            FAIR_TRY(b.grow(sizeof(double) * (cnt ? cnt : 1)));
            if (cnt) FAIR_CUDA(cudaMemcpyAsync(b.p, src, sizeof(double) * cnt, cudaMemcpyHostToDevice, s));
            return FAIR_OK;
        };
        (void)dat;
        FAIR_TRY(up(T.grid, grid.data(), grid.size()));
        FAIR_TRY(up(T.cth, ct.data() + a0, (size_t)(a1 - a0)));
        FAIR_TRY(up(T.sth, st.data() + a0, (size_t)(a1 - a0)));
        FAIR_TRY(up(T.bx0, x0.data(), x0.size()));
        FAIR_TRY(up(T.by0, y0.data(), y0.size()));
        FAIR_CUDA(cudaStreamSynchronize(s));  // the host tables may go after this
        return FAIR_OK;
    }
};

int build_f32(const fair_data *dat, int32_t block_angles, fair_csr h) {
    cudaStream_t s = h->stream;
    const int N = dat->n, p = dat->p, nth = dat->nth;
    ParTables P;
    P.N = N;
    P.p = p;
    P.x0.resize(p); P.y0.resize(p); P.grid.resize(N + 1); P.ct.resize(nth); P.st.resize(nth);
    const double d = p - 1;
    linspace_host(-.5 * d, .5 * d, p, P.x0.data());
    for (int j = 0; j < p; ++j) P.y0[j] = 0 * P.x0[j];
    linspace_host(-.5 * N, .5 * N, N + 1, P.grid.data());
    for (int i = 0; i < nth; ++i) {
        P.ct[i] = cos(dat->theta[i]);
        P.st[i] = sin(dat->theta[i]);
    }
    GeomTables T;
    TablesScope tscope{T};
    // phase 0: nonzeros per counting block of angles
    const int cb = 16;
    std::vector<int64_t> cnt;
    int64_t total = 0;
    for (int a0 = 0; a0 < nth; a0 += cb) {
        const int a1 = std::min(nth, a0 + cb);
        FAIR_TRY(P.make(dat, s, a0, a1, T));
        int64_t c = 0;
        FAIR_TRY(geometry_nnz(T, &c, s));
        cnt.push_back(c);
        total += c;
    }
    // build blocks: whole counting blocks up to the target size (or the asked
    // number of angles per block)
    const int64_t target = int64_t(1) << 28;
    std::vector<int> bounds{0};
    if (block_angles > 0) {
        for (int a = block_angles; a < nth; a += block_angles) bounds.push_back(a);
    } else {
        int64_t acc = 0;
        for (size_t k = 0; k < cnt.size(); ++k) {
            if (acc > 0 && acc + cnt[k] > target) {
                bounds.push_back((int)k * cb);
                acc = 0;
            }
            acc += cnt[k];
        }
    }
    bounds.push_back(nth);

    DevCSR &A = h->A;
    DevCSR &AT = h->AT;
    const int64_t m = (int64_t)nth * p, n = (int64_t)N * N;
    A.m = (int32_t)m;
    A.n = (int32_t)n;
    A.stride_hint = N;
    A.tstride_hint = p;
    FAIR_TRY(A.rowptr.grow(sizeof(int64_t) * (size_t)(m + 1)));
    FAIR_CUDA(cudaMemsetAsync(A.rowptr.p, 0, sizeof(int64_t), s));
    FAIR_TRY(alloc_f32(A, total, s));
    FAIR_TRY(A.rn1.grow(sizeof(double) * (size_t)(m + 1)));
    FAIR_TRY(A.rn2.grow(sizeof(double) * (size_t)(m + 1)));
    TmpBuf colcount;
    FAIR_TRY(colcount.grow(sizeof(int32_t) * (size_t)(n + 1)));
    FAIR_CUDA(cudaMemsetAsync(colcount.p, 0, sizeof(int32_t) * (size_t)(n + 1), s));

    // phase 1: the rows of A
    int64_t base = 0;
    for (size_t k = 0; k + 1 < bounds.size(); ++k) {
        const int a0 = bounds[k], a1 = bounds[k + 1];
        const int64_t r0 = (int64_t)a0 * p;
        FAIR_TRY(P.make(dat, s, a0, a1, T));
        DevCSR Ab;
        CsrScope ab_scope{Ab};
        FAIR_TRY(build_geometry(T, Ab, s));
        if (base + Ab.nnz > total) {
            set_detail("a block traced more nonzeros than its count");
            return FAIR_ERR_GEOMETRY;
        }
        k_s32_rows<<<s32_grid(Ab.m), 256, 0, s>>>(Ab.rowptr.as<int64_t>(), Ab.m, base,
                                                   A.rowptr.as<int64_t>() + r0);
        if (Ab.nnz)
            k_s32_entries<<<s32_grid(Ab.nnz), 256, 0, s>>>(Ab.col.as<int32_t>(), Ab.v64.as<double>(),
                                                            Ab.nnz, A.col.as<int32_t>() + base,
                                                            A.v32.as<float>() + base,
                                                            colcount.as<int32_t>());
        FAIR_CUDA(cudaGetLastError());
        FAIR_TRY(csr_row_norms(Ab, 1, A.rn1.as<double>() + r0, s));
        FAIR_TRY(csr_row_norms(Ab, 2, A.rn2.as<double>() + r0, s));
        A.max_row = std::max(A.max_row, Ab.max_row);
        base += Ab.nnz;
        FAIR_CUDA(cudaStreamSynchronize(s));  // before the block's buffers go
    }
    if (base != total) {
        set_detail("the blocks traced a different count than the count pass");
        return FAIR_ERR_GEOMETRY;
    }

    // A': row offsets from the column counts, then phase 2
    AT.m = (int32_t)n;
    AT.n = (int32_t)m;
    AT.stride_hint = A.tstride_hint;
    AT.tstride_hint = A.stride_hint;
    FAIR_TRY(AT.rowptr.grow(sizeof(int64_t) * (size_t)(n + 1)));
    FAIR_TRY(scan_counts(colcount.as<int32_t>(), n, AT.rowptr.as<int64_t>(), s));
    FAIR_TRY(alloc_f32(AT, total, s));
    FAIR_TRY(AT.rn1.grow(sizeof(double) * (size_t)(n + 1)));
    FAIR_TRY(AT.rn2.grow(sizeof(double) * (size_t)(n + 1)));
    FAIR_CUDA(cudaMemsetAsync(AT.rn1.p, 0, sizeof(double) * (size_t)(n + 1), s));
    FAIR_CUDA(cudaMemsetAsync(AT.rn2.p, 0, sizeof(double) * (size_t)(n + 1), s));
    FAIR_CUDA(cudaMemsetAsync(colcount.p, 0, sizeof(int32_t) * (size_t)(n + 1), s));  // the cursors
    for (size_t k = 0; k + 1 < bounds.size(); ++k) {
        const int a0 = bounds[k], a1 = bounds[k + 1];
        FAIR_TRY(P.make(dat, s, a0, a1, T));
        DevCSR Ab, Abt;
        CsrScope ab_scope{Ab}, abt_scope{Abt};
        FAIR_TRY(build_geometry(T, Ab, s));
        FAIR_TRY(csr_build_transpose(Ab, Abt, s));
        Ab.release();
        k_s32_append<<<s32_grid(n * 32), 256, 0, s>>>(
            Abt.rowptr.as<int64_t>(), (int32_t)n, Abt.col.as<int32_t>(), Abt.v64.as<double>(),
            (int32_t)((int64_t)a0 * p), AT.rowptr.as<int64_t>(), colcount.as<int32_t>(),
            AT.col.as<int32_t>(), AT.v32.as<float>(), AT.rn1.as<double>(), AT.rn2.as<double>());
        FAIR_CUDA(cudaGetLastError());
        FAIR_CUDA(cudaStreamSynchronize(s));
    }
    k_s32_sqrt<<<s32_grid(n), 256, 0, s>>>(AT.rn2.as<double>(), n);
    FAIR_CUDA(cudaGetLastError());
    FAIR_TRY(csr_max_row(AT, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    return FAIR_OK;
}

}  // namespace
}  // namespace fair

using namespace fair;

extern "C" int fair_paralleltomo_f32(const fair_data *dat, int32_t block_angles, fair_csr h) {
    if (!h) return FAIR_ERR_NULL;
    FAIR_CUDA(cudaSetDevice(h->device));
    if (!dat || !dat->theta) return FAIR_ERR_NULL;
    if (dat->n < 1 || dat->p < 1 || dat->nth < 1) {
        set_detail("n, p, nth must be positive");
        return FAIR_ERR_ARG;
    }
    if ((int64_t)dat->nth * dat->p > INT32_MAX || (int64_t)dat->n * dat->n > INT32_MAX) {
        set_detail("nth*p and n^2 must fit in 32-bit indices");
        return FAIR_ERR_ARG;
    }
    if (block_angles < 0) {
        set_detail("block_angles must be 0 (chosen by size) or positive");
        return FAIR_ERR_ARG;
    }
    FAIR_CUDA(cudaStreamSynchronize(h->stream));
    h->A.release();
    h->AT.release();
    h->at_valid = false;
    h->sirt_ready = false;
    const int st = build_f32(dat, block_angles, h);
    if (st != FAIR_OK) {
        cudaStreamSynchronize(h->stream);
        h->A.release();
        h->AT.release();
        return st;
    }
    h->at_valid = true;
    h->prec = FAIR_PREC_F32;
    return FAIR_OK;
}
