// packed.cu -- the packed index stream of the reduced-precision SIRT passes
// (format and decoder in rows.cuh).
//
// Built once per matrix on the GPU: groups of 4 entries per row and their
// offsets (device scan); one counting pass that scores several step codes
// (stride S, low-part width L) at once and keeps the one with the fewest
// escapes; the fill pass, where a group whose steps have no code claims a
// side-table slot with an atomic counter (the slot order varies between
// builds, the decoded columns do not); and, per reduced form, a padded copy
// of the values (4 per group, zeros in the padding), copied bit for bit from
// the unpadded form so both layouts hold the same numbers.
//
// Cost at the N=1024 parallel-beam problem (961M nonzeros): 8 bytes per
// group instead of 16 for the int32 column indices; with 16-bit values one
// group is 16 bytes instead of 24.
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "fair_internal.cuh"
#include "rows.cuh"

namespace fair {

namespace {

constexpr int kPkCand = 8;
struct PkCands {
    int n = 0;
    int S[kPkCand] = {};
    int L[kPkCand] = {};
};

int pk_grid(int64_t work_items) {
    int64_t b = (work_items + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 8;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}

__global__ void k_pk_groups(const int64_t *rowptr, int32_t m, int32_t *gcnt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x)
        gcnt[i] = (int32_t)((rowptr[i + 1] - rowptr[i] + 3) / 4);
}

// Columns of the group starting at entry k (row end e): c[t] for t < valid,
// repeated last column for the padding.
__device__ __forceinline__ int pk_cols(const int32_t *col, int64_t k, int64_t e, int (&c)[4]) {
    const int nv = e - k < 4 ? (int)(e - k) : 4;
    c[0] = col[k];
#pragma unroll
    for (int t = 1; t < 4; ++t) c[t] = t < nv ? col[k + t] : c[t - 1];
    return nv;
}

__global__ void k_pk_count(const int64_t *rowptr, int32_t m, const int32_t *col, PkCands C,
                           unsigned long long *esc) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned cnt[kPkCand];
#pragma unroll
    for (int c = 0; c < kPkCand; ++c) cnt[c] = 0;
    for (int64_t r = warp; r < m; r += nw) {
        const int64_t s = rowptr[r], e = rowptr[r + 1];
        for (int64_t k = s + 4 * lane; k < e; k += 128) {
            int cs[4];
            pk_cols(col, k, e, cs);
#pragma unroll
            for (int c = 0; c < kPkCand; ++c) {
                if (c >= C.n) break;
                uint32_t code;
                bool ok = true;
#pragma unroll
                for (int t = 1; t < 4; ++t)
                    ok = ok && pk_encode((int64_t)cs[t] - cs[t - 1], C.S[c], C.L[c], code);
                if (!ok) ++cnt[c];
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kPkCand; ++c) {
        unsigned v = cnt[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && c < C.n && v) atomicAdd(esc + c, (unsigned long long)v);
    }
}

__global__ void k_pk_fill(const int64_t *rowptr, int32_t m, const int32_t *col,
                          const int64_t *prow, int S, int L, uint2 *gidx, int4 *gside,
                          unsigned long long cap, unsigned long long *nesc) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < m; r += nw) {
        const int64_t s = rowptr[r], e = rowptr[r + 1], g0 = prow[r];
        for (int64_t j = lane; s + 4 * j < e; j += 32) {
            int cs[4];
            const int nv = pk_cols(col, s + 4 * j, e, cs);
            uint32_t y = (uint32_t)(nv - 1) << 24, code;
            bool ok = true;
#pragma unroll
            for (int t = 1; t < 4; ++t) {
                ok = ok && pk_encode((int64_t)cs[t] - cs[t - 1], S, L, code);
                if (ok) y |= code << (8 * (t - 1));
            }
            if (!ok) {
                const unsigned long long slot = atomicAdd(nesc, 1ull);
                y = ((uint32_t)(nv - 1) << 24) | kPkEsc | (uint32_t)(slot & 0xFFFFFFull);
                if (slot < cap) gside[slot] = make_int4(cs[1], cs[2], cs[3], 0);
            }
            gidx[g0 + j] = make_uint2((uint32_t)cs[0], y);
        }
    }
}

template <typename T>
__global__ void k_pk_values(const int64_t *rowptr, int32_t m, const int64_t *prow, const T *src,
                            T *dst) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < m; r += nw) {
        const int64_t s = rowptr[r], len = rowptr[r + 1] - s, d0 = 4 * prow[r];
        const int64_t padded = 4 * (prow[r + 1] - prow[r]);
        for (int64_t t = lane; t < padded; t += 32) dst[d0 + t] = t < len ? src[s + t] : T(0);
    }
}

// Fused records of a 2-byte form: {index word, the group's four values}.
__global__ void k_pk_fuse(const uint2 *gidx, const uint2 *vals, int64_t ng, uint4 *rec) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ng;
         j += (int64_t)gridDim.x * blockDim.x) {
        const uint2 w = gidx[j], v = vals[j];
        rec[j] = make_uint4(w.x, w.y, v.x, v.y);
    }
}

// Slots of each chunk in the sliced copy (rows.cuh), one warp per chunk: 32
// per step, the chunk's steps being the sum over its slices of R = 32/G rows
// of the slice's longest row in steps of G groups. G is the given one, or
// with G = 0 chosen per chunk from its rows' column steps: 8 lanes along
// each row when most steps are +-1 (neighbouring entries of a row are
// neighbours in x, so a row's lanes share cache sectors), else 1 lane per row
// (the rows' entries at one step are neighbours in x). lg[c] = log2 of the
// chunk's G.
__global__ void k_sl_len(const int64_t *prow, int32_t m, int64_t nch, int G, const uint2 *gidx,
                         int S, int L, int32_t *cnt, int8_t *lg) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nch; c += nw) {
        const int64_t r = 32 * c + lane;
        const int64_t ng = r < m ? prow[r + 1] - prow[r] : 0;
        int g = G;
        if (g == 0) {
            const int64_t s0 = prow[32 * c], s1 = prow[32 * c + 32 < m ? 32 * c + 32 : m];
            unsigned unit = 0, other = 0;
            for (int64_t j = s0 + lane; j < s1; j += 32) {
                const uint2 w = gidx[j];
                if (w.y & kPkEsc) { other += 3; continue; }
                const int cnt = (int)((w.y >> 24) & 3u);
                for (int t = 0; t < cnt; ++t) {
                    const int d = pk_step((w.y >> (8 * t)) & 0xFFu, S, L);
                    (d == 1 || d == -1 ? unit : other) += 1;
                }
            }
            unit = __reduce_add_sync(FULL, unit);
            other = __reduce_add_sync(FULL, other);
            g = unit > other ? 8 : 1;
        }
        const int R = 32 / g;
        const unsigned st = (unsigned)((ng + g - 1) / g);
        int64_t total = 0;
        for (int i = 0; i < g; ++i) total += __reduce_max_sync(FULL, lane / R == i ? st : 0u);
        if (lane == 0) {
            cnt[c] = (int32_t)(32 * total);
            lg[c] = (int8_t)(g == 8 ? 3 : g == 4 ? 2 : g == 2 ? 1 : 0);
        }
    }
}

// Tag every chunk's slot offset with its log2 G (offsets are multiples of 32).
__global__ void k_sl_tag(int64_t *soff, int64_t nch, const int8_t *lg) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nch;
         c += (int64_t)gridDim.x * blockDim.x)
        soff[c] |= lg[c];
}

// The slots of one chunk per warp: at step k of slice i, lane g*G + l gets
// group k*G + l of row 32c + i*R + g, or `hole` past the row's end.
template <typename T>
__global__ void k_sl_copy(const int64_t *prow, int32_t m, int64_t nch, const int64_t *soff,
                          const T *src, T *dst, T hole) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nch; c += nw) {
        const int G = 1 << (int)(soff[c] & 7), R = 32 / G, g = lane / G, gl = lane % G;
        int64_t pos = soff[c] & ~(int64_t)31;
        for (int i = 0; i < G; ++i) {
            const int64_t r = 32 * c + i * R + g;
            const int64_t g0 = r < m ? prow[r] : 0;
            const int64_t ng = r < m ? prow[r + 1] - g0 : 0;
            const unsigned st = (unsigned)((ng + G - 1) / G);
            const int64_t Ls = (int64_t)__reduce_max_sync(0xffffffffu, st);
            for (int64_t k = 0; k < Ls; ++k) {
                const int64_t j = k * G + gl;
                dst[pos + 32 * k + lane] = j < ng ? src[g0 + j] : hole;
            }
            pos += 32 * Ls;
        }
    }
}

// Four FP64 values of one group, copied as one unit.
struct alignas(16) Dbl4 {
    double2 a, b;
};

template <typename T>
int sl_copy(const DevCSR &A, const void *src, DevBuf &dst, T hole, cudaStream_t s) {
    FAIR_TRY(dst.grow(sizeof(T) * (size_t)std::max<int64_t>(A.nslots, 1)));
    const int64_t nch = ((int64_t)A.m + 31) / 32;
    k_sl_copy<T><<<pk_grid(nch * 32), 256, 0, s>>>(A.prow.as<int64_t>(), A.m, nch,
                                                   A.soff.as<int64_t>(),
                                                   static_cast<const T *>(src), dst.as<T>(), hole);
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int64_t isqrt64(int64_t v) {
    int64_t r = (int64_t)std::sqrt((double)v);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

template <typename T>
int pad_values(DevCSR &A, const DevBuf &src, DevBuf &dst, cudaStream_t s) {
    FAIR_TRY(dst.grow(sizeof(T) * 4 * (size_t)std::max<int64_t>(A.ngroups, 1)));
    k_pk_values<T><<<pk_grid((int64_t)A.m * 32), 256, 0, s>>>(
        A.rowptr.as<int64_t>(), A.m, A.prow.as<int64_t>(), src.as<T>(), dst.as<T>());
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int build_index(DevCSR &A, cudaStream_t s) {
    PkCands C;
    auto add = [&](int S, int L) {
        for (int c = 0; c < C.n; ++c)
            if (C.S[c] == S && C.L[c] == L) return;
        if (C.n < kPkCand) { C.S[C.n] = S; C.L[C.n] = L; ++C.n; }
    };
    if (A.stride_hint > 0)
        for (int L = 4; L <= 6; ++L) add(A.stride_hint, L);
    const int64_t sq = isqrt64(A.n);
    if (sq > 1 && sq * sq == A.n && sq < (1 << 30))
        for (int L = 4; L <= 5; ++L) add((int)sq, L);
    add(0, 7);

    TmpBuf gcnt, esc;
    FAIR_TRY(gcnt.grow(sizeof(int32_t) * ((size_t)A.m + 1)));
    FAIR_TRY(A.prow.grow(sizeof(int64_t) * ((size_t)A.m + 1)));
    FAIR_TRY(esc.grow(sizeof(unsigned long long) * (kPkCand + 1)));
    k_pk_groups<<<pk_grid(A.m), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, gcnt.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    FAIR_TRY(scan_counts(gcnt.as<int32_t>(), A.m, A.prow.as<int64_t>(), s));
    FAIR_CUDA(cudaMemsetAsync(esc.p, 0, sizeof(unsigned long long) * (kPkCand + 1), s));
    k_pk_count<<<pk_grid((int64_t)A.m * 32), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m,
                                                          A.col.as<int32_t>(), C,
                                                          esc.as<unsigned long long>());
    FAIR_CUDA(cudaGetLastError());
    unsigned long long hesc[kPkCand] = {};
    int64_t ng = 0;
    FAIR_CUDA(cudaMemcpyAsync(hesc, esc.p, sizeof(hesc), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaMemcpyAsync(&ng, A.prow.as<int64_t>() + A.m, sizeof(ng), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    gcnt.release();
    int best = 0;
    for (int c = 1; c < C.n; ++c)
        if (hesc[c] < hesc[best]) best = c;
    const unsigned long long nesc = hesc[best];
    // too many escapes: the side-table reads would cost more than the codes save
    if (nesc > (unsigned long long)(ng / 8) || nesc >= (1ull << 24)) {
        A.prow.release();
        return FAIR_OK;
    }
    FAIR_TRY(A.gidx.grow(sizeof(uint2) * (size_t)std::max<int64_t>(ng, 1)));
    FAIR_TRY(A.gside.grow(sizeof(int4) * (size_t)std::max<unsigned long long>(nesc, 1)));
    unsigned long long *ctr = esc.as<unsigned long long>() + kPkCand;
    k_pk_fill<<<pk_grid((int64_t)A.m * 32), 256, 0, s>>>(
        A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(), A.prow.as<int64_t>(), C.S[best],
        C.L[best], A.gidx.as<uint2>(), A.gside.as<int4>(), nesc, ctr);
    FAIR_CUDA(cudaGetLastError());
    unsigned long long used = 0;
    FAIR_CUDA(cudaMemcpyAsync(&used, ctr, sizeof(used), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    if (used != nesc) {  // the fill must meet exactly the escapes the count found
        set_detail("packed index: escape count mismatch");
        A.prow.release(); A.gidx.release(); A.gside.release();
        return FAIR_ERR_STATE;
    }
    A.ngroups = ng;
    A.nesc = (int64_t)nesc;
    A.pk_S = C.S[best];
    A.pk_L = C.L[best];
    A.haspk = true;
    return FAIR_OK;
}

}  // namespace

bool packed_enabled() {
    const char *e = getenv("FAIR_PACKED");
    return !(e && e[0] == '0');
}

int csr_make_packed(DevCSR &A, int prec, cudaStream_t s) {
    if (A.m == 0 || A.nnz == 0) return FAIR_OK;
    if (!A.pk_tried) {
        A.pk_tried = true;
        FAIR_TRY(build_index(A, s));
    }
    if (!A.haspk) return FAIR_OK;
    if (prec == FAIR_PREC_F64) {
        if (!A.hasp64) {
            FAIR_TRY(pad_values<double>(A, A.v64, A.pv64, s));
            A.hasp64 = true;
        }
        return FAIR_OK;
    }
    FAIR_TRY(csr_make_lowprec(A, prec, s));
    if (prec == FAIR_PREC_F32 && !A.hasp32) {
        FAIR_TRY(pad_values<float>(A, A.v32, A.pv32, s));
        A.hasp32 = true;
    } else if (prec == FAIR_PREC_F16 && !A.hasp16) {
        FAIR_TRY(pad_values<uint16_t>(A, A.v16, A.pv16, s));
        A.hasp16 = true;
    } else if (prec == FAIR_PREC_Q16 && !A.haspq) {
        FAIR_TRY(pad_values<uint16_t>(A, A.vq, A.pvq, s));
        A.haspq = true;
    }
    return FAIR_OK;
}

int csr_make_sliced(DevCSR &A, int prec, int G, cudaStream_t s) {
    if (!A.haspk || A.m == 0) return FAIR_OK;
    if (G != 0 && G != 1 && G != 2 && G != 4 && G != 8) {
        set_detail("sliced copy: lanes per row must be 0 (per chunk), 1, 2, 4 or 8");
        return FAIR_ERR_ARG;
    }
    // chunk slots and group offsets within a chunk stay below 2^31
    if (32 * (((int64_t)A.max_row + 3) / 4 + 8) >= (int64_t(1) << 31)) return FAIR_OK;
    if (A.hassl && A.sl_G != G) A.drop_sliced();
    const int64_t nch = ((int64_t)A.m + 31) / 32;
    if (!A.hassl) {
        TmpBuf cnt, lg;  // released after the synchronisation below
        FAIR_TRY(cnt.grow(sizeof(int32_t) * (size_t)(nch + 1)));
        FAIR_TRY(lg.grow((size_t)nch));
        FAIR_TRY(A.soff.grow(sizeof(int64_t) * (size_t)(nch + 1)));
        k_sl_len<<<pk_grid(nch * 32), 256, 0, s>>>(A.prow.as<int64_t>(), A.m, nch, G,
                                                   A.gidx.as<uint2>(), A.pk_S, A.pk_L,
                                                   cnt.as<int32_t>(), lg.as<int8_t>());
        FAIR_CUDA(cudaGetLastError());
        FAIR_TRY(scan_counts(cnt.as<int32_t>(), nch, A.soff.as<int64_t>(), s));
        k_sl_tag<<<pk_grid(nch), 256, 0, s>>>(A.soff.as<int64_t>(), nch, lg.as<int8_t>());
        FAIR_CUDA(cudaGetLastError());
        FAIR_CUDA(cudaMemcpyAsync(&A.nslots, A.soff.as<int64_t>() + nch, sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, s));
        FAIR_CUDA(cudaStreamSynchronize(s));
        A.sl_G = G;
        A.hassl = true;
    }
    if (prec == FAIR_PREC_F64 || prec == FAIR_PREC_F32) {
        FAIR_TRY(csr_make_packed(A, prec, s));
        if (!A.hassidx) {
            FAIR_TRY(sl_copy<uint2>(A, A.gidx.p, A.sidx, make_uint2(0u, kPkHole), s));
            A.hassidx = true;
        }
        if (prec == FAIR_PREC_F64 && A.hasp64 && !A.hassv64) {
            FAIR_TRY(sl_copy<Dbl4>(A, A.pv64.p, A.sv64, Dbl4{}, s));
            A.hassv64 = true;
        } else if (prec == FAIR_PREC_F32 && A.hasp32 && !A.hassv32) {
            FAIR_TRY(sl_copy<float4>(A, A.pv32.p, A.sv32, make_float4(0.f, 0.f, 0.f, 0.f), s));
            A.hassv32 = true;
        }
        return FAIR_OK;
    }
    const bool h = prec == FAIR_PREC_F16;
    if (h ? A.hassf16 : A.hassfq) return FAIR_OK;
    FAIR_TRY(csr_make_fused(A, prec, s));
    if (!(h ? A.hasf16 : A.hasfq)) return FAIR_OK;
    FAIR_TRY(sl_copy<uint4>(A, (h ? A.pf16 : A.pfq).p, h ? A.sf16 : A.sfq,
                            make_uint4(0u, kPkHole, 0u, 0u), s));
    (h ? A.hassf16 : A.hassfq) = true;
    return FAIR_OK;
}

int csr_make_fused(DevCSR &A, int prec, cudaStream_t s) {
    if (!A.haspk || (prec != FAIR_PREC_F16 && prec != FAIR_PREC_Q16)) return FAIR_OK;
    const bool h = prec == FAIR_PREC_F16;
    if (h ? A.hasf16 : A.hasfq) return FAIR_OK;
    FAIR_TRY(csr_make_packed(A, prec, s));
    DevBuf &dst = h ? A.pf16 : A.pfq;
    const DevBuf &src = h ? A.pv16 : A.pvq;
    FAIR_TRY(dst.grow(sizeof(uint4) * (size_t)std::max<int64_t>(A.ngroups, 1)));
    k_pk_fuse<<<pk_grid(A.ngroups), 256, 0, s>>>(A.gidx.as<uint2>(), src.as<uint2>(), A.ngroups,
                                                 dst.as<uint4>());
    FAIR_CUDA(cudaGetLastError());
    (h ? A.hasf16 : A.hasfq) = true;
    return FAIR_OK;
}

}  // namespace fair
