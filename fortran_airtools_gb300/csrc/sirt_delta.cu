// sirt_delta.cu -- the two SIRT passes (AIRMs.f90:1089-1110) on the delta
// copies of a matrix (layout codes 11-13).
//
// The sliced layout with one lane per row (rows.cuh, G = 1) reads each row
// from its first slot to its last in one lane, so a lane can carry the row's
// running column and a slot needs no column of its own: slot k of row 32c + l
// (at soff[c] + 32k + l) holds one 32-bit word of E column steps -- its first
// entry from the row's previous entry (from the row's anchor column for
// k = 0), the others from the entry before -- and the E values. A step code
// of B bits is a signed low part of L bits and a signed high part of B - L
// bits, delta = lo + hi*S, S the matrix's stride hint (the image side N for a
// ray matrix, the bins per angle for its transpose; L = B: the plain signed
// delta). A slot with a step outside the code range keeps its E columns in a
// side table (bit 31 set, the table slot in bits 0-29). Padding entries
// repeat the previous column with value 0.
//
// Two formats:
//   E = 4, B = 7: the word beside 4 FP32 or FP64 values (20 or 36 bytes per 4
//                 entries against 24 or 40 on the packed layouts);
//   E = 6, B = 5: one 16-byte record {word, six 2-byte values} for f16 and q16
//                 (2.67 bytes per entry against 4 on the fused records: a ray
//                 steps to a 4- or 8-neighbour pixel, delta in {+-1, +-N,
//                 +-N+-1}; the next ray through a pixel is the next bin or a
//                 bin a few away at the next angle, delta in {1, p-4 .. p+3}).
#include <algorithm>
#include <cmath>

#include "fair_internal.cuh"
#include "rows.cuh"
#include "sirt_epi.cuh"

namespace fair {

namespace {

constexpr uint32_t kDlEsc = kStepEsc;
constexpr uint32_t kDlSlot = kStepSlot;
constexpr int kDlCand = 8;
struct DlCands {
    int n = 0;
    int S[kDlCand] = {};
    int L[kDlCand] = {};
};

int dl_grid(int64_t work_items) {
    int64_t b = (work_items + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 8;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}

// The E columns of the slot starting at entry e0 of a row ending at e;
// entries past the row repeat the last column.
template <int E>
__device__ __forceinline__ void dl_cols(const int32_t *col, int64_t e0, int64_t e, int (&c)[E]) {
#pragma unroll
    for (int q = 0; q < E; ++q) c[q] = e0 + q < e ? col[e0 + q] : (q ? c[q - 1] : 0);
}

// Slots whose steps have no code, per candidate (one warp per row).
template <int E, int B>
__global__ void k_dl_count(const int64_t *rowptr, int32_t m, const int32_t *col, DlCands C,
                           unsigned long long *esc) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned cnt[kDlCand];
#pragma unroll
    for (int c = 0; c < kDlCand; ++c) cnt[c] = 0;
    for (int64_t r = warp; r < m; r += nw) {
        const int64_t s = rowptr[r], e = rowptr[r + 1];
        for (int64_t k0 = s + (int64_t)E * lane; k0 < e; k0 += 32 * E) {
            int cs[E];
            dl_cols<E>(col, k0, e, cs);
            const int prev = k0 > s ? col[k0 - 1] : cs[0];
#pragma unroll
            for (int c = 0; c < kDlCand; ++c) {
                if (c >= C.n) break;
                uint32_t w;
                if (!step_word<E, B>(cs, prev, C.S[c], C.L[c], w)) ++cnt[c];
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kDlCand; ++c) {
        unsigned v = cnt[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && c < C.n && v) atomicAdd(esc + c, (unsigned long long)v);
    }
}

// Slots of each chunk of 32 rows: 32 x its longest row in slots.
__global__ void k_dl_len(const int64_t *rowptr, int32_t m, int64_t nch, int E, int32_t *cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nch; c += nw) {
        const int64_t r = 32 * c + lane;
        const unsigned g = r < m ? (unsigned)((rowptr[r + 1] - rowptr[r] + E - 1) / E) : 0u;
        const unsigned mx = __reduce_max_sync(0xffffffffu, g);
        if (lane == 0) cnt[c] = (int32_t)(32 * mx);
    }
}

// Step words, anchors and side table (one warp per chunk, lane = row).
template <int E, int B>
__global__ void k_dl_fill(const int64_t *rowptr, int32_t m, const int32_t *col, int64_t nch,
                          const int64_t *soff, int S, int L, uint32_t *code, int32_t *anchor,
                          int4 *side, unsigned long long cap, unsigned long long *nesc) {
    constexpr int E4 = (E + 3) / 4;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nch; c += nw) {
        const int64_t r = 32 * c + lane;
        const int64_t s = r < m ? rowptr[r] : 0, e = r < m ? rowptr[r + 1] : 0;
        const int64_t base = soff[c], len = (soff[c + 1] - base) >> 5;
        int prev = e > s ? col[s] : 0;
        if (r < m) anchor[r] = prev;
        for (int64_t k = 0; k < len; ++k) {
            const int64_t e0 = s + (int64_t)E * k;
            uint32_t w = 0;  // past the row: zero steps
            if (e0 < e) {
                int cs[E];
                dl_cols<E>(col, e0, e, cs);
                if (!step_word<E, B>(cs, prev, S, L, w)) {
                    const unsigned long long slot = atomicAdd(nesc, 1ull);
                    if (slot < cap) {
                        int t[4 * E4];
#pragma unroll
                        for (int q = 0; q < 4 * E4; ++q) t[q] = q < E ? cs[q] : 0;
#pragma unroll
                        for (int h = 0; h < E4; ++h)
                            side[slot * E4 + h] = make_int4(t[4 * h], t[4 * h + 1], t[4 * h + 2], t[4 * h + 3]);
                    }
                    w = kDlEsc | (uint32_t)(slot & kDlSlot);
                }
                prev = cs[E - 1];
            }
            code[base + 32 * k + lane] = w;
        }
    }
}

// The 4 values of every slot of an E = 4 copy (zeros past a row).
template <typename T>
__global__ void k_dl_vals(const int64_t *rowptr, int32_t m, int64_t nch, const int64_t *soff,
                          const T *src, T *dst) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nch; c += nw) {
        const int64_t r = 32 * c + lane;
        const int64_t s = r < m ? rowptr[r] : 0, e = r < m ? rowptr[r + 1] : 0;
        const int64_t base = soff[c], len = (soff[c + 1] - base) >> 5;
        for (int64_t k = 0; k < len; ++k) {
            const int64_t slot = base + 32 * k + lane;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t j = s + 4 * k + q;
                dst[4 * slot + q] = j < e ? src[j] : T(0);
            }
        }
    }
}

// The records of an E = 6 copy: {word, six 2-byte codes}.
__global__ void k_dl_rec6(const int64_t *rowptr, int32_t m, int64_t nch, const int64_t *soff,
                          const uint32_t *code, const uint16_t *src, uint4 *rec) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nch; c += nw) {
        const int64_t r = 32 * c + lane;
        const int64_t s = r < m ? rowptr[r] : 0, e = r < m ? rowptr[r + 1] : 0;
        const int64_t base = soff[c], len = (soff[c + 1] - base) >> 5;
        for (int64_t k = 0; k < len; ++k) {
            const int64_t slot = base + 32 * k + lane;
            uint32_t h[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const int64_t j = s + 6 * k + q;
                h[q] = j < e ? src[j] : 0u;
            }
            rec[slot] = make_uint4(code[slot], h[0] | (h[1] << 16), h[2] | (h[3] << 16),
                                   h[4] | (h[5] << 16));
        }
    }
}

// ---- the passes ----------------------------------------------------------------
// A slot as loaded (Raw), its step word and its E values.
template <typename VT> struct DlSplit {  // E = 4: word + 4 FP32/FP64 values
    static constexpr int E = 4, B = 7;
    using Acc = VT;
    const uint32_t *code;
    const VT *val;
    struct Raw {
        uint32_t w;
        VBlk<VT> v;
    };
    __device__ __forceinline__ void load(int64_t j, Raw &r) const {
        r.w = ld_stream(code + j);
        r.v.ld(val + 4 * j);
    }
    __device__ __forceinline__ static uint32_t word(const Raw &r) { return r.w; }
    __device__ __forceinline__ static void vals(const Raw &r, VT (&v)[4]) { r.v.to(v); }
};
template <typename VT> struct DlRec6 {  // E = 6: one 16-byte record
    static constexpr int E = 6, B = 5;
    using Acc = float;
    const uint4 *rec;
    using Raw = uint4;
    __device__ __forceinline__ void load(int64_t j, Raw &r) const { r = ld_stream(rec + j); }
    __device__ __forceinline__ static uint32_t word(const Raw &r) { return r.x; }
    __device__ __forceinline__ static void vals(const Raw &r, float (&v)[6]) {
        Conv2B<VT>::two(r.y, v[0], v[1]);
        Conv2B<VT>::two(r.z, v[2], v[3]);
        Conv2B<VT>::two(r.w, v[4], v[5]);
    }
};

struct DlArgs {
    const int64_t *rowptr, *soff;
    const int32_t *anchor;
    const int4 *side;
    int S, L;
};

// Every chunk of 32 rows owned by this warp, lane l summing row base+l: D
// slots in flight; with PF the gathers of slot t+1 are issued before the
// products of slot t.
template <class LD, typename XT, int D, int PF, class Epi>
__device__ __forceinline__ void dl_rows(const DlArgs &P, const LD &ldr, int32_t m, const int *lut,
                                        const XT *__restrict__ x, Epi &epi, unsigned *sched) {
    constexpr int E = LD::E, B = LD::B, E4 = (E + 3) / 4;
    constexpr uint32_t mask = (1u << B) - 1u;
    using ACC = typename LD::Acc;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = ((int64_t)m + 31) >> 5;
    for (int64_t ch = sched ? next_chunk(sched, 0, nwarps, lane) : warp; ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int64_t row = (ch << 5) + lane;
        const int ns = row < m ? (int)((__ldg(P.rowptr + row + 1) - __ldg(P.rowptr + row) + E - 1) / E) : 0;
        int col = row < m ? __ldg(P.anchor + row) : 0;
        const int64_t s0 = __ldg(P.soff + ch) + lane;
        typename LD::Raw ring[D];
#pragma unroll
        for (int k = 0; k < D; ++k)
            if (k < ns) ldr.load(s0 + 32 * k, ring[k]);
        // the E columns of a word, moving the running column
        auto cols = [&](uint32_t w, int (&c)[E]) {
            if (w & kDlEsc) {
                const int4 *t = P.side + (int64_t)(w & kDlSlot) * E4;
                int u[4 * E4];
#pragma unroll
                for (int h = 0; h < E4; ++h) {
                    const int4 v = __ldg(t + h);
                    u[4 * h] = v.x; u[4 * h + 1] = v.y; u[4 * h + 2] = v.z; u[4 * h + 3] = v.w;
                }
#pragma unroll
                for (int q = 0; q < E; ++q) c[q] = u[q];
            } else {
                c[0] = col + lut[w & mask];
#pragma unroll
                for (int q = 1; q < E; ++q) c[q] = c[q - 1] + lut[(w >> (B * q)) & mask];
            }
            col = c[E - 1];
        };
        ACC acc = 0;
        ACC v[E], xv[E];
#pragma unroll
        for (int q = 0; q < E; ++q) v[q] = xv[q] = (ACC)0;
        if constexpr (PF) {
            if (ns > 0) {
                int c[E];
                cols(LD::word(ring[0]), c);
                LD::vals(ring[0], v);
#pragma unroll
                for (int q = 0; q < E; ++q) xv[q] = (ACC)__ldg(x + c[q]);
                if (D < ns) ldr.load(s0 + 32 * D, ring[0]);
            }
        }
        for (int t0 = 0; t0 < ns; t0 += D) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const int t = t0 + k;
                if (t >= ns) break;
                if constexpr (PF) {
                    const int kn = (k + 1) % D;  // ring slot of slot t+1 (fixed once unrolled)
                    ACC vn[E], xn[E];
#pragma unroll
                    for (int q = 0; q < E; ++q) vn[q] = xn[q] = (ACC)0;
                    if (t + 1 < ns) {
                        int c[E];
                        cols(LD::word(ring[kn]), c);
                        LD::vals(ring[kn], vn);
#pragma unroll
                        for (int q = 0; q < E; ++q) xn[q] = (ACC)__ldg(x + c[q]);
                        if (t + 1 + D < ns) ldr.load(s0 + 32 * (int64_t)(t + 1 + D), ring[kn]);
                    }
#pragma unroll
                    for (int q = 0; q < E; ++q) acc += xv[q] * v[q];
#pragma unroll
                    for (int q = 0; q < E; ++q) {
                        v[q] = vn[q];
                        xv[q] = xn[q];
                    }
                } else {
                    const typename LD::Raw cur = ring[k];
                    if (t + D < ns) ldr.load(s0 + 32 * (int64_t)(t + D), ring[k]);
                    int c[E];
                    cols(LD::word(cur), c);
                    LD::vals(cur, v);
#pragma unroll
                    for (int q = 0; q < E; ++q) acc += (ACC)__ldg(x + c[q]) * v[q];
                }
            }
        }
        if (row < m) epi(row, acc);
    }
    finish_chunks(sched, nwarps, lane);
}

// Resident CTAs per SM asked of the register allocator: with 2 slots in
// flight the 16-byte records fit 48 registers, so 5 CTAs (40 warps) gather
// through L1 together; the other variants keep their registers.
template <class LD, int D> constexpr int kDlMinBlocks = LD::E == 6 && D == 2 ? 5 : 1;

template <class LD, typename XT, int D, int PF, class Epi>
__global__ void __launch_bounds__(256, kDlMinBlocks<LD, D>) k_sirt_resid_dl(DlArgs P, LD ldr, int32_t m, const XT *x,
                                                       Epi epi, unsigned *sched) {
    __shared__ int lut[128];
    for (int t = threadIdx.x; t < (1 << LD::B); t += blockDim.x) lut[t] = step_decode<LD::B>((uint32_t)t, P.S, P.L);
    __syncthreads();
    dl_rows<LD, XT, D, PF>(P, ldr, m, lut, x, epi, sched);
}
template <class LD, typename XT, int D, int PF, class Epi>
__global__ void __launch_bounds__(256, kDlMinBlocks<LD, D>) k_sirt_update_dl(DlArgs P, LD ldr, int32_t m, const XT *r,
                                                        Epi epi, unsigned *sched) {
    __shared__ int lut[128];
    for (int t = threadIdx.x; t < (1 << LD::B); t += blockDim.x) lut[t] = step_decode<LD::B>((uint32_t)t, P.S, P.L);
    __syncthreads();
    dl_rows<LD, XT, D, PF>(P, ldr, m, lut, r, epi, sched);
}

// Code 11: 2 slots in flight; 12: 4 with the gathers one slot ahead; 13: 2
// with the gathers one slot ahead.
template <class LD, typename XT, class EpiR, class EpiU>
void dl_pass(const DevCSR &M, const DevCSR::Delta &dl, const LD &ldr, int pass, int code,
             const XT *x, const XT *r, const EpiR &er, const EpiU &eu, unsigned *sched,
             cudaStream_t s) {
    const DlArgs P{M.rowptr.as<int64_t>(), dl.soff.as<int64_t>(), dl.anchor.as<int32_t>(),
                   dl.side.as<int4>(), dl.S, dl.L};
    const int32_t m = M.m;
    auto go = [&](auto k, const XT *v, const auto &e) { k<<<chunk_grid(k, m), 256, 0, s>>>(P, ldr, m, v, e, sched); };
    if (pass == 1) {
        if (code == 12) go(k_sirt_resid_dl<LD, XT, 4, 1, EpiR>, x, er);
        else if (code == 13) go(k_sirt_resid_dl<LD, XT, 2, 1, EpiR>, x, er);
        else go(k_sirt_resid_dl<LD, XT, 2, 0, EpiR>, x, er);
    } else {
        if (code == 12) go(k_sirt_update_dl<LD, XT, 4, 1, EpiU>, r, eu);
        else if (code == 13) go(k_sirt_update_dl<LD, XT, 2, 1, EpiU>, r, eu);
        else go(k_sirt_update_dl<LD, XT, 2, 0, EpiU>, r, eu);
    }
}

// Index part of a delta copy with E entries per slot and B-bit steps.
template <int E, int B>
int dl_build(DevCSR &A, DevCSR::Delta &dl, cudaStream_t s) {
    dl.E = E;
    dl.bits = B;
    if (32 * (((int64_t)A.max_row + E - 1) / E) >= (int64_t(1) << 31)) return FAIR_OK;
    DlCands C;
    auto add = [&](int S, int L) {
        if (C.n < kDlCand) { C.S[C.n] = S; C.L[C.n] = L; ++C.n; }
    };
    if (A.stride_hint > 0)
        for (int L = 2; L <= B - 2; ++L) add(A.stride_hint, L);
    add(0, B);
    TmpBuf esc, cnt;
    FAIR_TRY(esc.grow(sizeof(unsigned long long) * (kDlCand + 1)));
    FAIR_CUDA(cudaMemsetAsync(esc.p, 0, sizeof(unsigned long long) * (kDlCand + 1), s));
    k_dl_count<E, B><<<dl_grid((int64_t)A.m * 32), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m,
                                                                A.col.as<int32_t>(), C,
                                                                esc.as<unsigned long long>());
    FAIR_CUDA(cudaGetLastError());
    unsigned long long hesc[kDlCand] = {};
    FAIR_CUDA(cudaMemcpyAsync(hesc, esc.p, sizeof(hesc), cudaMemcpyDeviceToHost, s));
    const int64_t nch = ((int64_t)A.m + 31) / 32;
    FAIR_TRY(cnt.grow(sizeof(int32_t) * (nch + 1)));
    FAIR_TRY(dl.soff.grow(sizeof(int64_t) * (nch + 1)));
    k_dl_len<<<dl_grid(nch * 32), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m, nch, E, cnt.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    FAIR_TRY(scan_counts(cnt.as<int32_t>(), nch, dl.soff.as<int64_t>(), s));
    FAIR_CUDA(cudaMemcpyAsync(&dl.nslots, dl.soff.as<int64_t>() + nch, sizeof(int64_t),
                              cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    int best = 0;
    for (int c = 1; c < C.n; ++c)
        if (hesc[c] < hesc[best]) best = c;
    const int64_t nslots_min = (A.nnz + E - 1) / E;
    // too many slots without codes: the side-table reads would cost more than the codes save
    if (hesc[best] > (unsigned long long)(nslots_min / 8) || hesc[best] > kDlSlot) {
        dl.soff.release();
        return FAIR_OK;
    }
    constexpr int E4 = (E + 3) / 4;
    const size_t ns = (size_t)std::max<int64_t>(dl.nslots, 1);
    FAIR_TRY(dl.code.grow(sizeof(uint32_t) * ns));
    FAIR_TRY(dl.anchor.grow(sizeof(int32_t) * (size_t)A.m));
    FAIR_TRY(dl.side.grow(sizeof(int4) * E4 * (size_t)std::max<unsigned long long>(hesc[best], 1)));
    unsigned long long *ctr = esc.as<unsigned long long>() + kDlCand;
    k_dl_fill<E, B><<<dl_grid(nch * 32), 256, 0, s>>>(
        A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(), nch, dl.soff.as<int64_t>(), C.S[best],
        C.L[best], dl.code.as<uint32_t>(), dl.anchor.as<int32_t>(), dl.side.as<int4>(), hesc[best], ctr);
    FAIR_CUDA(cudaGetLastError());
    unsigned long long used = 0;
    FAIR_CUDA(cudaMemcpyAsync(&used, ctr, sizeof(used), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    if (used != hesc[best]) {  // the fill must meet exactly the slots the count found
        set_detail("delta copy: side-table count mismatch");
        dl.release();
        dl.tried = true;
        return FAIR_ERR_STATE;
    }
    dl.S = C.S[best];
    dl.L = C.L[best];
    dl.nesc = (int64_t)hesc[best];
    dl.built = true;
    return FAIR_OK;
}

}  // namespace

int csr_make_delta(DevCSR &A, int prec, cudaStream_t s) {
    if (A.m == 0 || A.nnz == 0) return FAIR_OK;
    const bool two = prec == FAIR_PREC_F16 || prec == FAIR_PREC_Q16;
    DevCSR::Delta &dl = A.dl[two ? 1 : 0];
    if (!dl.tried) {
        dl.tried = true;
        const int st = two ? dl_build<6, 5>(A, dl, s) : dl_build<4, 7>(A, dl, s);
        if (st != FAIR_OK) return st;
    }
    if (!dl.built) return FAIR_OK;
    const int64_t nch = ((int64_t)A.m + 31) / 32;
    const size_t ns = (size_t)std::max<int64_t>(dl.nslots, 1);
    const int grid = dl_grid(nch * 32);
    const int64_t *rp = A.rowptr.as<int64_t>(), *so = dl.soff.as<int64_t>();
    if (prec == FAIR_PREC_F64 && !dl.has_v64) {
        FAIR_TRY(dl.v64.grow(sizeof(double) * 4 * ns));
        k_dl_vals<double><<<grid, 256, 0, s>>>(rp, A.m, nch, so, A.v64.as<double>(), dl.v64.as<double>());
        dl.has_v64 = true;
    } else if (prec == FAIR_PREC_F32 && !dl.has_v32) {
        FAIR_TRY(csr_make_lowprec(A, prec, s));
        FAIR_TRY(dl.v32.grow(sizeof(float) * 4 * ns));
        k_dl_vals<float><<<grid, 256, 0, s>>>(rp, A.m, nch, so, A.v32.as<float>(), dl.v32.as<float>());
        dl.has_v32 = true;
    } else if (two && !(prec == FAIR_PREC_F16 ? dl.has_r16 : dl.has_rq)) {
        FAIR_TRY(csr_make_lowprec(A, prec, s));
        const bool h = prec == FAIR_PREC_F16;
        DevBuf &dst = h ? dl.r16 : dl.rq;
        FAIR_TRY(dst.grow(sizeof(uint4) * ns));
        k_dl_rec6<<<grid, 256, 0, s>>>(rp, A.m, nch, so, dl.code.as<uint32_t>(),
                                        h ? A.v16.as<uint16_t>() : A.vq.as<uint16_t>(), dst.as<uint4>());
        (h ? dl.has_r16 : dl.has_rq) = true;
    }
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

bool sirt_pass_delta(const SirtDev &S, const DevCSR &M, int pass, int code, cudaStream_t s) {
    if (S.prec == FAIR_PREC_F64) {
        const DevCSR::Delta &dl = M.dl[0];
        if (!dl.built || !dl.has_v64) return false;
        dl_pass(M, dl, DlSplit<double>{dl.code.as<uint32_t>(), dl.v64.as<double>()}, pass, code, S.x,
                (const double *)S.r, EpiResidF64{S.b, S.Minv, (double *)S.r},
                EpiUpdateF64{S.D, S.x, S.omg, S.lb, S.ub, S.bmode}, S.sched, s);
        return true;
    }
    const double scale = S.prec == FAIR_PREC_Q16 ? M.qscale : 1.0;
    const EpiResidLP er{S.b, S.Minv, (float *)S.r, scale};
    const EpiUpdateLP eu{S.D, S.x, S.x32, S.omg, S.lb, S.ub, S.bmode, scale};
    const float *x = S.x32, *r = (const float *)S.r;
    if (S.prec == FAIR_PREC_F32) {
        const DevCSR::Delta &dl = M.dl[0];
        if (!dl.built || !dl.has_v32) return false;
        dl_pass(M, dl, DlSplit<float>{dl.code.as<uint32_t>(), dl.v32.as<float>()}, pass, code, x, r,
                er, eu, S.sched, s);
        return true;
    }
    const DevCSR::Delta &dl = M.dl[1];
    if (S.prec == FAIR_PREC_F16) {
        if (!dl.built || !dl.has_r16) return false;
        dl_pass(M, dl, DlRec6<__half>{dl.r16.as<uint4>()}, pass, code, x, r, er, eu, S.sched, s);
        return true;
    }
    if (!dl.built || !dl.has_rq) return false;
    if (M.qsigned)
        dl_pass(M, dl, DlRec6<int16_t>{dl.rq.as<uint4>()}, pass, code, x, r, er, eu, S.sched, s);
    else
        dl_pass(M, dl, DlRec6<uint16_t>{dl.rq.as<uint4>()}, pass, code, x, r, er, eu, S.sched, s);
    return true;
}

}  // namespace fair
