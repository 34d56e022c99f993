// rows.cuh -- the row-product engine shared by every CSR pass.
//
// A warp owns chunks of 32 consecutive rows (rays of one angle, or pixels of
// one image column for the transposed matrix, so the rows of a chunk have
// similar lengths). Within a chunk it works on 32/G rows at a time with G
// lanes per row; every lane reads 4 consecutive entries per step with one
// 128-bit load of column indices and one vector load of values, from the
// 16-byte-aligned window around the row, masking entries outside the row, and
// prefetches its next step before gathering x for the current one. The row
// sums are reduced over the G lanes and moved to lane (row mod 32), so the
// epilogue of a chunk runs once for its 32 rows with coalesced loads and
// stores: FP64 epilogue work (division, bounds) costs one warp instruction per
// 32 rows instead of one per row, which matters on a part whose FP64 pipe
// issues two lanes per clock.
//
// Column/value arrays are allocated with 4 spare entries so that the aligned
// window never reads past the allocation.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

namespace fair {

// Loads of the matrix streams (indices, values, records): read once per pass,
// so they bypass L1 (no allocation), which stays with the gathered vector,
// and ask L2 to fetch 256-byte blocks around each access.
#define FAIR_STREAM_L1_BYPASS 1
#if FAIR_STREAM_L1_BYPASS
__device__ __forceinline__ uint4 ld_stream(const uint4 *p) {
    uint4 r;
    asm("ld.global.nc.L1::no_allocate.L2::256B.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ int4 ld_stream(const int4 *p) {
    int4 r;
    asm("ld.global.nc.L1::no_allocate.L2::256B.v4.s32 {%0, %1, %2, %3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ unsigned ld_stream(const unsigned *p) {
    unsigned r;
    asm("ld.global.nc.L1::no_allocate.L2::256B.u32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
}
__device__ __forceinline__ uint2 ld_stream(const uint2 *p) {
    uint2 r;
    asm("ld.global.nc.L1::no_allocate.L2::256B.v2.u32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "l"(p));
    return r;
}
__device__ __forceinline__ float4 ld_stream(const float4 *p) {
    float4 r;
    asm("ld.global.nc.L1::no_allocate.L2::256B.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ double2 ld_stream(const double2 *p) {
    double2 r;
    asm("ld.global.nc.L1::no_allocate.L2::256B.v2.f64 {%0, %1}, [%2];" : "=d"(r.x), "=d"(r.y) : "l"(p));
    return r;
}
#else
template <typename T> __device__ __forceinline__ T ld_stream(const T *p) { return __ldcs(p); }
#endif

template <typename VT, typename AT> struct VLoad;
template <> struct VLoad<double, double> {
    static __device__ __forceinline__ void ld(const double *p, double (&o)[4]) {
        double2 a = ld_stream(reinterpret_cast<const double2 *>(p));
        double2 b = ld_stream(reinterpret_cast<const double2 *>(p) + 1);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    }
};
template <> struct VLoad<float, float> {
    static __device__ __forceinline__ void ld(const float *p, float (&o)[4]) {
        float4 t = ld_stream(reinterpret_cast<const float4 *>(p));
        o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
    }
};
template <> struct VLoad<__half, float> {
    static __device__ __forceinline__ void ld(const __half *p, float (&o)[4]) {
        uint2 t = ld_stream(reinterpret_cast<const uint2 *>(p));
        __half2 a = *reinterpret_cast<__half2 *>(&t.x), b = *reinterpret_cast<__half2 *>(&t.y);
        float2 fa = __half22float2(a), fb = __half22float2(b);
        o[0] = fa.x; o[1] = fa.y; o[2] = fb.x; o[3] = fb.y;
    }
};

// Next chunk for this warp. With `sched` (two zeroed counters) chunks are
// claimed dynamically, one atomic per chunk, which balances the warps when
// chunk costs differ (runs of empty edge rays); the last warp to run out
// resets the counters for the next launch on the stream. Without `sched`
// the warps stride over the chunks in a fixed order (used where block sums
// must not depend on scheduling).
__device__ __forceinline__ int64_t next_chunk(unsigned *sched, int64_t prev, int64_t nwarps,
                                              int lane) {
    if (!sched) return prev + nwarps;
    unsigned c = 0;
    if (lane == 0) c = atomicAdd(&sched[0], 1u);
    return (int64_t)__shfl_sync(0xffffffffu, c, 0);
}

__device__ __forceinline__ void finish_chunks(unsigned *sched, int64_t nwarps, int lane) {
    if (!sched || lane != 0) return;
    unsigned done = atomicAdd(&sched[1], 1u);
    if (done == (unsigned)(nwarps - 1)) {  // every warp has stopped claiming
        sched[0] = 0u;
        sched[1] = 0u;
    }
}

// 16-bit fixed-point values: the integer codes are accumulated as floats and
// the matrix scale is applied once per row in the epilogue. A code u becomes
// a float without the conversion pipe: the bytes of u under the exponent of
// 2^23 (one byte permute) are the float 2^23 + u, exact, minus 2^23 (one FP32
// add). Signed codes are first offset by 2^15 (flip of the sign bit).
// (The difference of the two exact floats is an integer below 2^24: exact.)
__device__ __forceinline__ float u16_lo(uint32_t w, float bias) {
    return __int_as_float((int)__byte_perm(w, 0x4B00u, 0x5410u)) - bias;
}
__device__ __forceinline__ float u16_hi(uint32_t w, float bias) {
    return __int_as_float((int)__byte_perm(w, 0x4B00u, 0x5432u)) - bias;
}
// Four 2-byte values held in two 32-bit words, to floats.
template <typename VT> struct Conv2B;
template <> struct Conv2B<uint16_t> {
    static __device__ __forceinline__ void two(uint32_t a, float &lo, float &hi) {
        constexpr float b = 8388608.0f;  // 2^23
        lo = u16_lo(a, b); hi = u16_hi(a, b);
    }
    static __device__ __forceinline__ void to(uint32_t a, uint32_t b2, float (&o)[4]) {
        two(a, o[0], o[1]);
        two(b2, o[2], o[3]);
    }
};
template <> struct Conv2B<int16_t> {
    static __device__ __forceinline__ void two(uint32_t a, float &lo, float &hi) {
        constexpr float b = 8421376.0f;  // 2^23 + 2^15
        a ^= 0x80008000u;
        lo = u16_lo(a, b); hi = u16_hi(a, b);
    }
    static __device__ __forceinline__ void to(uint32_t a, uint32_t b2, float (&o)[4]) {
        two(a, o[0], o[1]);
        two(b2, o[2], o[3]);
    }
};
template <> struct Conv2B<__half> {
    static __device__ __forceinline__ void two(uint32_t a, float &lo, float &hi) {
        const float2 f = __half22float2(*reinterpret_cast<__half2 *>(&a));
        lo = f.x; hi = f.y;
    }
    static __device__ __forceinline__ void to(uint32_t a, uint32_t b2, float (&o)[4]) {
        two(a, o[0], o[1]);
        two(b2, o[2], o[3]);
    }
};
template <> struct VLoad<uint16_t, float> {
    static __device__ __forceinline__ void ld(const uint16_t *p, float (&o)[4]) {
        uint2 t = ld_stream(reinterpret_cast<const uint2 *>(p));
        Conv2B<uint16_t>::to(t.x, t.y, o);
    }
};
template <> struct VLoad<int16_t, float> {
    static __device__ __forceinline__ void ld(const int16_t *p, float (&o)[4]) {
        uint2 t = ld_stream(reinterpret_cast<const uint2 *>(p));
        Conv2B<int16_t>::to(t.x, t.y, o);
    }
};

// Row sums of one chunk (rows base..base+31): returns, in lane l, the sum of
// row base+l. All lanes of the warp call it together.
// VT: stored value type; XT: gathered vector type; ACC: accumulator type.
// The sum of row `row` (0 past m) by the G lanes of its group, gl the lane's
// place in the group: each lane takes the 4-entry groups at (s & ~3) + 4 gl,
// then every 4 G entries, adding each group's products in order; the group's
// butterfly leaves the sum in every lane of the group.
template <typename VT, typename XT, typename ACC, int G>
__device__ __forceinline__ ACC csr_row_sum(const int64_t *__restrict__ rowptr, int32_t m,
                                           const int32_t *__restrict__ col,
                                           const VT *__restrict__ val,
                                           const XT *__restrict__ x, int64_t row, int gl) {
    int64_t s = 0, e = 0;
    if (row < m) {
        s = __ldg(rowptr + row);
        e = __ldg(rowptr + row + 1);
    }
    ACC acc = 0;
    int64_t k = (s & ~(int64_t)3) + 4 * gl;
    int4 cc = make_int4(0, 0, 0, 0);
    ACC vv[4] = {0, 0, 0, 0};
    if (k < e) {
        cc = ld_stream(reinterpret_cast<const int4 *>(col + k));
        VLoad<VT, ACC>::ld(val + k, vv);
    }
    while (k < e) {
        const int64_t kn = k + 4 * G;
        int4 cn = make_int4(0, 0, 0, 0);
        ACC vn[4] = {0, 0, 0, 0};
        if (kn < e) {
            cn = ld_stream(reinterpret_cast<const int4 *>(col + kn));
            VLoad<VT, ACC>::ld(val + kn, vn);
        }
        if (k >= s && k + 3 < e) {
            acc += (ACC)__ldg(x + cc.x) * vv[0];
            acc += (ACC)__ldg(x + cc.y) * vv[1];
            acc += (ACC)__ldg(x + cc.z) * vv[2];
            acc += (ACC)__ldg(x + cc.w) * vv[3];
        } else {
            if (k >= s && k < e) acc += (ACC)__ldg(x + cc.x) * vv[0];
            if (k + 1 >= s && k + 1 < e) acc += (ACC)__ldg(x + cc.y) * vv[1];
            if (k + 2 >= s && k + 2 < e) acc += (ACC)__ldg(x + cc.z) * vv[2];
            if (k + 3 >= s && k + 3 < e) acc += (ACC)__ldg(x + cc.w) * vv[3];
        }
        cc = cn;
#pragma unroll
        for (int t = 0; t < 4; ++t) vv[t] = vn[t];
        k = kn;
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// The sums of the 32 rows of a chunk, row base + lane in lane `lane`: 32/G
// rows at a time, one per group of G lanes.
template <typename VT, typename XT, typename ACC, int G>
__device__ __forceinline__ ACC csr_chunk_sums(const int64_t *__restrict__ rowptr, int32_t m,
                                              const int32_t *__restrict__ col,
                                              const VT *__restrict__ val,
                                              const XT *__restrict__ x, int64_t base) {
    constexpr int R = 32 / G;
    const int lane = threadIdx.x & 31, g = lane / G, gl = lane % G;
    ACC mine = 0;
#pragma unroll 1
    for (int sub = 0; sub < 32; sub += R) {
        const ACC acc = csr_row_sum<VT, XT, ACC, G>(rowptr, m, col, val, x, base + sub + g, gl);
        ACC r = __shfl_sync(0xffffffffu, acc, ((lane - sub) & (R - 1)) * G);
        if (lane >= sub && lane < sub + R) mine = r;
    }
    return mine;
}

// Sum over the rows of every chunk owned by this warp; calls epi(row, sum)
// from the lane that owns `row` (all lanes of the warp call epi together).
template <typename VT, typename XT, typename ACC, int G, class Epi>
__device__ __forceinline__ void chunk_rows(const int64_t *__restrict__ rowptr, int32_t m,
                                           const int32_t *__restrict__ col,
                                           const VT *__restrict__ val,
                                           const XT *__restrict__ x, Epi &epi,
                                           unsigned *sched = nullptr) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = ((int64_t)m + 31) >> 5;
    for (int64_t ch = sched ? next_chunk(sched, 0, nwarps, lane) : warp; ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int64_t base = ch << 5;
        const ACC mine = csr_chunk_sums<VT, XT, ACC, G>(rowptr, m, col, val, x, base);
        const int64_t row = base + lane;
        if (row < m) epi(row, mine);
    }
    finish_chunks(sched, nwarps, lane);
}

// The same row sums with each warp taking one group of 32/G consecutive rows
// at a time instead of a chunk of 32: G times the warps for the same rows, the
// same arithmetic per row (csr_row_sum), so the same results bit for bit.
// For matrices with too few 32-row chunks to fill the GPU.
template <typename VT, typename XT, typename ACC, int G, class Epi>
__device__ __forceinline__ void rows_by_group(const int64_t *__restrict__ rowptr, int32_t m,
                                              const int32_t *__restrict__ col,
                                              const VT *__restrict__ val,
                                              const XT *__restrict__ x, Epi &epi) {
    constexpr int R = 32 / G;
    const int lane = threadIdx.x & 31, g = lane / G, gl = lane % G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nunits = ((int64_t)m + R - 1) / R;
    for (int64_t u = warp; u < nunits; u += nwarps) {
        const int64_t row = u * R + g;
        const ACC acc = csr_row_sum<VT, XT, ACC, G>(rowptr, m, col, val, x, row, gl);
        if (gl == 0 && row < m) epi(row, acc);
    }
}

// ---- packed index stream ------------------------------------------------------
// One 8-byte word per group of 4 consecutive entries of a row (rows padded to
// whole groups): .x = column of the group's first entry; .y bits 0-23 = three
// 8-bit step codes (column of entry k minus column of entry k-1, k = 1..3) or,
// with bit 26 set, an index into a side table holding the three columns;
// bits 24-25 = entries in the group - 1. A step code is a signed low part of
// L bits and a signed high part of 8-L bits, delta = lo + hi*S, where S is the
// matrix's column step across the image: N for a ray matrix (a ray moves to a
// 4- or 8-neighbour pixel, delta in {+-1, +-N, +-N+-1}), the bins per angle
// for its transpose (the next ray through a pixel is the next bin or a bin
// of the next angle). With 16-bit values a group costs 16 bytes instead of 24.
constexpr uint32_t kPkEsc = 1u << 26;

__host__ __device__ inline bool pk_encode(int64_t d, int S, int L, uint32_t &code) {
    int64_t hi = 0;
    if (S > 0) hi = d >= 0 ? (d + S / 2) / S : -((-d + S / 2) / S);
    const int64_t lo = d - hi * S;
    const int64_t lmin = -(int64_t(1) << (L - 1)), lmax = (int64_t(1) << (L - 1)) - 1;
    const int64_t hmin = -(int64_t(1) << (7 - L)), hmax = (int64_t(1) << (7 - L)) - 1;
    if (lo < lmin || lo > lmax || hi < hmin || hi > hmax) return false;
    code = (uint32_t)(((hi << L) | (lo & ((int64_t(1) << L) - 1))) & 0xFF);
    return true;
}

__device__ __forceinline__ int pk_step(uint32_t b, int S, int L) {
    const int lo = (int)(b << (32 - L)) >> (32 - L);
    const int hi = (int)(b << 24) >> (24 + L);
    return lo + hi * S;
}

// Columns of one packed group (entries beyond the group's count repeat the
// previous column).
__device__ __forceinline__ void pk_decode(uint2 w, const int4 *__restrict__ gside, int S, int L,
                                          int (&c)[4]) {
    c[0] = (int)w.x;
    if (w.y & kPkEsc) {
        const int4 t = __ldg(gside + (w.y & 0xFFFFFFu));
        c[1] = t.x; c[2] = t.y; c[3] = t.z;
    } else {
        c[1] = c[0] + pk_step(w.y & 0xFFu, S, L);
        c[2] = c[1] + pk_step((w.y >> 8) & 0xFFu, S, L);
        c[3] = c[2] + pk_step((w.y >> 16) & 0xFFu, S, L);
    }
}

// Group loaders of the packed stream: the index word and the four values of
// group j. SplitLoad reads them from the index array and the padded value
// array (two loads); FusedLoad reads the 16-byte record {index word, four
// 2-byte values} of the fused layout (one load).
template <typename VT, typename ACC> struct SplitLoad {
    const uint2 *gidx;
    const VT *val;
    __device__ __forceinline__ void ld(int64_t j, uint2 &w, ACC (&v)[4]) const {
        w = ld_stream(gidx + j);
        VLoad<VT, ACC>::ld(val + 4 * j, v);
    }
};
template <typename VT> struct FusedLoad {
    const uint4 *rec;
    __device__ __forceinline__ void ld(int64_t j, uint2 &w, float (&v)[4]) const {
        const uint4 r = ld_stream(rec + j);
        w = make_uint2(r.x, r.y);
        Conv2B<VT>::to(r.z, r.w, v);
    }
};

// Row sums of one chunk over the packed index stream: every lane takes NG
// groups (4*NG entries) per step through the loader and issues the 4*NG
// gathers of a step together.
template <typename XT, typename ACC, int G, int NG, class LD>
__device__ __forceinline__ ACC pk_chunk_sums_ld(const int64_t *__restrict__ prow, int32_t m,
                                                const LD &ldr, const int4 *__restrict__ gside,
                                                int S, int L, const XT *__restrict__ x,
                                                int64_t base) {
    constexpr int R = 32 / G;
    const int lane = threadIdx.x & 31, g = lane / G, gl = lane % G;
    ACC mine = 0;
#pragma unroll 1
    for (int sub = 0; sub < 32; sub += R) {
        const int64_t row = base + sub + g;
        int64_t g0 = 0;
        int ng = 0;  // groups in the row
        if (row < m) {
            g0 = __ldg(prow + row);
            ng = (int)(__ldg(prow + row + 1) - g0);
        }
        ACC acc = 0;
        uint2 w[NG];
        ACC vv[NG][4];
#pragma unroll
        for (int q = 0; q < NG; ++q) {
            const int j = gl + q * G;
            w[q] = make_uint2(0u, 0u);
            vv[q][0] = vv[q][1] = vv[q][2] = vv[q][3] = 0;
            if (j < ng) ldr.ld(g0 + j, w[q], vv[q]);
        }
        for (int j = gl; j < ng; j += NG * G) {
            const int jn = j + NG * G;
            uint2 wn[NG];
            ACC vn[NG][4];
#pragma unroll
            for (int q = 0; q < NG; ++q) {
                wn[q] = make_uint2(0u, 0u);
                vn[q][0] = vn[q][1] = vn[q][2] = vn[q][3] = 0;
                if (jn + q * G < ng) ldr.ld(g0 + jn + q * G, wn[q], vn[q]);
            }
            int c[NG][4];
            ACC xv[NG][4];
#pragma unroll
            for (int q = 0; q < NG; ++q) {
                pk_decode(w[q], gside, S, L, c[q]);
                // entries past the group's count (and groups past the row)
                // read nothing and add zero
                const int cnt = j + q * G < ng ? (int)((w[q].y >> 24) & 3u) : -1;
#pragma unroll
                for (int t = 0; t < 4; ++t) xv[q][t] = t <= cnt ? (ACC)__ldg(x + c[q][t]) : (ACC)0;
            }
#pragma unroll
            for (int q = 0; q < NG; ++q)
#pragma unroll
                for (int t = 0; t < 4; ++t) acc += xv[q][t] * vv[q][t];
#pragma unroll
            for (int q = 0; q < NG; ++q) {
                w[q] = wn[q];
#pragma unroll
                for (int t = 0; t < 4; ++t) vv[q][t] = vn[q][t];
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        ACC r = __shfl_sync(0xffffffffu, acc, ((lane - sub) & (R - 1)) * G);
        if (lane >= sub && lane < sub + R) mine = r;
    }
    return mine;
}

// The split layout (index array + padded values).
template <typename VT, typename XT, typename ACC, int G, int NG>
__device__ __forceinline__ ACC pk_chunk_sums(const int64_t *__restrict__ prow, int32_t m,
                                             const uint2 *__restrict__ gidx,
                                             const int4 *__restrict__ gside, int S, int L,
                                             const VT *__restrict__ val,
                                             const XT *__restrict__ x, int64_t base) {
    const SplitLoad<VT, ACC> ldr{gidx, val};
    return pk_chunk_sums_ld<XT, ACC, G, NG>(prow, m, ldr, gside, S, L, x, base);
}

// chunk_rows over the fused 16-byte records (2-byte values).
template <typename VT, int G, int NG, class Epi>
__device__ __forceinline__ void chunk_rows_pkf(const int64_t *__restrict__ prow, int32_t m,
                                               const uint4 *__restrict__ rec,
                                               const int4 *__restrict__ gside, int S, int L,
                                               const float *__restrict__ x, Epi &epi,
                                               unsigned *sched) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = ((int64_t)m + 31) >> 5;
    const FusedLoad<VT> ldr{rec};
    for (int64_t ch = sched ? next_chunk(sched, 0, nwarps, lane) : warp; ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int64_t base = ch << 5;
        const float mine = pk_chunk_sums_ld<float, float, G, NG>(prow, m, ldr, gside, S, L, x, base);
        const int64_t row = base + lane;
        if (row < m) epi(row, mine);
    }
    finish_chunks(sched, nwarps, lane);
}

// chunk_rows over the packed index stream.
template <typename VT, typename XT, typename ACC, int G, int NG, class Epi>
__device__ __forceinline__ void chunk_rows_pk(const int64_t *__restrict__ prow, int32_t m,
                                              const uint2 *__restrict__ gidx,
                                              const int4 *__restrict__ gside, int S, int L,
                                              const VT *__restrict__ val,
                                              const XT *__restrict__ x, Epi &epi,
                                              unsigned *sched) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = ((int64_t)m + 31) >> 5;
    for (int64_t ch = sched ? next_chunk(sched, 0, nwarps, lane) : warp; ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int64_t base = ch << 5;
        const ACC mine = pk_chunk_sums<VT, XT, ACC, G, NG>(prow, m, gidx, gside, S, L, val, x, base);
        const int64_t row = base + lane;
        if (row < m) epi(row, mine);
    }
    finish_chunks(sched, nwarps, lane);
}

// ---- sliced copy of the packed stream --------------------------------------
// A chunk of 32 rows is cut into slices of R = 32/G rows with G lanes per row.
// Within a slice the rows' groups are interleaved by step: at step k lane
// g*G + l of the slice holds group k*G + l of its row g, all 32 slots of a
// step stored together, and every row is padded with hole records to the
// slice's longest row (in steps). The slices of a chunk follow one another,
// so the chunk is one contiguous run of slots, soff[chunk] .. soff[chunk+1],
// that the warp reads 32 slots (512 bytes of 16-byte records) per step with
// the loads of the next D steps in flight across slice boundaries. Every
// lane adds its own groups' products; at the end of a slice (a step count
// the whole warp knows) the G lanes of each row are summed and the row sum
// moves to the lane that owns the row. G = 1 is SELL-32: one lane per row,
// no lane sums. The rows of a slice are adjacent rays of one angle (or
// adjacent pixels of one image column for A'), so the gathers of one step
// reach neighbouring x entries.
constexpr uint32_t kPkHole = 1u << 27;  // padding slot of a sliced copy (no entries)

// Step codes to column steps for one (S, L), in shared memory: a table
// lookup instead of the shifts and multiply of pk_step.
__device__ __forceinline__ void pk_lut_fill(int *lut, int S, int L) {
    for (int t = threadIdx.x; t < 256; t += blockDim.x) lut[t] = pk_step((uint32_t)t, S, L);
    __syncthreads();
}
__device__ __forceinline__ void pk_decode_lut(uint2 w, const int4 *__restrict__ gside,
                                              const int *lut, int (&c)[4]) {
    c[0] = (int)w.x;
    c[1] = c[0] + lut[w.y & 0xFFu];
    c[2] = c[1] + lut[(w.y >> 8) & 0xFFu];
    c[3] = c[2] + lut[(w.y >> 16) & 0xFFu];
    if (w.y & kPkEsc) {
        const int4 t = __ldg(gside + (w.y & 0xFFFFFFu));
        c[1] = t.x; c[2] = t.y; c[3] = t.z;
    }
}

// Four padded values of one group as loaded (VBlk::ld) and converted (to).
template <typename VT> struct VBlk;
template <> struct VBlk<double> {
    double2 a, b;
    __device__ __forceinline__ void ld(const double *p) {
        a = ld_stream(reinterpret_cast<const double2 *>(p));
        b = ld_stream(reinterpret_cast<const double2 *>(p) + 1);
    }
    __device__ __forceinline__ void clear() { a = b = make_double2(0.0, 0.0); }
    __device__ __forceinline__ void to(double (&o)[4]) const { o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y; }
};
template <> struct VBlk<float> {
    float4 a;
    __device__ __forceinline__ void ld(const float *p) { a = ld_stream(reinterpret_cast<const float4 *>(p)); }
    __device__ __forceinline__ void clear() { a = make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ __forceinline__ void to(float (&o)[4]) const { o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; }
};

// Slot loaders of a sliced copy: Raw is what a lane holds for one group in
// flight.
template <typename VT> struct FusedRec {  // fused 16-byte records, 2-byte values
    const uint4 *rec;
    using Raw = uint4;
    __device__ __forceinline__ Raw load(int64_t j) const { return ld_stream(rec + j); }
    __device__ __forceinline__ static Raw none() { return make_uint4(0u, 0u, 0u, 0u); }
    __device__ __forceinline__ static void open(const Raw &r, uint2 &w, float (&v)[4]) {
        w = make_uint2(r.x, r.y);
        Conv2B<VT>::to(r.z, r.w, v);
    }
};
template <typename VT> struct SplitRec {  // index words + 4 FP32/FP64 values per slot
    const uint2 *gidx;
    const VT *val;
    struct Raw {
        uint2 w;
        VBlk<VT> v;
    };
    __device__ __forceinline__ Raw load(int64_t j) const {
        Raw r;
        r.w = ld_stream(gidx + j);
        r.v.ld(val + 4 * j);
        return r;
    }
    __device__ __forceinline__ static Raw none() {
        Raw r;
        r.w = make_uint2(0u, 0u);
        r.v.clear();
        return r;
    }
    __device__ __forceinline__ static void open(const Raw &r, uint2 &w, VT (&v)[4]) {
        w = r.w;
        r.v.to(v);
    }
};

// Every chunk owned by this warp: lane l sums row base+l over the sliced
// copy and calls epi(row, sum). A chunk's slot offset carries log2 of its
// lanes per row G in its low bits (offsets are multiples of 32), so G may
// differ from chunk to chunk; GF = 1 compiles the copy whose chunks all have
// G = 1 (no slices to track, no lane sums), GF = 0 reads G per chunk. With
// PF the gathers of step t+1 are issued before the products of step t, so a
// warp has two steps of gathers in flight (for vectors that miss L1). `lut`
// is the block's step-code table.
template <typename XT, typename ACC, int D, int GF, int PF, class LD, class Epi>
__device__ __forceinline__ void chunk_rows_sliced(const int64_t *__restrict__ prow,
                                                  const int64_t *__restrict__ soff, int32_t m,
                                                  const LD &ldr, const int4 *__restrict__ gside,
                                                  const int *lut, const XT *__restrict__ x,
                                                  Epi &epi, unsigned *sched) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = ((int64_t)m + 31) >> 5;
    // products of one slot: the group's values and its gathered x (zeros
    // past the group's entries and for holes)
    auto gather = [&](const typename LD::Raw &r, ACC (&v)[4], ACC (&xv)[4]) {
        uint2 w;
        LD::open(r, w, v);
        xv[0] = xv[1] = xv[2] = xv[3] = (ACC)0;
        if (!(w.y & kPkHole)) {
            int cc[4];
            pk_decode_lut(w, gside, lut, cc);
            const int cnt = (int)((w.y >> 24) & 3u);  // entries in the group - 1
            xv[0] = (ACC)__ldg(x + cc[0]);
#pragma unroll
            for (int q = 1; q < 4; ++q)
                if (q <= cnt) xv[q] = (ACC)__ldg(x + cc[q]);
        }
    };
    for (int64_t ch = sched ? next_chunk(sched, 0, nwarps, lane) : warp; ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int64_t o0 = __ldg(soff + ch), o1 = __ldg(soff + ch + 1);
        const int lg = GF == 1 ? 0 : (int)(o0 & 7);
        const int G = 1 << lg, R = 32 >> lg;  // lanes per row, rows per slice
        const int64_t row = (ch << 5) + lane;
        const int ng = row < m ? (int)(__ldg(prow + row + 1) - __ldg(prow + row)) : 0;
        const int steps = (ng + G - 1) >> lg;  // steps of row base+lane
        const int64_t s0 = (o0 & ~(int64_t)31) + lane;
        const int T = (int)(((o1 & ~(int64_t)31) - (o0 & ~(int64_t)31)) >> 5);  // chunk steps
        // steps of slice i: the longest of its R rows
        auto slice_steps = [&](int i) -> int {
            return (int)__reduce_max_sync(FULL, (unsigned)__shfl_sync(FULL, steps, i * R + (lane & (R - 1))));
        };
        typename LD::Raw ring[D];
#pragma unroll
        for (int k = 0; k < D; ++k) ring[k] = k < T ? ldr.load(s0 + 32 * k) : LD::none();
        ACC acc = 0, mine = 0;
        int i = 0, end = 0;  // current slice and the step that ends it
        if constexpr (GF != 1) {
            end = slice_steps(0);
            while (end == 0 && i < G - 1) end = slice_steps(++i);  // slices of empty rows
        }
        ACC v[4] = {0, 0, 0, 0}, xv[4] = {0, 0, 0, 0};  // step t's values and gathers (PF)
        if constexpr (PF) {
            if (T > 0) {
                gather(ring[0], v, xv);
                ring[0] = D < T ? ldr.load(s0 + 32 * D) : LD::none();
            }
        }
        for (int t0 = 0; t0 < T; t0 += D) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const int t = t0 + k;
                if (t >= T) break;
                if constexpr (PF) {
                    ACC vn[4] = {0, 0, 0, 0}, xn[4] = {0, 0, 0, 0};
                    const int kn = (k + 1) % D;  // ring slot of step t+1 (fixed once unrolled)
                    if (t + 1 < T) {
                        gather(ring[kn], vn, xn);
                        ring[kn] = t + 1 + D < T ? ldr.load(s0 + 32 * (int64_t)(t + 1 + D)) : LD::none();
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc += xv[q] * v[q];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        v[q] = vn[q];
                        xv[q] = xn[q];
                    }
                } else {
                    const typename LD::Raw cur = ring[k];
                    ring[k] = t + D < T ? ldr.load(s0 + 32 * (int64_t)(t + D)) : LD::none();
                    uint2 w;
                    LD::open(cur, w, v);
                    if (!(w.y & kPkHole)) {
                        int cc[4];
                        pk_decode_lut(w, gside, lut, cc);
                        const int cnt = (int)((w.y >> 24) & 3u);  // entries in the group - 1
                        acc += (ACC)__ldg(x + cc[0]) * v[0];
#pragma unroll
                        for (int q = 1; q < 4; ++q)
                            if (q <= cnt) acc += (ACC)__ldg(x + cc[q]) * v[q];
                    }
                }
                if constexpr (GF != 1) {
                    if (t + 1 == end) {  // slice i done: sum each row's G lanes
                        for (int o = G >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
                        const ACC r = __shfl_sync(FULL, acc, ((lane - i * R) & (R - 1)) << lg);
                        if (lane >= i * R && lane < i * R + R) mine = r;
                        acc = 0;
                        int add = 0;
                        while (add == 0 && i < G - 1) add = slice_steps(++i);
                        end += add;
                    }
                }
            }
        }
        if constexpr (GF == 1) mine = acc;
        if (row < m) epi(row, mine);
    }
    finish_chunks(sched, nwarps, lane);
}

// ---- column steps (delta copies) -------------------------------------------
// A B-bit step code: a signed low part of L bits and a signed high part of
// B - L bits, delta = lo + hi*S (L = B: the plain signed delta). A word holds
// E codes, code q in bits B*q .. B*q + B - 1.
template <int B>
__host__ __device__ inline bool step_encode(int64_t d, int S, int L, uint32_t &code) {
    constexpr uint32_t mask = (1u << B) - 1u;
    if (L >= B) {
        if (d < -(int64_t(1) << (B - 1)) || d >= (int64_t(1) << (B - 1))) return false;
        code = (uint32_t)d & mask;
        return true;
    }
    int64_t hi = 0;
    if (S > 0) hi = d >= 0 ? (d + S / 2) / S : -((-d + S / 2) / S);
    const int64_t lo = d - hi * S;
    const int64_t lmin = -(int64_t(1) << (L - 1)), lmax = (int64_t(1) << (L - 1)) - 1;
    const int64_t hmin = -(int64_t(1) << (B - 1 - L)), hmax = (int64_t(1) << (B - 1 - L)) - 1;
    if (lo < lmin || lo > lmax || hi < hmin || hi > hmax) return false;
    code = (uint32_t)((hi << L) | (lo & ((int64_t(1) << L) - 1))) & mask;
    return true;
}
template <int B>
__device__ __forceinline__ int step_decode(uint32_t b, int S, int L) {
    const int lo = (int)(b << (32 - L)) >> (32 - L);
    const int hi = L >= B ? 0 : (int)(b << (32 - B)) >> (32 - B + L);
    return lo + hi * S;
}
// The word of E steps from `prev` through c[0..E-1]; false when a step has no code.
template <int E, int B>
__device__ __forceinline__ bool step_word(const int (&c)[E], int prev, int S, int L, uint32_t &w) {
    uint32_t cd;
    bool ok = step_encode<B>((int64_t)c[0] - prev, S, L, cd);
    w = ok ? cd : 0u;
#pragma unroll
    for (int q = 1; q < E; ++q) {
        ok = ok && step_encode<B>((int64_t)c[q] - c[q - 1], S, L, cd);
        if (ok) w |= cd << (B * q);
    }
    return ok;
}
constexpr uint32_t kStepEsc = 1u << 31;         // the word's columns are in a side table
constexpr uint32_t kStepSlot = 0x3FFFFFFFu;     // its slot there

// Lanes per row used when none has been tuned.
constexpr int kDefaultLanesPerRow = 8;

}  // namespace fair
