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

template <typename VT, typename AT> struct VLoad;
template <> struct VLoad<double, double> {
    static __device__ __forceinline__ void ld(const double *p, double (&o)[4]) {
        double2 a = __ldcs(reinterpret_cast<const double2 *>(p));
        double2 b = __ldcs(reinterpret_cast<const double2 *>(p) + 1);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    }
};
template <> struct VLoad<float, float> {
    static __device__ __forceinline__ void ld(const float *p, float (&o)[4]) {
        float4 t = __ldcs(reinterpret_cast<const float4 *>(p));
        o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
    }
};
template <> struct VLoad<__half, float> {
    static __device__ __forceinline__ void ld(const __half *p, float (&o)[4]) {
        uint2 t = __ldcs(reinterpret_cast<const uint2 *>(p));
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
// the matrix scale is applied once per row in the epilogue.
template <> struct VLoad<uint16_t, float> {
    static __device__ __forceinline__ void ld(const uint16_t *p, float (&o)[4]) {
        uint2 t = __ldcs(reinterpret_cast<const uint2 *>(p));
        o[0] = (float)(t.x & 0xffffu); o[1] = (float)(t.x >> 16);
        o[2] = (float)(t.y & 0xffffu); o[3] = (float)(t.y >> 16);
    }
};
template <> struct VLoad<int16_t, float> {
    static __device__ __forceinline__ void ld(const int16_t *p, float (&o)[4]) {
        uint2 t = __ldcs(reinterpret_cast<const uint2 *>(p));
        o[0] = (float)(int16_t)(t.x & 0xffffu); o[1] = (float)(int16_t)(t.x >> 16);
        o[2] = (float)(int16_t)(t.y & 0xffffu); o[3] = (float)(int16_t)(t.y >> 16);
    }
};

// Sum over the rows of every chunk owned by this warp; calls epi(row, sum)
// from the lane that owns `row` (all lanes of the warp call epi together).
// VT: stored value type; XT: gathered vector type; ACC: accumulator type.
template <typename VT, typename XT, typename ACC, int G, class Epi>
__device__ __forceinline__ void chunk_rows(const int64_t *__restrict__ rowptr, int32_t m,
                                           const int32_t *__restrict__ col,
                                           const VT *__restrict__ val,
                                           const XT *__restrict__ x, Epi &epi,
                                           unsigned *sched = nullptr) {
    constexpr int R = 32 / G;
    const int lane = threadIdx.x & 31, g = lane / G, gl = lane % G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = ((int64_t)m + 31) >> 5;
    for (int64_t ch = sched ? next_chunk(sched, 0, nwarps, lane) : warp; ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int64_t base = ch << 5;
        ACC mine = 0;
#pragma unroll 1
        for (int sub = 0; sub < 32; sub += R) {
            const int64_t row = base + sub + g;
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
                cc = __ldcs(reinterpret_cast<const int4 *>(col + k));
                VLoad<VT, ACC>::ld(val + k, vv);
            }
            while (k < e) {
                const int64_t kn = k + 4 * G;
                int4 cn = make_int4(0, 0, 0, 0);
                ACC vn[4] = {0, 0, 0, 0};
                if (kn < e) {
                    cn = __ldcs(reinterpret_cast<const int4 *>(col + kn));
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
            ACC r = __shfl_sync(0xffffffffu, acc, ((lane - sub) & (R - 1)) * G);
            if (lane >= sub && lane < sub + R) mine = r;
        }
        const int64_t row = base + lane;
        if (row < m) epi(row, mine);
    }
    finish_chunks(sched, nwarps, lane);
}

// Lanes per row used when none has been tuned.
constexpr int kDefaultLanesPerRow = 8;

}  // namespace fair
