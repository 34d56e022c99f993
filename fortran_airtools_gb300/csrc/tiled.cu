// tiled.cu -- the SIRT passes (AIRMs.f90:1089-1110) on copies of A and A' cut
// by tiles whose part of the gathered vector fits in shared memory (layout
// codes 9, 10 and 14).
//
// The columns of a ray matrix are the pixels of an N x N image (column j =
// c*N + r). On the row layouts the x entries a warp gathers are scattered
// along whole rays, so half of them miss L1 and each costs a 32-byte sector
// from L2: more L2-to-SM bytes than the matrix itself. Here every row of A is
// cut into segments, one per T x T tile of the image that the ray crosses (a
// convex tile is crossed once, so a segment is a run of the row's entries).
// A' (rows = pixels, columns = rays a*p + b) is cut the other way round: by
// tiles of its rows (32 x 32 pixels) times blocks of angles, whose copy holds
// a window of residual bins per angle (TlGeo below).
// The segments of a tile are sorted by length (longest first; in row order the
// chunks mix lengths and idle more lanes: 20% slower) and stored in chunks of
// 32, one lane per segment, slot k of lane l at soff[chunk] + 32k +
// l (the sliced layout of rows.cuh with G = 1); a slot holds 4 entries as
// 16-bit indices into the tile's shared-memory copy (column stride T + 1, so
// that steps along rows and columns fall in different banks) plus their
// values. Padding entries and slots point at a zero cell with value 0.
// A work unit is a run of chunks of one tile: a CTA copies the tile of x into
// shared memory once and its warps work through the unit's chunks, every lane
// summing its segment into one partial (FP32, or FP64 for the FP64 form)
// stored at the segment's slot in row order; a second kernel adds each row's
// partials in that fixed order and applies the residual epilogue, so the
// result does not depend on scheduling. With 2 slots in flight (codes 9, 14)
// warp w of a CTA reads chunks w, w + W, ... of the unit as one stream, the
// loads of a chunk's first slots issued during the chunk before; its
// register use is capped so that 4 CTAs (64 warps) fit an SM. Code 10 keeps 4
// slots in flight per chunk and claims chunks dynamically.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

#include "fair_internal.cuh"
#include "rows.cuh"
#include "sirt_epi.cuh"

namespace fair {

namespace {

constexpr int kTile = 96;           // tile side T of A's image tiles (local indices < T*(T+1) + 1 < 2^16)
constexpr int kPixTile = 32;        // pixel tile side of A' (the residual windows stay small)
constexpr int kPixCells = 13000;    // most residuals in a tile of A' (NA * W; 52 KB in FP32)
constexpr int kUnitChunks = 128;    // most chunks per work unit (the tile copy is reloaded per unit)
constexpr int kTlThreads = 512;     // threads of a tile CTA

// N with N*N = n, or 0.
int64_t isqrt_exact(int64_t n) {
    int64_t r = (int64_t)std::sqrt((double)n);
    while (r * r > n) --r;
    while ((r + 1) * (r + 1) <= n) ++r;
    return r > 0 && r * r == n ? r : 0;
}

int tl_grid(int64_t work_items) {
    int64_t b = (work_items + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 8;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}

// Where an entry (row, col) falls: its tile, and its index in the tile's
// shared-memory copy of the gathered vector.
//  kind 0 (A, rows = rays, pass 1): the columns are the pixels of an N x N
//         image (col = c*N + r); a tile is T x T pixels and its copy holds the
//         tile's x values with column stride T + 1.
//  kind 1 (A', rows = pixels, pass 2): the rows are the pixels of an N x N
//         image and the columns the rays a*p + b (angle a, bin b); a tile is
//         T x T pixels times a block of NA angles, and its copy holds, for
//         each of those angles, the W residuals from bin bmin[pixel tile,
//         angle] on (W covers every bin the tile's pixels see at one angle).
struct TlGeo {
    int kind = 0;
    int N = 0, T = 0, ntr = 0;                  // image side, tile side, tiles per image column
    int p = 0, nth = 0, NA = 1, nab = 1, W = 0; // kind 1
    const int32_t *bmin = nullptr;              // kind 1: [ntr*ntr*nth]
    __host__ __device__ int cells() const { return kind == 0 ? T * (T + 1) : NA * W; }  // the zero cell
    __host__ __device__ int64_t ntiles() const { return (int64_t)ntr * ntr * (kind == 0 ? 1 : nab); }
    __device__ __forceinline__ int tile(int64_t row, int32_t col) const {
        if (kind == 0) {
            const int c = col / N, r = col - c * N;
            return (c / T) * ntr + r / T;
        }
        const int c = (int)(row / N), r = (int)(row - (int64_t)c * N);
        return ((c / T) * ntr + r / T) * nab + (col / p) / NA;
    }
    __device__ __forceinline__ uint32_t local(int64_t row, int32_t col) const {
        if (kind == 0) {
            const int c = col / N, r = col - c * N;
            return (uint32_t)((c % T) * (T + 1) + r % T);
        }
        const int c = (int)(row / N), r = (int)(row - (int64_t)c * N);
        const int pt = (c / T) * ntr + r / T, a = col / p, b = col - a * p;
        return (uint32_t)((a % NA) * W + (b - bmin[(int64_t)pt * nth + a]));
    }
};

// kind 1: first and last bin each pixel tile sees at each angle (one warp per row).
__global__ void k_tl_bins(const int64_t *rowptr, int32_t m, const int32_t *col, TlGeo G,
                          int32_t *bmin, int32_t *bmax) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = warp; row < m; row += nw) {
        const int c = (int)(row / G.N), r = (int)(row - (int64_t)c * G.N);
        const int64_t pt = (c / G.T) * G.ntr + r / G.T;
        for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += 32) {
            const int a = col[k] / G.p, b = col[k] - a * G.p;
            atomicMin(bmin + pt * G.nth + a, b);
            atomicMax(bmax + pt * G.nth + a, b);
        }
    }
}

// Segments per row (one warp per row): runs of entries in one tile.
__global__ void k_tl_count(const int64_t *rowptr, int32_t m, const int32_t *col, TlGeo G,
                           int32_t *nseg) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = warp; row < m; row += nw) {
        const int64_t s = rowptr[row], e = rowptr[row + 1];
        int carry = -1, count = 0;
        for (int64_t k0 = s; k0 < e; k0 += 32) {
            const int64_t k = k0 + lane;
            const int t = k < e ? G.tile(row, col[k]) : -2;
            int tp = __shfl_up_sync(FULL, t, 1);
            if (lane == 0) tp = carry;
            count += __popc(__ballot_sync(FULL, k < e && t != tp));
            carry = __shfl_sync(FULL, t, 31);
        }
        if (lane == 0) nseg[row] = count;
    }
}

// Segment s of row `row`: tile, first entry, row (segments in row order).
__global__ void k_tl_segs(const int64_t *rowptr, int32_t m, const int32_t *col, TlGeo G,
                          const int64_t *segbase, int32_t *stile, int64_t *sstart, int32_t *srow) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = warp; row < m; row += nw) {
        const int64_t s = rowptr[row], e = rowptr[row + 1];
        int64_t next = segbase[row];
        int carry = -1;
        for (int64_t k0 = s; k0 < e; k0 += 32) {
            const int64_t k = k0 + lane;
            const int t = k < e ? G.tile(row, col[k]) : -2;
            int tp = __shfl_up_sync(FULL, t, 1);
            if (lane == 0) tp = carry;
            const bool head = k < e && t != tp;
            const unsigned hm = __ballot_sync(FULL, head);
            if (head) {
                const int64_t sg = next + __popc(hm & ((1u << lane) - 1u));
                stile[sg] = t;
                sstart[sg] = k;
                srow[sg] = (int32_t)row;
            }
            next += __popc(hm);
            carry = __shfl_sync(FULL, t, 31);
        }
    }
}

// Groups of 4 entries of each segment; sort key = tile, then longest first.
__global__ void k_tl_keys(int64_t nseg, const int64_t *rowptr, const int64_t *segbase,
                          const int32_t *stile, const int64_t *sstart, const int32_t *srow,
                          int LB, int32_t *sglen, int32_t *key, unsigned *kcnt) {
    for (int64_t sg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sg < nseg;
         sg += (int64_t)gridDim.x * blockDim.x) {
        const int32_t row = srow[sg];
        const int64_t end = sg + 1 < segbase[row + 1] ? sstart[sg + 1] : rowptr[row + 1];
        const int64_t g = (end - sstart[sg] + 3) / 4;
        sglen[sg] = (int32_t)g;
        const int k = stile[sg] * LB + (LB - 1 - (int)(g < LB - 1 ? g : LB - 1));
        key[sg] = k;
        atomicAdd(kcnt + k, 1u);
    }
}

__global__ void k_tl_scatter(int64_t nseg, const int32_t *key, unsigned long long *kpos,
                             int32_t *perm) {
    for (int64_t sg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sg < nseg;
         sg += (int64_t)gridDim.x * blockDim.x)
        perm[atomicAdd(kpos + key[sg], 1ull)] = (int32_t)sg;
}

// Slots of each chunk: 32 x its longest segment (groups).
__global__ void k_tl_chunklen(int64_t nchunks, const int2 *chunks, const int32_t *perm,
                              const int32_t *sglen, int32_t *cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nchunks; c += nw) {
        const int2 ch = chunks[c];
        const unsigned g = lane < ch.y ? (unsigned)sglen[perm[ch.x + lane]] : 0u;
        const unsigned mx = __reduce_max_sync(0xffffffffu, g);
        if (lane == 0) cnt[c] = (int32_t)(32 * mx);
    }
}

// Segment of every chunk lane (-1 past the chunk's segments).
__global__ void k_tl_pslot(int64_t nchunks, const int2 *chunks, const int32_t *perm,
                           int32_t *pslot) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nchunks; c += nw) {
        const int2 ch = chunks[c];
        pslot[c * 32 + lane] = lane < ch.y ? perm[ch.x + lane] : -1;
    }
}

// End entry of every segment (the next segment's start, or the row's end).
__global__ void k_tl_ends(int64_t nseg, const int64_t *rowptr, const int64_t *segbase,
                          const int64_t *sstart, const int32_t *srow, int64_t *send) {
    for (int64_t sg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sg < nseg;
         sg += (int64_t)gridDim.x * blockDim.x) {
        const int32_t row = srow[sg];
        send[sg] = sg + 1 < segbase[row + 1] ? sstart[sg + 1] : rowptr[row + 1];
    }
}

// The slots of every chunk (one warp per chunk, lane l = segment pslot[32c+l]):
// slot k of a lane holds entries 4k..4k+3 of its segment. Writes the four
// local indices of each slot (idx, may be null) and the values through `put`
// (entries past the segment: the zero cell, source -1).
template <class Put>
__global__ void k_tl_fill(int64_t nchunks, const int64_t *soff, const int32_t *pslot,
                          const int64_t *sstart, const int64_t *send, const int32_t *srow,
                          const int32_t *col, TlGeo G, uint2 *idx, Put put) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t zero = (uint32_t)G.cells();
    for (int64_t c = warp; c < nchunks; c += nw) {
        const int64_t base = soff[c], len = (soff[c + 1] - base) >> 5;
        const int32_t sg = pslot[c * 32 + lane];
        const int64_t st = sg >= 0 ? sstart[sg] : 0, en = sg >= 0 ? send[sg] : 0;
        const int64_t row = sg >= 0 ? srow[sg] : 0;
        for (int64_t k = 0; k < len; ++k) {
            uint32_t li[4];
            int64_t src[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t e = st + 4 * k + q;
                const bool in = e < en;
                li[q] = in ? G.local(row, col[e]) : zero;
                src[q] = in ? e : -1;
            }
            const int64_t slot = base + 32 * k + lane;
            if (idx) idx[slot] = make_uint2(li[0] | (li[1] << 16), li[2] | (li[3] << 16));
            put(slot, li, src);
        }
    }
}

struct PutNone {
    __device__ void operator()(int64_t, const uint32_t (&)[4], const int64_t (&)[4]) const {}
};
struct Put2B {  // fused record {indices, four 2-byte codes}
    const uint16_t *v;
    uint4 *rec;
    __device__ void operator()(int64_t slot, const uint32_t (&li)[4], const int64_t (&src)[4]) const {
        uint32_t h[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) h[q] = src[q] >= 0 ? v[src[q]] : 0u;
        rec[slot] = make_uint4(li[0] | (li[1] << 16), li[2] | (li[3] << 16), h[0] | (h[1] << 16),
                               h[2] | (h[3] << 16));
    }
};
struct PutF32 {
    const float *v;
    float4 *out;
    __device__ void operator()(int64_t slot, const uint32_t (&)[4], const int64_t (&src)[4]) const {
        out[slot] = make_float4(src[0] >= 0 ? v[src[0]] : 0.f, src[1] >= 0 ? v[src[1]] : 0.f,
                                src[2] >= 0 ? v[src[2]] : 0.f, src[3] >= 0 ? v[src[3]] : 0.f);
    }
};
struct PutF64 {
    const double *v;
    double2 *out;  // two double2 per slot
    __device__ void operator()(int64_t slot, const uint32_t (&)[4], const int64_t (&src)[4]) const {
        out[2 * slot] = make_double2(src[0] >= 0 ? v[src[0]] : 0.0, src[1] >= 0 ? v[src[1]] : 0.0);
        out[2 * slot + 1] = make_double2(src[2] >= 0 ? v[src[2]] : 0.0, src[3] >= 0 ? v[src[3]] : 0.0);
    }
};

// ---- 6-entry step records (2-byte forms) ------------------------------------
// Slot k of a chunk lane holds entries 6k..6k+5 of its segment as six 5-bit
// steps of the tile-local index (the first from the entry before, from the
// segment's first index for k = 0) and six 2-byte values. Inside a tile a ray
// steps by +-1 (along a column) or +-(T+1) (to the next column of the shared
// copy), so the code with S = T + 1 covers every step of a ray matrix.
constexpr int kT6Cand = 3;
struct T6Cands {
    int n = 0;
    int S[kT6Cand] = {};
    int L[kT6Cand] = {};
};

__device__ __forceinline__ void t6_locals(const int32_t *col, int64_t row, int64_t e0, int64_t en,
                                          const TlGeo &G, int (&li)[6]) {
#pragma unroll
    for (int q = 0; q < 6; ++q) li[q] = e0 + q < en ? (int)G.local(row, col[e0 + q]) : (q ? li[q - 1] : 0);
}

// Slots of each chunk: 32 x its longest segment in 6-entry slots.
__global__ void k_t6_len(int64_t nchunks, const int32_t *pslot, const int64_t *sstart,
                         const int64_t *send, int32_t *cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nchunks; c += nw) {
        const int32_t sg = pslot[c * 32 + lane];
        const unsigned g = sg >= 0 ? (unsigned)((send[sg] - sstart[sg] + 5) / 6) : 0u;
        const unsigned mx = __reduce_max_sync(0xffffffffu, g);
        if (lane == 0) cnt[c] = (int32_t)(32 * mx);
    }
}

// Slots whose steps have no code, per candidate (one thread per segment).
__global__ void k_t6_count(int64_t nseg, const int64_t *sstart, const int64_t *send,
                           const int32_t *srow, const int32_t *col, TlGeo G, T6Cands C,
                           unsigned long long *esc) {
    unsigned cnt[kT6Cand] = {0, 0, 0};
    for (int64_t sg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sg < nseg;
         sg += (int64_t)gridDim.x * blockDim.x) {
        const int64_t st = sstart[sg], en = send[sg], row = srow[sg];
        int prev = (int)G.local(row, col[st]);
        for (int64_t e0 = st; e0 < en; e0 += 6) {
            int li[6];
            t6_locals(col, row, e0, en, G, li);
#pragma unroll
            for (int c = 0; c < kT6Cand; ++c) {
                uint32_t w;
                if (c < C.n && !step_word<6, 5>(li, prev, C.S[c], C.L[c], w)) ++cnt[c];
            }
            prev = li[5];
        }
    }
#pragma unroll
    for (int c = 0; c < kT6Cand; ++c)
        if (cnt[c]) atomicAdd(esc + c, (unsigned long long)cnt[c]);
}

// Step words, first indices and side table (one warp per chunk).
__global__ void k_t6_fill(int64_t nchunks, const int64_t *soff6, const int32_t *pslot,
                          const int64_t *sstart, const int64_t *send, const int32_t *srow,
                          const int32_t *col, TlGeo G, int S, int L, uint32_t *code, int32_t *anc,
                          int4 *side, unsigned long long cap, unsigned long long *nesc) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int zero = G.cells();
    for (int64_t c = warp; c < nchunks; c += nw) {
        const int32_t sg = pslot[c * 32 + lane];
        const int64_t st = sg >= 0 ? sstart[sg] : 0, en = sg >= 0 ? send[sg] : 0;
        const int64_t row = sg >= 0 ? srow[sg] : 0;
        const int64_t base = soff6[c], len = (soff6[c + 1] - base) >> 5;
        int prev = en > st ? (int)G.local(row, col[st]) : zero;
        anc[c * 32 + lane] = prev;
        for (int64_t k = 0; k < len; ++k) {
            const int64_t e0 = st + 6 * k;
            uint32_t w = 0;  // past the segment: zero steps
            if (e0 < en) {
                int li[6];
                t6_locals(col, row, e0, en, G, li);
                if (!step_word<6, 5>(li, prev, S, L, w)) {
                    const unsigned long long slot = atomicAdd(nesc, 1ull);
                    if (slot < cap) {
                        side[2 * slot] = make_int4(li[0], li[1], li[2], li[3]);
                        side[2 * slot + 1] = make_int4(li[4], li[5], 0, 0);
                    }
                    w = kStepEsc | (uint32_t)(slot & kStepSlot);
                }
                prev = li[5];
            }
            code[base + 32 * k + lane] = w;
        }
    }
}

// Records {word, six 2-byte codes} of one 2-byte form.
__global__ void k_t6_rec(int64_t nchunks, const int64_t *soff6, const int32_t *pslot,
                         const int64_t *sstart, const int64_t *send, const uint32_t *code,
                         const uint16_t *src, uint4 *rec) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nchunks; c += nw) {
        const int32_t sg = pslot[c * 32 + lane];
        const int64_t st = sg >= 0 ? sstart[sg] : 0, en = sg >= 0 ? send[sg] : 0;
        const int64_t base = soff6[c], len = (soff6[c + 1] - base) >> 5;
        for (int64_t k = 0; k < len; ++k) {
            const int64_t slot = base + 32 * k + lane;
            uint32_t h[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const int64_t j = st + 6 * k + q;
                h[q] = j < en ? src[j] : 0u;
            }
            rec[slot] = make_uint4(code[slot], h[0] | (h[1] << 16), h[2] | (h[3] << 16),
                                   h[4] | (h[5] << 16));
        }
    }
}

// ---- the pass ---------------------------------------------------------------
// Slot loaders: four local indices and four values.
// E entries per slot; State is what a lane carries from slot to slot; CTAS is
// the number of 512-thread CTAs per SM the pass is compiled for (its register
// budget: 4 -> 32 registers, 3 -> 40, 2 -> 64). Measured at N = 1024: 3 for the
// 2-byte forms and FP32 (FP32 pass 2 0.90 ms against 1.03 ms with 4; 2 is 20%
// slower), 2 for FP64 (64 registers, no spills at D = 2).
template <typename VT> struct TlFused {
    static constexpr int E = 4;
    static constexpr int CTAS = 3;
    const uint4 *rec;
    using Raw = uint4;
    struct State {};
    __device__ __forceinline__ State init(int64_t) const { return {}; }
    __device__ __forceinline__ Raw load(int64_t j) const { return ld_stream(rec + j); }
    __device__ __forceinline__ static Raw none() { return make_uint4(0u, 0u, 0u, 0u); }
    __device__ __forceinline__ void open(const Raw &r, State &, uint32_t (&li)[4], float (&v)[4]) const {
        li[0] = r.x & 0xFFFFu; li[1] = r.x >> 16; li[2] = r.y & 0xFFFFu; li[3] = r.y >> 16;
        Conv2B<VT>::to(r.z, r.w, v);
    }
};
// LB: bits of a code's low field (the copy's L6: 2, 3 or 5), a compile-time
// constant so that the decode's shifts are immediates.
template <typename VT, int LB> struct TlStep6 {  // 6-entry step records
    static constexpr int E = 6;
    static constexpr int CTAS = 3;
    const uint4 *rec;
    const int32_t *anc;
    const int4 *side;
    int hm;  // the high field's step S
    using Raw = uint4;
    struct State {
        int li;  // the lane's last local index
    };
    TlStep6(const uint4 *r, const int32_t *a, const int4 *sd, int S) : rec(r), anc(a), side(sd), hm(S) {}
    // the step of code q of word w: step_decode<5>((w >> 5q) & 31, S, LB) by
    // shifts alone (the signed low LB bits, the signed high 5 - LB bits)
    __device__ __forceinline__ int step(uint32_t w, int q) const {
        const int lo = (int)(w << (32 - LB - 5 * q)) >> (32 - LB);
        if constexpr (LB >= 5) {
            return lo;
        } else {
            const int hi = (int)(w << (27 - 5 * q)) >> (27 + LB);
            return lo + hi * hm;
        }
    }
    __device__ __forceinline__ State init(int64_t lanepos) const { return {__ldg(anc + lanepos)}; }
    __device__ __forceinline__ Raw load(int64_t j) const { return ld_stream(rec + j); }
    __device__ __forceinline__ static Raw none() { return make_uint4(0u, 0u, 0u, 0u); }
    __device__ __forceinline__ void open(const Raw &r, State &st, uint32_t (&li)[6], float (&v)[6]) const {
        const uint32_t w = r.x;
        if (w & kStepEsc) {
            const int4 a = __ldg(side + 2 * (int64_t)(w & kStepSlot));
            const int4 b = __ldg(side + 2 * (int64_t)(w & kStepSlot) + 1);
            li[0] = a.x; li[1] = a.y; li[2] = a.z; li[3] = a.w; li[4] = b.x; li[5] = b.y;
        } else {
            int d[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) d[q] = step(w, q);
            // running sums in a tree of depth 3 instead of a chain of 6
            const int s01 = d[0] + d[1], s23 = d[2] + d[3], s45 = d[4] + d[5];
            const int b1 = st.li + s01, b3 = b1 + s23;
            li[0] = (uint32_t)(st.li + d[0]);
            li[1] = (uint32_t)b1;
            li[2] = (uint32_t)(b1 + d[2]);
            li[3] = (uint32_t)b3;
            li[4] = (uint32_t)(b3 + d[4]);
            li[5] = (uint32_t)(b3 + s45);
        }
        st.li = (int)li[5];
        Conv2B<VT>::two(r.y, v[0], v[1]);
        Conv2B<VT>::two(r.z, v[2], v[3]);
        Conv2B<VT>::two(r.w, v[4], v[5]);
    }
};
template <typename VT> struct TlSplit {
    static constexpr int E = 4;
    static constexpr int CTAS = sizeof(VT) == 8 ? 2 : 3;
    const uint2 *idx;
    const VT *val;
    struct State {};
    __device__ __forceinline__ State init(int64_t) const { return {}; }
    struct Raw {
        uint2 w;
        VBlk<VT> v;
    };
    __device__ __forceinline__ Raw load(int64_t j) const {
        Raw r;
        r.w = ld_stream(idx + j);
        r.v.ld(val + 4 * j);
        return r;
    }
    __device__ __forceinline__ static Raw none() {
        Raw r;
        r.w = make_uint2(0u, 0u);
        r.v.clear();
        return r;
    }
    __device__ __forceinline__ void open(const Raw &r, State &, uint32_t (&li)[4], VT (&v)[4]) const {
        li[0] = r.w.x & 0xFFFFu; li[1] = r.w.x >> 16; li[2] = r.w.y & 0xFFFFu; li[3] = r.w.y >> 16;
        r.v.to(v);
    }
};

struct TlArgs {
    const int64_t *soff;
    const int32_t *pslot;
    const int4 *units;
    int32_t nunits;
    TlGeo G;
};

// One element from global to shared memory as an asynchronous copy (4 or 8
// bytes, `cp.async.ca`): a thread issues all its copies of a tile before any
// of them has to arrive, and waits once (cp_async_wait_all).
template <typename XT>
__device__ __forceinline__ void cp_async_elem(XT *dst, const XT *src) {
    static_assert(sizeof(XT) == 4 || sizeof(XT) == 8, "4- or 8-byte elements");
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(XT) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// The shared copy of unit U's tile of the gathered vector x (all threads of
// the CTA), zero cell included. Cells inside the image / sinogram arrive by
// asynchronous copies, the rest are stored as zeros; the caller's barrier
// follows each thread's cp_async_wait_all.
template <typename XT>
__device__ __forceinline__ void tl_fill_tile(const TlGeo &G, int4 U, const XT *__restrict__ x, XT *xs) {
    if (G.kind == 0) {  // the T x T pixels of the tile, column stride T + 1: a warp per
                        // column, its lanes along the column's T pixels (contiguous in x)
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        const int T = G.T, N = G.N;
        const int tc = U.x / G.ntr, tr = U.x - tc * G.ntr;
        for (int lc = wid; lc < T; lc += nw) {
            const int gc = tc * T + lc;
            XT *dst = xs + lc * (T + 1);
            for (int lr = lane; lr < T; lr += 32) {
                const int gr = tr * T + lr;
                if (gc < N && gr < N) cp_async_elem(dst + lr, x + (int64_t)gc * N + gr);
                else dst[lr] = (XT)0;
            }
        }
    } else {  // W bins per angle of the tile's angle block, one cell per thread in
              // turn (W is about 1.5 warps wide: a warp per angle would idle lanes);
              // the cell's angle and bin carried from step to step (no division)
        const int pt = U.x / G.nab, a0 = (U.x - pt * G.nab) * G.NA;
        const int W = G.W, dai = (int)blockDim.x / W, dr = (int)blockDim.x - dai * W;
        int ai = (int)threadIdx.x / W, r = (int)threadIdx.x - ai * W;
        for (int e = threadIdx.x; e < G.NA * W; e += blockDim.x) {
            const int a = a0 + ai;
            bool in = false;
            int b = 0;
            if (a < G.nth) {
                b = __ldg(G.bmin + (int64_t)pt * G.nth + a) + r;
                in = b < G.p;
            }
            if (in) cp_async_elem(xs + e, x + (int64_t)a * G.p + b);
            else xs[e] = (XT)0;
            ai += dai;
            r += dr;
            if (r >= W) {
                r -= W;
                ++ai;
            }
        }
    }
    if (threadIdx.x == 0) xs[G.cells()] = (XT)0;  // the zero cell of padding entries
    cp_async_wait_all();
}

// A segment's partial from its independent sums (one per ring slot), added
// in a fixed order: (k0 + k1) + (k2 + k3).
template <typename ACC, int K>
__device__ __forceinline__ ACC chain_sum(const ACC (&a)[K]) {
    ACC k[K];
#pragma unroll
    for (int i = 0; i < K; ++i) k[i] = a[i];
#pragma unroll
    for (int w = 1; w < K; w *= 2)
#pragma unroll
        for (int i = 0; i + w < K; i += 2 * w) k[i] += k[i + w];
    return k[0];
}

// The partial sums of warp `wid`'s chunks of work unit U, W warps sharing the
// unit (D = 2 slots in flight), the tile's copy of the gathered vector in xs.
template <class LD, typename XT, typename ACC>
__device__ __forceinline__ void tl_stream_chunks(const TlArgs &P, const LD &ldr, int4 U,
                                                 const XT *__restrict__ xs, ACC *__restrict__ part,
                                                 int W, int wid) {
    constexpr int E = LD::E;
    // independent sums: one per ring slot in the FP32 forms, one in FP64
    constexpr int KC = sizeof(ACC) == 8 ? 1 : 2;
    const int lane = threadIdx.x & 31;
    // the warp's chunks of the unit, one per group of W consecutive
    // chunks, in snake order (w in even groups, W - 1 - w in odd ones:
    // the chunks of a tile are sorted longest first, so the warps' sums
    // of lengths balance), as one stream of slots: the loads of the
    // next chunks' first slots start during the current chunk. With 2
    // slots in flight the window reaches at most one slot past the
    // current chunk: into the next chunk, or, when that chunk has a
    // single slot, into the first slot of the chunk after it (every
    // chunk has at least one slot).
    struct Meta {
        int64_t s0;
        int len, ps;
        typename LD::State st;
    };
    auto meta = [&](int c) -> Meta {
        Meta r{0, 0, -1, typename LD::State{}};
        if (c < U.z) {
            const int64_t o0 = __ldg(P.soff + c);
            r.s0 = o0 + lane;
            r.len = (int)((__ldg(P.soff + c + 1) - o0) >> 5);
            r.ps = __ldg(P.pslot + (int64_t)c * 32 + lane);
            r.st = ldr.init((int64_t)c * 32 + lane);
        }
        return r;
    };
    // chunk of group g (past the unit's end once one is: later groups
    // start after every chunk of group g)
    auto chunk_of = [&](int g) { return U.y + W * g + ((g & 1) ? W - 1 - wid : wid); };
    int g = 0, c = chunk_of(0);
    Meta cur = meta(c), nxt = meta(chunk_of(1));
    // slot q of the stream that starts at chunk c = chunk_of(g) (q <=
    // cur.len + 1); the chunk after nxt is looked up only when the
    // window reaches it (a 1-slot nxt: the tiles' shortest segments)
    auto fetch = [&](int q) {
        if (q < cur.len) return ldr.load(cur.s0 + 32 * (int64_t)q);
        q -= cur.len;
        if (q < nxt.len) return ldr.load(nxt.s0 + 32 * (int64_t)q);
        const int c2 = chunk_of(g + 2);
        return q == nxt.len && c2 < U.z ? ldr.load(__ldg(P.soff + c2) + lane) : LD::none();
    };
    typename LD::Raw ring[2] = {fetch(0), fetch(1)};
    while (c < U.z) {
        ACC acc[KC] = {};
        int t = 0;
        for (; t + 2 <= cur.len; t += 2) {  // slot pairs: both slots' work interleaves
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const typename LD::Raw r = ring[k];
                ring[k] = fetch(t + k + 2);
                uint32_t li[E];
                ACC v[E];
                ldr.open(r, cur.st, li, v);
#pragma unroll
                for (int q = 0; q < E; ++q) acc[k % KC] += (ACC)xs[li[q]] * v[q];
            }
        }
        if (t < cur.len) {  // an odd last slot, in ring[0]
            const typename LD::Raw r = ring[0];
            ring[0] = fetch(t + 2);
            uint32_t li[E];
            ACC v[E];
            ldr.open(r, cur.st, li, v);
#pragma unroll
            for (int q = 0; q < E; ++q) acc[0] += (ACC)xs[li[q]] * v[q];
            // the next chunk's slot 0 now sits in ring[1]
            const typename LD::Raw tmp = ring[0];
            ring[0] = ring[1];
            ring[1] = tmp;
        }
        if (cur.ps >= 0) part[cur.ps] = chain_sum<ACC, KC>(acc);
        ++g;
        c = chunk_of(g);
        cur = nxt;
        nxt = meta(chunk_of(g + 1));
    }
}

// Partial sums of all segments. Persistent CTAs take work units through
// ctr[0] (reset by the last CTA through ctr[1] for the next launch).
// One work unit U (a tile and a range of its chunks) by the whole CTA: the
// tile's shared copy, then the partial sums of the unit's segments; ends with
// a barrier (the tile is rewritten by the next unit).
template <class LD, typename XT, typename ACC, int D, bool CONT>
__device__ __forceinline__ void tl_unit(const TlArgs &P, const LD &ldr, const XT *__restrict__ x,
                                        ACC *__restrict__ part, int4 U, XT *xs, int &s_chunk) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int E = LD::E;
    // independent sums: one per ring slot in the FP32 forms, one in FP64 (whose
    // pass is bound by the FP64 pipe and keeps its registers for a second CTA
    // per SM)
    constexpr int KD = sizeof(ACC) == 8 ? 1 : D;
    const int lane = threadIdx.x & 31;
    {
        tl_fill_tile(P.G, U, x, xs);
        if (threadIdx.x == 0) s_chunk = U.y;
        __syncthreads();
        if constexpr (CONT) {
            static_assert(D == 2, "the continuous stream keeps 2 slots in flight");
            tl_stream_chunks<LD, XT, ACC>(P, ldr, U, xs, part, blockDim.x >> 5, (int)(threadIdx.x >> 5));
        } else {
            for (;;) {
                int c = 0;
                if (lane == 0) c = atomicAdd(&s_chunk, 1);
                c = __shfl_sync(FULL, c, 0);
                if (c >= U.z) break;
                const int64_t o0 = __ldg(P.soff + c);
                const int len = (int)((__ldg(P.soff + c + 1) - o0) >> 5);
                const int64_t s0 = o0 + lane;
                typename LD::Raw ring[D];
#pragma unroll
                for (int k = 0; k < D; ++k) ring[k] = k < len ? ldr.load(s0 + 32 * k) : LD::none();
                typename LD::State lst = ldr.init((int64_t)c * 32 + lane);
                ACC acc[KD] = {};
                for (int t0 = 0; t0 < len; t0 += D) {
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const int t = t0 + k;
                        if (t >= len) break;
                        const typename LD::Raw r = ring[k];
                        ring[k] = t + D < len ? ldr.load(s0 + 32 * (int64_t)(t + D)) : LD::none();
                        uint32_t li[E];
                        ACC v[E];
                        ldr.open(r, lst, li, v);
#pragma unroll
                        for (int q = 0; q < E; ++q) acc[k % KD] += (ACC)xs[li[q]] * v[q];
                    }
                }
                const int ps = __ldg(P.pslot + (int64_t)c * 32 + lane);
                if (ps >= 0) part[ps] = chain_sum<ACC, KD>(acc);
            }
        }
        __syncthreads();  // the tile is rewritten by the next unit
    }
}

template <class LD, typename XT, typename ACC, int D, bool CONT>
__global__ void __launch_bounds__(kTlThreads, LD::CTAS) k_tl_partials(TlArgs P, LD ldr,
                                                            const XT *__restrict__ x,
                                                            ACC *__restrict__ part, unsigned *ctr) {
    extern __shared__ __align__(16) unsigned char tl_smem[];
    XT *xs = reinterpret_cast<XT *>(tl_smem);
    __shared__ int s_unit, s_chunk;
    for (;;) {
        if (threadIdx.x == 0) s_unit = (int)atomicAdd(ctr, 1u);
        __syncthreads();
        const int u = s_unit;
        if (u >= P.nunits) break;
        tl_unit<LD, XT, ACC, D, CONT>(P, ldr, x, part, P.units[u], xs, s_chunk);
    }
    if (threadIdx.x == 0) {
        const unsigned done = atomicAdd(ctr + 1, 1u);
        if (done == gridDim.x - 1) {  // every CTA has stopped taking units
            ctr[0] = 0u;
            ctr[1] = 0u;
        }
    }
}

// Row sums of the partials (in row order) and the residual epilogue.
template <typename ACC, class Epi>
__global__ void k_tl_rows(int32_t m, const int64_t *__restrict__ segbase,
                          const ACC *__restrict__ part, Epi epi) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x) {
        ACC acc = 0;
        for (int64_t k = segbase[i]; k < segbase[i + 1]; ++k) acc += part[k];
        epi(i, acc);
    }
}

TlGeo tl_geo(const DevCSR::Tiled &tl) {
    TlGeo G;
    G.kind = tl.kind;
    G.N = tl.N;
    G.T = tl.T;
    G.ntr = tl.ntr;
    G.p = tl.p;
    G.nth = tl.nth;
    G.NA = tl.NA;
    G.nab = tl.nab;
    G.W = tl.W;
    G.bmin = tl.bmin.as<int32_t>();
    return G;
}

// Raise a kernel's dynamic shared-memory limit to `bytes` if it is lower
// (never lowers it: the tiled copies of A and A' launch the same kernels with
// tiles of different sizes).
cudaError_t smem_allow(const void *kernel, size_t bytes) {
    static std::mutex mu;
    static std::vector<std::pair<const void *, size_t>> set;
    std::lock_guard<std::mutex> lock(mu);
    for (auto &k : set)
        if (k.first == kernel) {
            if (bytes <= k.second) return cudaSuccess;
            const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            if (e == cudaSuccess) k.second = bytes;
            return e;
        }
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) set.emplace_back(kernel, bytes);
    return e;
}

// Launches one pass on the tiled copy (partials, then row sums); errors are
// left for the caller's cudaGetLastError.
template <class LD, typename XT, typename ACC, class Epi>
void launch_tl(const DevCSR &M, int code, const LD &ldr, const XT *x, const Epi &e,
               unsigned *ctr, cudaStream_t s) {
    const DevCSR::Tiled &tl = M.tl;
    const DevBuf &soff = LD::E == 6 ? tl.soff6 : tl.soff;
    const TlGeo G = tl_geo(tl);
    const TlArgs P{soff.as<int64_t>(), tl.pslot.as<int32_t>(), tl.units.as<int4>(), tl.nunits,
                   G};
    const size_t smem = sizeof(XT) * ((size_t)G.cells() + 1);
    ACC *part = tl.part.as<ACC>();
    auto run = [&](auto kernel) -> cudaError_t {
        const cudaError_t e = smem_allow(reinterpret_cast<const void *>(kernel), smem);
        if (e != cudaSuccess) return e;
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kTlThreads, smem);
        const int grid = std::max(1, std::min(sm_count() * std::max(occ, 1), (int)tl.nunits));
        kernel<<<grid, kTlThreads, smem, s>>>(P, ldr, x, part, ctr);
        return cudaPeekAtLastError();
    };
    const cudaError_t err = code == 10 ? run(k_tl_partials<LD, XT, ACC, 4, false>)
                                       : run(k_tl_partials<LD, XT, ACC, 2, true>);
    // the row sums only after partials that were launched; a failure stays
    // the runtime's last error, which the caller's check reports
    if (err == cudaSuccess)
        k_tl_rows<ACC, Epi><<<tl_grid(M.m), 256, 0, s>>>(M.m, tl.segbase.as<int64_t>(), part, e);
}

// Index part of the 6-entry step records (after the tiled copy is built).
int t6_build(DevCSR &A, cudaStream_t s) {
    DevCSR::Tiled &tl = A.tl;
    const int64_t nch = tl.nchunks;
    TmpBuf cnt, esc;
    FAIR_TRY(cnt.grow(sizeof(int32_t) * (nch + 1)));
    FAIR_TRY(tl.soff6.grow(sizeof(int64_t) * (nch + 1)));
    k_t6_len<<<tl_grid(nch * 32), 256, 0, s>>>(nch, tl.pslot.as<int32_t>(), tl.sstart.as<int64_t>(),
                                                tl.send.as<int64_t>(), cnt.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    FAIR_TRY(scan_counts(cnt.as<int32_t>(), nch, tl.soff6.as<int64_t>(), s));
    T6Cands C;
    const TlGeo G = tl_geo(tl);
    const int S6 = G.kind == 0 ? tl.T + 1 : tl.W;  // a step to the next column / angle of the copy
    C.S[0] = S6; C.L[0] = 2;
    C.S[1] = S6; C.L[1] = 3;
    C.S[2] = 0; C.L[2] = 5;
    C.n = 3;
    FAIR_TRY(esc.grow(sizeof(unsigned long long) * (kT6Cand + 1)));
    FAIR_CUDA(cudaMemsetAsync(esc.p, 0, sizeof(unsigned long long) * (kT6Cand + 1), s));
    k_t6_count<<<tl_grid(tl.nseg), 256, 0, s>>>(tl.nseg, tl.sstart.as<int64_t>(), tl.send.as<int64_t>(),
                                                  tl.srow.as<int32_t>(), A.col.as<int32_t>(), G, C,
                                                  esc.as<unsigned long long>());
    FAIR_CUDA(cudaGetLastError());
    unsigned long long hesc[kT6Cand] = {};
    FAIR_CUDA(cudaMemcpyAsync(hesc, esc.p, sizeof(hesc), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaMemcpyAsync(&tl.nslots6, tl.soff6.as<int64_t>() + nch, sizeof(int64_t),
                              cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    int best = 0;
    for (int c = 1; c < C.n; ++c)
        if (hesc[c] < hesc[best]) best = c;
    // too many slots without codes: the side-table reads would cost more than the codes save
    if (hesc[best] > (unsigned long long)(A.nnz / 6 / 8) || hesc[best] > kStepSlot) {
        tl.soff6.release();
        return FAIR_OK;
    }
    const size_t ns = (size_t)std::max<int64_t>(tl.nslots6, 1);
    FAIR_TRY(tl.code6.grow(sizeof(uint32_t) * ns));
    FAIR_TRY(tl.anc6.grow(sizeof(int32_t) * 32 * (size_t)std::max<int64_t>(nch, 1)));
    FAIR_TRY(tl.side6.grow(sizeof(int4) * 2 * (size_t)std::max<unsigned long long>(hesc[best], 1)));
    unsigned long long *ctr = esc.as<unsigned long long>() + kT6Cand;
    k_t6_fill<<<tl_grid(nch * 32), 256, 0, s>>>(
        nch, tl.soff6.as<int64_t>(), tl.pslot.as<int32_t>(), tl.sstart.as<int64_t>(),
        tl.send.as<int64_t>(), tl.srow.as<int32_t>(), A.col.as<int32_t>(), G, C.S[best], C.L[best],
        tl.code6.as<uint32_t>(), tl.anc6.as<int32_t>(), tl.side6.as<int4>(), hesc[best], ctr);
    FAIR_CUDA(cudaGetLastError());
    unsigned long long used = 0;
    FAIR_CUDA(cudaMemcpyAsync(&used, ctr, sizeof(used), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    if (used != hesc[best]) {  // the fill must meet exactly the slots the count found
        set_detail("tiled step records: side-table count mismatch");
        return FAIR_ERR_STATE;
    }
    tl.S6 = C.S[best];
    tl.L6 = C.L[best];
    tl.nesc6 = (int64_t)hesc[best];
    tl.built6 = true;
    return FAIR_OK;
}

}  // namespace

void tiled_shape(const DevCSR &M, int pass, int *side, int *cells) {
    const int dflt = pass == 1 ? kTile : kPixTile;
    *side = M.tile_req[0] > 0 ? M.tile_req[0] : dflt;
    *cells = pass == 1 ? 0 : (M.tile_req[1] > 0 ? M.tile_req[1] : kPixCells);
}

int csr_make_tiled(DevCSR &A, int prec, int pass, cudaStream_t s) {
    if (A.m == 0 || A.nnz == 0) return FAIR_OK;
    DevCSR::Tiled &tl = A.tl;
    const int kind = pass == 1 ? 0 : 1;
    int want_T = 0, want_cells = 0;
    tiled_shape(A, pass, &want_T, &want_cells);
    if (tl.built() && (tl.kind != kind || tl.T != want_T || (kind == 1 && tl.cells_cap != want_cells)))
        tl.release();
    if (!tl.built()) {
        TlGeo G;
        G.kind = kind;
        if (kind == 0) {
            const int64_t N = isqrt_exact(A.n);
            if (N <= 0) return FAIR_OK;  // the columns are not an image of N x N pixels
            G.N = (int)N;
            G.T = want_T;
            G.ntr = (int)((N + want_T - 1) / want_T);
        } else {
            const int64_t N = isqrt_exact(A.m);
            const int p = A.stride_hint;
            // the rows are not an N x N image, or the columns not rays of p bins per angle
            if (N <= 0 || p <= 0 || A.n % p != 0) return FAIR_OK;
            G.N = (int)N;
            G.T = want_T;
            G.ntr = (int)((N + want_T - 1) / want_T);
            G.p = p;
            G.nth = A.n / p;
            // the bins each pixel tile sees at each angle
            const size_t nb = (size_t)G.ntr * G.ntr * G.nth;
            TmpBuf bmax;
            FAIR_TRY(tl.bmin.grow(sizeof(int32_t) * nb));
            FAIR_TRY(bmax.grow(sizeof(int32_t) * nb));
            FAIR_CUDA(cudaMemsetAsync(tl.bmin.p, 0x7F, sizeof(int32_t) * nb, s));
            FAIR_CUDA(cudaMemsetAsync(bmax.p, 0xFF, sizeof(int32_t) * nb, s));
            k_tl_bins<<<tl_grid((int64_t)A.m * 32), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m,
                                                                 A.col.as<int32_t>(), G,
                                                                 tl.bmin.as<int32_t>(), bmax.as<int32_t>());
            FAIR_CUDA(cudaGetLastError());
            std::vector<int32_t> lo(nb), hi(nb);
            FAIR_CUDA(cudaMemcpyAsync(lo.data(), tl.bmin.p, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, s));
            FAIR_CUDA(cudaMemcpyAsync(hi.data(), bmax.p, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, s));
            FAIR_CUDA(cudaStreamSynchronize(s));
            int W = 0;
            for (size_t i = 0; i < nb; ++i) {
                if (hi[i] < 0) lo[i] = 0;  // no ray of the tile at this angle
                else W = std::max(W, hi[i] - lo[i] + 1);
            }
            if (W <= 0 || W > want_cells) { tl.release(); return FAIR_OK; }
            FAIR_CUDA(cudaMemcpyAsync(tl.bmin.p, lo.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice, s));
            FAIR_CUDA(cudaStreamSynchronize(s));
            G.W = W;
            G.NA = std::max(1, std::min(G.nth, want_cells / W));
            G.nab = (G.nth + G.NA - 1) / G.NA;
            G.bmin = tl.bmin.as<int32_t>();
        }
        const int T = G.T;
        const int64_t ntiles = G.ntiles();
        // length classes of the sort: a ray crosses T x T pixels in up to 2T entries; a
        // pixel sees up to ~3 rays per angle
        const int LB = (kind == 0 ? T / 2 : G.NA) + 2;
        if (ntiles * LB >= (int64_t(1) << 31)) { tl.release(); return FAIR_OK; }
        // segments
        TmpBuf nseg;
        FAIR_TRY(nseg.grow(sizeof(int32_t) * ((size_t)A.m + 1)));
        FAIR_TRY(tl.segbase.grow(sizeof(int64_t) * ((size_t)A.m + 1)));
        k_tl_count<<<tl_grid((int64_t)A.m * 32), 256, 0, s>>>(A.rowptr.as<int64_t>(), A.m,
                                                              A.col.as<int32_t>(), G, nseg.as<int32_t>());
        FAIR_CUDA(cudaGetLastError());
        FAIR_TRY(scan_counts(nseg.as<int32_t>(), A.m, tl.segbase.as<int64_t>(), s));
        int64_t S = 0;
        FAIR_CUDA(cudaMemcpyAsync(&S, tl.segbase.as<int64_t>() + A.m, sizeof(S),
                                  cudaMemcpyDeviceToHost, s));
        FAIR_CUDA(cudaStreamSynchronize(s));
        if (S <= 0 || S >= (int64_t(1) << 31)) { tl.release(); return FAIR_OK; }
        TmpBuf stile, sstart, sglen, key, kcnt, kpos, perm;
        DevBuf &srow = tl.srow;
        FAIR_TRY(stile.grow(sizeof(int32_t) * S));
        FAIR_TRY(sstart.grow(sizeof(int64_t) * S));
        FAIR_TRY(srow.grow(sizeof(int32_t) * S));
        FAIR_TRY(sglen.grow(sizeof(int32_t) * S));
        FAIR_TRY(key.grow(sizeof(int32_t) * S));
        FAIR_TRY(perm.grow(sizeof(int32_t) * S));
        const int64_t nkeys = ntiles * LB;
        FAIR_TRY(kcnt.grow(sizeof(unsigned) * (nkeys + 1)));
        FAIR_TRY(kpos.grow(sizeof(unsigned long long) * (nkeys + 1)));
        FAIR_CUDA(cudaMemsetAsync(kcnt.p, 0, sizeof(unsigned) * (nkeys + 1), s));
        k_tl_segs<<<tl_grid((int64_t)A.m * 32), 256, 0, s>>>(
            A.rowptr.as<int64_t>(), A.m, A.col.as<int32_t>(), G, tl.segbase.as<int64_t>(),
            stile.as<int32_t>(), sstart.as<int64_t>(), srow.as<int32_t>());
        k_tl_keys<<<tl_grid(S), 256, 0, s>>>(S, A.rowptr.as<int64_t>(), tl.segbase.as<int64_t>(),
                                              stile.as<int32_t>(), sstart.as<int64_t>(),
                                              srow.as<int32_t>(), LB, sglen.as<int32_t>(),
                                              key.as<int32_t>(), kcnt.as<unsigned>());
        FAIR_CUDA(cudaGetLastError());
        // bucket offsets on the host (ntiles * LB counters)
        std::vector<unsigned> hc((size_t)nkeys);
        FAIR_CUDA(cudaMemcpyAsync(hc.data(), kcnt.p, sizeof(unsigned) * nkeys,
                                  cudaMemcpyDeviceToHost, s));
        FAIR_CUDA(cudaStreamSynchronize(s));
        std::vector<unsigned long long> ho((size_t)nkeys + 1, 0ull);
        for (int64_t k = 0; k < nkeys; ++k) ho[k + 1] = ho[k] + hc[k];
        // a tile's segments longest first (chunks of similar lengths)
        FAIR_CUDA(cudaMemcpyAsync(kpos.p, ho.data(), sizeof(unsigned long long) * nkeys,
                                  cudaMemcpyHostToDevice, s));
        k_tl_scatter<<<tl_grid(S), 256, 0, s>>>(S, key.as<int32_t>(), kpos.as<unsigned long long>(),
                                                 perm.as<int32_t>());
        FAIR_CUDA(cudaGetLastError());
        // chunks of 32 segments per tile; units of up to kUnitChunks chunks,
        // fewer when that leaves under a dozen units per SM to balance
        std::vector<int2> chunks;
        std::vector<int4> units;
        for (int64_t t = 0; t < ntiles; ++t) {
            const int64_t a = (int64_t)ho[t * LB], b = (int64_t)ho[(t + 1) * LB];
            for (int64_t p = a; p < b; p += 32)
                chunks.push_back(make_int2((int)p, (int)std::min<int64_t>(32, b - p)));
        }
        const int64_t per_unit = std::max<int64_t>(
            8, std::min<int64_t>(kUnitChunks, (int64_t)chunks.size() / ((int64_t)sm_count() * 12)));
        for (int64_t t = 0, c0 = 0; t < ntiles; ++t) {
            const int64_t c1 = c0 + ((int64_t)ho[(t + 1) * LB] - (int64_t)ho[t * LB] + 31) / 32;
            for (int64_t c = c0; c < c1; c += per_unit)
                units.push_back(make_int4((int)t, (int)c, (int)std::min<int64_t>(c + per_unit, c1), 0));
            c0 = c1;
        }
        // most work first: units of longer segments lead within a tile already
        const int64_t nch = (int64_t)chunks.size();
        TmpBuf dch, ccnt;
        FAIR_TRY(dch.grow(sizeof(int2) * std::max<int64_t>(nch, 1)));
        FAIR_TRY(ccnt.grow(sizeof(int32_t) * (nch + 1)));
        FAIR_TRY(tl.soff.grow(sizeof(int64_t) * (nch + 1)));
        FAIR_TRY(tl.pslot.grow(sizeof(int32_t) * 32 * std::max<int64_t>(nch, 1)));
        FAIR_TRY(tl.units.grow(sizeof(int4) * std::max<size_t>(units.size(), 1)));
        FAIR_CUDA(cudaMemcpyAsync(dch.p, chunks.data(), sizeof(int2) * nch, cudaMemcpyHostToDevice, s));
        FAIR_CUDA(cudaMemcpyAsync(tl.units.p, units.data(), sizeof(int4) * units.size(),
                                  cudaMemcpyHostToDevice, s));
        k_tl_chunklen<<<tl_grid(nch * 32), 256, 0, s>>>(nch, dch.as<int2>(), perm.as<int32_t>(),
                                                         sglen.as<int32_t>(), ccnt.as<int32_t>());
        FAIR_CUDA(cudaGetLastError());
        FAIR_TRY(scan_counts(ccnt.as<int32_t>(), nch, tl.soff.as<int64_t>(), s));
        int64_t nslots = 0;
        FAIR_CUDA(cudaMemcpyAsync(&nslots, tl.soff.as<int64_t>() + nch, sizeof(nslots),
                                  cudaMemcpyDeviceToHost, s));
        FAIR_CUDA(cudaStreamSynchronize(s));
        FAIR_TRY(tl.sstart.grow(sizeof(int64_t) * S));
        FAIR_TRY(tl.send.grow(sizeof(int64_t) * S));
        FAIR_CUDA(cudaMemcpyAsync(tl.sstart.p, sstart.p, sizeof(int64_t) * S,
                                  cudaMemcpyDeviceToDevice, s));
        k_tl_ends<<<tl_grid(S), 256, 0, s>>>(S, A.rowptr.as<int64_t>(), tl.segbase.as<int64_t>(),
                                              sstart.as<int64_t>(), srow.as<int32_t>(),
                                              tl.send.as<int64_t>());
        k_tl_pslot<<<tl_grid(nch * 32), 256, 0, s>>>(nch, dch.as<int2>(), perm.as<int32_t>(),
                                                      tl.pslot.as<int32_t>());
        FAIR_CUDA(cudaGetLastError());
        // index words (read by the FP32 and FP64 forms)
        FAIR_TRY(tl.idx.grow(sizeof(uint2) * std::max<int64_t>(nslots, 1)));
        k_tl_fill<PutNone><<<tl_grid(nch * 32), 256, 0, s>>>(
            nch, tl.soff.as<int64_t>(), tl.pslot.as<int32_t>(), tl.sstart.as<int64_t>(),
            tl.send.as<int64_t>(), tl.srow.as<int32_t>(), A.col.as<int32_t>(), G, tl.idx.as<uint2>(),
            PutNone{});
        FAIR_CUDA(cudaGetLastError());
        FAIR_TRY(tl.part.grow(sizeof(double) * S));
        tl.kind = G.kind;
        tl.T = G.T;
        tl.N = G.N;
        tl.ntr = G.ntr;
        tl.p = G.p;
        tl.nth = G.nth;
        tl.NA = G.NA;
        tl.nab = G.nab;
        tl.W = G.W;
        tl.cells_cap = want_cells;
        tl.nseg = S;
        tl.nchunks = nch;
        tl.nslots = nslots;
        tl.nunits = (int32_t)units.size();
        tl.has_idx = true;
        FAIR_CUDA(cudaStreamSynchronize(s));  // before the scratch buffers go
    }
    // the values of the form, slot by slot
    const TlGeo G = tl_geo(tl);
    const int64_t nch = tl.nchunks;
    const int grid = tl_grid(nch * 32);
    const int64_t *soff = tl.soff.as<int64_t>(), *st = tl.sstart.as<int64_t>(), *en = tl.send.as<int64_t>();
    const int32_t *ps = tl.pslot.as<int32_t>(), *col = A.col.as<int32_t>();
    const size_t ns = (size_t)std::max<int64_t>(tl.nslots, 1);
    if (prec == FAIR_PREC_F64 && !tl.has_v64) {
        FAIR_TRY(tl.v64.grow(sizeof(double) * 4 * ns));
        k_tl_fill<PutF64><<<grid, 256, 0, s>>>(nch, soff, ps, st, en, tl.srow.as<int32_t>(), col, G, nullptr,
                                                PutF64{A.v64.as<double>(), tl.v64.as<double2>()});
        tl.has_v64 = true;
    } else if (prec == FAIR_PREC_F32 && !tl.has_v32) {
        FAIR_TRY(csr_make_lowprec(A, prec, s));
        FAIR_TRY(tl.v32.grow(sizeof(float) * 4 * ns));
        k_tl_fill<PutF32><<<grid, 256, 0, s>>>(nch, soff, ps, st, en, tl.srow.as<int32_t>(), col, G, nullptr,
                                                PutF32{A.v32.as<float>(), tl.v32.as<float4>()});
        tl.has_v32 = true;
    } else if ((prec == FAIR_PREC_F16 && !tl.has_r16) || (prec == FAIR_PREC_Q16 && !tl.has_rq)) {
        FAIR_TRY(csr_make_lowprec(A, prec, s));
        const bool h = prec == FAIR_PREC_F16;
        DevBuf &dst = h ? tl.r16 : tl.rq;
        FAIR_TRY(dst.grow(sizeof(uint4) * ns));
        const uint16_t *v = h ? A.v16.as<uint16_t>() : A.vq.as<uint16_t>();
        k_tl_fill<Put2B><<<grid, 256, 0, s>>>(nch, soff, ps, st, en, tl.srow.as<int32_t>(), col, G, nullptr,
                                               Put2B{v, dst.as<uint4>()});
        (h ? tl.has_r16 : tl.has_rq) = true;
    }
    FAIR_CUDA(cudaGetLastError());
    if (prec == FAIR_PREC_F16 || prec == FAIR_PREC_Q16) {  // the 6-entry step records
        if (!tl.tried6) {
            tl.tried6 = true;
            FAIR_TRY(t6_build(A, s));
        }
        const bool h = prec == FAIR_PREC_F16;
        if (tl.built6 && !(h ? tl.has6_16 : tl.has6_q)) {
            DevBuf &dst = h ? tl.r6_16 : tl.r6_q;
            FAIR_TRY(dst.grow(sizeof(uint4) * (size_t)std::max<int64_t>(tl.nslots6, 1)));
            k_t6_rec<<<tl_grid(nch * 32), 256, 0, s>>>(
                nch, tl.soff6.as<int64_t>(), ps, st, en, tl.code6.as<uint32_t>(),
                h ? A.v16.as<uint16_t>() : A.vq.as<uint16_t>(), dst.as<uint4>());
            FAIR_CUDA(cudaGetLastError());
            (h ? tl.has6_16 : tl.has6_q) = true;
        }
    }
    return FAIR_OK;
}

bool sirt_pass_tiled(const SirtDev &S, const DevCSR &M, int pass, int code, cudaStream_t s) {
    const DevCSR::Tiled &tl = M.tl;
    // the work-unit counters are S.sched; pass 1 reads a copy of A, pass 2 one of A'.
    // Once launched, the pass is not repeated on another layout: a launch error
    // stays the runtime's last error for the caller to report.
    if (!tl.built() || !S.sched || tl.kind != (pass == 1 ? 0 : 1)) return false;
    if (S.prec == FAIR_PREC_F64) {
        if (!tl.has_v64) return false;
        const TlSplit<double> ld{tl.idx.as<uint2>(), tl.v64.as<double>()};
        if (pass == 1)
            launch_tl<TlSplit<double>, double, double>(M, code, ld, S.x, EpiResidF64{S.b, S.Minv, (double *)S.r},
                                                       S.sched, s);
        else
            launch_tl<TlSplit<double>, double, double>(M, code, ld, (const double *)S.r,
                                                       EpiUpdateF64{S.D, S.x, S.omg, S.lb, S.ub, S.bmode},
                                                       S.sched, s);
        return true;
    }
    const double scale = S.prec == FAIR_PREC_Q16 ? M.qscale : 1.0;
    const float *xv = pass == 1 ? S.x32 : (const float *)S.r;
    auto run = [&](const auto &ld) -> bool {
        using LD = std::decay_t<decltype(ld)>;
        if (pass == 1)
            launch_tl<LD, float, float>(M, code, ld, xv, EpiResidLP{S.b, S.Minv, (float *)S.r, scale}, S.sched, s);
        else
            launch_tl<LD, float, float>(M, code, ld, xv,
                                        EpiUpdateLP{S.D, S.x, S.x32, S.omg, S.lb, S.ub, S.bmode, scale}, S.sched,
                                        s);
        return true;
    };
    if (S.prec == FAIR_PREC_F32) {
        if (!tl.has_v32) return false;
        return run(TlSplit<float>{tl.idx.as<uint2>(), tl.v32.as<float>()});
    }
    const bool h = S.prec == FAIR_PREC_F16;
    if (code == 14 && tl.built6 && (h ? tl.has6_16 : tl.has6_q)) {
        const int32_t *anc = tl.anc6.as<int32_t>();
        const int4 *side = tl.side6.as<int4>();
        // the copy's step code: L6 is one of the builder's candidates 2, 3, 5
        auto run6 = [&](auto vt) -> bool {
            using VT = decltype(vt);
            const uint4 *rec = (h ? tl.r6_16 : tl.r6_q).as<uint4>();
            if (tl.L6 == 2) return run(TlStep6<VT, 2>(rec, anc, side, tl.S6));
            if (tl.L6 == 3) return run(TlStep6<VT, 3>(rec, anc, side, tl.S6));
            return run(TlStep6<VT, 5>(rec, anc, side, tl.S6));
        };
        if (h) return run6(__half());
        if (M.qsigned) return run6(int16_t());
        return run6(uint16_t());
    }
    if (h) {
        if (!tl.has_r16) return false;
        return run(TlFused<__half>{tl.r16.as<uint4>()});
    }
    if (!tl.has_rq) return false;
    if (M.qsigned) return run(TlFused<int16_t>{tl.rq.as<uint4>()});
    return run(TlFused<uint16_t>{tl.rq.as<uint4>()});
}

// ---- batches: the tiled passes of many problems in one launch ---------------
namespace {

// One problem's tiled pass (device table entry).
struct TlbDesc {
    TlArgs P;                  // its chunks, units and tile geometry
    const void *idx, *val;     // split copy: local indices and values; fused: records
    const void *x;             // the gathered vector
    void *part;                // its partial sums
    const int64_t *segbase;
    const double *b, *M;       // pass 1 epilogue
    void *r;
    const double *D;           // pass 2 epilogue
    double *x64;
    float *x32;
    double scale;              // 1, or the fixed-point scale of 16-bit codes
};

// last p in [0, np) with off[p] <= v (off[0] = 0 <= v < off[np])
__device__ __forceinline__ int tlb_owner(const int64_t *__restrict__ off, int np, int64_t v) {
    int lo = 0, hi = np;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= v) lo = mid; else hi = mid;
    }
    return lo;
}

template <class LD> struct TlbMake;
template <typename VT> struct TlbMake<TlSplit<VT>> {
    __device__ static TlSplit<VT> make(const TlbDesc &d) {
        return TlSplit<VT>{(const uint2 *)d.idx, (const VT *)d.val};
    }
};
template <typename VT> struct TlbMake<TlFused<VT>> {
    __device__ static TlFused<VT> make(const TlbDesc &d) { return TlFused<VT>{(const uint4 *)d.idx}; }
};

// The units of all problems numbered consecutively (uoff): a CTA takes the
// next unit, finds its problem and runs the single-problem unit body on it, so
// problems of any sizes share the GPU without tails.
template <class LD, typename XT, typename ACC>
__global__ void __launch_bounds__(kTlThreads, LD::CTAS) k_tlb_partials(const TlbDesc *__restrict__ desc,
                                                             const int64_t *__restrict__ uoff, int np,
                                                             unsigned *ctr) {
    extern __shared__ __align__(16) unsigned char tl_smem[];
    XT *xs = reinterpret_cast<XT *>(tl_smem);
    __shared__ int s_unit, s_chunk;
    const int64_t total = __ldg(uoff + np);
    for (;;) {
        if (threadIdx.x == 0) s_unit = (int)atomicAdd(ctr, 1u);
        __syncthreads();
        const int64_t u = s_unit;
        if (u >= total) break;
        const int p = tlb_owner(uoff, np, u);
        const TlbDesc &d = desc[p];
        const TlArgs P = d.P;
        tl_unit<LD, XT, ACC, 2, true>(P, TlbMake<LD>::make(d), (const XT *)d.x, (ACC *)d.part,
                                      P.units[u - __ldg(uoff + p)], xs, s_chunk);
    }
    if (threadIdx.x == 0) {
        const unsigned done = atomicAdd(ctr + 1, 1u);
        if (done == gridDim.x - 1) {  // every CTA has stopped taking units
            ctr[0] = 0u;
            ctr[1] = 0u;
        }
    }
}

// Row sums of the partials (in row order) and each problem's epilogue.
template <int PASS, typename ACC>
__global__ void k_tlb_rows(const TlbDesc *__restrict__ desc, const int64_t *__restrict__ roff, int np,
                           double omg, double lb, double ub, int bmode) {
    const int64_t total = __ldg(roff + np);
    // a thread's rows only grow, so its problem is looked up (and its
    // pointers loaded) only when a row passes the current problem's end
    int64_t lo = 0, hi = 0;
    const int64_t *segbase = nullptr;
    const ACC *part = nullptr;
    const double *b = nullptr, *M = nullptr, *D = nullptr;
    void *r = nullptr;
    double *x64 = nullptr;
    float *x32 = nullptr;
    double scale = 1.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= hi) {
            const int p = tlb_owner(roff, np, i);
            const TlbDesc &d = desc[p];
            lo = __ldg(roff + p);
            hi = __ldg(roff + p + 1);
            segbase = d.segbase;
            part = (const ACC *)d.part;
            b = d.b; M = d.M; r = d.r;
            D = d.D; x64 = d.x64; x32 = d.x32;
            scale = d.scale;
        }
        const int64_t row = i - lo;
        ACC acc = 0;
        for (int64_t k = segbase[row]; k < segbase[row + 1]; ++k) acc += part[k];
        if constexpr (sizeof(ACC) == 8) {
            if (PASS == 1) EpiResidF64{b, M, (double *)r}(row, acc);
            else EpiUpdateF64{D, x64, omg, lb, ub, bmode}(row, acc);
        } else {
            if (PASS == 1) EpiResidLP{b, M, (float *)r, scale}(row, acc);
            else EpiUpdateLP{D, x64, x32, omg, lb, ub, bmode, scale}(row, acc);
        }
    }
}

// Resident CTAs of a partials kernel at `smem` bytes, looked up once (so no
// occupancy query runs while a graph is captured).
int tlb_occupancy(const void *kernel, size_t smem) {
    static std::mutex mu;
    static std::map<std::pair<const void *, size_t>, int> table;
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_pair(kernel, smem);
    const auto it = table.find(key);
    if (it != table.end()) return it->second;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kTlThreads, smem);
    table[key] = std::max(occ, 1);
    return table[key];
}

template <class LD, typename XT, typename ACC>
int tlb_run(const TlBatch &T, int pass, double omg, double lb, double ub, int bmode, unsigned *ctr,
            cudaStream_t s, bool dry) {
    auto kernel = k_tlb_partials<LD, XT, ACC>;
    const void *kp = reinterpret_cast<const void *>(kernel);
    FAIR_CUDA(smem_allow(kp, T.smem));
    const int occ = tlb_occupancy(kp, T.smem);
    if (dry) return FAIR_OK;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sm_count() * occ, T.units));
    const TlbDesc *d = T.desc.as<TlbDesc>();
    kernel<<<grid, kTlThreads, T.smem, s>>>(d, T.uoff.as<int64_t>(), T.np, ctr);
    if (pass == 1)
        k_tlb_rows<1, ACC><<<tl_grid(T.rows), 256, 0, s>>>(d, T.roff.as<int64_t>(), T.np, omg, lb, ub, bmode);
    else
        k_tlb_rows<2, ACC><<<tl_grid(T.rows), 256, 0, s>>>(d, T.roff.as<int64_t>(), T.np, omg, lb, ub, bmode);
    return FAIR_OK;
}

}  // namespace

bool tl_batch_ready(const DevCSR &M, int prec) {
    const DevCSR::Tiled &tl = M.tl;
    if (!tl.built() || (!tl.has_idx && (prec == FAIR_PREC_F64 || prec == FAIR_PREC_F32))) return false;
    switch (prec) {
        case FAIR_PREC_F64: return tl.has_v64;
        case FAIR_PREC_F32: return tl.has_v32;
        case FAIR_PREC_F16: return tl.has_r16;
        default: return tl.has_rq && !M.qsigned;
    }
}

void tl_drop_build(DevCSR &M) {
    DevCSR::Tiled &tl = M.tl;
    tl.srow.release();
    tl.sstart.release();
    tl.send.release();
    // the 6-entry step records (a batched pass reads the 4-entry slots)
    tl.soff6.release(); tl.anc6.release(); tl.code6.release(); tl.side6.release();
    tl.r6_16.release(); tl.r6_q.release();
    tl.built6 = tl.has6_16 = tl.has6_q = false;
    tl.tried6 = true;
}

int tl_batch_bind(TlBatch &T, int prec, const std::vector<TlBatchProb> &probs) {
    const int np = (int)probs.size();
    std::vector<TlbDesc> d(np);
    std::vector<int64_t> uo(np + 1, 0), ro(np + 1, 0);
    int64_t cells = 1;
    for (int p = 0; p < np; ++p) {
        const DevCSR &M = *probs[p].M;
        const DevCSR::Tiled &tl = M.tl;
        if (!tl_batch_ready(M, prec)) {
            set_detail("batched tiled pass: a problem without its tiled copy");
            return FAIR_ERR_STATE;
        }
        TlbDesc &e = d[p];
        e.P = TlArgs{tl.soff.as<int64_t>(), tl.pslot.as<int32_t>(), tl.units.as<int4>(), tl.nunits, tl_geo(tl)};
        switch (prec) {
            case FAIR_PREC_F64: e.idx = tl.idx.p; e.val = tl.v64.p; break;
            case FAIR_PREC_F32: e.idx = tl.idx.p; e.val = tl.v32.p; break;
            case FAIR_PREC_F16: e.idx = tl.r16.p; e.val = nullptr; break;
            default: e.idx = tl.rq.p; e.val = nullptr; break;
        }
        e.x = probs[p].xin;
        e.part = tl.part.p;
        e.segbase = tl.segbase.as<int64_t>();
        e.b = probs[p].b;
        e.M = probs[p].Minv;
        e.r = probs[p].r;
        e.D = probs[p].D;
        e.x64 = probs[p].x;
        e.x32 = probs[p].x32;
        e.scale = prec == FAIR_PREC_Q16 ? M.qscale : 1.0;
        uo[p + 1] = uo[p] + tl.nunits;
        ro[p + 1] = ro[p] + M.m;
        cells = std::max<int64_t>(cells, (int64_t)e.P.G.cells() + 1);
    }
    FAIR_TRY(T.desc.grow(sizeof(TlbDesc) * std::max(np, 1)));
    FAIR_TRY(T.uoff.grow(sizeof(int64_t) * (np + 1)));
    FAIR_TRY(T.roff.grow(sizeof(int64_t) * (np + 1)));
    // synchronous copies: the host tables go out of scope on return
    FAIR_CUDA(cudaMemcpy(T.desc.p, d.data(), sizeof(TlbDesc) * np, cudaMemcpyHostToDevice));
    FAIR_CUDA(cudaMemcpy(T.uoff.p, uo.data(), sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice));
    FAIR_CUDA(cudaMemcpy(T.roff.p, ro.data(), sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice));
    T.np = np;
    T.units = uo[np];
    T.rows = ro[np];
    T.smem = (size_t)cells * (prec == FAIR_PREC_F64 ? sizeof(double) : sizeof(float));
    return FAIR_OK;
}

int tl_batch_launch(const TlBatch &T, int prec, int pass, double omg, double lb, double ub, int bmode,
                    unsigned *ctr, cudaStream_t s, bool dry) {
    if (T.np == 0) return FAIR_OK;
    switch (prec) {
        case FAIR_PREC_F64:
            return tlb_run<TlSplit<double>, double, double>(T, pass, omg, lb, ub, bmode, ctr, s, dry);
        case FAIR_PREC_F32:
            return tlb_run<TlSplit<float>, float, float>(T, pass, omg, lb, ub, bmode, ctr, s, dry);
        case FAIR_PREC_F16:
            return tlb_run<TlFused<__half>, float, float>(T, pass, omg, lb, ub, bmode, ctr, s, dry);
        default:
            return tlb_run<TlFused<uint16_t>, float, float>(T, pass, omg, lb, ub, bmode, ctr, s, dry);
    }
}

}  // namespace fair
