// kaczmarz.cu -- the ordered row-action sweep of basic_sweep
// (AIRMs.f90:813-858) on the GPU.
//
// The sweep is strictly sequential (adjacent rays share pixels), so one
// thread block walks the reference's row order; its W warps share each row's
// dot product (csr_matrowvec, sparse_matrices.f90:252-270) and bounded update
// (add_mult_row, :795-822). Row k+1 starts only after row k's update is
// visible, so the iterate follows the reference's sequence of projections.
// Three roundings differ from the reference: a_i.x - b_i is exact before its
// one rounding (the reference rounds each term of its ordered sum), the
// update is one fused multiply-add, and the coefficient is formed as
// (b_i - a_i.x) * (omega / nrA_i) instead of omega * (b_i - a_i.x) / nrA_i
// (AIRMs.f90:842).
//
// On GB300 every FP64 warp instruction holds its SM sub-partition's FP64 pipe
// for 64 cycles (measured: a dependent and an independent chain of DFMA both
// issue one per 64 cycles per warp), whatever its active lanes, and a
// row-action sweep runs on one SM; a row is a dependent chain (dot product,
// reduction, coefficient, update). The kernel therefore spends FP64
// instructions only where the arithmetic needs them:
//  * a row's entries are spread densely over the block (len / (32 W)
//    instructions per lane, skipped by a block-uniform branch past the end);
//  * the row sum a_i.x - b_i is formed exactly on the integer pipes (the
//    lanes' partials as 64-bit fixed point in a common frame, added by warp
//    reductions) and rounded once, so the reduction tree and the subtraction
//    of b_i use no FP64 instruction; each warp adds the W warp sums itself,
//    so one barrier per row suffices;
//  * omega / nrA_i, b_i and each step's entry range come from a parallel
//    schedule kernel, together with the row sampled by row probability
//    (AIRMs.f90:830-835);
//  * the box constraints are applied with integer comparisons on an
//    order-preserving key of the IEEE bits (the gfortran MAX/MIN semantics:
//    a NaN operand loses, +0 and -0 compare equal).
// The step record two rows ahead and the next row's column indices and
// values are prefetched while the current row is worked on, and the gathered
// values of x stay in registers for the update.
//
// When the iterate fits in shared memory it is kept there for the whole
// sweep; otherwise it stays in global memory (L2-resident at these sizes).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "fair_internal.cuh"

namespace fair {

namespace {

struct RowStep {
    int64_t s;    // first entry of the row
    int32_t len;  // entries
    int32_t pad;
    double b;     // b(ri)
    double w;     // omega / nrA(ri)
};

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

__global__ void k_sweep_schedule(const int32_t *ord, int32_t nord, int dir, int rowprob,
                                 const double *cumul, int32_t m, uint64_t seed, uint64_t ctr,
                                 const int64_t *rowptr, const double *b, const double *nrA,
                                 double omg, RowStep *steps) {
    for (int32_t ii = blockIdx.x * blockDim.x + threadIdx.x; ii < nord;
         ii += gridDim.x * blockDim.x) {
        int32_t ri = rowprob ? sample_row(cumul, m, uniform01(seed, ctr + (uint64_t)ii))
                             : ord[dir > 0 ? ii : nord - 1 - ii] - 1;
        int64_t s = rowptr[ri];
        steps[ii] = RowStep{s, (int32_t)(rowptr[ri + 1] - s), 0, b[ri], __ddiv_rn(omg, nrA[ri])};
    }
}

// Order-preserving key of a non-NaN double: key(-x) = -key(x), key(+-0) = 0.
__host__ __device__ __forceinline__ long long okey(long long bits) {
    long long mag = bits & 0x7FFFFFFFFFFFFFFFLL;
    return bits < 0 ? -mag : mag;
}
__device__ __forceinline__ bool is_nan_bits(long long bits) {
    return (bits & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL;
}

struct Box {
    int mode;  // bit0: upper bound, bit1: lower bound
    long long klb, kub;
    double lb, ub;
    // add_mult_row (sparse_matrices.f90:812-818): MAX(t, lb) first, then
    // MIN(t, ub); MAX/MIN return the non-NaN operand
    __device__ __forceinline__ double apply(double t) const {
        if (mode & 2) {
            long long tb = __double_as_longlong(t);
            if (klb > okey(tb) || is_nan_bits(tb)) t = lb;
        }
        if (mode & 1) {
            long long tb = __double_as_longlong(t);
            if (kub < okey(tb) || is_nan_bits(tb)) t = ub;
        }
        return t;
    }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---- exact sums of doubles on the integer pipes ------------------------------
// A finite double with exponent field e and significand m (53 bits with the
// implicit one; e = 0: no implicit one, scale as e = 1) is m * 2^(e - 1075).
// In the frame E (at least every term's e) it becomes the integer m >> (E - e),
// which drops less than one unit 2^(E - 1075): an ulp of the largest term. A
// warp adds its lanes' integers exactly as three 26-bit limbs with
// __reduce_add_sync, the warps' sums are aligned to the largest frame, and the
// total is rounded to double once (round to nearest even). A row of up to
// 8 x 32 lanes x 2 partials + b stays below 2^63.
__device__ __forceinline__ int fx_exp(double v) {
    const int e = (int)((__double_as_longlong(v) >> 52) & 0x7FF);
    return e > 1 ? e : 1;
}
__device__ __forceinline__ long long fx_of(double v, int E) {
    const long long b = __double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF);
    long long m = b & 0xFFFFFFFFFFFFFLL;
    if (e) m |= 1LL << 52;
    const int sh = E - (e > 1 ? e : 1);
    const long long f = sh < 64 ? (m >> sh) : 0LL;
    return b < 0 ? -f : f;
}
__device__ __forceinline__ long long fx_warp_sum(long long F) {  // |F| < 2^55 per lane
    const unsigned l0 = __reduce_add_sync(0xffffffffu, (unsigned)(F & 0x3FFFFFF));
    const unsigned l1 = __reduce_add_sync(0xffffffffu, (unsigned)((F >> 26) & 0x3FFFFFF));
    const int l2 = __reduce_add_sync(0xffffffffu, (int)(F >> 52));
    return (long long)l2 * (1LL << 52) + (long long)l1 * (1LL << 26) + (long long)l0;
}
// total * 2^(E - 1075) rounded to nearest even, once. Below the normal range
// the value is exact: the frame's unit 2^(E - 1075) (E >= 1) is a multiple of
// the smallest subnormal 2^-1074, and such a total has fewer than 53 - E + 1
// bits, so it is the subnormal significand shifted by E - 1. Above it the
// rounded value overflows to infinity.
__device__ __forceinline__ double fx_to_double(long long total, int E) {
    if (total == 0) return 0.0;
    const bool neg = total < 0;
    unsigned long long a = neg ? 0ull - (unsigned long long)total : (unsigned long long)total;
    int nb = 64 - __clzll((long long)a);
    unsigned long long mant;
    if (nb <= 53) {
        mant = a << (53 - nb);
    } else {
        const int sh = nb - 53;
        mant = a >> sh;
        const unsigned long long rem = a & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (mant & 1ull))) ++mant;
        if (mant == (1ull << 53)) {
            mant >>= 1;
            ++nb;
        }
    }
    const int field = nb + E - 53;
    unsigned long long bits;
    if (field < 1) bits = a << (E - 1);  // nb <= 53 - E here: no rounding above, < 2^52
    else if (field > 2046) bits = 0x7FF0000000000000ull;
    else bits = ((unsigned long long)field << 52) | (mant & 0xFFFFFFFFFFFFFull);
    if (neg) bits |= 1ull << 63;
    return __longlong_as_double((long long)bits);
}
// A warp's share of a row sum: its integer sum in its frame, or (when a term
// is Inf or NaN, frame 0x7FF) its FP64 sum.
struct FxPart {
    long long s;
    double d;
    int e;
    int pad;
};
__device__ __forceinline__ FxPart fx_warp_part(double p0, double p1, double p2) {
    int e = max(max(fx_exp(p0), fx_exp(p1)), fx_exp(p2));
    FxPart r{0, 0.0, (int)__reduce_max_sync(0xffffffffu, (unsigned)e), 0};
    if (r.e < 0x7FF) r.s = fx_warp_sum(fx_of(p0, r.e) + fx_of(p1, r.e) + fx_of(p2, r.e));
    else r.d = warp_sum(p0 + p1 + p2);
    return r;
}
// The row sum from the warps' shares (FP64 sum of the non-finite shares when
// there are any: an Inf or NaN term decides the result).
template <int W>
__device__ __forceinline__ double fx_total(const FxPart *part) {
    int E = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) E = max(E, part[w].e);
    if (E >= 0x7FF) {
        double d = 0.0;
#pragma unroll
        for (int w = 0; w < W; ++w)
            if (part[w].e >= 0x7FF) d += part[w].d;
        return d;
    }
    long long t = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int sh = E - part[w].e;
        if (sh < 64) t += part[w].s >> sh;
    }
    return fx_to_double(t, E);
}

// dup: when given and set, some row repeats a column (found by the level
// set-up); thread 0 then applies each row's updates one entry after the other,
// so that a repeated column takes both updates in order as in add_mult_row.
// only_if_dup: the level sweep ran; this kernel runs only for such a matrix.
template <int W, int CACHE, bool SMEM_X>
__global__ void __launch_bounds__(32 * W) k_sweep(const RowStep *__restrict__ steps, int32_t nord,
                                                  const int32_t *__restrict__ col,
                                                  const double *__restrict__ val, double *xg,
                                                  int32_t n, Box box, const int *dup,
                                                  int only_if_dup) {
    constexpr int T = 32 * W;
    extern __shared__ double xs[];
    __shared__ FxPart part_s[W];
    const bool serial_update = dup && *dup;
    if (only_if_dup && !serial_update) return;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    double *x = SMEM_X ? xs : xg;
    if (SMEM_X) {
        for (int32_t j = tid; j < n; j += T) xs[j] = xg[j];
        __syncthreads();
    }
    if (nord <= 0) return;
    const RowStep none{0, 0, 0, 0.0, 0.0};
    // three-stage pipeline: the step record two rows ahead, the entries of
    // the next row, the current row
    RowStep cur = steps[0];
    RowStep nxt = nord > 1 ? steps[1] : none;
    int32_t cc[CACHE];
    double vv[CACHE];
    int nq = (cur.len + T - 1) / T;
#pragma unroll
    for (int q = 0; q < CACHE; ++q) {
        if (q >= nq) break;
        int k = tid + q * T;
        cc[q] = k < cur.len ? __ldg(col + cur.s + k) : 0;
        vv[q] = k < cur.len ? __ldg(val + cur.s + k) : 0.0;
    }
    for (int32_t ii = 0; ii < nord; ++ii) {
        const RowStep nxt2 = ii + 2 < nord ? steps[ii + 2] : none;
        const int nqn = (nxt.len + T - 1) / T;
        int32_t nc[CACHE];
        double nv[CACHE];
#pragma unroll
        for (int q = 0; q < CACHE; ++q) {
            if (q >= nqn) break;
            int k = tid + q * T;
            nc[q] = k < nxt.len ? __ldg(col + nxt.s + k) : 0;
            nv[q] = k < nxt.len ? __ldg(val + nxt.s + k) : 0.0;
        }
        // dot product of the row with x (two independent accumulators)
        double xo[CACHE];
        double p0 = 0.0, p1 = 0.0;
#pragma unroll
        for (int q = 0; q < CACHE; ++q) {
            if (q >= nq) break;
            int k = tid + q * T;
            xo[q] = k < cur.len ? x[cc[q]] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < CACHE; ++q) {
            if (q >= nq) break;
            if (q & 1) p1 = fma(xo[q], vv[q], p1); else p0 = fma(xo[q], vv[q], p0);
        }
        for (int k = tid + CACHE * T; k < cur.len; k += T)
            p0 = fma(x[__ldg(col + cur.s + k)], __ldg(val + cur.s + k), p0);
        // a_i.x - b_i, summed exactly on the integer pipes (-b_i is a term of
        // thread 0) and rounded once; every warp forms the same total, so the
        // coefficient needs no second barrier
        const FxPart mine = fx_warp_part(p0, p1, tid == 0 ? -cur.b : 0.0);
        double resid;
        if (W > 1) {
            if (lane == 0) part_s[wid] = mine;
            __syncthreads();
            resid = fx_total<W>(part_s);
        } else {
            resid = fx_total<1>(&mine);
        }
        const double coeff = __dmul_rn(-resid, cur.w);
        if (serial_update) {
            // every thread's reads of x for this row are done (the barrier above,
            // or the warp's reductions)
            if (tid == 0)
                for (int k = 0; k < cur.len; ++k) {
                    const int32_t c = __ldg(col + cur.s + k);
                    x[c] = box.apply(fma(coeff, __ldg(val + cur.s + k), x[c]));
                }
        } else {
#pragma unroll
            for (int q = 0; q < CACHE; ++q) {
                if (q >= nq) break;
                int k = tid + q * T;
                if (k < cur.len) x[cc[q]] = box.apply(fma(coeff, vv[q], xo[q]));
            }
            for (int k = tid + CACHE * T; k < cur.len; k += T) {
                int32_t c = __ldg(col + cur.s + k);
                x[c] = box.apply(fma(coeff, __ldg(val + cur.s + k), x[c]));
            }
        }
        if (W > 1) __syncthreads(); else __syncwarp();
        cur = nxt;
        nxt = nxt2;
        nq = nqn;
#pragma unroll
        for (int q = 0; q < CACHE; ++q) { cc[q] = nc[q]; vv[q] = nv[q]; }
    }
    if (SMEM_X) {
        __syncthreads();
        for (int32_t j = tid; j < n; j += T) xg[j] = xs[j];
    }
}

template <int W, int CACHE>
int launch(const SweepDev &S, const RowStep *steps, bool smem, size_t smem_bytes, const Box &box,
           const int *dup, int only_if_dup, cudaStream_t s) {
    const DevCSR &A = *S.A;
    if (smem) {
        auto kern = k_sweep<W, CACHE, true>;
        FAIR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem_bytes));
        kern<<<1, 32 * W, smem_bytes, s>>>(steps, S.nord, A.col.as<int32_t>(), A.v64.as<double>(),
                                          S.x, A.n, box, dup, only_if_dup);
    } else {
        k_sweep<W, CACHE, false><<<1, 32 * W, 0, s>>>(steps, S.nord, A.col.as<int32_t>(),
                                                     A.v64.as<double>(), S.x, A.n, box, dup,
                                                     only_if_dup);
    }
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

long long host_key(double v) {
    long long bits;
    memcpy(&bits, &v, sizeof bits);
    return okey(bits);
}

// Warps per row: FAIR_SWEEP_WARPS (1, 2, 4 or 8) when set, else 4. Measured
// on GB300 (host call, rows/s for 1, 2, 4, 8 warps): fan beam N=128, x in
// shared memory, Kaczmarz 0.83M, 0.97M, 1.00M, 0.94M; fan beam N=512, x in
// global memory, symmetric Kaczmarz 0.18M, 0.33M, 0.44M, 0.39M and random
// Kaczmarz 0.17M, 0.30M, 0.43M, 0.42M.
int sweep_warps() {
    const char *env = getenv("FAIR_SWEEP_WARPS");
    if (env) {
        int w = atoi(env);
        if (w == 1 || w == 2 || w == 4 || w == 8) return w;
    }
    return 4;
}

// ---- level-scheduled sweep ------------------------------------------------------
// Two steps of a sweep commute when their rows share no column: neither reads
// what the other writes. Give step k the level 1 + max(level of every earlier
// step sharing a column with it); then every step's reads come after all
// earlier steps that write those columns and before all later ones, so running
// the levels in order, the steps of one level in parallel, gives exactly the
// sequence of bounded projections of basic_sweep (AIRMs.f90:813-858): the
// same row sums (exact fixed-point sums of the lanes' FP64 partials, rounded
// once) and the same updates in the same order per column. For a ray order
// that walks the bins of one angle and then the next, the levels form a
// wavefront: a ray waits for its neighbour bin and for the few rays of the
// previous angle that cross its pixels, so about 30 (fan beam N=128) to 80
// (N=512) steps share a level.
//
// The levels are exact, computed per sweep order in windows of 32 steps:
//   k_lvl_setup (every SM, windows in parallel): each entry swaps a stamp
//     into its column's cell of the block's table; a stamp of an earlier step
//     of the window makes the entry "shared" and that step a predecessor; the
//     step's entries are written in groups [first touch in the window and
//     last | first, not last | shared, not last | shared and last], and the
//     longest paths between the window's steps (predecessor chains) as one
//     byte per pair;
//   k_lvl_levels (one block; k_lvl_levels_cluster for tables that do not fit
//     shared memory, on a 16-block cluster), windows in order: a step's level
//     is the largest, over the steps a of its window with a path to it, of
//     base(a) + the path's length, base(a) = 1 + the table's level over a's
//     first-touch columns; the last touches write the levels into the table;
//   counting sort of the steps by level (level pointers, steps in level order).
// The sweep (k_lvl_sweep) runs a group of G warps per step, the steps of a
// level spread over the groups, on one thread-block cluster (a cluster barrier
// between levels; x in the cluster's distributed shared memory when its parts
// fit, else in global memory read past L1) or, when a level outgrows the
// cluster, on a cooperative grid of up to one block per SM (a software grid
// barrier between levels; x in global memory).

struct WinRow {
    int64_t off;              // first entry of the step in the grouped column array
    int32_t len, c1, c2, c3;  // entries; groups [0,c1) [c1,c2) [c2,c3) [c3,len)
};
static_assert(sizeof(WinRow) == 24, "WinRow layout");

constexpr int kWinRows = 32;      // steps per window (one predecessor bit each)
constexpr int kMinStepsPerLevel = 4;
constexpr int kSetupThreads = 512;
constexpr int kSetupWarps = kSetupThreads / 32;
// Window stamps of the set-up's column tables: window id (36 bits), step in
// the window (8 bits), entry position in the window (20 bits). All ones marks
// an empty cell.
constexpr int kStampPosBits = 20;
constexpr unsigned long long kStampIdLimit = (1ull << 36) - 1ull;

__device__ __forceinline__ unsigned long long win_stamp(unsigned long long id, int r, int pos) {
    return (id << 28) | ((unsigned long long)r << kStampPosBits) | (unsigned long long)pos;
}
// group of an entry from its flags (bit 0: a later step has the column; bit 1: an earlier one)
__device__ __forceinline__ int win_group(unsigned f) {
    return (f & 2u) ? ((f & 1u) ? 2 : 3) : (int)f;
}

// total * 2^(E - 1075), rounded once: the integer converted to double (round
// to nearest even) and rescaled by its exponent field when the result is a
// normal number; otherwise fx_to_double.
__device__ __forceinline__ double fx_to_double_fast(long long total, int E) {
    if (total == 0) return 0.0;
    const long long bits = __double_as_longlong(__ll2double_rn(total));
    const int field = (int)((bits >> 52) & 0x7FF) + E - 1075;
    if (field >= 1 && field <= 2046)
        return __longlong_as_double(bits + ((long long)(E - 1075) << 52));
    return fx_to_double(total, E);
}
__device__ __forceinline__ double fx_part_double(const FxPart &p) {
    return p.e >= 0x7FF ? p.d : fx_to_double_fast(p.s, p.e);
}

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Exclusive scan of n counts (n from *n_dev when given) into out[0..n], one
// block.
__global__ void __launch_bounds__(1024) k_scan_excl(const int32_t *__restrict__ in, int64_t n_host,
                                                   const int *__restrict__ n_dev,
                                                   int64_t *__restrict__ out) {
    __shared__ int64_t wsum[32];
    __shared__ int64_t carry;
    const int64_t n = n_dev ? (int64_t)*n_dev : n_host;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int64_t b = 0; b < n; b += 1024) {
        const int64_t i = b + tid;
        int64_t v = i < n ? in[i] : 0, inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[wid] = inc;
        __syncthreads();
        if (wid == 0) {
            int64_t w = wsum[lane], wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
            wsum[lane] = wi - w;
        }
        __syncthreads();
        const int64_t c = carry;
        if (i < n) out[i] = c + wsum[wid] + inc - v;
        __syncthreads();
        if (tid == 1023) carry = c + wsum[31] + inc;
        __syncthreads();
    }
    if (tid == 0) out[n] = carry;
}

__global__ void k_step_lengths(const RowStep *__restrict__ steps, int32_t nord,
                               int32_t *__restrict__ lens) {
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nord; k += gridDim.x * blockDim.x)
        lens[k] = steps[k].len;
}

// Set-up of the windows (one block per window at a time, a table per block).
// The steps of a window are taken in order; each entry swaps its stamp into
// its column's cell, and the stamp it finds tells whether an earlier step of
// the window has the column (this entry is then shared, that one not last,
// and that step a predecessor of this one). A stamp of the same step means the
// row repeats a column: *err is set and the single-block kernel applies the
// sweep's updates in order instead. From the predecessors, the longest path
// between every two steps of the window (dpath: 32 bytes per step).
__global__ void __launch_bounds__(kSetupThreads) k_lvl_setup(
        const RowStep *__restrict__ steps, const int64_t *__restrict__ eoff, int32_t nord,
        const int32_t *__restrict__ col, unsigned long long *__restrict__ tabs, int32_t n,
        unsigned long long id0, int32_t *__restrict__ oidx, WinRow *__restrict__ rec,
        signed char *__restrict__ dpath, int *err) {
    extern __shared__ __align__(16) unsigned char fl[];  // [entries of a window]
    __shared__ int rb[kWinRows + 1];
    __shared__ uint32_t msk[kWinRows];              // predecessor steps in the window
    __shared__ signed char dps[kWinRows][kWinRows];  // longest path a -> r, -1: none
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    unsigned long long *tab = tabs + (size_t)blockIdx.x * (size_t)n;
    const int nwin = (nord + kWinRows - 1) / kWinRows;
    for (int q = blockIdx.x; q < nwin; q += gridDim.x) {
        const int k0 = q * kWinRows, nr = min(kWinRows, nord - k0);
        const int64_t wbase = eoff[k0];
        if (tid < kWinRows) {
            rb[tid + 1] = tid < nr ? (int)(eoff[k0 + tid + 1] - wbase) : 0;
            msk[tid] = 0;
            if (tid == 0) rb[0] = 0;
        }
        __syncthreads();
        const unsigned long long id = id0 + (unsigned long long)q;
        for (int r = 0; r < nr; ++r) {
            const int64_t s0 = steps[k0 + r].s;
            const int base = rb[r], len = rb[r + 1] - base;
            for (int e = tid; e < len; e += kSetupThreads) {
                const int32_t c = col[s0 + e];
                const int pos = base + e;
                const unsigned long long old = atomicExch(tab + c, win_stamp(id, r, pos));
                unsigned char f = 0;
                if ((old >> 28) == id) {
                    const int orow = (int)((old >> kStampPosBits) & 0xFFull);
                    if (orow == r) {
                        atomicExch(err, 1);
                    } else {
                        f = 2;
                        fl[old & ((1ull << kStampPosBits) - 1ull)] |= 1;  // its one writer
                        atomicOr(&msk[r], 1u << orow);
                    }
                }
                fl[pos] = f;
            }
            __syncthreads();
        }
        if (wid == 0) {  // longest paths within the window (rows in order)
            for (int r = 0; r < nr; ++r) {
                int v = lane == r ? 0 : -1;
                for (uint32_t bits = msk[r]; bits; bits &= bits - 1u) {
                    const int d = dps[__ffs(bits) - 1][lane];
                    if (d >= 0) v = max(v, d + 1);
                }
                dps[r][lane] = (signed char)v;
                __syncwarp();
            }
            for (int r = 0; r < nr; ++r) dpath[(size_t)(k0 + r) * kWinRows + lane] = dps[r][lane];
        }
        const unsigned lt = (1u << lane) - 1u;
        for (int r = wid; r < nr; r += kSetupWarps) {
            const int64_t s0 = steps[k0 + r].s;
            const int base = rb[r], len = rb[r + 1] - base;
            int n0 = 0, n1 = 0, n2 = 0;
            for (int e0 = 0; e0 < len; e0 += 32) {
                const int e = e0 + lane;
                const int g = e < len ? win_group(fl[base + e]) : -1;
                n0 += __popc(__ballot_sync(0xffffffffu, g == 0));
                n1 += __popc(__ballot_sync(0xffffffffu, g == 1));
                n2 += __popc(__ballot_sync(0xffffffffu, g == 2));
            }
            int o0 = 0, o1 = n0, o2 = n0 + n1, o3 = n0 + n1 + n2;
            const int64_t ro = wbase + base;
            for (int e0 = 0; e0 < len; e0 += 32) {
                const int e = e0 + lane;
                const int g = e < len ? win_group(fl[base + e]) : -1;
                const unsigned b0 = __ballot_sync(0xffffffffu, g == 0);
                const unsigned b1 = __ballot_sync(0xffffffffu, g == 1);
                const unsigned b2 = __ballot_sync(0xffffffffu, g == 2);
                const unsigned b3 = __ballot_sync(0xffffffffu, g == 3);
                if (g >= 0) {
                    const int d = g == 0 ? o0 + __popc(b0 & lt)
                                : g == 1 ? o1 + __popc(b1 & lt)
                                : g == 2 ? o2 + __popc(b2 & lt)
                                         : o3 + __popc(b3 & lt);
                    oidx[ro + d] = col[s0 + e];
                }
                o0 += __popc(b0);
                o1 += __popc(b1);
                o2 += __popc(b2);
                o3 += __popc(b3);
            }
            if (lane == 0) rec[k0 + r] = WinRow{ro, len, n0, n0 + n1, n0 + n1 + n2};
        }
        __syncthreads();  // fl, rb, msk and dps belong to the next window
    }
}

// The steps' levels, windows in order (one block of 1024 threads). lv: the
// last level written into each column (shared memory when it fits, else
// global memory, zeroed by the caller). A step's level is the largest, over
// the steps a of its window with a path to it, of base(a) + the path's length,
// where base(a) = 1 + the table's level over a's first-touch columns. The next
// window's records are loaded while a window runs.
template <bool SMEM>
__global__ void __launch_bounds__(1024, 1) k_lvl_levels(
        const WinRow *__restrict__ rec, const signed char *__restrict__ dpath,
        const int32_t *__restrict__ oidx, int32_t nord, int32_t *lvg, int32_t n,
        int32_t *__restrict__ lvl, int *__restrict__ nlev) {
    extern __shared__ int32_t lvs[];
    __shared__ int32_t base[kWinRows], lvw[kWinRows];
    int32_t *lv = SMEM ? lvs : lvg;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (SMEM)
        for (int32_t j = tid; j < n; j += 1024) lvs[j] = 0;
    const WinRow none{0, 0, 0, 0, 0};
    const int nwin = (nord + kWinRows - 1) / kWinRows;
    int nr1 = min(kWinRows, nord);
    WinRow wn = wid < nr1 ? rec[wid] : none;
    uint4 dn0 = make_uint4(0, 0, 0, 0), dn1 = dn0;
    if (wid == 0 && lane < nr1) {
        const uint4 *d = reinterpret_cast<const uint4 *>(dpath + (size_t)lane * kWinRows);
        dn0 = d[0];
        dn1 = d[1];
    }
    __syncthreads();
    int top = 0;
    for (int q = 0; q < nwin; ++q) {
        const int k0 = q * kWinRows, nr = nr1;
        const WinRow w = wn;
        const uint4 d0 = dn0, d1 = dn1;
        if (q + 1 < nwin) {
            nr1 = min(kWinRows, nord - k0 - kWinRows);
            wn = wid < nr1 ? rec[k0 + kWinRows + wid] : none;
            if (wid == 0 && lane < nr1) {
                const uint4 *d = reinterpret_cast<const uint4 *>(
                    dpath + (size_t)(k0 + kWinRows + lane) * kWinRows);
                dn0 = d[0];
                dn1 = d[1];
            }
        }
        if (wid < nr) {  // 1 + the table's level over the step's first-touch columns
            int m = 0;
            for (int e0 = lane; e0 < w.c2; e0 += 32 * 8) {  // 8 independent loads per lane
                int32_t j[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) j[t] = e0 + 32 * t < w.c2 ? oidx[w.off + e0 + 32 * t] : -1;
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    if (j[t] >= 0) m = max(m, SMEM ? lvs[j[t]] : __ldcg(lvg + j[t]));
            }
            m = (int)__reduce_max_sync(0xffffffffu, (unsigned)m);
            if (lane == 0) base[wid] = m + 1;
        }
        __syncthreads();
        if (wid == 0) {  // the longest paths within the window
            const uint32_t dw[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
            int L = 0;
#pragma unroll
            for (int a = 0; a < kWinRows; ++a) {
                const int dv = (int)(signed char)(dw[a >> 2] >> (8 * (a & 3)));
                if (a < nr && dv >= 0) L = max(L, base[a] + dv);
            }
            if (lane < nr) {
                lvw[lane] = L;
                lvl[k0 + lane] = L;
            }
            top = max(top, (int)__reduce_max_sync(0xffffffffu, lane < nr ? (unsigned)L : 0u));
        }
        __syncthreads();
        if (wid < nr) {  // the last touches of the window write the step's level
            const int L = lvw[wid];
            for (int e0 = lane; e0 < w.len; e0 += 32 * 8) {
                int32_t j[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const int e = e0 + 32 * t;
                    j[t] = e < w.len && (e < w.c1 || e >= w.c3) ? oidx[w.off + e] : -1;
                }
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    if (j[t] >= 0) lv[j[t]] = L;
            }
        }
        __syncthreads();
    }
    if (tid == 0) *nlev = top;
}

// The same on a cluster of CS blocks (512 threads each), for a level table
// in global memory: block c takes the steps c, c + CS, ... of every window
// (16 * CS / 32 warps per step), so the scattered table reads and writes are
// spread over CS SMs. The steps' bases meet in distributed shared memory; a
// cluster barrier after the bases and one after the table writes keep the
// windows in order. *nlev must be zero at the start.
template <int CS>
__global__ void __launch_bounds__(512, 1) k_lvl_levels_cluster(
        const WinRow *__restrict__ rec, const signed char *__restrict__ dpath,
        const int32_t *__restrict__ oidx, int32_t nord, int32_t *lv, int32_t *__restrict__ lvl,
        int *__restrict__ nlev) {
    constexpr int RW = (kWinRows + CS - 1) / CS;  // steps per block and window
    constexpr int WPR = 16 / RW;                  // warps per step
    static_assert(WPR >= 1 && RW * WPR <= 16, "cluster shape");
    __shared__ int32_t base[RW], lvw[RW];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int rank = (int)cluster_rank();
    const int i = wid / WPR, sw = wid - i * WPR;  // the warp's step slot, warp in the step
    const WinRow none{0, 0, 0, 0, 0};
    const int nwin = (nord + kWinRows - 1) / kWinRows;
    int top = 0;
    // distributed shared memory address of the base of step `lane` of a window
    uint32_t lane_base;
    {
        const uint32_t a = (uint32_t)__cvta_generic_to_shared(base);
        asm("mapa.shared::cluster.u32 %0, %1, %2;"
            : "=r"(lane_base)
            : "r"(a + 4u * (uint32_t)(lane / CS)), "r"((uint32_t)(lane % CS)));
    }
    for (int q = 0; q < nwin; ++q) {
        const int k0 = q * kWinRows, nr = min(kWinRows, nord - k0);
        const int r = rank + CS * i;  // this warp's step in the window
        const bool mine = i < RW && r < nr;
        const WinRow w = mine ? rec[k0 + r] : none;
        if (sw == 0 && lane == 0 && i < RW) base[i] = 0;
        if (q + 1 < nwin && mine) {  // the next window's step of this warp: its columns into L2
            const int r1 = r;
            if (k0 + kWinRows + r1 < nord) {
                const WinRow wn = rec[k0 + kWinRows + r1];
                const char *c0 = reinterpret_cast<const char *>(oidx + wn.off);
                const int nl = (wn.len * 4 + 127) >> 7;
                for (int l = sw * 32 + lane; l < nl; l += 32 * WPR)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(c0 + ((size_t)l << 7)));
            }
        }
        __syncthreads();
        if (mine) {  // 1 + the table's level over the step's first-touch columns
            int m = 0;
            for (int e0 = sw * 32 + lane; e0 < w.c2; e0 += 32 * WPR * 4) {
                int32_t j[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int e = e0 + 32 * WPR * t;
                    j[t] = e < w.c2 ? oidx[w.off + e] : -1;
                }
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    if (j[t] >= 0) m = max(m, __ldcg(lv + j[t]));
            }
            m = (int)__reduce_max_sync(0xffffffffu, (unsigned)m);
            if (lane == 0) atomicMax(&base[i], m + 1);
        }
        cluster_barrier();
        if (mine && sw == 0) {  // the longest paths within the window
            const uint4 *dp = reinterpret_cast<const uint4 *>(dpath + (size_t)(k0 + r) * kWinRows);
            const uint4 d0 = dp[0], d1 = dp[1];
            const uint32_t dw[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
            int dv = 0;
#pragma unroll
            for (int a = 0; a < kWinRows; ++a)
                if (a == lane) dv = (int)(signed char)(dw[a >> 2] >> (8 * (a & 3)));
            int bv = 0;
            if (lane < nr && dv >= 0)
                asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(bv) : "r"(lane_base));
            const int L = (int)__reduce_max_sync(0xffffffffu, (lane < nr && dv >= 0) ? (unsigned)(bv + dv) : 0u);
            if (lane == 0) {
                lvw[i] = L;
                lvl[k0 + r] = L;
            }
            top = max(top, L);
        }
        __syncthreads();
        if (mine) {  // the last touches of the window write the step's level
            const int L = lvw[i];
            for (int e0 = sw * 32 + lane; e0 < w.len; e0 += 32 * WPR * 4) {
                int32_t j[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int e = e0 + 32 * WPR * t;
                    j[t] = e < w.len && (e < w.c1 || e >= w.c3) ? oidx[w.off + e] : -1;
                }
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    if (j[t] >= 0) lv[j[t]] = L;
            }
        }
        cluster_barrier();
    }
    if (lane == 0 && top > 0) atomicMax(nlev, top);
}

__global__ void k_lvl_count(const int32_t *__restrict__ lvl, int32_t nord, int32_t *cnt) {
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nord; k += gridDim.x * blockDim.x)
        atomicAdd(cnt + lvl[k] - 1, 1);
}
// steps in level order (any order within a level: its steps share no column)
__global__ void k_lvl_scatter(const RowStep *__restrict__ steps, const int32_t *__restrict__ lvl,
                              int32_t nord, const int64_t *__restrict__ lptr, int32_t *cnt,
                              RowStep *__restrict__ sched) {
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nord; k += gridDim.x * blockDim.x) {
        const int l = lvl[k] - 1;
        sched[lptr[l] + atomicSub(cnt + l, 1) - 1] = steps[k];
    }
}


// Where the level sweep keeps x: global memory read past L1 (XG), the
// block's shared memory (XS, one block), or the cluster's distributed shared
// memory (XD: block r holds x[r * 2^cb, (r + 1) * 2^cb)). XS and XD address x
// by 32-bit shared-window addresses.
enum { XG = 0, XS = 1, XD = 2 };
template <int XM> struct XAcc;
template <> struct XAcc<XG> {
    double *x;
    using R = double *;
    __device__ __forceinline__ R ref(int32_t j) const { return x + j; }
    __device__ __forceinline__ double ld(R p) const { return __ldcg(p); }
    __device__ __forceinline__ void st(R p, double v) const { *p = v; }
};
template <> struct XAcc<XS> {
    uint32_t base;  // shared-window address of x
    using R = uint32_t;
    __device__ __forceinline__ R ref(int32_t j) const { return base + ((uint32_t)j << 3); }
    __device__ __forceinline__ double ld(R a) const {
        double v;
        asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"(a));
        return v;
    }
    __device__ __forceinline__ void st(R a, double v) const {
        asm volatile("st.shared.f64 [%0], %1;" ::"r"(a), "d"(v));
    }
};
template <> struct XAcc<XD> {
    uint32_t base;  // shared-window address of this block's part
    int cb;         // log2 of the part's length
    using R = uint32_t;
    __device__ __forceinline__ R ref(int32_t j) const {  // an address, no memory access
        const uint32_t a = base + (((uint32_t)j & ((1u << cb) - 1u)) << 3);
        uint32_t r;
        asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"((uint32_t)j >> cb));
        return r;
    }
    // volatile keeps these in program order among themselves and against the
    // barriers (also volatile asm), the only ordering the sweep needs
    __device__ __forceinline__ double ld(R a) const {
        double v;
        asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a));
        return v;
    }
    __device__ __forceinline__ void st(R a, double v) const {
        asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v));
    }
};

// One step by a group of G warps: the row's chunks of 32 entries are dealt
// to the group's warps in turn (chunk q to warp q mod G), CACHE chunks per
// warp held in registers and the rest loaded in batches of four. Each warp's
// part of a.x - b is an exact fixed-point sum (fx_warp_part); the G parts meet
// in shared memory behind the group's named barrier, are added exactly and
// rounded once; then the coefficient (b - a.x) * (omega / nrA) and the bounded
// updates.
// A warp's first CACHE chunks of a step (column and value of entry lane of
// each chunk; column 0 and value 0 past the row's end).
template <int CACHE> struct LvlChunks {
    int32_t c[CACHE];
    double v[CACHE];
};
template <int CACHE>
__device__ __forceinline__ void lvl_load_chunks(const RowStep &st, const int32_t *__restrict__ col,
                                                const double *__restrict__ val, int lane, int G,
                                                int wg, LvlChunks<CACHE> &k) {
    const int nq = (st.len + 31) >> 5;
    const int nmine = nq > wg ? (nq - wg + G - 1) / G : 0;
#pragma unroll
    for (int i = 0; i < CACHE; ++i) {
        const int e = (wg + G * i) * 32 + lane;
        const bool h = i < nmine && e < st.len;
        k.c[i] = h ? __ldg(col + st.s + e) : 0;
        k.v[i] = h ? __ldg(val + st.s + e) : 0.0;
    }
}

template <int XM, int CACHE>
__device__ __forceinline__ void lvl_row(const RowStep &st, const int32_t *__restrict__ col,
                                        const double *__restrict__ val, const XAcc<XM> &X,
                                        const Box &box, int lane, int G, int wg, FxPart *parts,
                                        int bar, const LvlChunks<CACHE> &pre) {
    using R = typename XAcc<XM>::R;
    constexpr int B = 4;  // chunks per batch beyond the cached ones
    R cr[CACHE];
    double vv[CACHE], xo[CACHE];
    const int nq = (st.len + 31) >> 5;                      // chunks of the row
    const int nmine = nq > wg ? (nq - wg + G - 1) / G : 0;  // this warp's chunks
    int32_t cj[CACHE];
#pragma unroll
    for (int i = 0; i < CACHE; ++i) {
        cj[i] = pre.c[i];
        vv[i] = pre.v[i];
    }
#pragma unroll
    for (int i = 0; i < CACHE; ++i) {
        if (i >= nmine) break;
        cr[i] = X.ref(cj[i]);
    }
#pragma unroll
    for (int i = 0; i < CACHE; ++i) {
        if (i >= nmine) break;
        xo[i] = (wg + G * i) * 32 + lane < st.len ? X.ld(cr[i]) : 0.0;
    }
    double p0 = 0.0, p1 = 0.0;
#pragma unroll
    for (int i = 0; i < CACHE; ++i) {
        if (i >= nmine) break;
        if (i & 1) p1 = fma(xo[i], vv[i], p1);
        else p0 = fma(xo[i], vv[i], p0);
    }
    for (int i0 = CACHE; i0 < nmine; i0 += B) {
        R tr[B];
        bool th[B];
        double tv[B], tx[B];
        int32_t tj[B];
#pragma unroll
        for (int t = 0; t < B; ++t) {
            const int e = (wg + G * (i0 + t)) * 32 + lane;
            th[t] = i0 + t < nmine && e < st.len;
            tj[t] = th[t] ? __ldg(col + st.s + e) : 0;
            tv[t] = th[t] ? __ldg(val + st.s + e) : 0.0;
        }
#pragma unroll
        for (int t = 0; t < B; ++t) tr[t] = X.ref(tj[t]);
#pragma unroll
        for (int t = 0; t < B; ++t) tx[t] = th[t] ? X.ld(tr[t]) : 0.0;
#pragma unroll
        for (int t = 0; t < B; ++t) {
            if (t & 1) p1 = fma(tx[t], tv[t], p1);
            else p0 = fma(tx[t], tv[t], p0);
        }
    }
    const FxPart part = fx_warp_part(p0, p1, (wg == 0 && lane == 0) ? -st.b : 0.0);
    double resid;
    if (G > 1) {
        if (lane == 0) parts[wg] = part;
        asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(32 * G) : "memory");
        int E = 0;
        for (int w = 0; w < G; ++w) E = max(E, parts[w].e);
        if (E >= 0x7FF) {
            resid = 0.0;
            for (int w = 0; w < G; ++w)
                if (parts[w].e >= 0x7FF) resid += parts[w].d;
        } else {
            long long t = 0;
            for (int w = 0; w < G; ++w) {
                const int sh = E - parts[w].e;
                if (sh < 64) t += parts[w].s >> sh;
            }
            resid = fx_to_double_fast(t, E);
        }
    } else {
        resid = fx_part_double(part);
    }
    const double c = __dmul_rn(-resid, st.w);
#pragma unroll
    for (int i = 0; i < CACHE; ++i) {
        if (i >= nmine) break;
        if ((wg + G * i) * 32 + lane < st.len) X.st(cr[i], box.apply(fma(c, vv[i], xo[i])));
    }
    for (int i0 = CACHE; i0 < nmine; i0 += B) {
        R tr[B];
        bool th[B];
        double tv[B], tx[B];
        int32_t tj[B];
#pragma unroll
        for (int t = 0; t < B; ++t) {
            const int e = (wg + G * (i0 + t)) * 32 + lane;
            th[t] = i0 + t < nmine && e < st.len;
            tj[t] = th[t] ? __ldg(col + st.s + e) : 0;
            tv[t] = th[t] ? __ldg(val + st.s + e) : 0.0;
        }
#pragma unroll
        for (int t = 0; t < B; ++t) tr[t] = X.ref(tj[t]);
#pragma unroll
        for (int t = 0; t < B; ++t) tx[t] = th[t] ? X.ld(tr[t]) : 0.0;
#pragma unroll
        for (int t = 0; t < B; ++t)
            if (th[t]) X.st(tr[t], box.apply(fma(c, tv[t], tx[t])));
    }
}


// The levels in order on one cluster of gridDim.x blocks (CLUSTER) or one
// block. Groups of G consecutive warps take the steps of a level in turn; each
// group's first step of a level is known two levels ahead and its first
// chunks are loaded one level ahead (in registers). With x in
// (distributed) shared memory (XM = XS or XD, cb = log2 of a block's part), x
// is loaded at the start and written back at the end.
// A barrier of all blocks of a cooperative launch on one counter, gbar[0]
// (zero at the launch): block 0 adds 2^31 - (blocks - 1), every other block
// 1, so the counter's top bit flips exactly when the last block arrives -- one
// atomic per block and nothing to reset (the counter wraps). The arrival
// follows a fence (the block's writes of the level are visible first); the
// waiting thread reads the counter with acquire semantics. A block that waits
// more than kGridSpinLimit polls, or sees *gerr set (checked every 1024
// polls), sets *gerr and returns false; the sweep then stops, and the host
// reports the error.
constexpr unsigned long long kGridSpinLimit = 1ull << 26;
enum { SYNC_BLOCK = 0, SYNC_CLUSTER = 1, SYNC_GRID = 2 };

__device__ __forceinline__ bool grid_barrier(unsigned *gbar, int *gerr) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) : 1u;
        int ok = 1;
        __threadfence();
        const unsigned old = atomicAdd(gbar, add);
        for (unsigned long long it = 1;; ++it) {
            unsigned cur;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(gbar) : "memory");
            if ((cur ^ old) & 0x80000000u) break;
            if ((it & 1023u) == 0 && (it > kGridSpinLimit || *(volatile int *)gerr)) {
                atomicExch(gerr, 1);
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

template <int SYNC, int XM, int CACHE, int NT>
__global__ void __launch_bounds__(NT, 1) k_lvl_sweep(
        const RowStep *__restrict__ sched, const int64_t *__restrict__ lptr,
        const int *__restrict__ nlevp, const int32_t *__restrict__ col,
        const double *__restrict__ val, double *x, int32_t n, int cb, Box box, int G,
        const int *__restrict__ err, unsigned *gbar, int *gerr) {
    constexpr int NW = NT / 32;
    constexpr bool CLUSTER = SYNC == SYNC_CLUSTER;
    extern __shared__ __align__(16) double xsm[];
    __shared__ FxPart parts[2][NW];  // per group: two rows' parts (by parity), G each
    if (*err) return;
    const int nlev = *nlevp;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    XAcc<XM> X;
    int64_t part0 = 0, plen = 0;  // this block's part of x (XS: all of it)
    if constexpr (XM == XG) {
        X.x = x;
    } else {
        X.base = (uint32_t)__cvta_generic_to_shared(xsm);
        if constexpr (XM == XD) {
            X.cb = cb;
            part0 = (int64_t)cluster_rank() << cb;
            plen = (int64_t)1 << cb;
        } else {
            plen = n;
        }
        for (int64_t i = threadIdx.x; i < plen; i += NT)
            xsm[i] = part0 + i < n ? x[part0 + i] : 0.0;
    }
    if (CLUSTER) cluster_barrier();
    else __syncthreads();
    const int gl = wid / G, wg = wid - gl * G;  // group in the block, warp in the group
    const int64_t grp = (int64_t)blockIdx.x * (NW / G) + gl;
    const int64_t NG = (int64_t)gridDim.x * (NW / G);
    const int bar = 1 + gl;
    const RowStep none{0, 0, 0, 0.0, 0.0};
    // State at the start of level l: the bounds of levels l, l+1, l+2
    // ([a0, a1), [a1, a2), [a2, a3)); this group's first step of level l (cur,
    // its first chunks in pc) and of level l+1 (nxt). During level l the group
    // loads the bound after a3, its first step of level l+2 and the first
    // chunks of nxt, so that no level waits for a load of its own bounds,
    // steps or first entries; the rest of nxt's entries are prefetched into L2.
    auto bound = [&](int q) -> int64_t { return q <= nlev ? lptr[q] : lptr[nlev]; };
    int64_t a0 = 0, a1 = bound(1), a2 = bound(2), a3 = bound(3);
    RowStep cur = grp < a1 ? sched[grp] : none;
    RowStep nxt = a1 + grp < a2 ? sched[a1 + grp] : none;
    LvlChunks<CACHE> pc;
    lvl_load_chunks<CACHE>(cur, col, val, lane, G, wg, pc);
    for (int l = 0; l < nlev; ++l) {
        const int64_t a4 = bound(l + 4);
        const RowStep nxt2 = a2 + grp < a3 ? sched[a2 + grp] : none;
        LvlChunks<CACHE> pn;
        lvl_load_chunks<CACHE>(nxt, col, val, lane, G, wg, pn);
        int par = 0;
        for (int64_t k = a0 + grp; k < a1; k += NG, par ^= 1) {
            if (k == a0 + grp) {
                lvl_row<XM, CACHE>(cur, col, val, X, box, lane, G, wg, parts[par] + gl * G, bar, pc);
            } else {
                const RowStep st = sched[k];
                LvlChunks<CACHE> pk;
                lvl_load_chunks<CACHE>(st, col, val, lane, G, wg, pk);
                lvl_row<XM, CACHE>(st, col, val, X, box, lane, G, wg, parts[par] + gl * G, bar, pk);
            }
        }
        if (nxt.len > 32 * G * CACHE) {  // the rest of the next level's first step: into L2
            const char *c0 = reinterpret_cast<const char *>(col + nxt.s);
            const char *v0 = reinterpret_cast<const char *>(val + nxt.s);
            const int nc = (nxt.len * 4 + 127) >> 7, nv = (nxt.len * 8 + 127) >> 7;
            for (int i = wg * 32 + lane; i < nc + nv; i += 32 * G) {
                const char *p = i < nc ? c0 + ((size_t)i << 7) : v0 + ((size_t)(i - nc) << 7);
                asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
            }
        }
        if (SYNC == SYNC_CLUSTER) cluster_barrier();
        else if (SYNC == SYNC_GRID) {
            if (!grid_barrier(gbar, gerr)) return;
        } else {
            __syncthreads();
        }
        a0 = a1;
        a1 = a2;
        a2 = a3;
        a3 = a4;
        cur = nxt;
        nxt = nxt2;
        pc = pn;
    }
    if constexpr (XM != XG) {
        for (int64_t i = threadIdx.x; i < plen; i += NT)
            if (part0 + i < n) x[part0 + i] = xsm[i];
    }
}

int env_int(const char *name, int dflt) {
    const char *v = getenv(name);
    return v && *v ? atoi(v) : dflt;
}

// log2 of the power-of-two part of x per block when cs blocks hold n entries
int part_log2(int cs, int32_t n) {
    int cb = 0;
    while (((int64_t)cs << cb) < (int64_t)n) ++cb;
    return cb;
}

// The cluster shape of the level sweep: the largest of 16, 8, 4, 2 blocks
// (at most `want`) that the device can co-schedule, each with its part of x
// in shared memory (XD: 8 << part_log2 bytes, at most `room`) or none (XG);
// 1 if none can be had.
template <int XM, int CACHE, int NT>
int lvl_cluster_size(int want, int32_t n, size_t room) {
    auto kern = k_lvl_sweep<SYNC_CLUSTER, XM, CACHE, NT>;
    for (int cs = 16; cs >= 2; cs >>= 1) {
        if (cs > want) continue;
        const size_t smem = XM == XD ? (size_t)8 << part_log2(cs, n) : 0;
        if (XM == XD && smem > room) continue;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
            (cs > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(NT);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, kern, &cfg) == cudaSuccess && nc >= 1) return cs;
        cudaGetLastError();
    }
    return 1;
}

template <int XM, int CACHE, int NT>
int lvl_launch_cluster(int cs, size_t smem, const RowStep *sched, const int64_t *lptr,
                       const int *nlev, const int32_t *col, const double *val, double *x,
                       int32_t n, int cb, const Box &box, int G, const int *err, cudaStream_t s) {
    auto kern = k_lvl_sweep<SYNC_CLUSTER, XM, CACHE, NT>;
    FAIR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (cs > 8) FAIR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    FAIR_CUDA(cudaLaunchKernelEx(&cfg, kern, sched, lptr, nlev, col, val, x, n, cb, box, G, err,
                                 (unsigned *)nullptr, (int *)nullptr));
    return FAIR_OK;
}

// Launches the level sweep: x in the distributed shared memory of a cluster
// when its parts (a power of two per block) fit, else in global memory; one
// block with x in its shared memory when no cluster can be had.
// FAIR_SWEEP_CLUSTER caps the cluster size (1: one block), FAIR_SWEEP_XMEM
// picks x's place (0: global, 1: shared/distributed).
// The level sweep on a cooperative grid of nb blocks (x in global memory, the
// software grid barrier between levels); gsync: {barrier counter, unused, error}.
template <int CACHE, int NT>
int lvl_launch_grid(int nb, const RowStep *sched, const int64_t *lptr, const int *nlev,
                    const int32_t *col, const double *val, double *x, int32_t n, const Box &box,
                    int G, const int *err, int *gsync, cudaStream_t s) {
    auto kern = k_lvl_sweep<SYNC_GRID, XG, CACHE, NT>;
    FAIR_CUDA(cudaMemsetAsync(gsync, 0, 4 * sizeof(int), s));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(nb);
    cfg.blockDim = dim3(NT);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    FAIR_CUDA(cudaLaunchKernelEx(&cfg, kern, sched, lptr, nlev, col, val, x, n, 0, box, G, err,
                                 (unsigned *)gsync, gsync + 2));
    int gerr = 0;
    FAIR_CUDA(cudaMemcpyAsync(&gerr, gsync + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    if (gerr) {
        set_detail("Kaczmarz level sweep: a grid barrier timed out");
        return FAIR_ERR_CUDA;
    }
    return FAIR_OK;
}

// Blocks of a cooperative grid for a level sweep whose levels hold `spl`
// steps of G warps on average (room for twice that: the wavefront's levels
// vary), at most the co-resident blocks; 0 when the grid would not exceed the
// cluster (cs blocks).
template <int CACHE, int NT>
int lvl_grid_blocks(double spl, int G, int cs) {
    int want = (int)std::ceil(spl * 2.0 * G / (NT / 32));
    // FAIR_SWEEP_GRID_BLOCKS sets the count instead (tuning measurements),
    // still capped at the co-resident blocks
    const int forced = env_int("FAIR_SWEEP_GRID_BLOCKS", 0);
    if (forced > 0) want = forced;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_lvl_sweep<SYNC_GRID, XG, CACHE, NT>, NT, 0) !=
            cudaSuccess || occ < 1) {
        cudaGetLastError();
        return 0;
    }
    const int nb = std::min(want, occ * sm_count());
    return nb > cs ? nb : 0;
}

template <int CACHE, int NT>
int lvl_launch(const SweepDev &S, const RowStep *sched, const int64_t *lptr, const int *nlev,
               const Box &box, int G, const int *err, double spl, cudaStream_t s) {
    // cluster sizes found per device, x placement and image size (host
    // threads may sweep on different handles at once)
    static struct { int32_t n = -1; int want = 0, cs = 0; } cache[128][2];
    static std::mutex cache_mu;
    int dev = 0, optin = 0;
    FAIR_CUDA(cudaGetDevice(&dev));
    FAIR_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const int want = std::max(1, env_int("FAIR_SWEEP_CLUSTER", 16));
    const bool xmem = env_int("FAIR_SWEEP_XMEM", 1) != 0;
    const int32_t n = S.A->n;
    const int32_t *col = S.A->col.as<int32_t>();
    const double *val = S.A->v64.as<double>();
    const size_t room = (size_t)optin - 8192;  // beside the static parts
    auto cluster = [&](int xd) {
        std::lock_guard<std::mutex> lk(cache_mu);
        auto &c = cache[dev & 127][xd];
        if (c.n != n || c.want != want) {
            c.cs = xd ? lvl_cluster_size<XD, CACHE, NT>(want, n, room)
                      : lvl_cluster_size<XG, CACHE, NT>(want, n, room);
            c.n = n;
            c.want = want;
        }
        return c.cs;
    };
    // levels with more steps than one round of the cluster's groups: a
    // cooperative grid (FAIR_SWEEP_GRID=0 keeps the cluster, 1 forces the grid)
    {
        const int gmode = env_int("FAIR_SWEEP_GRID", -1);
        const int cs = cluster(xmem ? 1 : 0);
        int nb = gmode == 0 ? 0 : lvl_grid_blocks<CACHE, NT>(spl, G, std::max(cs, 1));
        if (gmode == 1 && nb == 0) nb = std::min(2 * std::max(cs, 1), sm_count());
        if (nb > 0 && S.work)
            return lvl_launch_grid<CACHE, NT>(nb, sched, lptr, nlev, col, val, S.x, n, box, G, err,
                                              S.work->gsync.as<int>(), s);
    }
    if (xmem) {
        const int cs = cluster(1);
        if (cs >= 2) {
            const int cb = part_log2(cs, n);
            return lvl_launch_cluster<XD, CACHE, NT>(cs, (size_t)8 << cb, sched, lptr, nlev, col, val,
                                                     S.x, n, cb, box, G, err, s);
        }
        if ((size_t)8 * n <= room) {
            auto kern = k_lvl_sweep<SYNC_BLOCK, XS, CACHE, NT>;
            FAIR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(8 * (size_t)n)));
            kern<<<1, NT, 8 * (size_t)n, s>>>(sched, lptr, nlev, col, val, S.x, n, 0, box, G, err, nullptr,
                                               nullptr);
            FAIR_CUDA(cudaGetLastError());
            return FAIR_OK;
        }
    }
    const int cs = cluster(0);
    if (cs <= 1) {
        k_lvl_sweep<SYNC_BLOCK, XG, CACHE, NT><<<1, NT, 0, s>>>(sched, lptr, nlev, col, val, S.x, n,
                                                               0, box, G, err, nullptr, nullptr);
        FAIR_CUDA(cudaGetLastError());
        return FAIR_OK;
    }
    return lvl_launch_cluster<XG, CACHE, NT>(cs, 0, sched, lptr, nlev, col, val, S.x, n, 0, box, G,
                                             err, s);
}

// The levels on a 16-block cluster (the level table in global memory);
// false when no such cluster can be had (FAIR_SWEEP_CLUSTER below 16 also
// keeps the single block).
bool lvl_levels_cluster(SweepWork &W, int32_t nord, int *nlev, cudaStream_t s) {
    if (env_int("FAIR_SWEEP_CLUSTER", 16) < 16) return false;
    auto kern = k_lvl_levels_cluster<16>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(512);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 16;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, kern, &cfg) != cudaSuccess || nc < 1) {
        cudaGetLastError();
        return false;
    }
    if (cudaMemsetAsync(nlev, 0, sizeof(int), s) != cudaSuccess ||
        cudaLaunchKernelEx(&cfg, kern, (const WinRow *)W.rec.as<WinRow>(),
                           (const signed char *)W.dpath.as<signed char>(),
                           (const int32_t *)W.idx.as<int32_t>(), nord, W.lvtab.as<int32_t>(),
                           W.lvl.as<int32_t>(), nlev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return true;
}

// Builds (or takes from the cache of this sweep order) the level schedule and
// launches the level sweep. Returns FAIR_OK with *done = false (nothing
// launched) when its buffers cannot be had; the caller then runs the
// single-block kernel alone.
int lvl_sweep(const SweepDev &S, int dir, const RowStep *steps, const Box &box, bool *done,
              cudaStream_t s) {
    *done = false;
    SweepWork &W = *S.work;
    const DevCSR &A = *S.A;
    const int slot = dir > 0 ? 0 : 1;
    SweepWork::Levels &C = W.lev[slot];
    const bool cached = S.order_key != 0 && C.key == S.order_key && C.nord == S.nord;
    // orders drawn anew in every sweep get no levels, only (once per call) the
    // set-up's check for rows that repeat a column
    const bool want = S.order_key != 0 || env_int("FAIR_SWEEP_LEVELS_ALWAYS", 0);
    if (!want && W.err_valid) return FAIR_OK;
    if (!cached) {
        C.key = 0;
        const int32_t nord = S.nord;
        const int nwin = (nord + kWinRows - 1) / kWinRows;
        const size_t tab_row = (size_t)std::max<int32_t>(A.n, 1) * sizeof(unsigned long long);
        int blocks = std::min(nwin, 2 * sm_count());
        blocks = (int)std::max<size_t>(1, std::min<size_t>((size_t)blocks, ((size_t)2 << 30) / tab_row));
        const int64_t max_win = (int64_t)kWinRows * std::max(A.max_row, 1);
        if (max_win >= (1 << kStampPosBits)) return FAIR_OK;
        // the entries of this sweep: an upper bound from the longest row
        const size_t ent = (size_t)nord * (size_t)std::max(A.max_row, 1);
        if (W.lens.grow(4 * ((size_t)nord + 1)) || W.eoff.grow(8 * ((size_t)nord + 1)) ||
            W.idx.grow(4 * ent) || W.rec.grow(sizeof(WinRow) * (size_t)nord) ||
            W.dpath.grow((size_t)kWinRows * ((size_t)nord + kWinRows)) || W.lvl.grow(4 * (size_t)nord) ||
            W.cnt.grow(4 * ((size_t)nord + 1)) || W.err.grow(sizeof(int)) ||
            C.sched.grow(sizeof(RowStep) * (size_t)nord) || C.lptr.grow(8 * ((size_t)nord + 2)) ||
            C.dnlev.grow(sizeof(int))) {
            W.release();
            return FAIR_OK;
        }
        if (W.tab_n != A.n || W.tab_blocks < blocks || W.uid + (uint64_t)nwin >= kStampIdLimit) {
            W.tabs.release();
            W.tab_n = 0;
            W.tab_blocks = 0;
            if (W.tabs.grow(tab_row * (size_t)blocks)) return FAIR_OK;
            FAIR_CUDA(cudaMemsetAsync(W.tabs.p, 0xFF, tab_row * (size_t)blocks, s));
            W.tab_n = A.n;
            W.tab_blocks = blocks;
            W.uid = 0;
        }
        int dev = 0, optin = 0;
        FAIR_CUDA(cudaGetDevice(&dev));
        FAIR_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        const int g = (int)std::min<int64_t>((nord + 255) / 256, (int64_t)sm_count() * 4);
        k_step_lengths<<<g, 256, 0, s>>>(steps, nord, W.lens.as<int32_t>());
        k_scan_excl<<<1, 1024, 0, s>>>(W.lens.as<int32_t>(), nord, nullptr, W.eoff.as<int64_t>());
        FAIR_CUDA(cudaMemsetAsync(W.err.p, 0, sizeof(int), s));
        const size_t setup_smem = (size_t)max_win;
        if (setup_smem + 1024 > (size_t)optin) return FAIR_OK;
        FAIR_CUDA(cudaFuncSetAttribute(k_lvl_setup, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)setup_smem));
        k_lvl_setup<<<blocks, kSetupThreads, setup_smem, s>>>(
            steps, W.eoff.as<int64_t>(), nord, A.col.as<int32_t>(), W.tabs.as<unsigned long long>(),
            A.n, W.uid, W.idx.as<int32_t>(), W.rec.as<WinRow>(), W.dpath.as<signed char>(),
            W.err.as<int>());
        FAIR_CUDA(cudaGetLastError());
        W.err_valid = true;
        W.uid += (uint64_t)nwin;
        if (!want) return FAIR_OK;
        const size_t lv_bytes = 4 * (size_t)std::max<int32_t>(A.n, 1);
        if (lv_bytes + 2048 <= (size_t)optin) {
            FAIR_CUDA(cudaFuncSetAttribute(k_lvl_levels<true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lv_bytes));
            k_lvl_levels<true><<<1, 1024, lv_bytes, s>>>(W.rec.as<WinRow>(), W.dpath.as<signed char>(),
                                                        W.idx.as<int32_t>(), nord, nullptr, A.n,
                                                        W.lvl.as<int32_t>(), C.dnlev.as<int>());
        } else {
            if (W.lvtab.grow(lv_bytes)) {
                W.release();
                return FAIR_OK;
            }
            FAIR_CUDA(cudaMemsetAsync(W.lvtab.p, 0, lv_bytes, s));
            if (!lvl_levels_cluster(W, nord, C.dnlev.as<int>(), s))
                k_lvl_levels<false><<<1, 1024, 0, s>>>(W.rec.as<WinRow>(), W.dpath.as<signed char>(),
                                                      W.idx.as<int32_t>(), nord,
                                                      W.lvtab.as<int32_t>(), A.n,
                                                      W.lvl.as<int32_t>(), C.dnlev.as<int>());
        }
        FAIR_CUDA(cudaGetLastError());
        FAIR_CUDA(cudaMemsetAsync(W.cnt.p, 0, 4 * ((size_t)nord + 1), s));
        k_lvl_count<<<g, 256, 0, s>>>(W.lvl.as<int32_t>(), nord, W.cnt.as<int32_t>());
        k_scan_excl<<<1, 1024, 0, s>>>(W.cnt.as<int32_t>(), 0, C.dnlev.as<int>(), C.lptr.as<int64_t>());
        k_lvl_scatter<<<g, 256, 0, s>>>(steps, W.lvl.as<int32_t>(), nord, C.lptr.as<int64_t>(),
                                        W.cnt.as<int32_t>(), C.sched.as<RowStep>());
        FAIR_CUDA(cudaGetLastError());
        // levels pay when they hold several steps each (the ray orders: 30-80);
        // an order whose steps nearly all depend on the one before runs on the
        // single-block kernel
        FAIR_CUDA(cudaMemcpyAsync(&C.nlev, C.dnlev.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        FAIR_CUDA(cudaMemcpyAsync(&C.entries, W.eoff.as<int64_t>() + nord, sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, s));
        FAIR_CUDA(cudaStreamSynchronize(s));
        C.use = (int64_t)nord >= (int64_t)kMinStepsPerLevel * std::max(C.nlev, 1) ||
                env_int("FAIR_SWEEP_LEVELS_ALWAYS", 0);
        C.key = S.order_key;
        C.nord = nord;
    }
    if (!C.use) return FAIR_OK;
    const RowStep *sched = C.sched.as<RowStep>();
    const int64_t *lptr = C.lptr.as<int64_t>();
    const int *nlev = C.dnlev.as<int>();
    const int *err = W.err.as<int>();
    // warps per step: a long row (twice the mean, at most the longest) in 2
    // chunks of 32 entries per warp, at most 16 warps (a block): a warp's
    // FP64 instructions per step (64 cycles each) are on the level's critical
    // path. Measured (GB300, 10 sweeps of fan N=128 on the cluster, s): G = 1
    // 0.061, 2 0.041, 4 0.036, 8 0.038; 20 sweeps of fan N=512 symmetric on
    // the cooperative grid (s, blocks): G = 4 0.66 (26), 8 0.58 (51) / 0.52
    // (152), 16 0.47 (101) / 0.42 (152). FAIR_SWEEP_GROUP overrides (1, 2, 4,
    // 8 or 16).
    const double avg = S.nord > 0 ? (double)C.entries / S.nord : 0.0;
    int G = 1;
    while (G < 16 && 64.0 * G < std::min(2.0 * avg, (double)A.max_row)) G *= 2;
    const int Ge = env_int("FAIR_SWEEP_GROUP", 0);
    if (Ge == 1 || Ge == 2 || Ge == 4 || Ge == 8 || Ge == 16) G = Ge;
    if (W.gsync.grow(4 * sizeof(int))) return FAIR_OK;
    const double spl = C.nlev > 0 ? (double)S.nord / C.nlev : 1.0;
    FAIR_TRY((lvl_launch<2, 512>(S, sched, lptr, nlev, box, G, err, spl, s)));
    *done = true;
    return FAIR_OK;
}

}  // namespace

void SweepWork::release() {
    steps.release();
    lens.release();
    eoff.release();
    idx.release();
    rec.release();
    dpath.release();
    lvl.release();
    cnt.release();
    lvtab.release();
    err.release();
    tabs.release();
    gsync.release();
    for (Levels &L : lev) {
        L.sched.release();
        L.lptr.release();
        L.dnlev.release();
        L.key = 0;
        L.nord = L.nlev = 0;
        L.entries = 0;
        L.use = false;
    }
    tab_n = tab_blocks = 0;
    uid = 0;
    err_valid = false;
}

int kaczmarz_sweep(const SweepDev &S, int dir, cudaStream_t s) {
    if (S.nord <= 0) return FAIR_OK;
    SweepWork local;
    SweepWork &W = S.work ? *S.work : local;
    SweepDev SW = S;
    SW.work = &W;
    FAIR_TRY(W.steps.grow(sizeof(RowStep) * (size_t)S.nord));
    RowStep *steps = W.steps.as<RowStep>();
    const DevCSR &A = *S.A;
    int grid = (int)std::min<int64_t>(((int64_t)S.nord + 255) / 256, (int64_t)sm_count() * 8);
    k_sweep_schedule<<<grid, 256, 0, s>>>(S.ord, S.nord, dir, S.rand_rowprob ? 1 : 0, S.cumul, A.m,
                                          S.seed, S.ctr, A.rowptr.as<int64_t>(), S.b, S.nrA,
                                          S.omg, steps);
    FAIR_CUDA(cudaGetLastError());
    Box box;
    // a NaN bound leaves t unchanged unless t is NaN (MAX/MIN semantics); the
    // bound is then dropped, which differs only in the NaN payload
    box.mode = (S.bmode & 2) && !std::isnan(S.lb) ? 2 : 0;
    box.mode |= (S.bmode & 1) && !std::isnan(S.ub) ? 1 : 0;
    box.lb = S.lb;
    box.ub = S.ub;
    box.klb = host_key(S.lb);
    box.kub = host_key(S.ub);
    // the level sweep, and the single-block kernel behind it for a matrix
    // whose rows repeat a column (it runs only if the set-up said so);
    // FAIR_SWEEP_LEGACY=1 runs the single-block kernel alone
    bool leveled = false;
    const int *dup = nullptr;
    if (!env_int("FAIR_SWEEP_LEGACY", 0)) {
        FAIR_TRY(lvl_sweep(SW, dir, steps, box, &leveled, s));
        if (W.err_valid) dup = W.err.as<int>();
    }
    int dev = 0, optin = 0;
    FAIR_CUDA(cudaGetDevice(&dev));
    FAIR_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t need = sizeof(double) * (size_t)A.n;
    const bool smem = need + 4096 <= (size_t)optin;
    const int Wl = sweep_warps();
    const int oid = leveled ? 1 : 0;
    // entries per lane held in registers (longer rows finish in a loop)
    const int per_lane = (A.max_row + 32 * Wl - 1) / (32 * Wl);
    int st;
    switch (Wl) {
    case 1: st = per_lane <= 8 ? launch<1, 8>(SW, steps, smem, need, box, dup, oid, s)
                               : launch<1, 16>(SW, steps, smem, need, box, dup, oid, s);
        break;
    case 2: st = per_lane <= 8 ? launch<2, 8>(SW, steps, smem, need, box, dup, oid, s)
                               : launch<2, 16>(SW, steps, smem, need, box, dup, oid, s);
        break;
    case 4: st = per_lane <= 4 ? launch<4, 4>(SW, steps, smem, need, box, dup, oid, s)
                               : launch<4, 8>(SW, steps, smem, need, box, dup, oid, s);
        break;
    default: st = per_lane <= 2 ? launch<8, 2>(SW, steps, smem, need, box, dup, oid, s)
                                : launch<8, 4>(SW, steps, smem, need, box, dup, oid, s);
    }
    if (!S.work) {
        cudaStreamSynchronize(s);
        local.release();
    }
    return st;
}

}  // namespace fair
