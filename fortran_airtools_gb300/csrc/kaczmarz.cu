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

template <int W, int CACHE, bool SMEM_X>
__global__ void __launch_bounds__(32 * W) k_sweep(const RowStep *__restrict__ steps, int32_t nord,
                                                  const int32_t *__restrict__ col,
                                                  const double *__restrict__ val, double *xg,
                                                  int32_t n, Box box) {
    constexpr int T = 32 * W;
    extern __shared__ double xs[];
    __shared__ FxPart part_s[W];
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
           cudaStream_t s) {
    const DevCSR &A = *S.A;
    if (smem) {
        auto kern = k_sweep<W, CACHE, true>;
        FAIR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem_bytes));
        kern<<<1, 32 * W, smem_bytes, s>>>(steps, S.nord, A.col.as<int32_t>(), A.v64.as<double>(),
                                          S.x, A.n, box);
    } else {
        k_sweep<W, CACHE, false><<<1, 32 * W, 0, s>>>(steps, S.nord, A.col.as<int32_t>(),
                                                     A.v64.as<double>(), S.x, A.n, box);
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

}  // namespace

int kaczmarz_sweep(const SweepDev &S, int dir, cudaStream_t s) {
    if (S.nord <= 0) return FAIR_OK;
    static thread_local DevBuf stepbuf;  // schedule of one sweep (grown on demand)
    FAIR_TRY(stepbuf.grow(sizeof(RowStep) * (size_t)S.nord));
    RowStep *steps = stepbuf.as<RowStep>();
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
    int dev = 0, optin = 0;
    FAIR_CUDA(cudaGetDevice(&dev));
    FAIR_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t need = sizeof(double) * (size_t)A.n;
    const bool smem = need + 4096 <= (size_t)optin;
    const int W = sweep_warps();
    // entries per lane held in registers (longer rows finish in a loop)
    const int per_lane = (A.max_row + 32 * W - 1) / (32 * W);
    switch (W) {
    case 1: return per_lane <= 8 ? launch<1, 8>(S, steps, smem, need, box, s)
                                 : launch<1, 16>(S, steps, smem, need, box, s);
    case 2: return per_lane <= 8 ? launch<2, 8>(S, steps, smem, need, box, s)
                                 : launch<2, 16>(S, steps, smem, need, box, s);
    case 4: return per_lane <= 4 ? launch<4, 4>(S, steps, smem, need, box, s)
                                 : launch<4, 8>(S, steps, smem, need, box, s);
    default: return per_lane <= 2 ? launch<8, 2>(S, steps, smem, need, box, s)
                                  : launch<8, 4>(S, steps, smem, need, box, s);
    }
}

}  // namespace fair
