// mfree.cu -- matrix-free projector / backprojector pairs (parallel beam and
// fan beam) and SIRT on them (include/fair_mf.h).
//
// Geometry of paralleltomo (system_generation.f90:309-492): ray (angle i,
// bin j) is the line with unit normal n_i = (cos th_i, sin th_i) at offset
// x0_j = j - (p-1)/2 (linspace(-(p-1)/2, (p-1)/2, p), unit bins), direction
// (-sin, cos). Pixel (ix, iy) (ix from the left, iy from the bottom, both
// 0..N-1) is the unit square centred at (ix + 1/2 - N/2, iy + 1/2 - N/2) and
// is column ix*N + (N-1-iy) of the matrix (JA = floor(xm)*N + (N - floor(ym))).
//
// The ray's length inside a unit square is a function of the signed distance
// d between the square's centre and the line (the chord of a unit square):
// with c = max(|cos|, |sin|), s = min(...):
//   L = 1/c                      for |d| <= (c - s)/2,
//   L = ((c + s)/2 - |d|)/(c s)  for (c - s)/2 < |d| < (c + s)/2,  else 0,
// which is the segment length the ray tracer measures between consecutive
// crossings; segments of 1e-10 or less are dropped, as there. An axis-aligned
// ray on a grid line (s = 0, |d| = 1/2) belongs to the pixel on the positive
// side, as the reference's floor-of-midpoint rule gives.
//
// d = ix*cos + iy*sin + K_i - j with K_i = (1/2 - N/2)(cos + sin) + (p-1)/2,
// evaluated in 64-bit fixed point with 46 fractional bits (N <= 8192 and
// p <= 16384 keep every term below 2^60): exact integer
// arithmetic, so every kernel computes bit-identical entries whatever the
// order it meets the (ray, pixel) pairs in. The projector runs one thread
// per ray and walks the image along the ray's faster axis (per column when
// |sin| >= |cos|, else per row); at each step the only pixels within H2 of
// the ray are the two that bracket its crossing, which the walk tracks
// exactly with one 64-bit add per step. The backprojector runs one thread per
// 4 pixels of an image column and, per angle, evaluates the two rays whose
// offsets bracket each pixel's. Both keep only pairs with L > 0, so they sum
// the same entries: an exact adjoint pair, deterministic, without atomics.
//
// Fan beam (fanlineartomo, system_generation.f90:79-307): ray (i, j) is the
// line through the rotated source P_i with direction u_ij = R(omega_j) u0_i,
// computed on the host exactly as the reference does (cos/sin of the bin
// angles, the same products and sums). Its unit normal n = (b, -a)/|u| and
// K_ij = n . ((1/2 - N/2, 1/2 - N/2) - P_i) give d = ix*n_x + iy*n_y + K_ij,
// the same fixed-point form, one record per ray. The projector walks each ray
// as above (and the rays that walk image rows read a transposed copy of x, so
// that a warp's rays gather adjacent addresses); the backprojector finds, per
// pixel and angle, the rays whose bin
// angle omega_j lies within asin(0.7072/|c - P_i|) (+ 2e-4) of the angle of
// the pixel centre c seen from the source (a binary search over the bin
// angles, sorted once: the reference's odd-p angles are not monotone in j),
// and tests them with the exact distance.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "fair_internal.cuh"
#include "fair_mf.h"
#include "sirt_epi.cuh"

namespace fair {

namespace {

constexpr int kFix = 46;
constexpr double kOne = 70368744177664.0;  // 2^46

// The first 48 bytes hold what the FP32 backprojector reads per angle (three
// 16-byte loads), the next 32 what FP64 adds.
struct __align__(16) MfAngle {
    long long C, S;      // cos, sin in fixed point
    long long K, H2;     // K_i; (c + s)/2 in fixed point
    int H2s;             // H2 truncated to 30 fractional bits (FP32 entries)
    float inv_c;         // 1/c
    float ramp30;        // 2^-30 / s (0 when s = 0)
    int tie;             // s = 0: +1 / -1 = sign of d that keeps |d| = 1/2; 0 otherwise
    long long H1;        // (c - s)/2 in fixed point
    long long Hcut;      // |d| >= Hcut leaves a segment of at most 1e-10: dropped
    double inv_c64, scale_ramp64;
    float Cf, Sf, Kf;    // float copies for the walk's step range
    int by_column;       // 1: walk columns (|sin| >= |cos|)
};
static_assert(sizeof(MfAngle) == 96, "MfAngle layout");

// The fields of record p that a backprojector of entries T reads: the first
// 48 bytes (FP32), or 80 (FP64), by 16-byte loads.
template <typename T>
__device__ __forceinline__ MfAngle mf_load(const MfAngle *p) {
    const int4 *q = reinterpret_cast<const int4 *>(p);
    auto ll = [](int lo, int hi) { return (long long)(((unsigned long long)(unsigned)hi << 32) | (unsigned)lo); };
    MfAngle A;
    const int4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    A.C = ll(a.x, a.y);
    A.S = ll(a.z, a.w);
    A.K = ll(b.x, b.y);
    A.H2 = ll(b.z, b.w);
    A.H2s = c.x;
    A.inv_c = __int_as_float(c.y);
    A.ramp30 = __int_as_float(c.z);
    A.tie = c.w;
    if constexpr (sizeof(T) == 8) {
        const int4 d = __ldg(q + 3), e = __ldg(q + 4);
        A.H1 = ll(d.x, d.y);
        A.Hcut = ll(d.z, d.w);
        A.inv_c64 = __hiloint2double(e.y, e.x);
        A.scale_ramp64 = __hiloint2double(e.w, e.z);
    }
    return A;
}

template <typename T> struct Chord;
// The chord of a unit pixel at |d| = ad < 2^47 from the line: ramp() for s > 0,
// tied() for an axis-aligned line (s = 0), where tu = H2 when a ray on the
// pixel's edge, on this side of it, keeps the pixel (else -1); at() picks one.
// FP32 entries evaluate the ramp on the exact distance truncated to 30
// fractional bits, as (1/c) sat((H2 - |d|) / s) with sat() the clamp to
// [0, 1] (two multiplies on the FMA pipe; the cut of segments below 1e-10 is
// left to the FP64 entries); every kernel evaluates the same expression on
// the same exact value, so they agree bit for bit.
template <> struct Chord<float> {
    static __device__ __forceinline__ float ramp(const MfAngle &A, long long ad) {
        const int u = (int)(ad >> 16);
        return A.inv_c * __saturatef((float)(A.H2s - u) * A.ramp30);
    }
    static __device__ __forceinline__ float tied(const MfAngle &A, long long ad, long long tu) {
        return ad < A.H2 || ad == tu ? A.inv_c : 0.f;
    }
    static __device__ __forceinline__ float at(const MfAngle &A, long long ad, long long tu) {
        return A.tie != 0 ? tied(A, ad, tu) : ramp(A, ad);
    }
    static __device__ __forceinline__ float of(const MfAngle &A, long long d) {
        const long long ad = d < 0 ? -d : d;
        if (ad >= (1LL << 47)) return 0.f;  // more than two pixels away
        return at(A, ad, A.tie == (d > 0 ? 1 : -1) ? A.H2 : -1);
    }
};
template <> struct Chord<double> {
    static __device__ __forceinline__ double ramp(const MfAngle &A, long long ad) {
        const double w = ad <= A.H1 ? A.inv_c64 : (double)(A.H2 - ad) * A.scale_ramp64;
        return ad < A.Hcut ? w : 0.0;
    }
    static __device__ __forceinline__ double tied(const MfAngle &A, long long ad, long long tu) {
        return ad < A.H2 || ad == tu ? A.inv_c64 : 0.0;
    }
    static __device__ __forceinline__ double at(const MfAngle &A, long long ad, long long tu) {
        return A.tie != 0 ? tied(A, ad, tu) : ramp(A, ad);
    }
    static __device__ __forceinline__ double of(const MfAngle &A, long long d) {
        const long long ad = d < 0 ? -d : d;
        return at(A, ad, A.tie == (d > 0 ? 1 : -1) ? A.H2 : -1);
    }
};

// ---- epilogues of the projector (per ray) and backprojector (per pixel) ---------
template <typename T> struct EpiStore {  // y = A x (or A' r)
    T *y;
    __device__ void operator()(int64_t i, T acc) const { y[i] = acc; }
};
struct EpiCimminoW {  // M = m * sum_j a_ij^2 (the sum arrives in acc)
    double *M;
    double m;
    __device__ void operator()(int64_t i, double acc) const { M[i] = m * acc; }
};

// One entry a_rq = w of a pass (valid: pixel q exists): MODE 0 adds w * v_q
// (v read only for w > 0, as a stored matrix reads only its entries), MODE 1
// adds w, MODE 2 w^2, MODE 3 counts w > 0.
template <typename VT, typename ACC, int MODE>
__device__ __forceinline__ void mf_add(ACC &acc, ACC w, bool valid, const VT *__restrict__ v,
                                       int64_t q) {
    if (MODE == 0) {
        const ACC vq = valid && w > (ACC)0 ? (ACC)__ldg(v + q) : (ACC)0;
        acc += w * vq;
    } else if (MODE == 1) {
        acc += valid ? w : (ACC)0;
    } else if (MODE == 2) {
        acc += valid ? w * w : (ACC)0;
    } else {
        acc += valid && w > (ACC)0 ? (ACC)1 : (ACC)0;
    }
}

// The steps of one ray (see k_mf_project): E = |d| at pixel ua, Qa - E at
// ua + 1; a step lowers E by Fw and moves ua down by one when E leaves
// [0, Qa). TIE: an axis-aligned ray (tied chords). Two steps per iteration,
// so that their gathers are in flight together.
template <typename XT, typename ACC, int MODE, bool TIE>
__device__ __forceinline__ ACC mf_walk(const MfAngle &A, long long E, int ua, long long Qa,
                                       long long Fw, const XT *__restrict__ xv, int qt, int su,
                                       int dqt, int N, int cnt, long long tua, long long tub) {
    ACC acc = 0;
    auto step = [&](ACC &wa, ACC &wb, int &qa, bool &va, bool &vb) {
        if constexpr (TIE) {
            wa = Chord<ACC>::tied(A, E, tua);
            wb = Chord<ACC>::tied(A, Qa - E, tub);
        } else {
            wa = Chord<ACC>::ramp(A, E);
            wb = Chord<ACC>::ramp(A, Qa - E);
        }
        qa = qt + ua * su;
        va = (unsigned)ua < (unsigned)N;
        vb = (unsigned)(ua + 1) < (unsigned)N;
        E -= Fw;
        if (E < 0) {
            --ua;
            E += Qa;
        }
        qt += dqt;
    };
    for (; cnt >= 2; cnt -= 2) {
        ACC w0, w1, w2, w3;
        int q0, q1;
        bool v0, v1, v2, v3;
        step(w0, w1, q0, v0, v1);
        step(w2, w3, q1, v2, v3);
        mf_add<XT, ACC, MODE>(acc, w0, v0, xv, q0);
        mf_add<XT, ACC, MODE>(acc, w1, v1, xv, q0 + su);
        mf_add<XT, ACC, MODE>(acc, w2, v2, xv, q1);
        mf_add<XT, ACC, MODE>(acc, w3, v3, xv, q1 + su);
    }
    if (cnt > 0) {
        ACC w0, w1;
        int q0;
        bool v0, v1;
        step(w0, w1, q0, v0, v1);
        mf_add<XT, ACC, MODE>(acc, w0, v0, xv, q0);
        mf_add<XT, ACC, MODE>(acc, w1, v1, xv, q0 + su);
    }
    return acc;
}

// Per ray r: MODE 0 sums a_rj * x_j, MODE 1 sums a_rj, MODE 2 sums a_rj^2,
// MODE 3 counts the pixels with a_rj > 0 (x unused for MODE 1-3).
// FAN: ang holds one record per ray (K its own offset), else one per angle
// (ray j of angle i at offset K - j).
//
// The ray walks its faster axis t (|F| <= |Q|): with g = sign(Q) d =
// t Fp + u Qa + Gk, the pixels u of step t with |d| <= H2 (< Qa) lie within
// one pixel of u* = -(t Fp + Gk)/Qa, so they are ua = floor(u*) and ua + 1,
// at |d| = -g(t, ua) in [0, Qa) and Qa - that. The walk keeps ua and that
// distance exactly: a step changes g by |Fp| (the walk runs in the direction
// that makes the change non-negative). Only steps whose candidates can lie
// in the image are walked (a float bound, widened).
//
// x is read as x[ix*N + N-1-iy] by the rays that walk columns (a warp's
// adjacent rays then gather adjacent pixels of one column) and as its
// transpose xt[(N-1-iy)*N + ix] by those that walk rows (adjacent pixels of
// one row).
template <typename XT, typename ACC, int MODE, bool FAN, class Epi>
__global__ void __launch_bounds__(128) k_mf_project(const MfAngle *__restrict__ ang, int nth,
                                                    int p, int N, const XT *__restrict__ x,
                                                    const XT *__restrict__ xt, Epi epi) {
    const int64_t m = (int64_t)nth * p;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(r / p), j = (int)(r - (int64_t)i * p);
        const MfAngle &A = ang[FAN ? r : i];
        const long long K = FAN ? A.K : A.K - ((long long)j << kFix);
        const float Kf = FAN ? A.Kf : A.Kf - (float)j;
        const bool col = A.by_column != 0;
        const long long F = col ? A.C : A.S, Q = col ? A.S : A.C;
        const float Ff = col ? A.Cf : A.Sf, Qf = col ? A.Sf : A.Cf;
        const int sq = Q > 0 ? 1 : -1;
        const long long Qa = Q > 0 ? Q : -Q, Fp = sq * F, Gk = sq * K;
        const float Qaf = fabsf(Qf), Fpf = sq * Ff, Gkf = sq * Kf;
        // steps with u* in [-1, N): -N Qa < t Fp + Gk <= Qa (widened by 0.05)
        const float lo = -(float)N * Qaf - 0.05f - Gkf, hi = Qaf + 0.05f - Gkf;
        float ta = 0.f, tb = (float)(N - 1);
        if (Fpf > 0.f) {
            ta = fmaxf(ta, lo / Fpf);
            tb = fminf(tb, hi / Fpf);
        } else if (Fpf < 0.f) {
            ta = fmaxf(ta, hi / Fpf);
            tb = fminf(tb, lo / Fpf);
        } else if (!(lo < 0.f && hi >= 0.f)) {
            tb = -1.f;
        }
        const int t0 = max(0, (int)floorf(ta)), t1 = min(N - 1, (int)ceilf(tb));
        ACC acc = 0;
        if (t0 <= t1) {
            const int dir = Fp >= 0 ? 1 : -1;
            const long long Fw = Fp >= 0 ? Fp : -Fp;
            const int ts = dir > 0 ? t0 : t1;
            const long long G = (long long)ts * Fp + Gk;
            int ua = (int)floorf(-(float)G / (float)Qa);
            long long e = G + (long long)ua * Qa;
            while (e > 0) { --ua; e -= Qa; }
            while (e <= -Qa) { ++ua; e += Qa; }
            // pixel (t, u): element qt + u su of xv
            const XT *__restrict__ xv = col ? x : xt;
            const int su = col ? -1 : 1, dqt = col ? dir * N : -dir * N;
            const int qt = col ? ts * N + N - 1 : (N - 1 - ts) * N;
            if (A.tie != 0) {
                // d at ua is sign(Q) e <= 0, at ua + 1 sign(Q) (e + Qa) > 0
                const long long tua = A.tie == -sq ? A.H2 : -1, tub = A.tie == sq ? A.H2 : -1;
                acc = mf_walk<XT, ACC, MODE, true>(A, -e, ua, Qa, Fw, xv, qt, su, dqt, N,
                                                   t1 - t0 + 1, tua, tub);
            } else {
                acc = mf_walk<XT, ACC, MODE, false>(A, -e, ua, Qa, Fw, xv, qt, su, dqt, N,
                                                    t1 - t0 + 1, -1, -1);
            }
        }
        epi(r, acc);
    }
}

// xt = the transpose of x viewed as an N x N array (32 x 32 tiles through
// shared memory, both sides coalesced).
template <typename T>
__global__ void __launch_bounds__(256) k_mf_transpose(const T *__restrict__ x, T *__restrict__ xt,
                                                      int N) {
    __shared__ T tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = r0 + k, c = c0 + threadIdx.x;
        if (r < N && c < N) tile[k][threadIdx.x] = x[(int64_t)r * N + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = c0 + k, c = r0 + threadIdx.x;
        if (r < N && c < N) xt[(int64_t)r * N + c] = tile[threadIdx.x][k];
    }
}

// Sum over the rays through pixel q of a_rq * y_r, for every pixel; MODE 1
// sums a_rq (y unused). A thread takes PB vertically adjacent pixels of one
// image column (iy0, iy0 - 1, ...), which share the per-angle set-up. With
// D = ix C + iy S + K = jh 2^46 + dl (0 <= dl < 2^46), the rays j with
// |D - j 2^46| <= H2 (< 2^46) are jh (d = dl) and jh + 1 (d = dl - 2^46).
template <typename YT, typename ACC, int MODE, int PB, bool TIE>
__device__ __forceinline__ void bp_angle(const MfAngle &A, long long D, int p,
                                         const YT *__restrict__ yi, ACC (&acc)[PB]) {
    constexpr long long kMask = (1LL << kFix) - 1;
    const long long t0 = TIE && A.tie == 1 ? A.H2 : -1, t1 = TIE && A.tie == -1 ? A.H2 : -1;
#pragma unroll
    for (int b = 0; b < PB; ++b, D -= A.S) {
        const int jh = (int)(D >> kFix);
        const long long dl = D & kMask;
        ACC w0, w1;
        if constexpr (TIE) {
            w0 = Chord<ACC>::tied(A, dl, t0);
            w1 = Chord<ACC>::tied(A, (1LL << kFix) - dl, t1);
        } else {
            w0 = Chord<ACC>::ramp(A, dl);
            w1 = Chord<ACC>::ramp(A, (1LL << kFix) - dl);
        }
        mf_add<YT, ACC, MODE>(acc[b], w0, (unsigned)jh < (unsigned)p, yi, jh);
        mf_add<YT, ACC, MODE>(acc[b], w1, (unsigned)(jh + 1) < (unsigned)p, yi, jh + 1);
    }
}

template <typename YT, typename ACC, int MODE, int PB, class Epi>
__global__ void __launch_bounds__(128) k_mf_backproject(const MfAngle *__restrict__ ang,
                                                        int nth, int p, int N,
                                                        const YT *__restrict__ y, Epi epi) {
    const int groups = (N + PB - 1) / PB;  // pixel groups per image column
    const int64_t ngr = (int64_t)N * groups;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ngr;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(t / groups), k = (int)(t - (int64_t)ix * groups);
        const int iy0 = N - 1 - PB * k;  // pixel q = ix*N + PB*k + b is iy0 - b
        ACC acc[PB];
#pragma unroll
        for (int b = 0; b < PB; ++b) acc[b] = 0;
        for (int i = 0; i < nth; ++i) {
            const MfAngle A = mf_load<ACC>(ang + i);
            const YT *__restrict__ yi = y + (int64_t)i * p;
            const long long D = (long long)ix * A.C + (long long)iy0 * A.S + A.K;
            if (A.tie != 0) bp_angle<YT, ACC, MODE, PB, true>(A, D, p, yi, acc);
            else bp_angle<YT, ACC, MODE, PB, false>(A, D, p, yi, acc);
        }
        const int64_t q0 = (int64_t)ix * N + PB * k;
#pragma unroll
        for (int b = 0; b < PB; ++b)
            if (iy0 - b >= 0) epi(q0 + b, acc[b]);
    }
}

// Per angle of a fan: the source P and the unit direction u0 towards the
// origin (floats, for the candidate search only).
struct MfFanAngle {
    float px, py, ux, uy;
};

// The sorted bin angles oms and, for a uniform grid of L cells over
// [oms[0], oms[p-1]], the first sorted index at or past each cell's start
// (tab[L] = p): the search for an angle starts one cell before the cell it
// falls in (the last cell past the grid), whose start lies below it, and
// steps forward.
struct MfBins {
    const float *oms;
    const int *omj;
    const int *tab;
    float om0, inv_cell;
    int L;
    // the first k with oms[k] >= lo
    __device__ __forceinline__ int first(float lo, int p) const {
        const float t = (lo - om0) * inv_cell;
        const int k = t < 1.f ? 0 : (t >= (float)L ? L - 1 : (int)t - 1);
        int a = __ldg(tab + k);
        while (a < p && __ldg(oms + a) < lo) ++a;
        return a;
    }
};

// The rays of angle i through pixel (ix, iy): bin angles within the pixel's
// angular half-width of its centre's angle from the source (oms sorted, omj
// their bins), each tested with the exact fixed-point distance. TANK: the
// keys are tan(bin angle) (a source at least 1.42 N from the centre: every
// pixel lies within 30 degrees of the central ray, where tan is monotone), and
// the window is the tangent of the angle window, t = tan(alpha) = cross/dot
// and tan(de) = 0.7072/sqrt(|v|^2 - 0.7072^2) + 2.5e-4 combined by the
// tangent addition formula -- no arctangent or arcsine.
template <typename YT, typename ACC, int MODE, bool TANK>
__device__ __forceinline__ void bp_fan_rays(const MfAngle *__restrict__ rays, const MfFanAngle &F,
                                            const MfBins &B, int i, int p, int ix, int iy, float cx,
                                            float cy, const YT *__restrict__ y, ACC &acc) {
    const float vx = cx - F.px, vy = cy - F.py;
    const float cr = fmaf(F.ux, vy, -F.uy * vx), dt = fmaf(F.ux, vx, F.uy * vy);
    float lo, hi;
    if constexpr (TANK) {
        const float t = __fdividef(cr, dt);
        const float tau = 0.7072f * rsqrtf(fmaf(vx, vx, fmaf(vy, vy, -0.50014f))) + 2.5e-4f;
        lo = __fdividef(t - tau, fmaf(t, tau, 1.f));
        hi = __fdividef(t + tau, fmaf(-t, tau, 1.f));
    } else {
        const float al = atan2f(cr, dt);
        const float de = asinf(fminf(1.f, 0.7072f * rsqrtf(fmaf(vx, vx, vy * vy)))) + 2e-4f;
        lo = al - de;
        hi = al + de;
    }
    for (int k = B.first(lo, p); k < p && __ldg(B.oms + k) <= hi; ++k) {
        const int j = __ldg(B.omj + k);
        const int64_t r = (int64_t)i * p + j;
        const MfAngle A = mf_load<ACC>(rays + r);
        const long long d = (long long)ix * A.C + (long long)iy * A.S + A.K;
        const ACC w = Chord<ACC>::of(A, d);
        if (w > (ACC)0) {
            if (MODE == 0) acc += w * (ACC)__ldg(y + r);
            else acc += w;
        }
    }
}

template <typename YT, typename ACC, int MODE, bool TANK, class Epi>
__global__ void __launch_bounds__(128) k_mf_backproject_fan(
        const MfAngle *__restrict__ rays, const MfFanAngle *__restrict__ fa, MfBins B, int nth,
        int p, int N, const YT *__restrict__ y, Epi epi) {
    const int half = (N + 1) / 2;  // pixel pairs per image column
    const int64_t npairs = (int64_t)N * half;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < npairs;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(t / half), k = (int)(t - (int64_t)ix * half);
        const int iy0 = N - 1 - 2 * k;  // pixel q0 = ix*N + 2k
        const bool two = iy0 >= 1;      // and q0 + 1 (iy0 - 1) when it exists
        const float cx = (float)ix + 0.5f - 0.5f * (float)N;
        const float cy0 = (float)iy0 + 0.5f - 0.5f * (float)N;
        ACC acc0 = 0, acc1 = 0;
        for (int i = 0; i < nth; ++i) {
            const MfFanAngle F = fa[i];
            bp_fan_rays<YT, ACC, MODE, TANK>(rays, F, B, i, p, ix, iy0, cx, cy0, y, acc0);
            if (two) bp_fan_rays<YT, ACC, MODE, TANK>(rays, F, B, i, p, ix, iy0 - 1, cx, cy0 - 1.f, y, acc1);
        }
        const int64_t q0 = (int64_t)ix * N + 2 * k;
        epi(q0, acc0);
        if (two) epi(q0 + 1, acc1);
    }
}

constexpr int kMfPB = 4;  // pixels per backprojector thread (parallel beam)

int grid_for(int64_t items, int threads) {
    int64_t b = (items + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm_count() * 32));
}

}  // namespace
}  // namespace fair

struct fair_mf_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int prec = FAIR_PREC_F32;
    int N = 0, p = 0, nth = 0;
    int kind = 0;                      // 0: parallel beam, 1: fan beam
    fair::DevBuf ang;                  // MfAngle [nth] (parallel) or [nth*p] (fan: per ray)
    fair::DevBuf fang, oms, omj, omt;  // fan: MfFanAngle [nth], sorted bin angles, their bins,
                                       // first sorted index per cell of the angle grid
    float om0 = 0.f, om_inv = 0.f;     // the grid: start, 1 / cell width, cells
    int om_L = 1;
    bool tan_keys = false;             // oms holds tan(bin angle) (the backprojector's TANK)
    fair::DevBuf w_in, w_out;          // host-call staging (FP64)
    fair::DevBuf xt;                   // the projector's transposed copy of x
    fair::DevBuf v_a, v_b;             // reduced-precision staging
    // SIRT state
    bool ready = false, sart = false;
    double omg = 1.0, lb = 0.0, ub = 0.0;
    int bmode = 0;
    fair::DevBuf M_sart, M_cim, D;     // FP64 weights (computed on first use)
    bool have_sart = false, have_cim = false;
    fair::DevBuf x32, r, w_b, w_x;
    std::mutex mu;
};

namespace fair {
namespace {

// Projector / backprojector launches of either geometry.
// The transposed copy of x that the projector reads (N^2 elements of the
// operator's precision), grown before a pass that reads x.
int mf_grow_xt(fair_mf A) {
    const size_t es = A->prec == FAIR_PREC_F64 ? sizeof(double) : sizeof(float);
    return A->xt.grow(es * (size_t)A->N * A->N);
}

template <typename XT, typename ACC, int MODE, class Epi>
void mf_project(fair_mf A, const XT *x, Epi epi, cudaStream_t s) {
    const int64_t m = (int64_t)A->nth * A->p;
    const int N = A->N;
    const MfAngle *ang = A->ang.as<MfAngle>();
    const XT *xt = nullptr;
    if (MODE == 0) {  // the rays that walk rows read the transpose (mf_grow_xt)
        const int nb = (N + 31) / 32;
        k_mf_transpose<XT><<<dim3(nb, nb), dim3(32, 8), 0, s>>>(x, A->xt.as<XT>(), N);
        xt = A->xt.as<XT>();
    }
    if (A->kind == 1)
        k_mf_project<XT, ACC, MODE, true><<<grid_for(m, 128), 128, 0, s>>>(ang, A->nth, A->p, N, x, xt, epi);
    else
        k_mf_project<XT, ACC, MODE, false><<<grid_for(m, 128), 128, 0, s>>>(ang, A->nth, A->p, N, x, xt, epi);
}
template <typename YT, typename ACC, int MODE, class Epi>
void mf_backproject(fair_mf A, const YT *y, Epi epi, cudaStream_t s) {
    const int64_t n = (int64_t)A->N * A->N;
    const MfAngle *ang = A->ang.as<MfAngle>();
    if (A->kind == 1) {
        const MfBins B{A->oms.as<float>(), A->omj.as<int>(), A->omt.as<int>(), A->om0, A->om_inv, A->om_L};
        if (A->tan_keys)
            k_mf_backproject_fan<YT, ACC, MODE, true><<<grid_for(n / 2 + 1, 128), 128, 0, s>>>(
                ang, A->fang.as<MfFanAngle>(), B, A->nth, A->p, A->N, y, epi);
        else
            k_mf_backproject_fan<YT, ACC, MODE, false><<<grid_for(n / 2 + 1, 128), 128, 0, s>>>(
                ang, A->fang.as<MfFanAngle>(), B, A->nth, A->p, A->N, y, epi);
    }
    else
        k_mf_backproject<YT, ACC, MODE, kMfPB><<<grid_for(n / kMfPB + A->N, 128), 128, 0, s>>>(
            ang, A->nth, A->p, A->N, y, epi);
}

int mf_weights(fair_mf A, bool sart, cudaStream_t s) {
    const int64_t m = (int64_t)A->nth * A->p, n = (int64_t)A->N * A->N;
    if (sart && !A->have_sart) {
        FAIR_TRY(A->M_sart.grow(sizeof(double) * (m + 1)));
        FAIR_TRY(A->D.grow(sizeof(double) * (n + 1)));
        EpiStore<double> e1{A->M_sart.as<double>()};
        mf_project<double, double, 1>(A, (const double *)nullptr, e1, s);
        EpiStore<double> e2{A->D.as<double>()};
        mf_backproject<double, double, 1>(A, (const double *)nullptr, e2, s);
        FAIR_CUDA(cudaGetLastError());
        FAIR_TRY(vec_reciprocal(A->M_sart.as<double>(), m, s));  // the epilogues multiply
        FAIR_TRY(vec_reciprocal(A->D.as<double>(), n, s));
        A->have_sart = true;
    }
    if (!sart && !A->have_cim) {
        FAIR_TRY(A->M_cim.grow(sizeof(double) * (m + 1)));
        EpiCimminoW e{A->M_cim.as<double>(), (double)m};
        mf_project<double, double, 2>(A, (const double *)nullptr, e, s);
        FAIR_CUDA(cudaGetLastError());
        FAIR_TRY(vec_reciprocal(A->M_cim.as<double>(), m, s));
        A->have_cim = true;
    }
    return FAIR_OK;
}

// One projector / backprojector pass of a SIRT iteration.
void mf_pass(fair_mf A, int pass, const double *d_b, double *d_x, cudaStream_t s) {
    const double *M = A->sart ? A->M_sart.as<double>() : A->M_cim.as<double>();
    const double *D = A->sart ? A->D.as<double>() : nullptr;
    if (A->prec == FAIR_PREC_F64) {
        if (pass == 1) {
            EpiResidF64 e{d_b, M, A->r.as<double>()};
            mf_project<double, double, 0>(A, (const double *)d_x, e, s);
        } else {
            EpiUpdateF64 e{D, d_x, A->omg, A->lb, A->ub, A->bmode};
            mf_backproject<double, double, 0>(A, (const double *)A->r.as<double>(), e, s);
        }
    } else {
        if (pass == 1) {
            EpiResidLP e{d_b, M, A->r.as<float>(), 1.0};
            mf_project<float, float, 0>(A, (const float *)A->x32.as<float>(), e, s);
        } else {
            EpiUpdateLP e{D, d_x, A->x32.as<float>(), A->omg, A->lb, A->ub, A->bmode, 1.0};
            mf_backproject<float, float, 0>(A, (const float *)A->r.as<float>(), e, s);
        }
    }
}

}  // namespace
}  // namespace fair

#define MENTER(A)                                                  \
    do {                                                           \
        if (!(A)) { fair::set_detail("null operator"); return FAIR_ERR_NULL; } \
        FAIR_CUDA(cudaSetDevice((A)->device));                     \
    } while (0)

extern "C" {

}  // extern "C"

namespace fair {
namespace {

// The constants of the line with unit normal (C, S) and d = ix*C + iy*S + K
// for pixel (ix, iy): fixed-point terms, chord thresholds, walk axis, floats.
void mf_line(double C, double S, double K, MfAngle &a) {
    const double c = std::max(fabs(C), fabs(S)), s = std::min(fabs(C), fabs(S));
    a = MfAngle{};
    a.C = llround(C * kOne);
    a.S = llround(S * kOne);
    a.K = llround(K * kOne);
    a.H1 = llround(0.5 * (c - s) * kOne);
    a.H2 = llround(0.5 * (c + s) * kOne);
    a.Cf = (float)C;
    a.Sf = (float)S;
    a.Kf = (float)K;
    a.by_column = fabs(S) >= fabs(C) ? 1 : 0;
    a.inv_c = (float)(1.0 / c);
    a.inv_c64 = 1.0 / c;
    a.scale_ramp64 = s > 0 ? 1.0 / (kOne * c * s) : 0.0;
    a.tie = 0;
    if (a.S == 0) a.tie = C > 0 ? 1 : -1;        // vertical ray, normal (+-1, 0)
    else if (a.C == 0) a.tie = S > 0 ? 1 : -1;   // horizontal ray, normal (0, +-1)
    if (a.tie != 0) a.H1 = a.H2;                 // s = 0: no ramp
    // segments of 1e-10 or less are dropped, as the ray tracer does
    // (system_generation.f90:393-394)
    a.Hcut = a.tie != 0 ? a.H2 : a.H2 - (long long)floor(1e-10 * c * s * kOne);
    a.H2s = (int)(a.H2 >> 16);
    a.ramp30 = s > 0 ? (float)(1.0 / (1073741824.0 * s)) : 0.f;
}

// A new operator handle with its own stream, or a status.
int mf_new(fair_mf *out, const fair_data *dat, int32_t prec, int kind) {
    if (!out || !dat || !dat->theta) return FAIR_ERR_NULL;
    *out = nullptr;
    if (prec != FAIR_PREC_F64 && prec != FAIR_PREC_F32) {
        set_detail("the matrix-free operator runs in FP64 or FP32");
        return FAIR_ERR_ARG;
    }
    const int N = dat->n, p = dat->p, nth = dat->nth;
    if (N < 1 || p < 2 || nth < 1) { set_detail("n >= 1, p >= 2, nth >= 1 required"); return FAIR_ERR_ARG; }
    if ((int64_t)nth * p > INT32_MAX || N > 8192 || p > 16384) {
        set_detail("the matrix-free operator needs n <= 8192, p <= 16384, nth*p < 2^31");
        return FAIR_ERR_ARG;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_detail(e != cudaSuccess ? cudaGetErrorString(e) : "no CUDA device");
        return FAIR_ERR_NOGPU;
    }
    fair_mf A = new (std::nothrow) fair_mf_s();
    if (!A) return FAIR_ERR_ALLOC;
    cudaGetDevice(&A->device);
    A->prec = prec;
    A->N = N;
    A->p = p;
    A->nth = nth;
    A->kind = kind;
    e = cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete A;
        return cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    A->own_stream = true;
    *out = A;
    return FAIR_OK;
}

template <typename T>
int mf_upload(DevBuf &d, const std::vector<T> &v) {
    if (d.grow(sizeof(T) * std::max<size_t>(v.size(), 1)) != FAIR_OK) return FAIR_ERR_ALLOC;
    if (cudaMemcpy(d.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        return FAIR_ERR_ALLOC;
    }
    return FAIR_OK;
}

}  // namespace
}  // namespace fair

extern "C" {

int fair_mf_create_parallel(fair_mf *out, const fair_data *dat, int32_t prec) {
    FAIR_TRY(fair::mf_new(out, dat, prec, 0));
    fair_mf A = *out;
    const int N = dat->n, p = dat->p, nth = dat->nth;
    // per-angle constants (cos/sin from the host libm, as paralleltomo)
    std::vector<fair::MfAngle> t(nth);
    for (int i = 0; i < nth; ++i) {
        const double C = cos(dat->theta[i]), S = sin(dat->theta[i]);
        const double K = (0.5 - 0.5 * N) * (C + S) + 0.5 * (p - 1);
        fair::mf_line(C, S, K, t[i]);
    }
    if (fair::mf_upload(A->ang, t) != FAIR_OK) {
        fair_mf_destroy(A);
        *out = nullptr;
        return FAIR_ERR_ALLOC;
    }
    return FAIR_OK;
}

int fair_mf_create_fan(fair_mf *out, const fair_data *dat, int32_t geometry_fix, int32_t prec) {
    FAIR_TRY(fair::mf_new(out, dat, prec, 1));
    fair_mf A = *out;
    const int N = dat->n, p = dat->p, nth = dat->nth;
    const double pi = 3.141592653589793;  // 4*atan(1d0), system_generation.f90:4
    // the bin angles and the rotated source and central direction, as
    // fanlineartomo computes them (system_generation.f90:98-157)
    const double R = dat->r * N, dwn = dat->dw * N, sdn = dat->sd * N;
    const double dew = dwn / p;
    std::vector<double> omega(p), com(p), som(p);
    if (p % 2 == 1) {
        const int hh = (p - 1) / 2;
        for (int i = 1; i <= hh; ++i) {
            const double dep = i * dew;
            omega[hh - i] = atan(sdn / dep) - (geometry_fix ? .5 * pi : .5);  // :122
            omega[hh + i] = .5 * pi - atan(sdn / dep);
        }
        omega[hh] = 0.0;
    } else {
        const int hh = p / 2;
        for (int i = 1; i <= hh; ++i) {
            const double dep = (i - .5) * dew;
            omega[hh - i] = atan(sdn / dep) - .5 * pi;  // :129
            omega[hh + i - 1] = .5 * pi - atan(sdn / dep);
        }
    }
    for (int j = 0; j < p; ++j) {
        com[j] = cos(omega[j]);
        som[j] = sin(omega[j]);
    }
    std::vector<fair::MfAngle> rays((size_t)nth * p);
    std::vector<fair::MfFanAngle> fa(nth);
    for (int i = 0; i < nth; ++i) {
        const double c = cos(dat->theta[i]), s = sin(dat->theta[i]);
        const double x0th = c * 0.0 - s * R, y0th = s * 0.0 + c * R;
        const double ath = -x0th / R, bth = -y0th / R;
        fa[i] = fair::MfFanAngle{(float)x0th, (float)y0th, (float)ath, (float)bth};
        for (int j = 0; j < p; ++j) {
            // the ray direction of the reference's tracer (:163-166)
            const double a = com[j] * ath - som[j] * bth;
            const double b = som[j] * ath + com[j] * bth;
            const double nu = sqrt(a * a + b * b);
            const double C = b / nu, S = -a / nu;  // unit normal
            const double K = C * (0.5 - 0.5 * N - x0th) + S * (0.5 - 0.5 * N - y0th);
            fair::mf_line(C, S, K, rays[(size_t)i * p + j]);
        }
    }
    // the bin angles sorted (the odd-p angles of :122 are not monotone in j)
    std::vector<int> order(p);
    for (int j = 0; j < p; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(),
                     [&](int u, int v) { return (float)omega[u] < (float)omega[v]; });
    // keys: tan of the bin angles when the source is at least 1.42 N from the
    // centre (every pixel within 30 degrees of the central ray) and every bin
    // angle below 1.5 rad, else the angles
    bool tk = R >= 1.42 * N;
    for (int j = 0; j < p; ++j) tk = tk && std::fabs(omega[j]) < 1.5;
    A->tan_keys = tk;
    std::vector<float> oms(p);
    for (int k = 0; k < p; ++k) oms[k] = (float)(tk ? std::tan(omega[order[k]]) : omega[order[k]]);
    // a grid of 4p cells over the sorted angles; tab[c] = first k with oms[k] >=
    // om0 + c / inv (the device starts one cell early and steps forward)
    const int L = 4 * p;
    const double span = (double)oms[p - 1] - (double)oms[0];
    A->om0 = oms[0];
    A->om_inv = span > 0 ? (float)(L / span) : 0.f;
    A->om_L = L;
    std::vector<int> tab(L + 1);
    for (int c = 0, k = 0; c <= L; ++c) {
        const double start = (double)oms[0] + (span > 0 ? c * span / L : 0.0);
        while (k < p && (double)oms[k] < start) ++k;
        tab[c] = c == L ? p : k;
    }
    if (fair::mf_upload(A->ang, rays) != FAIR_OK || fair::mf_upload(A->fang, fa) != FAIR_OK ||
        fair::mf_upload(A->oms, oms) != FAIR_OK || fair::mf_upload(A->omj, order) != FAIR_OK ||
        fair::mf_upload(A->omt, tab) != FAIR_OK) {
        fair_mf_destroy(A);
        *out = nullptr;
        return FAIR_ERR_ALLOC;
    }
    return FAIR_OK;
}

int fair_mf_destroy(fair_mf A) {
    if (!A) return FAIR_OK;
    cudaSetDevice(A->device);
    cudaStreamSynchronize(A->stream);
    for (fair::DevBuf *d : {&A->ang, &A->fang, &A->oms, &A->omj, &A->omt, &A->w_in, &A->w_out, &A->v_a,
                            &A->v_b, &A->M_sart, &A->M_cim, &A->D, &A->x32, &A->r, &A->w_b,
                            &A->w_x, &A->xt})
        d->release();
    if (A->own_stream) cudaStreamDestroy(A->stream);
    delete A;
    return FAIR_OK;
}

int fair_mf_set_stream(fair_mf A, void *cuda_stream) {
    MENTER(A);
    std::lock_guard<std::mutex> lk(A->mu);
    FAIR_CUDA(cudaStreamSynchronize(A->stream));
    if (A->own_stream) cudaStreamDestroy(A->stream);
    if (cuda_stream) {
        A->stream = (cudaStream_t)cuda_stream;
        A->own_stream = false;
    } else {
        FAIR_CUDA(cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking));
        A->own_stream = true;
    }
    return FAIR_OK;
}

int fair_mf_info(fair_mf A, int32_t *m, int32_t *n) {
    if (!A) return FAIR_ERR_NULL;
    if (m) *m = A->nth * A->p;
    if (n) *n = A->N * A->N;
    return FAIR_OK;
}

static int mf_apply(fair_mf A, bool back, const double *in, double *out) {
    MENTER(A);
    if (!in || !out) return FAIR_ERR_NULL;
    std::lock_guard<std::mutex> lk(A->mu);
    const int64_t m = (int64_t)A->nth * A->p, n = (int64_t)A->N * A->N;
    const int64_t nin = back ? m : n, nout = back ? n : m;
    cudaStream_t s = A->stream;
    FAIR_TRY(A->w_in.grow(sizeof(double) * (nin + 1)));
    FAIR_TRY(A->w_out.grow(sizeof(double) * (nout + 1)));
    if (!back) FAIR_TRY(fair::mf_grow_xt(A));
    FAIR_CUDA(cudaMemcpyAsync(A->w_in.p, in, sizeof(double) * nin, cudaMemcpyHostToDevice, s));
    if (A->prec == FAIR_PREC_F64) {
        fair::EpiStore<double> e{A->w_out.as<double>()};
        const double *vin = A->w_in.as<double>();
        if (back) fair::mf_backproject<double, double, 0>(A, vin, e, s);
        else fair::mf_project<double, double, 0>(A, vin, e, s);
        FAIR_CUDA(cudaGetLastError());
    } else {
        FAIR_TRY(A->v_a.grow(sizeof(float) * (nin + 1)));
        FAIR_TRY(A->v_b.grow(sizeof(float) * (nout + 1)));
        FAIR_TRY(fair::vec_to_f32(A->w_in.as<double>(), nin, A->v_a.as<float>(), s));
        fair::EpiStore<float> e{A->v_b.as<float>()};
        const float *vin = A->v_a.as<float>();
        if (back) fair::mf_backproject<float, float, 0>(A, vin, e, s);
        else fair::mf_project<float, float, 0>(A, vin, e, s);
        FAIR_CUDA(cudaGetLastError());
        FAIR_TRY(fair::vec_to_f64(A->v_b.as<float>(), nout, A->w_out.as<double>(), s));
    }
    FAIR_CUDA(cudaMemcpyAsync(out, A->w_out.p, sizeof(double) * nout, cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    return FAIR_OK;
}

int fair_mf_nnz(fair_mf A, int64_t *nnz) {
    MENTER(A);
    if (!nnz) return FAIR_ERR_NULL;
    std::lock_guard<std::mutex> lk(A->mu);
    const int64_t m = (int64_t)A->nth * A->p;
    cudaStream_t s = A->stream;
    FAIR_TRY(A->w_out.grow(sizeof(double) * (m + 1)));
    fair::EpiStore<double> e{A->w_out.as<double>()};
    fair::mf_project<double, double, 3>(A, (const double *)nullptr, e, s);
    FAIR_CUDA(cudaGetLastError());
    std::vector<double> c(m);
    FAIR_CUDA(cudaMemcpyAsync(c.data(), A->w_out.p, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    int64_t t = 0;
    for (double v : c) t += (int64_t)v;
    *nnz = t;
    return FAIR_OK;
}

int fair_mf_project(fair_mf A, const double *x, double *y) { return mf_apply(A, false, x, y); }
int fair_mf_backproject(fair_mf A, const double *y, double *x) { return mf_apply(A, true, y, x); }

int fair_mf_sirt_prepare(fair_mf A, const char *sirt_method, const fair_opts *options) {
    MENTER(A);
    if (!sirt_method) return FAIR_ERR_NULL;
    bool sart;
    if (!strcmp(sirt_method, "cimmino")) sart = false;
    else if (!strcmp(sirt_method, "sart")) sart = true;
    else { fair::set_detail("Not a recognised SIRT method."); return FAIR_ERR_METHOD; }
    std::lock_guard<std::mutex> lk(A->mu);
    fair_opts o;
    if (options) o = *options;
    else FAIR_TRY(fair_opts_initialise(&o));
    A->sart = sart;
    A->omg = o.relaxpar;
    A->lb = o.lbound;
    A->ub = o.ubound;
    A->bmode = (o.upb ? 1 : 0) | (o.lwrb ? 2 : 0);
    const int64_t m = (int64_t)A->nth * A->p, n = (int64_t)A->N * A->N;
    const bool red = A->prec != FAIR_PREC_F64;
    FAIR_TRY(A->r.grow((red ? sizeof(float) : sizeof(double)) * (m + 1)));
    if (red) FAIR_TRY(A->x32.grow(sizeof(float) * (n + 1)));
    FAIR_TRY(fair::mf_grow_xt(A));
    FAIR_TRY(fair::mf_weights(A, sart, A->stream));
    FAIR_CUDA(cudaStreamSynchronize(A->stream));
    A->ready = true;
    return FAIR_OK;
}

static int mf_iterations(fair_mf A, const double *d_b, double *d_x, int32_t K, float *ms1,
                         float *ms2) {
    if (!A->ready) {
        fair::set_detail("call fair_mf_sirt_prepare first");
        return FAIR_ERR_STATE;
    }
    if (!d_b || !d_x) return FAIR_ERR_NULL;
    if (K < 0) { fair::set_detail("K >= 0 required"); return FAIR_ERR_ARG; }
    cudaStream_t s = A->stream;
    const int64_t n = (int64_t)A->N * A->N;
    if (A->prec != FAIR_PREC_F64) FAIR_TRY(fair::vec_to_f32(d_x, n, A->x32.as<float>(), s));
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    if (ms1)
        for (auto &e : ev) FAIR_CUDA(cudaEventCreate(&e));
    float t1 = 0.f, t2 = 0.f;
    int st = FAIR_OK;
    for (int it = 0; it < K; ++it) {
        if (ms1) cudaEventRecord(ev[0], s);
        fair::mf_pass(A, 1, d_b, d_x, s);
        if (ms1) cudaEventRecord(ev[1], s);
        fair::mf_pass(A, 2, d_b, d_x, s);
        if (ms1) {
            cudaEventRecord(ev[2], s);
            cudaError_t e = cudaEventSynchronize(ev[2]);
            if (e != cudaSuccess) { st = fair::cuda_fail(e, "matrix-free pass", __FILE__, __LINE__); break; }
            float a = 0.f, b = 0.f;
            cudaEventElapsedTime(&a, ev[0], ev[1]);
            cudaEventElapsedTime(&b, ev[1], ev[2]);
            t1 += a;
            t2 += b;
        }
    }
    if (ms1) {
        for (auto &e : ev) cudaEventDestroy(e);
        *ms1 = t1;
        *ms2 = t2;
    }
    if (st != FAIR_OK) return st;
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int fair_mf_sirt_run_device(fair_mf A, const double *d_b, double *d_x, int32_t K) {
    MENTER(A);
    std::lock_guard<std::mutex> lk(A->mu);
    return mf_iterations(A, d_b, d_x, K, nullptr, nullptr);
}

int fair_mf_sirt_run_device_timed(fair_mf A, const double *d_b, double *d_x, int32_t K,
                                  float *ms_project, float *ms_backproject) {
    MENTER(A);
    if (!ms_project || !ms_backproject) return FAIR_ERR_NULL;
    std::lock_guard<std::mutex> lk(A->mu);
    return mf_iterations(A, d_b, d_x, K, ms_project, ms_backproject);
}

int fair_mf_sirt(fair_mf A, const char *sirt_method, const double *b, int32_t K,
                 const double *x0, const fair_opts *options, double *x) {
    MENTER(A);
    if (!b || !x) return FAIR_ERR_NULL;
    FAIR_TRY(fair_mf_sirt_prepare(A, sirt_method, options));
    std::lock_guard<std::mutex> lk(A->mu);
    const int64_t m = (int64_t)A->nth * A->p, n = (int64_t)A->N * A->N;
    cudaStream_t s = A->stream;
    FAIR_TRY(A->w_b.grow(sizeof(double) * (m + 1)));
    FAIR_TRY(A->w_x.grow(sizeof(double) * (n + 1)));
    FAIR_CUDA(cudaMemcpyAsync(A->w_b.p, b, sizeof(double) * m, cudaMemcpyHostToDevice, s));
    if (x0) FAIR_CUDA(cudaMemcpyAsync(A->w_x.p, x0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    else FAIR_CUDA(cudaMemsetAsync(A->w_x.p, 0, sizeof(double) * n, s));
    FAIR_TRY(mf_iterations(A, A->w_b.as<double>(), A->w_x.as<double>(), K, nullptr, nullptr));
    FAIR_CUDA(cudaMemcpyAsync(x, A->w_x.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    return FAIR_OK;
}

}  // extern "C"
