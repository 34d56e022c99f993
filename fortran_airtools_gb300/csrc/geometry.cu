// geometry.cu -- ray-traced system matrix (paralleltomo / fanlineartomo) on
// the GPU, one thread per ray, two passes (count, scan, fill) like the
// reference (system_generation.f90:138-212 count, :214-302 fill).
//
// Per ray the reference computes the 2N+2 crossings with the grid lines,
// quicksorts them by the ray parameter t, keeps the points inside the square
// and emits one nonzero per pair of consecutive points further apart than
// 1e-10 (system_generation.f90:163-203, :357-397). Here the two crossing
// families are already monotone in t, so the fast path merges them instead of
// sorting: the in-box points of each family form one index interval (found by
// binary search on the monotone other coordinate), and the merge yields the
// same sequence as the sort whenever no two in-box keys are equal. A ray whose
// keys contain a NaN (a == 0 or b == 0 with the ray on a grid line, where the
// reference's quicksort no longer sorts) or an exact tie between the families
// (where the unstable sort picks the order) is sent to the exact path, which
// replays the reference's Hoare quicksort on that ray.
//
// Every product, sum and quotient on the ray uses explicit round-to-nearest
// intrinsics so that no multiply-add is fused: the results then match the
// reference's separately rounded operations bit for bit.
#include <vector>

#include "fair_internal.cuh"

namespace fair {

namespace {

struct GeomDev {
    int kind, N, nth, p;
    const double *grid;
    const double *cth, *sth, *bx0, *by0;
    const double *ax0th, *ay0th, *aath, *abth, *com, *som;
};

struct Ray {
    double a, b, x0th, y0th;
    bool excluded;
};

// system_generation.f90:348-353 (parallel) and :146-157 (fan).
__device__ __forceinline__ Ray ray_params(const GeomDev &G, int i, int j) {
    Ray r;
    if (G.kind == 0) {
        double ct = G.cth[i], st = G.sth[i], x0 = G.bx0[j], y0 = G.by0[j];
        r.x0th = __dsub_rn(__dmul_rn(ct, x0), __dmul_rn(st, y0));
        r.y0th = __dadd_rn(__dmul_rn(st, x0), __dmul_rn(ct, y0));
        r.a = -st;
        r.b = ct;
        const double h = 0.5 * G.N;
        // boundary rays excluded by :393-394 / :466-467
        r.excluded = (r.b == 0.0 && fabs(__dsub_rn(r.y0th, h)) < 1e-15) ||
                     (r.a == 0.0 && fabs(__dsub_rn(r.x0th, h)) < 1e-15);
    } else {
        r.x0th = G.ax0th[i];
        r.y0th = G.ay0th[i];
        double ath = G.aath[i], bth = G.abth[i], co = G.com[j], so = G.som[j];
        r.a = __dsub_rn(__dmul_rn(co, ath), __dmul_rn(so, bth));
        r.b = __dadd_rn(__dmul_rn(so, ath), __dmul_rn(co, bth));
        r.excluded = false;
    }
    return r;
}

// Crossing with the vertical grid line x = g[k]: tx, yx of :163-164 / :357-358.
__device__ __forceinline__ void eval_x(const double *g, const Ray &r, int k, double &t,
                                       double &px, double &py) {
    px = g[k];
    t = __ddiv_rn(__dsub_rn(px, r.x0th), r.a);
    py = __dadd_rn(__dmul_rn(r.b, t), r.y0th);
}
// Crossing with the horizontal grid line y = g[l]: ty, xy of :168-169 / :362-363.
__device__ __forceinline__ void eval_y(const double *g, const Ray &r, int l, double &t,
                                       double &px, double &py) {
    py = g[l];
    t = __ddiv_rn(__dsub_rn(py, r.y0th), r.b);
    px = __dadd_rn(__dmul_rn(r.a, t), r.x0th);
}

// Smallest k in [0, N] with pred(k) true (pred monotone false..true); N+1 if none.
template <class P>
__device__ __forceinline__ int first_true(int N, P pred) {
    int L = 0, R = N + 1;
    while (L < R) {
        int mid = (L + R) >> 1;
        if (pred(mid)) R = mid; else L = mid + 1;
    }
    return L;
}

struct CountSink {
    __device__ __forceinline__ void emit(int64_t, double, int) {}
};

struct WriteSink {
    int32_t *col;
    double *val;
    int64_t cap;     // nonzeros reserved for this row by the count pass
    int32_t ncols;
    int *err;
    __device__ __forceinline__ void emit(int64_t k, double d, int ja) {
        if (ja < 1 || ja > ncols) {  // "++ Something went wrong" (:293, :478)
            atomicOr(err, 1);
            return;
        }
        if (k < cap) {
            col[k] = ja - 1;
            val[k] = d;
        }
    }
};

// Segment between consecutive in-box points (:199-203 / :279-297).
template <class Sink>
__device__ __forceinline__ void segment(int N, double px0, double py0, double px1, double py1,
                                        int64_t &cnt, Sink &sink) {
    double dx = __dsub_rn(px0, px1), dy = __dsub_rn(py0, py1);
    double d = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    if (d > 1e-10) {
        double xm = __dmul_rn(0.5, __dadd_rn(__dadd_rn(px0, px1), (double)N));
        double ym = __dmul_rn(0.5, __dadd_rn(__dadd_rn(py0, py1), (double)N));
        int ja = (int)floor(xm) * N + (N - (int)floor(ym));
        sink.emit(cnt, d, ja);
        cnt++;
    }
}

// Fast path. Returns the nonzero count, or -1 when the ray needs the exact path.
template <class Sink>
__device__ int64_t trace_merge(const GeomDev &G, const Ray &r, Sink &sink) {
    if (r.excluded) return 0;
    const int N = G.N;
    const double *g = G.grid;
    const double lo = -0.5 * N, hi = 0.5 * N;

    // x-crossings: in-box interval [kx0, kx1] of k (py monotone in k)
    int kx0 = 0, kx1 = -1;
    if (r.a != 0.0) {
        double t, px, py0, pyN;
        eval_x(g, r, 0, t, px, py0);
        eval_x(g, r, N, t, px, pyN);
        auto py = [&](int k) { double tt, xx, yy; eval_x(g, r, k, tt, xx, yy); return yy; };
        if (py0 <= pyN) {
            kx0 = first_true(N, [&](int k) { return py(k) >= lo; });
            kx1 = first_true(N, [&](int k) { return py(k) > hi; }) - 1;
        } else {
            kx0 = first_true(N, [&](int k) { return py(k) <= hi; });
            kx1 = first_true(N, [&](int k) { return py(k) < lo; }) - 1;
        }
    } else {
        for (int k = 0; k <= N; ++k)
            if (g[k] == r.x0th) return -1;  // 0/0 = NaN key
    }
    // y-crossings: in-box interval [ly0, ly1] of l (px monotone in l)
    int ly0 = 0, ly1 = -1;
    if (r.b != 0.0) {
        double t, py, px0, pxN;
        eval_y(g, r, 0, t, px0, py);
        eval_y(g, r, N, t, pxN, py);
        auto px = [&](int l) { double tt, xx, yy; eval_y(g, r, l, tt, xx, yy); return xx; };
        if (px0 <= pxN) {
            ly0 = first_true(N, [&](int l) { return px(l) >= lo; });
            ly1 = first_true(N, [&](int l) { return px(l) > hi; }) - 1;
        } else {
            ly0 = first_true(N, [&](int l) { return px(l) <= hi; });
            ly1 = first_true(N, [&](int l) { return px(l) < lo; }) - 1;
        }
    } else {
        for (int l = 0; l <= N; ++l)
            if (g[l] == r.y0th) return -1;
    }

    int nx = kx1 >= kx0 ? kx1 - kx0 + 1 : 0;
    int ny = ly1 >= ly0 ? ly1 - ly0 + 1 : 0;
    // t increases with k when a > 0 and with l when b > 0
    int kx = r.a > 0.0 ? kx0 : kx1, sx = r.a > 0.0 ? 1 : -1;
    int ly = r.b > 0.0 ? ly0 : ly1, sy = r.b > 0.0 ? 1 : -1;
    double tX = 0, xX = 0, yX = 0, tY = 0, xY = 0, yY = 0;
    if (nx) eval_x(g, r, kx, tX, xX, yX);
    if (ny) eval_y(g, r, ly, tY, xY, yY);

    int64_t cnt = 0;
    bool have = false;
    double ppx = 0, ppy = 0;
    while (nx > 0 || ny > 0) {
        bool takeX;
        if (nx > 0 && ny > 0) {
            if (tX == tY) return -1;  // unstable-sort tie: exact path
            takeX = tX < tY;
        } else {
            takeX = nx > 0;
        }
        double px, py;
        if (takeX) {
            px = xX; py = yX;
            if (--nx) { kx += sx; eval_x(g, r, kx, tX, xX, yX); }
        } else {
            px = xY; py = yY;
            if (--ny) { ly += sy; eval_y(g, r, ly, tY, xY, yY); }
        }
        // in-box test of :188 / :382 (the grid coordinate is inside by construction)
        if (px >= lo && px <= hi && py >= lo && py <= hi) {
            if (have) segment(N, ppx, ppy, px, py, cnt, sink);
            ppx = px; ppy = py; have = true;
        }
    }
    return cnt;
}

// Exact path: the reference's quicksort (system_generation.f90:37-77) on the
// full key array of one ray, held in per-ray scratch.
struct RayScratch {
    double *t, *xxy, *yxy;
    int32_t *ind;
};

__device__ void quicksort_emul(double *a, int32_t *ind, int nt) {
    // The two recursive calls of :75-76 act on disjoint index ranges, so any
    // processing order gives the same result; the larger range is stacked.
    int stk_f[64], stk_l[64];
    int top = 0;
    stk_f[top] = 0; stk_l[top] = nt - 1; top++;
    while (top > 0) {
        --top;
        int f = stk_f[top], l = stk_l[top];
        while (f < l) {
            double x = a[(f + l) >> 1];  // 1-based (f+l)/2 maps to the same element
            int i = f, j = l;
            for (;;) {
                while (i < l && a[i] < x) i++;
                while (j > f && x < a[j]) j--;
                if (i >= j) break;
                double tt = a[i]; a[i] = a[j]; a[j] = tt;
                int32_t m = ind[i]; ind[i] = ind[j]; ind[j] = m;
                i++;
                j--;
            }
            int lf = f, ll = i - 1, rf = j + 1, rl = l;
            bool hasL = lf < ll, hasR = rf < rl;
            if (hasL && hasR) {
                if (ll - lf > rl - rf) {
                    if (top < 64) { stk_f[top] = lf; stk_l[top] = ll; top++; }
                    f = rf; l = rl;
                } else {
                    if (top < 64) { stk_f[top] = rf; stk_l[top] = rl; top++; }
                    f = lf; l = ll;
                }
            } else if (hasL) {
                f = lf; l = ll;
            } else if (hasR) {
                f = rf; l = rl;
            } else {
                break;
            }
        }
    }
}

template <class Sink>
__device__ int64_t trace_exact(const GeomDev &G, const Ray &r, RayScratch s, Sink &sink) {
    if (r.excluded) return 0;
    const int N = G.N, np = N + 1, nt = 2 * N + 2;
    const double *g = G.grid;
    for (int k = 0; k < np; ++k) {
        double tx, xx, yx, ty, xy, yy;
        eval_x(g, r, k, tx, xx, yx);
        eval_y(g, r, k, ty, xy, yy);
        s.t[k] = tx;       s.t[np + k] = ty;
        s.xxy[k] = xx;     s.xxy[np + k] = xy;
        s.yxy[k] = yx;     s.yxy[np + k] = yy;
        s.ind[k] = k;      s.ind[np + k] = np + k;
    }
    quicksort_emul(s.t, s.ind, nt);
    const double lo = -0.5 * N, hi = 0.5 * N;
    int64_t cnt = 0;
    bool have = false;
    double ppx = 0, ppy = 0;
    for (int k = 0; k < nt; ++k) {
        double px = s.xxy[s.ind[k]], py = s.yxy[s.ind[k]];
        if (px >= lo && px <= hi && py >= lo && py <= hi) {
            if (have) segment(N, ppx, ppy, px, py, cnt, sink);
            ppx = px; ppy = py; have = true;
        }
    }
    return cnt;
}

__global__ void k_geom_count(GeomDev G, int32_t *counts, int32_t *special, int32_t *nspecial) {
    int64_t m = (int64_t)G.nth * G.p;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
         r += (int64_t)gridDim.x * blockDim.x) {
        int i = (int)(r / G.p), j = (int)(r % G.p);
        Ray ray = ray_params(G, i, j);
        CountSink cs;
        int64_t c = trace_merge(G, ray, cs);
        if (c < 0) {
            int slot = atomicAdd(nspecial, 1);
            special[slot] = (int32_t)r;
            c = 0;
        }
        counts[r] = (int32_t)c;
    }
}

__global__ void k_geom_count_exact(GeomDev G, const int32_t *special, int32_t nsp,
                                   double *scr_d, int32_t *scr_i, int32_t *counts) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsp) return;
    const int nt = 2 * G.N + 2;
    RayScratch s{scr_d + (size_t)q * 3 * nt, scr_d + (size_t)q * 3 * nt + nt,
                 scr_d + (size_t)q * 3 * nt + 2 * nt, scr_i + (size_t)q * nt};
    int32_t r = special[q];
    Ray ray = ray_params(G, r / G.p, r % G.p);
    CountSink cs;
    counts[r] = (int32_t)trace_exact(G, ray, s, cs);
}

__global__ void k_geom_fill(GeomDev G, const int64_t *rowptr, int32_t *col, double *val,
                            int32_t ncols, int *err) {
    int64_t m = (int64_t)G.nth * G.p;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
         r += (int64_t)gridDim.x * blockDim.x) {
        int i = (int)(r / G.p), j = (int)(r % G.p);
        Ray ray = ray_params(G, i, j);
        int64_t s0 = rowptr[r], cap = rowptr[r + 1] - s0;
        WriteSink ws{col + s0, val + s0, cap, ncols, err};
        int64_t c = trace_merge(G, ray, ws);
        if (c >= 0 && c != cap) atomicOr(err, 2);  // "Didn't hit all elements" (:304)
    }
}

__global__ void k_geom_fill_exact(GeomDev G, const int32_t *special, int32_t nsp, double *scr_d,
                                  int32_t *scr_i, const int64_t *rowptr, int32_t *col,
                                  double *val, int32_t ncols, int *err) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsp) return;
    const int nt = 2 * G.N + 2;
    RayScratch s{scr_d + (size_t)q * 3 * nt, scr_d + (size_t)q * 3 * nt + nt,
                 scr_d + (size_t)q * 3 * nt + 2 * nt, scr_i + (size_t)q * nt};
    int32_t r = special[q];
    Ray ray = ray_params(G, r / G.p, r % G.p);
    int64_t s0 = rowptr[r], cap = rowptr[r + 1] - s0;
    WriteSink ws{col + s0, val + s0, cap, ncols, err};
    int64_t c = trace_exact(G, ray, s, ws);
    if (c != cap) atomicOr(err, 2);
}

GeomDev to_dev(const GeomTables &T) {
    GeomDev G;
    G.kind = T.kind; G.N = T.N; G.nth = T.nth; G.p = T.p;
    G.grid = T.grid.as<double>();
    G.cth = T.cth.as<double>(); G.sth = T.sth.as<double>();
    G.bx0 = T.bx0.as<double>(); G.by0 = T.by0.as<double>();
    G.ax0th = T.ax0th.as<double>(); G.ay0th = T.ay0th.as<double>();
    G.aath = T.aath.as<double>(); G.abth = T.abth.as<double>();
    G.com = T.com.as<double>(); G.som = T.som.as<double>();
    return G;
}

constexpr int kExactBatch = 2048;  // special rays traced per launch (scratch bound)

}  // namespace

namespace {
// The count pass (k_geom_count, then the exact path for the rays whose keys
// need the quicksort replay): entries per ray into counts [m]; the special
// rays, their number and the exact path's scratch stay for the fill.
struct GeomCount {
    DevBuf counts, special, nsp, scr_d, scr_i;
    int32_t h_nsp = 0, batch = 0;
    int blocks = 1;
    static constexpr int threads = 128;
    void release() {
        counts.release(); special.release(); nsp.release(); scr_d.release(); scr_i.release();
    }
};

int geometry_count(const GeomTables &T, const GeomDev &G, GeomCount &C, cudaStream_t s) {
    const int64_t m = (int64_t)T.nth * T.p;
    FAIR_TRY(C.counts.grow(sizeof(int32_t) * (m > 0 ? m : 1)));
    FAIR_TRY(C.special.grow(sizeof(int32_t) * (m > 0 ? m : 1)));
    FAIR_TRY(C.nsp.grow(sizeof(int32_t)));
    FAIR_CUDA(cudaMemsetAsync(C.nsp.p, 0, sizeof(int32_t), s));
    int64_t blocks64 = (m + C.threads - 1) / C.threads;
    C.blocks = (int)(blocks64 < (int64_t)sm_count() * 64 ? (blocks64 > 0 ? blocks64 : 1)
                                                         : (int64_t)sm_count() * 64);
    k_geom_count<<<C.blocks, C.threads, 0, s>>>(G, C.counts.as<int32_t>(), C.special.as<int32_t>(),
                                                C.nsp.as<int32_t>());
    FAIR_CUDA(cudaGetLastError());
    FAIR_CUDA(cudaMemcpyAsync(&C.h_nsp, C.nsp.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    // Scratch for the exact path: keys, two coordinate arrays, permutation.
    const int nt = 2 * T.N + 2;
    C.batch = C.h_nsp < kExactBatch ? C.h_nsp : kExactBatch;
    if (C.h_nsp > 0) {
        FAIR_TRY(C.scr_d.grow(sizeof(double) * 3 * (size_t)nt * C.batch));
        FAIR_TRY(C.scr_i.grow(sizeof(int32_t) * (size_t)nt * C.batch));
        for (int32_t q0 = 0; q0 < C.h_nsp; q0 += C.batch) {
            int32_t nq = C.h_nsp - q0 < C.batch ? C.h_nsp - q0 : C.batch;
            k_geom_count_exact<<<(nq + 63) / 64, 64, 0, s>>>(G, C.special.as<int32_t>() + q0, nq,
                                                            C.scr_d.as<double>(),
                                                            C.scr_i.as<int32_t>(),
                                                            C.counts.as<int32_t>());
            FAIR_CUDA(cudaGetLastError());
        }
    }
    return FAIR_OK;
}
}  // namespace

int geometry_nnz(const GeomTables &T, int64_t *nnz, cudaStream_t s) {
    const int64_t m = (int64_t)T.nth * T.p;
    GeomDev G = to_dev(T);
    GeomCount C;
    FAIR_TRY(geometry_count(T, G, C, s));
    DevBuf rp;
    FAIR_TRY(rp.grow(sizeof(int64_t) * (m + 1)));
    FAIR_TRY(scan_counts(C.counts.as<int32_t>(), m, rp.as<int64_t>(), s));
    FAIR_CUDA(cudaMemcpyAsync(nnz, rp.as<int64_t>() + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    return FAIR_OK;
}

int build_geometry(const GeomTables &T, DevCSR &A, cudaStream_t s) {
    const int64_t m = (int64_t)T.nth * T.p;
    const int32_t ncols = T.N * T.N;
    GeomDev G = to_dev(T);
    A.release();
    A.m = (int32_t)m;
    A.n = ncols;
    A.stride_hint = T.N;   // pixel (x, y) is column x*N + (N - y)
    A.tstride_hint = T.p;  // ray (angle i, bin j) is row i*p + j

    GeomCount C;
    FAIR_TRY(geometry_count(T, G, C, s));
    DevBuf err;
    FAIR_TRY(err.grow(sizeof(int)));
    FAIR_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    DevBuf &counts = C.counts, &special = C.special, &scr_d = C.scr_d, &scr_i = C.scr_i;
    const int32_t h_nsp = C.h_nsp, batch = C.batch;
    const int blocks = C.blocks, threads = C.threads;

    FAIR_TRY(A.rowptr.grow(sizeof(int64_t) * (m + 1)));
    FAIR_TRY(scan_counts(counts.as<int32_t>(), m, A.rowptr.as<int64_t>(), s));
    int64_t nnz = 0;
    FAIR_CUDA(cudaMemcpyAsync(&nnz, A.rowptr.as<int64_t>() + m, sizeof(int64_t),
                              cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    A.nnz = nnz;
    FAIR_TRY(A.alloc_entries(nnz, s));

    k_geom_fill<<<blocks, threads, 0, s>>>(G, A.rowptr.as<int64_t>(), A.col.as<int32_t>(),
                                           A.v64.as<double>(), ncols, err.as<int>());
    FAIR_CUDA(cudaGetLastError());
    for (int32_t q0 = 0; q0 < h_nsp; q0 += batch) {
        int32_t nq = h_nsp - q0 < batch ? h_nsp - q0 : batch;
        k_geom_fill_exact<<<(nq + 63) / 64, 64, 0, s>>>(
            G, special.as<int32_t>() + q0, nq, scr_d.as<double>(), scr_i.as<int32_t>(),
            A.rowptr.as<int64_t>(), A.col.as<int32_t>(), A.v64.as<double>(), ncols, err.as<int>());
        FAIR_CUDA(cudaGetLastError());
    }
    int h_err = 0;
    FAIR_CUDA(cudaMemcpyAsync(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    C.release();
    err.release();
    if (h_err) {
        set_detail(h_err & 1 ? "column index outside 1..N^2 while tracing a ray"
                             : "fill pass wrote a different count than the count pass");
        A.release();
        return FAIR_ERR_GEOMETRY;
    }
    FAIR_TRY(csr_max_row(A, s));
    return FAIR_OK;
}

}  // namespace fair
