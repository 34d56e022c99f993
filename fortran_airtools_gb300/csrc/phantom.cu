// phantom.cu -- phantoms and measurement noise on the GPU (include/fair_phantom.h).
//
// One thread per pixel. Pixel (i, j) of the reference's N x N image (row i,
// column j, 0-based) is element j*N + i of the vectorised image. Random
// parameters (seeds, centres) are few: they are drawn on the host from the
// library stream in the reference's order and passed to the kernels. Noise:
// one thread per entry draws its uniform at its stream position and runs the
// reference's Newton iteration; the two norms are deterministic FP64 block
// reductions.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fair_internal.cuh"
#include "fair_phantom.h"

namespace fair {
namespace {

struct Ellipse {
    double A, a2, b2, x0, y0, c, s;
};

// x(i,j) = lx(j), y(i,j) = ly(i): meshgrid on [-1,1]^2 (phantomgallery.f90:17-56)
__global__ void k_shepplogan(const Ellipse *__restrict__ E, int ne, const double *lx,
                             const double *ly, int N, double *v) {
    const int64_t n = (int64_t)N * N;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(q / N), i = (int)(q - (int64_t)j * N);
        const double x = lx[j], y = ly[i];
        double acc = 0.0;
        for (int k = 0; k < ne; ++k) {
            const Ellipse e = E[k];
            const double dx = __dsub_rn(x, e.x0), dy = __dsub_rn(y, e.y0);
            const double u = __dadd_rn(__dmul_rn(dx, e.c), __dmul_rn(dy, e.s));
            const double w = __dsub_rn(__dmul_rn(dy, e.c), __dmul_rn(dx, e.s));
            const double t = __dadd_rn(__ddiv_rn(__dmul_rn(u, u), e.a2), __ddiv_rn(__dmul_rn(w, w), e.b2));
            if (t <= 1.0) acc = __dadd_rn(acc, e.A);
        }
        v[q] = acc;
    }
}

// smooth (:166-199): integer mesh xc(i,j) = j+1, yc(i,j) = i+1
__global__ void k_smooth(const double *__restrict__ c1, const double *__restrict__ c2,
                         const double *__restrict__ a, int p, double sx2, double sy2, int N,
                         double *v) {
    const int64_t n = (int64_t)N * N;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(q / N), i = (int)(q - (int64_t)j * N);
        const double xc = j + 1, yc = i + 1;
        double acc = 0.0;
        for (int k = 0; k < p; ++k) {
            const double dx = __dsub_rn(xc, c1[k]), dy = __dsub_rn(yc, c2[k]);
            const double arg = __dsub_rn(-__ddiv_rn(__dmul_rn(dx, dx), sx2),
                                         __ddiv_rn(__dmul_rn(dy, dy), sy2));
            acc = __dadd_rn(acc, __dmul_rn(a[k], exp(arg)));
        }
        v[q] = acc;
    }
}

// grains (:529-600): index (1-based) of the nearest seed, first on ties
__global__ void k_grains(const double *__restrict__ sx, const double *__restrict__ sy, int p,
                         const double *lx, const double *ly, int N, double *v) {
    const int64_t n = (int64_t)N * N;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(q / N), i = (int)(q - (int64_t)j * N);
        const double x = lx[j], y = ly[i];
        double dmin = 1.7976931348623157e308;
        int kmin = 0;
        for (int k = 0; k < p; ++k) {
            const double dx = __dsub_rn(x, sx[k]), dy = __dsub_rn(y, sy[k]);
            const double d = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
            if (d < dmin) {
                dmin = d;
                kmin = k + 1;
            }
        }
        v[q] = kmin;
    }
}

__device__ __forceinline__ double cube(double t) { return __dmul_rn(__dmul_rn(t, t), t); }

// threephases (:201-254): mesh xc(i,j) = lx(j) on [1,N], yc(i,j) = ly(i) on [1,N]
__global__ void k_threephases(const double *__restrict__ c1x, const double *__restrict__ c1y,
                              const double *__restrict__ c2x, const double *__restrict__ c2y,
                              int p, double s1c, double s2s, const double *lx, const double *ly,
                              int N, double *v) {
    const int64_t n = (int64_t)N * N;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(q / N), i = (int)(q - (int64_t)j * N);
        const double xc = lx[j], yc = ly[i];
        double im1 = 0.0, im2 = 0.0;
        for (int k = 0; k < p; ++k) {
            const double a = __dsub_rn(-__ddiv_rn(cube(fabs(__dsub_rn(xc, c1x[k]))), s1c),
                                       __ddiv_rn(cube(fabs(__dsub_rn(yc, c1y[k]))), s1c));
            im1 = __dadd_rn(im1, exp(a));
        }
        for (int k = 0; k < p; ++k) {
            // the reference divides these cubes by a square (:243)
            const double a = __dsub_rn(-__ddiv_rn(cube(fabs(__dsub_rn(xc, c2x[k]))), s2s),
                                       __ddiv_rn(cube(fabs(__dsub_rn(yc, c2y[k]))), s2s));
            im2 = __dadd_rn(im2, exp(a));
        }
        im1 = im1 < 0.35 ? 0.0 : 2.0;
        im2 = im2 < 0.55 ? 0.0 : 1.0;
        double t = im1 + im2;
        v[q] = t == 3.0 ? 1.0 : t;
    }
}

__global__ void k_block_max(const double *v, int64_t n, double *part) {
    __shared__ double sh[256];
    double m = -1.7976931348623157e308;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, v[q]);
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_divide_by_max(double *v, int64_t n, const double *part, int nb) {
    __shared__ double mx;
    if (threadIdx.x == 0) {
        double m = part[0];
        for (int b = 1; b < nb; ++b) m = fmax(m, part[b]);
        mx = m;
    }
    __syncthreads();
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x)
        v[q] = __ddiv_rn(v[q], mx);
}

// e_k: inverse normal CDF of the stream's draw by Newton (system_generation.f90:725-739)
__global__ void k_noise(double *e, int64_t m, uint64_t seed, uint64_t ctr, int *fail) {
    const double pi = 3.141592653589793, tol = 1e-14;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double u = uniform01(seed, ctr + (uint64_t)k);
        double x = 0.0;
        for (int i = 1; i <= 100; ++i) {
            const double f = .5 * (1 + erf(x / sqrt(2.0))) - u;
            const double df = sqrt(2.0 / pi) * exp(-.5 * (x * x));
            if (fabs(f / df) < tol) break;
            if (i == 100 && fabs(f / df) > tol) atomicExch(fail, 1);
            x = x - f / df;
        }
        e[k] = x;
    }
}

// per-block sums of squares of a and b (fixed order)
__global__ void k_sumsq2(const double *a, const double *b, int64_t m, double *pa, double *pb) {
    __shared__ double sa[256], sb[256];
    double x = 0.0, y = 0.0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m;
         k += (int64_t)gridDim.x * blockDim.x) {
        x += a[k] * a[k];
        y += b[k] * b[k];
    }
    sa[threadIdx.x] = x;
    sb[threadIdx.x] = y;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sa[threadIdx.x] += sa[threadIdx.x + o];
            sb[threadIdx.x] += sb[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        pa[blockIdx.x] = sa[0];
        pb[blockIdx.x] = sb[0];
    }
}

__global__ void k_noise_apply(double *bt, double *e, const double *b, int64_t m, double eta,
                              const double *pa, const double *pb, int nb) {
    __shared__ double sc, ne;
    if (threadIdx.x == 0) {
        double sbb = 0.0, see = 0.0;
        for (int k = 0; k < nb; ++k) {
            sbb += pa[k];
            see += pb[k];
        }
        sc = eta * sqrt(sbb);
        ne = sqrt(see);
    }
    __syncthreads();
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double v = sc * e[k] / ne;
        e[k] = v;
        bt[k] = b[k] + v;
    }
}

constexpr int kBlocks = 512;

int grid_for(int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 16));
}

void linspace(double a, double b, int n, double *x) {  // system_generation.f90:17-35
    const double c = (b - a) / (n - 1), d = a - c;
    for (int i = 1; i <= n; ++i) x[i - 1] = c * i + d;
}

std::vector<double> draws(uint64_t count) {
    uint64_t seed, ctr;
    rng_take(count, &seed, &ctr);
    std::vector<double> u(count);
    for (uint64_t k = 0; k < count; ++k) u[k] = uniform01(seed, ctr + k);
    return u;
}

int normalise(double *d_x, int64_t n, cudaStream_t s) {
    DevBuf part;
    FAIR_TRY(part.grow(sizeof(double) * kBlocks));
    k_block_max<<<kBlocks, 256, 0, s>>>(d_x, n, part.as<double>());
    k_divide_by_max<<<grid_for(n), 256, 0, s>>>(d_x, n, part.as<double>(), kBlocks);
    FAIR_CUDA(cudaGetLastError());
    FAIR_CUDA(cudaStreamSynchronize(s));
    part.release();
    return FAIR_OK;
}

int make_phantom(const std::string &name, int N, double *d_x, cudaStream_t s) {
    const int64_t n = (int64_t)N * N;
    DevBuf t1, t2, t3, t4, t5;
    auto up = [&](DevBuf &b, const std::vector<double> &h) -> int {
        FAIR_TRY(b.grow(sizeof(double) * std::max<size_t>(h.size(), 1)));
        FAIR_CUDA(cudaMemcpyAsync(b.p, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, s));
        return FAIR_OK;
    };
    int st = FAIR_OK;
    if (name == "shepplogan") {
        static const double e[10][6] = {
            {1, .69, .92, 0, 0, 0},          {-.8, .6624, .874, 0, -.0184, 0},
            {-.2, .11, .31, .22, 0, -18},    {-.2, .16, .41, -.22, 0, 18},
            {.1, .21, .25, 0, .35, 0},       {.1, .046, .046, 0, .1, 0},
            {.1, .046, .046, 0, -.1, 0},     {.1, .046, .023, -.08, -.605, 0},
            {.1, .023, .023, 0, -.606, 0},   {.1, .023, .046, .06, -.605, 0}};
        const double pi = 3.141592653589793;
        std::vector<Ellipse> E(10);
        for (int q = 0; q < 10; ++q) {
            const double phi = e[q][5] * pi / 180.0;
            E[q] = Ellipse{e[q][0], e[q][1] * e[q][1], e[q][2] * e[q][2], e[q][3], e[q][4],
                           cos(phi), sin(phi)};
        }
        std::vector<double> lx(N), ly(N);
        linspace(-1.0, 1.0, N, lx.data());
        linspace(1.0, -1.0, N, ly.data());
        FAIR_TRY(t1.grow(sizeof(Ellipse) * 10));
        FAIR_CUDA(cudaMemcpyAsync(t1.p, E.data(), sizeof(Ellipse) * 10, cudaMemcpyHostToDevice, s));
        FAIR_TRY(up(t2, lx));
        FAIR_TRY(up(t3, ly));
        k_shepplogan<<<grid_for(n), 256, 0, s>>>(t1.as<Ellipse>(), 10, t2.as<double>(),
                                                 t3.as<double>(), N, d_x);
        FAIR_CUDA(cudaGetLastError());
        FAIR_CUDA(cudaStreamSynchronize(s));
    } else if (name == "smooth") {
        // centres (:183-186): rows 2-4 are single-precision literals times N
        const double sigma = 0.25 * N;
        std::vector<double> c1 = {0.6 * N, (double)(0.5f * (float)N), (double)(0.2f * (float)N),
                                  (double)(0.8f * (float)N)};
        std::vector<double> c2 = {0.6 * N, (double)(0.3f * (float)N), (double)(0.7f * (float)N),
                                  (double)(0.2f * (float)N)};
        std::vector<double> a = {1.0, 0.5, 0.7, 0.9};
        FAIR_TRY(up(t1, c1));
        FAIR_TRY(up(t2, c2));
        FAIR_TRY(up(t3, a));
        const double sx = 1.2 * sigma;
        k_smooth<<<grid_for(n), 256, 0, s>>>(t1.as<double>(), t2.as<double>(), t3.as<double>(),
                                             4, sx * sx, sigma * sigma, N, d_x);
        FAIR_CUDA(cudaGetLastError());
        st = normalise(d_x, n, s);
    } else if (name == "grains") {
        const int p = (int)(3 * sqrt(N * 1.0));
        // random_number(x0) on x0(2,p) in element order, then random_number(vals)
        std::vector<double> u = draws(2 * (uint64_t)p);
        draws((uint64_t)p);  // vals: drawn, unused (:577)
        std::vector<double> sx(p), sy(p);
        for (int k = 0; k < p; ++k) {
            sx[k] = 1.5 * (2.0 * u[2 * k] - 1.0);
            sy[k] = 1.5 * (2.0 * u[2 * k + 1] - 1.0);
        }
        std::vector<double> lx(N), ly(N);
        linspace(-1.0, 1.0, N, lx.data());
        linspace(1.0, -1.0, N, ly.data());
        FAIR_TRY(up(t1, sx));
        FAIR_TRY(up(t2, sy));
        FAIR_TRY(up(t3, lx));
        FAIR_TRY(up(t4, ly));
        k_grains<<<grid_for(n), 256, 0, s>>>(t1.as<double>(), t2.as<double>(), p, t3.as<double>(),
                                             t4.as<double>(), N, d_x);
        FAIR_CUDA(cudaGetLastError());
        st = normalise(d_x, n, s);
    } else if (name == "3phases") {
        const int p = 100;
        // random_number(c) on c(p,2): column 1 (x) then column 2 (y), times N
        std::vector<double> u1 = draws(2 * (uint64_t)p), u2 = draws(2 * (uint64_t)p);
        std::vector<double> c1x(p), c1y(p), c2x(p), c2y(p);
        for (int k = 0; k < p; ++k) {
            c1x[k] = u1[k] * N;
            c1y[k] = u1[p + k] * N;
            c2x[k] = u2[k] * N;
            c2y[k] = u2[p + k] * N;
        }
        // meshgrid(xc, yc, N, (/1,N,N,1/)): x = linspace(1, N), y = linspace(1, N) (:222)
        std::vector<double> lx(N), ly(N);
        linspace(1.0, (double)N, N, lx.data());
        linspace(1.0, (double)N, N, ly.data());
        const double s1 = 0.025 * N, s2 = 0.025 * N;
        const double s1c = (2.5 * s1) * (2.5 * s1) * (2.5 * s1), s2s = (2.5 * s2) * (2.5 * s2);
        FAIR_TRY(up(t1, c1x));
        FAIR_TRY(up(t2, c1y));
        FAIR_TRY(up(t3, c2x));
        FAIR_TRY(up(t4, c2y));
        DevBuf t6;
        FAIR_TRY(up(t5, lx));
        FAIR_TRY(up(t6, ly));
        k_threephases<<<grid_for(n), 256, 0, s>>>(t1.as<double>(), t2.as<double>(),
                                                  t3.as<double>(), t4.as<double>(), p, s1c, s2s,
                                                  t5.as<double>(), t6.as<double>(), N, d_x);
        FAIR_CUDA(cudaGetLastError());
        st = normalise(d_x, n, s);
        FAIR_CUDA(cudaStreamSynchronize(s));
        t6.release();
    } else {
        set_detail("Not a recognised phantom.");
        return FAIR_ERR_ARG;
    }
    FAIR_CUDA(cudaStreamSynchronize(s));
    for (DevBuf *b : {&t1, &t2, &t3, &t4, &t5}) b->release();
    return st;
}

}  // namespace
}  // namespace fair

extern "C" {

int fair_phantom_device(const char *name, int32_t N, double *d_x, void *cuda_stream) {
    if (!name || !d_x) return FAIR_ERR_NULL;
    if (N < 2) { fair::set_detail("N >= 2 required"); return FAIR_ERR_ARG; }
    return fair::make_phantom(name, N, d_x, (cudaStream_t)cuda_stream);
}

int fair_phantom(const char *name, int32_t N, double *x) {
    if (!name || !x) return FAIR_ERR_NULL;
    if (N < 2) { fair::set_detail("N >= 2 required"); return FAIR_ERR_ARG; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        fair::set_detail("no CUDA device");
        return FAIR_ERR_NOGPU;
    }
    const int64_t n = (int64_t)N * N;
    fair::DevBuf d;
    FAIR_TRY(d.grow(sizeof(double) * n));
    int st = fair::make_phantom(name, N, d.as<double>(), nullptr);
    if (st == FAIR_OK) {
        cudaError_t e = cudaMemcpy(x, d.p, sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = fair::cuda_fail(e, "cudaMemcpy", __FILE__, __LINE__);
    }
    d.release();
    return st;
}

int fair_add_white_noise_device(double *d_bt, double *d_e, const double *d_b, int64_t m,
                                double eta, void *cuda_stream) {
    if (!d_bt || !d_e || !d_b) return FAIR_ERR_NULL;
    if (m <= 0) return FAIR_OK;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    uint64_t seed, ctr;
    fair::rng_take((uint64_t)m, &seed, &ctr);
    fair::DevBuf flag, pa, pb;
    FAIR_TRY(flag.grow(sizeof(int)));
    FAIR_TRY(pa.grow(sizeof(double) * fair::kBlocks));
    FAIR_TRY(pb.grow(sizeof(double) * fair::kBlocks));
    FAIR_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), s));
    fair::k_noise<<<fair::grid_for(m), 256, 0, s>>>(d_e, m, seed, ctr, flag.as<int>());
    fair::k_sumsq2<<<fair::kBlocks, 256, 0, s>>>(d_b, d_e, m, pa.as<double>(), pb.as<double>());
    fair::k_noise_apply<<<fair::grid_for(m), 256, 0, s>>>(d_bt, d_e, d_b, m, eta, pa.as<double>(),
                                                          pb.as<double>(), fair::kBlocks);
    FAIR_CUDA(cudaGetLastError());
    int hf = 0;
    FAIR_CUDA(cudaMemcpyAsync(&hf, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    flag.release();
    pa.release();
    pb.release();
    return hf ? FAIR_ERR_NEWTON : FAIR_OK;
}

}  // extern "C"
