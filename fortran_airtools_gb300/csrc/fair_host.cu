// fair_host.cu -- the extern "C" entry points of include/fair_gpu.h.
//
// Host code here only validates arguments, computes the small geometry
// tables the reference computes with libm (cos/sin/atan per angle and per
// detector bin), runs the reference's O(m) set-up logic (row filters,
// permutations, probability tables) and moves the caller's vectors to and
// from the device. All O(nnz) work runs in the CUDA kernels of geometry.cu,
// sparse.cu, solvers.cu and kaczmarz.cu; there is no CPU fallback.
//
// This file is compiled with -ffp-contract=off for the host compiler so that
// the geometry tables round every product separately, like the reference.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "fair_gpu_ext.h"
#include "fair_internal.cuh"

namespace fair {

static thread_local std::string g_detail;

void set_detail(const std::string &s) { g_detail = s; }

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_detail = buf;
    if (e == cudaErrorMemoryAllocation) return FAIR_ERR_ALLOC;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FAIR_ERR_NOGPU;
    return FAIR_ERR_CUDA;
}

int DevBuf::grow(size_t need) {
    if (need == 0) need = 1;
    if (p && need <= bytes) return FAIR_OK;
    release();
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
        p = nullptr;
        bytes = 0;
        cudaGetLastError();
        return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
    }
    bytes = need;
    return FAIR_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

void DevCSR::drop_sliced() {
    soff.release(); sidx.release(); sv64.release(); sv32.release(); sf16.release(); sfq.release();
    nslots = 0;
    sl_G = 0;
    hassl = hassidx = hassv64 = hassv32 = hassf16 = hassfq = false;
}

void DevCSR::Tiled::release() {
    segbase.release(); soff.release(); pslot.release(); units.release(); idx.release();
    v64.release(); v32.release(); r16.release(); rq.release(); part.release();
    sstart.release(); send.release(); bmin.release(); srow.release();
    kind = p = nth = W = 0;
    cells_cap = 0;
    NA = nab = 1;
    soff6.release(); anc6.release(); code6.release(); side6.release(); r6_16.release(); r6_q.release();
    S6 = 0;
    L6 = 5;
    nslots6 = nesc6 = 0;
    tried6 = built6 = has6_16 = has6_q = false;
    T = N = ntr = 0;
    nseg = nchunks = nslots = 0;
    nunits = 0;
    has_idx = has_v64 = has_v32 = has_r16 = has_rq = false;
}

void DevCSR::Delta::release() {
    soff.release(); anchor.release(); code.release(); side.release();
    v64.release(); v32.release(); r16.release(); rq.release();
    S = 0;
    L = 7;
    nslots = nesc = 0;
    tried = built = false;
    has_v64 = has_v32 = has_r16 = has_rq = false;
}

void DevCSR::release() {
    drop_sliced();
    tl.release();
    dl[0].release();
    dl[1].release();
    rowptr.release(); col.release(); v64.release(); v32.release(); v16.release(); vq.release();
    has32 = has16 = hasq = false;
    rn1.release(); rn2.release();
    f32_only = false;
    prow.release(); gidx.release(); gside.release();
    pv64.release(); pv32.release(); pv16.release(); pvq.release();
    pf16.release(); pfq.release();
    pk_tried = haspk = hasp64 = hasp32 = hasp16 = haspq = hasf16 = hasfq = false;
    for (int &g : sirt_lanes) g = 8;
    for (int &g : sirt_groups) g = 1;
    tile_req[0] = tile_req[1] = 0;
    sirt_groups[FAIR_PREC_F64] = 0;
    ngroups = nesc = 0;
    stride_hint = tstride_hint = 0;
    m = n = 0;
    nnz = 0;
    max_row = 0;
}

int DevCSR::alloc_entries(int64_t nnz_, cudaStream_t s) {
    FAIR_TRY(col.grow(sizeof(int32_t) * (size_t)(nnz_ + kEntryPad)));
    FAIR_TRY(v64.grow(sizeof(double) * (size_t)(nnz_ + kEntryPad)));
    FAIR_CUDA(cudaMemsetAsync(col.as<int32_t>() + nnz_, 0, sizeof(int32_t) * kEntryPad, s));
    FAIR_CUDA(cudaMemsetAsync(v64.as<double>() + nnz_, 0, sizeof(double) * kEntryPad, s));
    return FAIR_OK;
}

void GeomTables::release() {
    grid.release(); cth.release(); sth.release(); bx0.release(); by0.release();
    ax0th.release(); ay0th.release(); aath.release(); abth.release();
    com.release(); som.release();
}

int sm_count() {
    static int cache[128] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 128) dev = 0;
    if (!cache[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

// ---- the library random stream ---------------------------------------------
static std::mutex g_rng_mu;
static uint64_t g_seed = 0, g_ctr = 0;

static double rng_next() { return uniform01(g_seed, g_ctr++); }

// `count` consecutive draws of the library stream, for a consumer that
// evaluates them itself (on the device): the stream's seed and first counter.
void rng_take(uint64_t count, uint64_t *seed, uint64_t *ctr) {
    std::lock_guard<std::mutex> lk(g_rng_mu);
    *seed = g_seed;
    *ctr = g_ctr;
    g_ctr += count;
}
static uint64_t rng_reserve(uint64_t k) {
    uint64_t c = g_ctr;
    g_ctr += k;
    return c;
}

// scramble, AIRMs.f90:1175-1212: two passes of swaps with j = 1 + floor(n*u).
static void scramble_host(int32_t n, int32_t *arr) {
    for (int32_t i = 0; i < n; ++i) arr[i] = i + 1;
    for (int k = 0; k < 2; ++k) {
        for (int32_t i = 1; i <= n; ++i) {
            double u = rng_next();
            int32_t j = 1 + (int32_t)std::floor(n * u);
            std::swap(arr[j - 1], arr[i - 1]);
        }
    }
}

// linspace, system_generation.f90:17-35
void linspace_host(double a, double b, int n, double *x) {
    double c = (b - a) / (n - 1);
    double d = a - c;
    for (int i = 1; i <= n; ++i) x[i - 1] = c * i + d;
}

template <typename T>
static int upload(DevBuf &buf, const T *src, size_t count, cudaStream_t s) {
    FAIR_TRY(buf.grow(sizeof(T) * (count ? count : 1)));
    if (count) FAIR_CUDA(cudaMemcpyAsync(buf.p, src, sizeof(T) * count, cudaMemcpyHostToDevice, s));
    return FAIR_OK;
}

template <typename T>
static int download(T *dst, const void *src, size_t count, cudaStream_t s) {
    if (count) FAIR_CUDA(cudaMemcpyAsync(dst, src, sizeof(T) * count, cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    return FAIR_OK;
}

static int ensure_transpose(fair_csr h) {
    if (h->at_valid) return FAIR_OK;
    FAIR_TRY(csr_build_transpose(h->A, h->AT, h->stream));
    h->at_valid = true;
    return FAIR_OK;
}

static void invalidate_transpose(fair_csr h) {
    h->AT.release();
    h->at_valid = false;
    h->sirt_ready = false;
}

struct OptVals {
    bool upb = false, lwrb = false, rowprob = false, verbose = false;
    double ub = 0.0, lb = 1.0, dmp = 0.0, omg = 1.0;
    int bmode() const { return (upb ? 1 : 0) | (lwrb ? 2 : 0); }
};

static OptVals read_opts(const fair_opts *o) {
    OptVals v;
    if (o) {
        v.upb = o->upb != 0;
        v.lwrb = o->lwrb != 0;
        v.ub = o->ubound;
        v.lb = o->lbound;
        v.dmp = o->damp;
        v.omg = o->relaxpar;
        v.rowprob = o->rowprobability != 0;
        v.verbose = o->verbose != 0;
    }
    return v;
}

}  // namespace fair

using namespace fair;

#define ENTER(h)                                                  \
    do {                                                          \
        if (!(h)) { set_detail("null handle"); return FAIR_ERR_NULL; } \
        FAIR_CUDA(cudaSetDevice((h)->device));                    \
    } while (0)

#define NEED_MATRIX(h)                                                   \
    do {                                                                 \
        if ((h)->A.empty()) { set_detail("handle holds no matrix"); return FAIR_ERR_STATE; } \
    } while (0)

// Entry points that read FP64 values refuse a matrix held in FP32 only
// (fair_paralleltomo_f32).
#define NEED_F64(h)                                                                         \
    do {                                                                                    \
        if ((h)->A.f32_only) {                                                              \
            set_detail("the matrix is held in FP32 only (fair_paralleltomo_f32): no FP64 values"); \
            return FAIR_ERR_STATE;                                                          \
        }                                                                                   \
    } while (0)

extern "C" {

const char *fair_error_string(int status) {
    switch (status) {
        case FAIR_OK: return "ok";
        case FAIR_ERR_SIZE: return "Vector input size incorrect.";
        case FAIR_ERR_METHOD: return "Unknown method or stopping rule.";
        case FAIR_ERR_GEOMETRY: return "++ Something went wrong";
        case FAIR_ERR_ARG: return "Invalid argument.";
        case FAIR_ERR_NEWTON: return "Newton method did not converge.";
        case FAIR_ERR_ALLOC: return "Allocation failed.";
        case FAIR_ERR_CUDA: return "CUDA error.";
        case FAIR_ERR_NULL: return "Null handle or pointer.";
        case FAIR_ERR_STATE: return "Handle holds no matrix.";
        case FAIR_ERR_NOGPU: return "No CUDA device available.";
        default: return "Unknown status.";
    }
}

const char *fair_last_error_detail(void) { return g_detail.c_str(); }

// ---------------------------------------------------------------- handles ----
int fair_csr_create(fair_csr *out) {
    if (!out) return FAIR_ERR_NULL;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_detail(e != cudaSuccess ? cudaGetErrorString(e) : "no CUDA device");
        return FAIR_ERR_NOGPU;
    }
    fair_csr h = new (std::nothrow) fair_csr_s();
    if (!h) return FAIR_ERR_ALLOC;
    cudaGetDevice(&h->device);
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    h->own_stream = true;
    if (h->w_sched.grow(4 * sizeof(unsigned)) != FAIR_OK ||
        cudaMemset(h->w_sched.p, 0, 4 * sizeof(unsigned)) != cudaSuccess) {
        fair_csr_destroy(h);
        return FAIR_ERR_ALLOC;
    }
    *out = h;
    return FAIR_OK;
}

int fair_csr_destroy(fair_csr h) {
    if (!h) return FAIR_OK;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    h->A.release();
    h->AT.release();
    DevBuf *bufs[] = {&h->w_in, &h->w_out, &h->w_b, &h->w_x, &h->w_x32, &h->w_r, &h->w_M,
                      &h->w_D, &h->w_xn, &h->w_tmp, &h->w_part, &h->w_flag, &h->w_ord,
                      &h->w_cumul, &h->w_nrA, &h->w_y, &h->s_M, &h->s_D, &h->s_r, &h->s_x32, &h->w_sched};
    for (DevBuf *b : bufs) b->release();
    h->w_sweep.release();
    if (h->own_stream) cudaStreamDestroy(h->stream);
    delete h;
    return FAIR_OK;
}

int fair_csr_set_stream(fair_csr h, void *cuda_stream) {
    ENTER(h);
    FAIR_CUDA(cudaStreamSynchronize(h->stream));
    if (h->own_stream) cudaStreamDestroy(h->stream);
    if (cuda_stream) {
        h->stream = (cudaStream_t)cuda_stream;
        h->own_stream = false;
    } else {
        FAIR_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    return FAIR_OK;
}

int fair_csr_info(fair_csr h, int32_t *m, int32_t *n, int64_t *nnz) {
    if (!h) return FAIR_ERR_NULL;
    if (m) *m = h->A.m;
    if (n) *n = h->A.n;
    if (nnz) *nnz = h->A.nnz;
    return FAIR_OK;
}

int fair_csr_set_precision(fair_csr h, int32_t prec) {
    if (!h) return FAIR_ERR_NULL;
    if (prec != FAIR_PREC_F64 && prec != FAIR_PREC_F32 && prec != FAIR_PREC_F16 &&
        prec != FAIR_PREC_Q16) {
        set_detail("precision must be FAIR_PREC_F64, _F32, _F16 or _Q16");
        return FAIR_ERR_ARG;
    }
    if (h->A.f32_only && prec != FAIR_PREC_F32) {
        set_detail("the matrix is held in FP32 only (fair_paralleltomo_f32)");
        return FAIR_ERR_STATE;
    }
    h->prec = prec;
    return FAIR_OK;
}

// ------------------------------------------------------------- matrix I/O ----
static int upload_csr(fair_csr h, int32_t m, int32_t n, int64_t nnz, const double *vA,
                      const int64_t *IA64, const int32_t *IA32, const int32_t *JA) {
    if (m < 0 || n < 0 || nnz < 0) { set_detail("negative size"); return FAIR_ERR_ARG; }
    if ((!IA64 && !IA32) || (nnz > 0 && (!vA || !JA))) return FAIR_ERR_NULL;
    std::vector<int64_t> ia;
    const int64_t *rp = IA64;
    if (IA32) {
        ia.resize((size_t)m + 1);
        for (int64_t i = 0; i <= m; ++i) ia[i] = IA32[i];
        rp = ia.data();
    }
    if (rp[0] != 0 || rp[m] != nnz) { set_detail("IA(0) must be 0 and IA(m) = nnz"); return FAIR_ERR_ARG; }
    invalidate_transpose(h);
    h->A.release();
    h->A.m = m;
    h->A.n = n;
    h->A.nnz = nnz;
    cudaStream_t s = h->stream;
    FAIR_TRY(upload(h->A.rowptr, rp, (size_t)m + 1, s));
    FAIR_TRY(h->A.alloc_entries(nnz, s));
    if (nnz) {
        FAIR_CUDA(cudaMemcpyAsync(h->A.col.p, JA, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, s));
        FAIR_CUDA(cudaMemcpyAsync(h->A.v64.p, vA, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    }
    int st = csr_check_upload(h->A, s);
    if (st) h->A.release();
    return st;
}

int fair_construct_csr_matrix(int32_t m, int32_t n, const double *vA, const int32_t *IA,
                              const int32_t *JA, fair_csr h) {
    ENTER(h);
    if (!IA) return FAIR_ERR_NULL;
    return upload_csr(h, m, n, m >= 0 ? IA[m] : 0, vA, nullptr, IA, JA);
}

int fair_construct_csr_matrix64(int32_t m, int32_t n, const double *vA, const int64_t *IA,
                                const int32_t *JA, fair_csr h) {
    ENTER(h);
    if (!IA) return FAIR_ERR_NULL;
    return upload_csr(h, m, n, m >= 0 ? IA[m] : 0, vA, IA, nullptr, JA);
}

int fair_csr_download(fair_csr h, double *vA, int64_t *IA, int32_t *JA) {
    ENTER(h);
    NEED_MATRIX(h);
    cudaStream_t s = h->stream;
    if (IA) FAIR_TRY(download<int64_t>(IA, h->A.rowptr.p, (size_t)h->A.m + 1, s));
    if (vA) NEED_F64(h);
    if (vA) FAIR_TRY(download<double>(vA, h->A.v64.p, (size_t)h->A.nnz, s));
    if (JA) {
        FAIR_TRY(download<int32_t>(JA, h->A.col.p, (size_t)h->A.nnz, s));
        for (int64_t k = 0; k < h->A.nnz; ++k) JA[k] += 1;
    }
    return FAIR_OK;
}

// ---------------------------------------------------------------- geometry ----
int fair_linspace(double a, double b, int32_t n, double *x) {
    if (!x) return FAIR_ERR_NULL;
    if (n < 1) return FAIR_ERR_ARG;
    linspace_host(a, b, n, x);
    return FAIR_OK;
}

static int check_data(const fair_data *dat) {
    if (!dat || !dat->theta) return FAIR_ERR_NULL;
    if (dat->n < 1 || dat->p < 1 || dat->nth < 1) { set_detail("n, p, nth must be positive"); return FAIR_ERR_ARG; }
    if ((int64_t)dat->nth * dat->p > INT32_MAX || (int64_t)dat->n * dat->n > INT32_MAX) {
        set_detail("nth*p and n^2 must fit in 32-bit indices");
        return FAIR_ERR_ARG;
    }
    return FAIR_OK;
}

int fair_paralleltomo(const fair_data *dat, fair_csr h) {
    ENTER(h);
    FAIR_TRY(check_data(dat));
    const int N = dat->n, p = dat->p, nth = dat->nth;
    // system_generation.f90:328-331
    std::vector<double> x0(p), y0(p), grid(N + 1), ct(nth), st(nth);
    double d = p - 1;
    linspace_host(-.5 * d, .5 * d, p, x0.data());  // p = 1 gives 0/0 = NaN, as the reference
    for (int j = 0; j < p; ++j) y0[j] = 0 * x0[j];
    linspace_host(-.5 * N, .5 * N, N + 1, grid.data());
    for (int i = 0; i < nth; ++i) {
        ct[i] = cos(dat->theta[i]);
        st[i] = sin(dat->theta[i]);
    }
    GeomTables T;
    T.kind = 0; T.N = N; T.nth = nth; T.p = p;
    cudaStream_t s = h->stream;
    FAIR_TRY(upload(T.grid, grid.data(), grid.size(), s));
    FAIR_TRY(upload(T.cth, ct.data(), ct.size(), s));
    FAIR_TRY(upload(T.sth, st.data(), st.size(), s));
    FAIR_TRY(upload(T.bx0, x0.data(), x0.size(), s));
    FAIR_TRY(upload(T.by0, y0.data(), y0.size(), s));
    invalidate_transpose(h);
    int stt = build_geometry(T, h->A, s);
    FAIR_CUDA(cudaStreamSynchronize(s));
    T.release();
    return stt;
}

int fair_fanlineartomo(const fair_data *dat, int32_t geometry_fix, fair_csr h) {
    ENTER(h);
    FAIR_TRY(check_data(dat));
    const int N = dat->n, p = dat->p, nth = dat->nth;
    const double pi = 3.141592653589793;  // 4*atan(1d0), system_generation.f90:4
    // system_generation.f90:98-130
    const double R = dat->r * N, dwn = dat->dw * N, sdn = dat->sd * N;
    const double dew = dwn / p;
    std::vector<double> grid(N + 1), omega(p), com(p), som(p);
    for (int i = 1; i <= N + 1; ++i) grid[i - 1] = i - .5 * N - 1.0;
    if (p % 2 == 1) {
        int hh = (p - 1) / 2;
        for (int i = 1; i <= hh; ++i) {
            double dep = i * dew;
            omega[hh - i] = atan(sdn / dep) - (geometry_fix ? .5 * pi : .5);  // :122
            omega[hh + i] = .5 * pi - atan(sdn / dep);
        }
        omega[hh] = 0.0;
    } else {
        int hh = p / 2;
        for (int i = 1; i <= hh; ++i) {
            double dep = (i - .5) * dew;
            omega[hh - i] = atan(sdn / dep) - .5 * pi;  // :129
            omega[hh + i - 1] = .5 * pi - atan(sdn / dep);
        }
    }
    for (int j = 0; j < p; ++j) {
        com[j] = cos(omega[j]);
        som[j] = sin(omega[j]);
    }
    // per angle: rotated source (0,R) and unit direction towards the origin (:146-152)
    std::vector<double> ax0th(nth), ay0th(nth), aath(nth), abth(nth);
    for (int i = 0; i < nth; ++i) {
        double c = cos(dat->theta[i]), s = sin(dat->theta[i]);
        double x0th = c * 0.0 - s * R;
        double y0th = s * 0.0 + c * R;
        ax0th[i] = x0th;
        ay0th[i] = y0th;
        aath[i] = -x0th / R;
        abth[i] = -y0th / R;
    }
    GeomTables T;
    T.kind = 1; T.N = N; T.nth = nth; T.p = p;
    cudaStream_t s = h->stream;
    FAIR_TRY(upload(T.grid, grid.data(), grid.size(), s));
    FAIR_TRY(upload(T.com, com.data(), com.size(), s));
    FAIR_TRY(upload(T.som, som.data(), som.size(), s));
    FAIR_TRY(upload(T.ax0th, ax0th.data(), ax0th.size(), s));
    FAIR_TRY(upload(T.ay0th, ay0th.data(), ay0th.size(), s));
    FAIR_TRY(upload(T.aath, aath.data(), aath.size(), s));
    FAIR_TRY(upload(T.abth, abth.data(), abth.size(), s));
    invalidate_transpose(h);
    int stt = build_geometry(T, h->A, s);
    FAIR_CUDA(cudaStreamSynchronize(s));
    T.release();
    return stt;
}

int fair_add_white_noise(double *bt, double *e, const double *b, int64_t m, double eta) {
    if (!bt || !e || !b) return FAIR_ERR_NULL;
    const double pi = 3.141592653589793, tol = 1e-14;
    std::lock_guard<std::mutex> lk(g_rng_mu);
    // system_generation.f90:725-743
    for (int64_t k = 0; k < m; ++k) {
        double u = rng_next();
        double x = 0.0;
        for (int i = 1; i <= 100; ++i) {
            double f = .5 * (1 + erf(x / sqrt(2.0))) - u;
            double df = sqrt(2.0 / pi) * exp(-.5 * (x * x));
            if (fabs(f / df) < tol) break;
            if (i == 100 && fabs(f / df) > tol) return FAIR_ERR_NEWTON;
            x = x - f / df;
        }
        e[k] = x;
    }
    double nb = 0, ne = 0;
    for (int64_t k = 0; k < m; ++k) nb += b[k] * b[k];
    for (int64_t k = 0; k < m; ++k) ne += e[k] * e[k];
    nb = sqrt(nb);
    ne = sqrt(ne);
    double sc = eta * nb;
    for (int64_t k = 0; k < m; ++k) {
        e[k] = sc * e[k] / ne;
        bt[k] = b[k] + e[k];
    }
    return FAIR_OK;
}

// --------------------------------------------------------------- operators ----
static int apply_op(fair_csr h, const DevCSR &M, const double *v, double *w) {
    cudaStream_t s = h->stream;
    FAIR_TRY(upload(h->w_in, v, (size_t)M.n, s));
    FAIR_TRY(h->w_out.grow(sizeof(double) * ((size_t)M.m + 1)));
    if (h->prec == FAIR_PREC_F64) {
        FAIR_TRY(spmv(M, FAIR_PREC_F64, h->w_in.p, h->w_out.p, s, h->w_sched.as<unsigned>()));
    } else {
        FAIR_TRY(h->w_x32.grow(sizeof(float) * ((size_t)M.n + 1)));
        FAIR_TRY(h->w_tmp.grow(sizeof(float) * ((size_t)M.m + 1)));
        FAIR_TRY(vec_to_f32(h->w_in.as<double>(), M.n, h->w_x32.as<float>(), s));
        FAIR_TRY(spmv(M, h->prec, h->w_x32.p, h->w_tmp.p, s, h->w_sched.as<unsigned>()));
        FAIR_TRY(vec_to_f64(h->w_tmp.as<float>(), M.m, h->w_out.as<double>(), s));
    }
    return download<double>(w, h->w_out.p, (size_t)M.m, s);
}

int fair_matvecmul(fair_csr h, const double *v, int64_t size_v, double *w) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!v || !w) return FAIR_ERR_NULL;
    if (size_v != h->A.n) return FAIR_ERR_SIZE;  // sparse_matrices.f90:284-288
    return apply_op(h, h->A, v, w);
}

int fair_transvecmul(fair_csr h, const double *v, int64_t size_v, double *w) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!v || !w) return FAIR_ERR_NULL;
    if (size_v != h->A.m) return FAIR_ERR_SIZE;  // sparse_matrices.f90:315-319
    FAIR_TRY(ensure_transpose(h));
    return apply_op(h, h->AT, v, w);
}

int fair_rowvecmult(fair_csr h, int32_t k, const double *v, int64_t size_v, double *f) {
    ENTER(h);
    NEED_MATRIX(h);
    NEED_F64(h);
    if (!v || !f) return FAIR_ERR_NULL;
    if (k < 1 || k > h->A.m) { set_detail("row index outside 1..m"); return FAIR_ERR_ARG; }
    if (size_v != h->A.n) return FAIR_ERR_SIZE;
    cudaStream_t s = h->stream;
    FAIR_TRY(upload(h->w_in, v, (size_t)h->A.n, s));
    FAIR_TRY(h->w_out.grow(sizeof(double)));
    FAIR_TRY(csr_row_dot(h->A, k - 1, h->w_in.as<double>(), h->w_out.as<double>(), s));
    return download<double>(f, h->w_out.p, 1, s);
}

int fair_add_scalar_mult_row(fair_csr h, int32_t k, double c, double *w, int64_t size_w,
                             const double *lwrb, const double *upb) {
    ENTER(h);
    NEED_MATRIX(h);
    NEED_F64(h);
    if (!w) return FAIR_ERR_NULL;
    if (k < 1 || k > h->A.m) { set_detail("row index outside 1..m"); return FAIR_ERR_ARG; }
    if (size_w != h->A.n) return FAIR_ERR_SIZE;
    cudaStream_t s = h->stream;
    FAIR_TRY(upload(h->w_in, w, (size_t)h->A.n, s));
    int bmode = (upb ? 1 : 0) | (lwrb ? 2 : 0);
    FAIR_TRY(csr_add_mult_row(h->A, k - 1, c, h->w_in.as<double>(), bmode, lwrb ? *lwrb : 0.0,
                              upb ? *upb : 0.0, s));
    return download<double>(w, h->w_in.p, (size_t)h->A.n, s);
}

int fair_row_norms(fair_csr h, int32_t p, double *nrA) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!nrA) return FAIR_ERR_NULL;
    if (p < 1) { set_detail("p must be a positive integer"); return FAIR_ERR_ARG; }
    cudaStream_t s = h->stream;
    FAIR_TRY(h->w_out.grow(sizeof(double) * ((size_t)h->A.m + 1)));
    FAIR_TRY(csr_row_norms(h->A, p, h->w_out.as<double>(), s));
    return download<double>(nrA, h->w_out.p, (size_t)h->A.m, s);
}

int fair_column_norms(fair_csr h, int32_t p, double *ncA) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!ncA) return FAIR_ERR_NULL;
    if (p < 1) { set_detail("p must be a positive integer"); return FAIR_ERR_ARG; }
    FAIR_TRY(ensure_transpose(h));
    cudaStream_t s = h->stream;
    FAIR_TRY(h->w_out.grow(sizeof(double) * ((size_t)h->A.n + 1)));
    FAIR_TRY(csr_row_norms(h->AT, p, h->w_out.as<double>(), s));
    return download<double>(ncA, h->w_out.p, (size_t)h->A.n, s);
}

int fair_transpose(fair_csr h) {
    ENTER(h);
    NEED_MATRIX(h);
    FAIR_TRY(ensure_transpose(h));
    std::swap(h->A, h->AT);
    h->sirt_ready = false;
    return FAIR_OK;
}

int fair_multiply_by_scalar(fair_csr h, double c) {
    ENTER(h);
    NEED_MATRIX(h);
    NEED_F64(h);
    h->sirt_ready = false;
    FAIR_TRY(csr_scale(h->A, c, h->stream));
    if (h->at_valid) FAIR_TRY(csr_scale(h->AT, c, h->stream));
    FAIR_CUDA(cudaStreamSynchronize(h->stream));
    return FAIR_OK;
}

// ----------------------------------------------------------------- options ----
int fair_opts_initialise(fair_opts *o) {
    if (!o) return FAIR_ERR_NULL;
    // AIRMs.f90:29-36
    o->upb = 0; o->lwrb = 0; o->ubound = 0.0; o->lbound = 1.0;
    o->damp = 0.0; o->relaxpar = 1.0; o->verbose = 0; o->rowprobability = 0;
    return FAIR_OK;
}
int fair_opts_set_ubound(fair_opts *o, double ubound) {
    if (!o) return FAIR_ERR_NULL;
    o->upb = 1;
    o->ubound = ubound;
    return FAIR_OK;
}
int fair_opts_set_lbound(fair_opts *o, double lbound) {
    if (!o) return FAIR_ERR_NULL;
    o->lwrb = 1;
    o->lbound = lbound;
    return FAIR_OK;
}

// -------------------------------------------------------------------- SIRT ----
int fair_sirt(double *xout, const char *sirt_method, fair_csr h, const double *b,
              const int32_t *Kin, int32_t nK, const double *x0, const fair_opts *options) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!xout || !sirt_method || !b || !Kin) return FAIR_ERR_NULL;
    if (nK < 1) { set_detail("Kin is empty"); return FAIR_ERR_ARG; }
    bool sart;
    if (!strcmp(sirt_method, "cimmino")) sart = false;
    else if (!strcmp(sirt_method, "sart")) sart = true;
    else { set_detail("Not a recognised SIRT method."); return FAIR_ERR_METHOD; }  // AIRMs.f90:1082
    int32_t maxits = 0;
    for (int32_t l = 0; l < nK; ++l) maxits = std::max(maxits, Kin[l]);
    OptVals o = read_opts(options);
    const int32_t m = h->A.m, n = h->A.n;
    cudaStream_t s = h->stream;
    FAIR_TRY(ensure_transpose(h));
    FAIR_TRY(upload(h->w_b, b, (size_t)m, s));
    FAIR_TRY(h->w_x.grow(sizeof(double) * ((size_t)n + 1)));
    if (x0) FAIR_CUDA(cudaMemcpyAsync(h->w_x.p, x0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    else FAIR_CUDA(cudaMemsetAsync(h->w_x.p, 0, sizeof(double) * n, s));
    FAIR_TRY(h->w_M.grow(sizeof(double) * ((size_t)m + 1)));
    FAIR_TRY(h->w_D.grow(sizeof(double) * ((size_t)n + 1)));
    FAIR_TRY(h->w_r.grow(sizeof(double) * ((size_t)m + 1)));
    FAIR_TRY(h->w_x32.grow(sizeof(float) * ((size_t)n + 1)));
    FAIR_TRY(sirt_weights_recip(h->A, h->AT, sart, h->w_M.as<double>(), h->w_D.as<double>(), s));
    SirtDev S;
    S.prec = h->prec;
    S.m = m; S.n = n;
    S.A = &h->A; S.AT = &h->AT;
    S.b = h->w_b.as<double>();
    S.Minv = h->w_M.as<double>();
    S.D = sart ? h->w_D.as<double>() : nullptr;  // Cimmino: Ddiag = 1
    S.x = h->w_x.as<double>();
    S.x32 = h->w_x32.as<float>();
    S.r = h->w_r.p;
    S.omg = o.omg;
    S.bmode = o.bmode();
    S.lb = o.lb;
    S.ub = o.ub;
    S.sched = h->w_sched.as<unsigned>();
    FAIR_TRY(sirt_prepare_shadow(S, s));
    FAIR_TRY(sirt_iterations(S, maxits, s));
    return download<double>(xout, h->w_x.p, (size_t)n, s);
}

// ------------------------------------------------------ normest / gradient ----
static int normest_dev(fair_csr h, double tol, int maxit, double *sigma) {
    const int32_t m = h->A.m, n = h->A.n;
    cudaStream_t s = h->stream;
    FAIR_TRY(ensure_transpose(h));
    FAIR_TRY(h->w_x.grow(sizeof(double) * ((size_t)n + 1)));
    FAIR_TRY(h->w_xn.grow(sizeof(double) * ((size_t)n + 1)));
    FAIR_TRY(h->w_y.grow(sizeof(double) * ((size_t)m + 1)));
    FAIR_TRY(h->w_part.grow(sizeof(double) * (kReduceBlocks + 8)));
    FAIR_TRY(h->w_flag.grow(sizeof(int) * 4));
    uint64_t ctr;
    {
        std::lock_guard<std::mutex> lk(g_rng_mu);
        ctr = rng_reserve((uint64_t)n);  // call random_number(v), AIRMs.f90:1157
    }
    FAIR_TRY(fill_uniform(h->w_x.as<double>(), n, g_seed, ctr, s));
    return normest_run(h->A, h->AT, h->w_x.as<double>(), h->w_xn.as<double>(),
                       h->w_y.as<double>(), h->w_part.as<double>(), h->w_flag.as<int>(), tol,
                       maxit, sigma, s);
}

int fair_normest(fair_csr h, const double *tolerance, const int32_t *max_its, double *sigma) {
    ENTER(h);
    NEED_MATRIX(h);
    NEED_F64(h);
    if (!sigma) return FAIR_ERR_NULL;
    return normest_dev(h, tolerance ? *tolerance : 1e-5, max_its ? *max_its : 100, sigma);
}

int fair_gradient_descent(double *xout, fair_csr h, const double *b, const int32_t *max_iter,
                          const double *x0, const double *rho_in, const double *tolerance,
                          const fair_opts *options, int32_t *iters_done) {
    ENTER(h);
    NEED_MATRIX(h);
    NEED_F64(h);
    if (!xout || !b) return FAIR_ERR_NULL;
    OptVals o = read_opts(options);
    int maxiter = max_iter ? *max_iter : 100;
    double rho = rho_in ? *rho_in : 1.5;
    double tol = tolerance ? *tolerance : 1e-6;
    if (tol < 0.0) { set_detail("Must use positive tolerance."); return FAIR_ERR_ARG; }
    const int32_t m = h->A.m, n = h->A.n;
    cudaStream_t s = h->stream;
    double sigma = 0.0;
    FAIR_TRY(normest_dev(h, 1e-5, 100, &sigma));  // AIRMs.f90:945
    sigma = sigma * sigma;
    FAIR_TRY(upload(h->w_b, b, (size_t)m, s));
    FAIR_TRY(h->w_x.grow(sizeof(double) * ((size_t)n + 1)));
    FAIR_TRY(h->w_xn.grow(sizeof(double) * ((size_t)n + 1)));
    FAIR_TRY(h->w_r.grow(sizeof(double) * ((size_t)m + 1)));
    if (x0) FAIR_CUDA(cudaMemcpyAsync(h->w_x.p, x0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    else FAIR_CUDA(cudaMemsetAsync(h->w_x.p, 0, sizeof(double) * n, s));
    GdDev G;
    G.A = &h->A; G.AT = &h->AT;
    G.b = h->w_b.as<double>();
    G.x = h->w_x.as<double>();
    G.xn = h->w_xn.as<double>();
    G.r = h->w_r.as<double>();
    G.partials = h->w_part.as<double>();
    G.flag = h->w_flag.as<int>();
    G.step = rho / sigma;
    G.tol = tol;
    G.bmode = o.upb || o.lwrb ? o.bmode() : 0;
    G.lb = o.lb;
    G.ub = o.ub;
    FAIR_TRY(gd_run(G, maxiter, s));
    int flag[2] = {0, 0};
    FAIR_TRY(download<int>(flag, h->w_flag.p, 2, s));
    if (iters_done) *iters_done = flag[1];
    return download<double>(xout, h->w_x.p, (size_t)n, s);
}

// --------------------------------------------------------------------- ART ----
namespace {

struct ArtState {
    std::vector<int32_t> ord;
    std::vector<double> nrA, cumul;
    std::vector<int32_t> Kuse;
    int32_t nord = 0;
    bool isrand = false, issym = false;
    uint64_t order_key = 0;  // changes whenever ord changes (sweep schedules are cached by it)
};

uint64_t new_order_key() {
    static std::atomic<uint64_t> next{1};
    return next++;
}

// AIRMs.f90:217-312 (art) / :525-628 (twin_art)
int art_setup(fair_csr h, const char *method, const int32_t *Kin, int32_t nK,
              const int32_t *order, int32_t nord_in, const OptVals &o, ArtState &st) {
    const int32_t m = h->A.m;
    cudaStream_t s = h->stream;
    for (int32_t l = 1; l < nK; ++l)
        if (Kin[l] < Kin[l - 1]) { set_detail("Kin must be ascending"); return FAIR_ERR_ARG; }
    st.Kuse.assign(Kin, Kin + nK);
    bool kacz = !strcmp(method, "kaczmarz"), sym = !strcmp(method, "symkaczmarz"),
         rnd = !strcmp(method, "randkaczmarz");
    if (!kacz && !sym && !rnd) {
        set_detail("Unknown ART method. Use kaczmarz, symkaczmarz or randkaczmarz");
        return FAIR_ERR_METHOD;
    }
    if (sym) {
        for (int32_t l = 0; l < nK; ++l)
            if (Kin[l] % 2 == 1) { set_detail("Kin should all be multiples of 2."); return FAIR_ERR_ARG; }
        for (auto &k : st.Kuse) k /= 2;
    }
    st.issym = sym;
    st.isrand = rnd;
    st.ord.assign((size_t)m + 1, 0);
    if (order) {
        if (nord_in < 0 || nord_in > m) { set_detail("order longer than m"); return FAIR_ERR_ARG; }
        for (int32_t i = 0; i < nord_in; ++i) {
            if (order[i] < 1 || order[i] > m) { set_detail("order entry outside 1..m"); return FAIR_ERR_ARG; }
            st.ord[i] = order[i];
        }
        st.nord = nord_in;
    } else {
        for (int32_t i = 0; i < m; ++i) st.ord[i] = i + 1;
        st.nord = m;
    }
    // nrA = row_norms(2)**2 + damp*maxval (AIRMs.f90:273-275), rows on the GPU
    st.nrA.resize(m);
    FAIR_TRY(h->w_nrA.grow(sizeof(double) * ((size_t)m + 1)));
    FAIR_TRY(csr_row_norms(h->A, 2, h->w_nrA.as<double>(), s));
    FAIR_TRY(download<double>(st.nrA.data(), h->w_nrA.p, (size_t)m, s));
    double mx = -INFINITY;
    for (int32_t i = 0; i < m; ++i) {
        st.nrA[i] = st.nrA[i] * st.nrA[i];
        mx = std::max(mx, st.nrA[i]);
    }
    for (int32_t i = 0; i < m; ++i) st.nrA[i] = st.nrA[i] + o.dmp * mx;
    // nonzero rows only (:279-287)
    int32_t k = 0;
    for (int32_t i = 0; i < st.nord; ++i)
        if (st.nrA[st.ord[i] - 1] > 0) st.ord[k++] = st.ord[i];
    st.nord = k;
    st.cumul.assign(m, 0.0);
    if (st.isrand) {
        std::lock_guard<std::mutex> lk(g_rng_mu);
        scramble_host(st.nord, st.ord.data());  // :297
        if (o.rowprob) {  // :302-308 (indexed by position, as the reference)
            double cs = 0;
            for (int32_t i = 0; i < st.nord; ++i) { cs = cs + st.nrA[i]; st.cumul[i] = cs; }
            double tot = 0;
            for (int32_t i = 0; i < m; ++i) tot += st.nrA[i];
            for (int32_t i = 0; i < st.nord; ++i) st.cumul[i] = st.cumul[i] / tot;
            for (int32_t i = st.nord; i < m; ++i) st.cumul[i] = 1.0;
        }
    }
    st.order_key = new_order_key();
    FAIR_TRY(upload(h->w_nrA, st.nrA.data(), (size_t)m, s));
    FAIR_TRY(upload(h->w_cumul, st.cumul.data(), (size_t)m, s));
    FAIR_TRY(upload(h->w_ord, st.ord.data(), (size_t)std::max<int32_t>(st.nord, 1), s));
    return FAIR_OK;
}

int sweep(fair_csr h, const ArtState &st, const OptVals &o, const double *d_b, double *d_x,
          int dir) {
    SweepDev S;
    S.work = &h->w_sweep;
    S.A = &h->A;
    S.b = d_b;
    S.nrA = h->w_nrA.as<double>();
    S.cumul = h->w_cumul.as<double>();
    S.x = d_x;
    S.ord = h->w_ord.as<int32_t>();
    S.nord = st.nord;
    S.rand_rowprob = st.isrand && o.rowprob;
    // random orders are drawn anew in every sweep: no level schedule is kept
    S.order_key = st.isrand ? 0 : st.order_key;
    S.omg = o.omg;
    S.bmode = o.bmode();
    S.lb = o.lb;
    S.ub = o.ub;
    if (S.rand_rowprob) {
        std::lock_guard<std::mutex> lk(g_rng_mu);
        S.seed = g_seed;
        S.ctr = rng_reserve((uint64_t)st.nord);  // one random_number per step (:830)
    }
    return kaczmarz_sweep(S, dir, h->stream);
}

// Releases the sweep buffers when a Kaczmarz call returns (on every path):
// the windowed sweep's reordered entries are of the size of the matrix.
struct SweepRelease {
    SweepWork &w;
    ~SweepRelease() { w.release(); }
};

int rescramble(fair_csr h, ArtState &st) {
    {
        std::lock_guard<std::mutex> lk(g_rng_mu);
        scramble_host(st.nord, st.ord.data());
    }
    st.order_key = new_order_key();
    return upload(h->w_ord, st.ord.data(), (size_t)std::max<int32_t>(st.nord, 1), h->stream);
}

double host_norm_diff(fair_csr h, const double *a, const double *b, int64_t n, int &st) {
    double out = 0.0;
    st = dev_sumsq_diff(a, b, n, h->w_part.as<double>(), h->w_part.as<double>() + kReduceBlocks,
                        h->stream);
    if (!st) st = download<double>(&out, h->w_part.as<double>() + kReduceBlocks, 1, h->stream);
    return sqrt(out);
}

double host_dot(fair_csr h, const double *a, const double *b, int64_t n, int &st) {
    double out = 0.0;
    st = dev_dot(a, b, n, h->w_part.as<double>(), h->w_part.as<double>() + kReduceBlocks,
                 h->stream);
    if (!st) st = download<double>(&out, h->w_part.as<double>() + kReduceBlocks, 1, h->stream);
    return out;
}

}  // namespace

int fair_art(double *Xout, const char *art_method, fair_csr h, const double *b,
             const int32_t *Kin, int32_t nK, const double *x0, const double *xref,
             const int32_t *order, int32_t nord, const fair_opts *options) {
    ENTER(h);
    NEED_MATRIX(h);
    NEED_F64(h);
    if (!Xout || !art_method || !b || !Kin) return FAIR_ERR_NULL;
    if (nK < 1) { set_detail("Kin is empty"); return FAIR_ERR_ARG; }
    OptVals o = read_opts(options);
    ArtState st;
    SweepRelease sweep_guard{h->w_sweep};
    FAIR_TRY(art_setup(h, art_method, Kin, nK, order, nord, o, st));
    const int32_t m = h->A.m, n = h->A.n;
    cudaStream_t s = h->stream;
    FAIR_TRY(upload(h->w_b, b, (size_t)m, s));
    FAIR_TRY(h->w_x.grow(sizeof(double) * ((size_t)n + 1)));
    FAIR_TRY(h->w_xn.grow(sizeof(double) * ((size_t)n + 1)));
    FAIR_TRY(h->w_part.grow(sizeof(double) * (kReduceBlocks + 8)));
    if (x0) FAIR_CUDA(cudaMemcpyAsync(h->w_x.p, x0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    else FAIR_CUDA(cudaMemsetAsync(h->w_x.p, 0, sizeof(double) * n, s));
    if (xref) FAIR_TRY(upload(h->w_y, xref, (size_t)n, s));
    memset(Xout, 0, sizeof(double) * (size_t)n * nK);
    int32_t maxiter = 0;
    for (int32_t k : st.Kuse) maxiter = std::max(maxiter, k);
    double *dx = h->w_x.as<double>(), *dxp = h->w_xn.as<double>();
    const double *db = h->w_b.as<double>();
    int32_t l = 0;
    for (int32_t iter = 1; iter <= maxiter; ++iter) {
        if (st.isrand) FAIR_TRY(rescramble(h, st));  // :320
        if (xref) FAIR_CUDA(cudaMemcpyAsync(dxp, dx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        FAIR_TRY(sweep(h, st, o, db, dx, +1));
        if (st.issym) FAIR_TRY(sweep(h, st, o, db, dx, -1));
        if (xref) {  // oracle stop (:330-333)
            int e1 = 0, e2 = 0;
            double n1 = host_norm_diff(h, dx, h->w_y.as<double>(), n, e1);
            double n0 = host_norm_diff(h, dxp, h->w_y.as<double>(), n, e2);
            if (e1 || e2) return e1 ? e1 : e2;
            if (n1 > n0) {
                FAIR_TRY(download<double>(Xout + (size_t)n * (nK - 1), dxp, (size_t)n, s));
                break;
            }
        }
        if (l < nK && iter == st.Kuse[l]) {
            FAIR_TRY(download<double>(Xout + (size_t)n * l, dx, (size_t)n, s));
            l++;
        }
    }
    FAIR_CUDA(cudaStreamSynchronize(s));
    return FAIR_OK;
}

int fair_twin_art(double *xout, int32_t *final_it, double *Xstore, double *Ystore, double *EG,
                  const char *art_method, const char *stoprule, fair_csr h, const double *b,
                  const int32_t *Kin, int32_t nK, const double *x0, const double *y0,
                  const int32_t *order, int32_t nord, int32_t slack, const fair_opts *options) {
    ENTER(h);
    NEED_MATRIX(h);
    NEED_F64(h);
    if (!xout || !final_it || !Xstore || !Ystore || !EG || !art_method || !stoprule || !b || !Kin)
        return FAIR_ERR_NULL;
    if (nK < 1) { set_detail("Kin is empty"); return FAIR_ERR_ARG; }
    bool eg = !strcmp(stoprule, "errorgauge"), ms = !strcmp(stoprule, "mutualstep");
    OptVals o = read_opts(options);
    ArtState st;
    SweepRelease sweep_guard{h->w_sweep};
    FAIR_TRY(art_setup(h, art_method, Kin, nK, order, nord, o, st));
    if (!eg && !ms) {  // AIRMs.f90:584
        set_detail("Unknown stopping rule. Use errorgauge or mutualstep.");
        return FAIR_ERR_METHOD;
    }
    const int slck = slack >= 0 ? slack : 7;
    const int32_t m = h->A.m, n = h->A.n;
    cudaStream_t s = h->stream;
    int32_t maxK = 0;
    for (int32_t l = 0; l < nK; ++l) maxK = std::max(maxK, Kin[l]);
    memset(Xstore, 0, sizeof(double) * (size_t)n * nK);
    memset(Ystore, 0, sizeof(double) * (size_t)n * nK);
    memset(EG, 0, sizeof(double) * (size_t)std::max(maxK, 1));
    FAIR_TRY(upload(h->w_b, b, (size_t)m, s));
    FAIR_TRY(h->w_part.grow(sizeof(double) * (kReduceBlocks + 8)));
    // x, y, v, w, d in one allocation
    FAIR_TRY(h->w_tmp.grow(sizeof(double) * 5 * ((size_t)n + 1)));
    double *dx = h->w_tmp.as<double>(), *dy = dx + n + 1, *dv = dy + n + 1, *dw = dv + n + 1,
           *dd = dw + n + 1;
    FAIR_CUDA(cudaMemsetAsync(h->w_tmp.p, 0, sizeof(double) * 5 * ((size_t)n + 1), s));
    const double *db = h->w_b.as<double>();
    int e = 0;
    int startiter;
    if (x0 && y0) {
        FAIR_CUDA(cudaMemcpyAsync(dx, x0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        FAIR_CUDA(cudaMemcpyAsync(dy, y0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        double d0 = host_norm_diff(h, dx, dy, n, e);
        if (e) return e;
        if (d0 < 1e-10) { set_detail("Initial conditions x0 and y0 too close."); return FAIR_ERR_ARG; }
        startiter = 1;
    } else {
        const double *s0 = x0 ? x0 : y0;
        if (s0) {
            FAIR_CUDA(cudaMemcpyAsync(dx, s0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            FAIR_CUDA(cudaMemcpyAsync(dy, s0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        }
        FAIR_TRY(sweep(h, st, o, db, dx, +1));
        if (st.issym) FAIR_TRY(sweep(h, st, o, db, dx, -1));
        FAIR_TRY(sweep(h, st, o, db, dy, -1));
        if (st.issym) FAIR_TRY(sweep(h, st, o, db, dy, +1));
        EG[0] = host_norm_diff(h, dx, dy, n, e);
        if (e) return e;
        startiter = 2;
    }
    int32_t maxiter = 0;
    for (int32_t k : st.Kuse) maxiter = std::max(maxiter, k);
    int32_t l = 0, trck = 0, iter;
    double minEG = 1.79769313486231570815e308;  // huge(minEG)
    *final_it = 0;
    for (iter = startiter; iter <= maxiter; ++iter) {
        if (st.isrand) FAIR_TRY(rescramble(h, st));
        if (ms) FAIR_CUDA(cudaMemcpyAsync(dv, dx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        FAIR_TRY(sweep(h, st, o, db, dx, +1));
        if (st.issym) FAIR_TRY(sweep(h, st, o, db, dx, -1));
        if (ms) {  // v = x - v; x = x - v (:709-712)
            FAIR_TRY(vec_op(VEC_SUB, dv, dx, dv, 0.0, n, s));
            FAIR_TRY(vec_op(VEC_SUB, dx, dx, dv, 0.0, n, s));
            FAIR_CUDA(cudaMemcpyAsync(dw, dy, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        }
        FAIR_TRY(sweep(h, st, o, db, dy, -1));
        if (st.issym) FAIR_TRY(sweep(h, st, o, db, dy, +1));
        if (ms) {
            FAIR_TRY(vec_op(VEC_SUB, dw, dy, dw, 0.0, n, s));
            FAIR_TRY(vec_op(VEC_SUB, dy, dy, dw, 0.0, n, s));
        }
        if (eg) {  // :725-737
            double g = host_norm_diff(h, dx, dy, n, e);
            if (e) return e;
            EG[iter - 1] = g;
            if (g < minEG) {
                minEG = g;
                FAIR_CUDA(cudaMemcpyAsync(dv, dx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
                FAIR_CUDA(cudaMemcpyAsync(dw, dy, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
                trck = 0;
                *final_it = iter;
            } else {
                trck = trck + 1;
                if (trck >= slck) break;
            }
        } else {  // mutual step, :739-758
            double nw = host_norm_diff(h, dw, nullptr, n, e);
            if (e) return e;
            double nv = host_norm_diff(h, dv, nullptr, n, e);
            if (e) return e;
            FAIR_TRY(vec_op(VEC_DIV, dw, dw, nullptr, nw, n, s));
            FAIR_TRY(vec_op(VEC_DIV, dv, dv, nullptr, nv, n, s));
            FAIR_TRY(vec_op(VEC_SUB, dd, dx, dy, 0.0, n, s));
            int e1 = 0, e2 = 0, e3 = 0, e4 = 0, e5 = 0;
            double mat1 = host_dot(h, dv, dv, n, e1), mat2 = host_dot(h, dw, dw, n, e2);
            double mat3 = -host_dot(h, dv, dw, n, e3);
            double rhs1 = -host_dot(h, dv, dd, n, e4), rhs2 = host_dot(h, dw, dd, n, e5);
            if (e1 || e2 || e3 || e4 || e5) return FAIR_ERR_CUDA;
            double det = mat1 * mat2 - mat3 * mat3;
            double alph = (rhs1 * mat2 - rhs2 * mat3) / det;
            double bet = (mat1 * rhs2 - mat3 * rhs1) / det;
            FAIR_TRY(vec_op(VEC_AXPY, dx, dx, dv, alph, n, s));
            FAIR_TRY(vec_op(VEC_AXPY, dy, dy, dw, bet, n, s));
            double g = host_norm_diff(h, dx, dy, n, e);
            if (e) return e;
            EG[iter - 1] = g;
            if (fabs(alph) + fabs(bet) < 1e-5) break;
        }
        if (l < nK && iter == st.Kuse[l]) {
            FAIR_TRY(download<double>(Xstore + (size_t)n * l, dx, (size_t)n, s));
            FAIR_TRY(download<double>(Ystore + (size_t)n * l, dy, (size_t)n, s));
            l++;
        }
    }
    if (eg) {
        FAIR_TRY(vec_op(VEC_MEAN, dd, dv, dw, 0.0, n, s));
    } else {
        FAIR_TRY(vec_op(VEC_MEAN, dd, dx, dy, 0.0, n, s));
        *final_it = iter;
    }
    return download<double>(xout, dd, (size_t)n, s);
}

int fair_scramble(int32_t n, int32_t *out) {
    if (!out) return FAIR_ERR_NULL;
    if (n < 0) return FAIR_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_rng_mu);
    scramble_host(n, out);
    return FAIR_OK;
}

int fair_random_seed(uint64_t seed) {
    std::lock_guard<std::mutex> lk(g_rng_mu);
    g_seed = seed;
    g_ctr = 0;
    return FAIR_OK;
}

int fair_random_number(double *u, int64_t k) {
    if (!u && k > 0) return FAIR_ERR_NULL;
    std::lock_guard<std::mutex> lk(g_rng_mu);
    for (int64_t i = 0; i < k; ++i) u[i] = rng_next();
    return FAIR_OK;
}

// shepplogan, phantomgallery.f90:116-164 on meshgrid (:17-56), vectorised.
int fair_shepplogan(int32_t N, double *v) {
    if (!v) return FAIR_ERR_NULL;
    if (N < 2) return FAIR_ERR_ARG;
    static const double e[10][6] = {
        {1, .69, .92, 0, 0, 0},          {-.8, .6624, .874, 0, -.0184, 0},
        {-.2, .11, .31, .22, 0, -18},    {-.2, .16, .41, -.22, 0, 18},
        {.1, .21, .25, 0, .35, 0},       {.1, .046, .046, 0, .1, 0},
        {.1, .046, .046, 0, -.1, 0},     {.1, .046, .023, -.08, -.605, 0},
        {.1, .023, .023, 0, -.606, 0},   {.1, .023, .046, .06, -.605, 0}};
    const double pi = 3.141592653589793;
    std::vector<double> lx(N), ly(N);
    linspace_host(-1.0, 1.0, N, lx.data());
    linspace_host(1.0, -1.0, N, ly.data());
    std::fill(v, v + (size_t)N * N, 0.0);
    for (int q = 0; q < 10; ++q) {
        double A = e[q][0], a2 = e[q][1] * e[q][1], b2 = e[q][2] * e[q][2];
        double x0 = e[q][3], y0 = e[q][4], phi = e[q][5] * pi / 180.0;
        double c = cos(phi), sn = sin(phi);
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double u = (lx[j] - x0) * c + (ly[i] - y0) * sn;
                double w = (ly[i] - y0) * c - (lx[j] - x0) * sn;
                if (u * u / a2 + w * w / b2 <= 1.0) v[(size_t)j * N + i] += A;
            }
    }
    return FAIR_OK;
}

// ------------------------------------------------ device-resident entry points ----
int fair_sirt_prepare(fair_csr h, const char *sirt_method, const fair_opts *options) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!sirt_method) return FAIR_ERR_NULL;
    bool sart;
    if (!strcmp(sirt_method, "cimmino")) sart = false;
    else if (!strcmp(sirt_method, "sart")) sart = true;
    else { set_detail("Not a recognised SIRT method."); return FAIR_ERR_METHOD; }
    OptVals o = read_opts(options);
    const int32_t m = h->A.m, n = h->A.n;
    cudaStream_t s = h->stream;
    FAIR_TRY(ensure_transpose(h));
    FAIR_TRY(h->s_M.grow(sizeof(double) * ((size_t)m + 1)));
    FAIR_TRY(h->s_D.grow(sizeof(double) * ((size_t)n + 1)));
    FAIR_TRY(h->s_r.grow(sizeof(double) * ((size_t)m + 1)));
    FAIR_TRY(h->s_x32.grow(sizeof(float) * ((size_t)n + 1)));
    FAIR_TRY(sirt_weights_recip(h->A, h->AT, sart, h->s_M.as<double>(), h->s_D.as<double>(), s));
    FAIR_TRY(sirt_make_forms(h->A, h->AT, h->prec, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    h->sirt_sart = sart;
    h->sirt_prec = h->prec;
    h->sirt_omg = o.omg;
    h->sirt_bmode = o.bmode();
    h->sirt_lb = o.lb;
    h->sirt_ub = o.ub;
    h->sirt_ready = true;
    return FAIR_OK;
}

static int device_sirt(fair_csr h, const double *d_b, double *d_x, SirtDev &S) {
    if (!h->sirt_ready || h->sirt_prec != h->prec) {
        set_detail("call fair_sirt_prepare first (after any change of matrix or precision)");
        return FAIR_ERR_STATE;
    }
    if (!d_b || !d_x) return FAIR_ERR_NULL;
    S.prec = h->prec;
    S.m = h->A.m; S.n = h->A.n;
    S.A = &h->A; S.AT = &h->AT;
    S.b = d_b;
    S.Minv = h->s_M.as<double>();
    S.D = h->sirt_sart ? h->s_D.as<double>() : nullptr;
    S.x = d_x;
    S.x32 = h->s_x32.as<float>();
    S.r = h->s_r.p;
    S.omg = h->sirt_omg;
    S.bmode = h->sirt_bmode;
    S.lb = h->sirt_lb;
    S.ub = h->sirt_ub;
    S.sched = h->w_sched.as<unsigned>();
    return sirt_prepare_shadow(S, h->stream);
}

int fair_sirt_run_device(fair_csr h, const double *d_b, double *d_x, int32_t K) {
    ENTER(h);
    SirtDev S;
    FAIR_TRY(device_sirt(h, d_b, d_x, S));
    return sirt_iterations(S, K, h->stream);
}

int fair_sirt_run_device_timed(fair_csr h, const double *d_b, double *d_x, int32_t K,
                               float *ms_pass1, float *ms_pass2) {
    ENTER(h);
    if (!ms_pass1 || !ms_pass2) return FAIR_ERR_NULL;
    SirtDev S;
    FAIR_TRY(device_sirt(h, d_b, d_x, S));
    return sirt_iterations_timed(S, K, h->stream, ms_pass1, ms_pass2);
}

int fair_sirt_autotune(fair_csr h, const double *d_b, double *d_x, int32_t reps,
                       int32_t *config) {
    ENTER(h);
    if (reps < 1) { set_detail("reps >= 1 required"); return FAIR_ERR_ARG; }
    SirtDev S;
    FAIR_TRY(device_sirt(h, d_b, d_x, S));
    FAIR_TRY(sirt_autotune(S, h->A, h->AT, reps, h->stream, nullptr));
    if (config) {
        config[0] = h->A.sirt_lanes[h->prec];
        config[1] = h->AT.sirt_lanes[h->prec];
        config[2] = h->A.sirt_groups[h->prec];
        config[3] = h->AT.sirt_groups[h->prec];
    }
    return FAIR_OK;
}

int fair_sirt_set_lanes(fair_csr h, const int32_t *config) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!config) return FAIR_ERR_NULL;
    // lanes per row: 4-32 on the row layouts (codes 0-4); 1-8, or 0 (chosen
    // per chunk), on the sliced copy (5-8)
    auto ok = [](int32_t g, int32_t code) {
        if (code >= 0 && code <= 4) return g == 4 || g == 8 || g == 16 || g == 32;
        if (code >= 5 && code <= 8) return g == 0 || g == 1 || g == 2 || g == 4 || g == 8;
        if (code >= 9 && code <= 14) return g == 4 || g == 8 || g == 16 || g == 32;
        return false;
    };
    if (!ok(config[0], config[2]) || !ok(config[1], config[3])) {
        set_detail("layout code must be 0-14, with 4, 8, 16 or 32 lanes per row for codes 0-4 "
                   "and 9-14 and 0, 1, 2, 4 or 8 for codes 5-8");
        return FAIR_ERR_ARG;
    }
    FAIR_TRY(ensure_transpose(h));
    h->A.sirt_lanes[h->prec] = config[0];
    h->AT.sirt_lanes[h->prec] = config[1];
    h->A.sirt_groups[h->prec] = config[2];
    h->AT.sirt_groups[h->prec] = config[3];
    return FAIR_OK;
}

int fair_sirt_adjoint(fair_csr h, const char *sirt_method, int32_t nrhs, const double *b,
                      const double *x0, int32_t K, const double *lambda, const fair_opts *options,
                      const double *gx, double *xK, double *gb, double *gx0, double *glam) {
    ENTER(h);
    NEED_MATRIX(h);
    NEED_F64(h);
    if (!sirt_method || !b || !lambda || !gx || !gb || !gx0 || !glam) return FAIR_ERR_NULL;
    bool sart;
    if (!strcmp(sirt_method, "cimmino")) sart = false;
    else if (!strcmp(sirt_method, "sart")) sart = true;
    else { set_detail("Not a recognised SIRT method."); return FAIR_ERR_METHOD; }
    if (nrhs < 1 || K < 0) { set_detail("nrhs >= 1 and K >= 0 required"); return FAIR_ERR_ARG; }
    if (h->prec != FAIR_PREC_F64 && h->prec != FAIR_PREC_F32) {
        set_detail("the adjoint runs in FP64 or FP32");
        return FAIR_ERR_ARG;
    }
    OptVals o = read_opts(options);
    FAIR_TRY(ensure_transpose(h));
    return sirt_adjoint(h, sart, nrhs, b, x0, K, lambda, o.bmode(), o.lb, o.ub, gx, xK, gb, gx0,
                        glam);
}

int fair_sirt_launches(fair_csr h, int32_t K, int64_t *launches) {
    if (!h || !launches) return FAIR_ERR_NULL;
    // one FP32 shadow conversion per call in reduced precision, one kernel per
    // pass and iteration (two for a pass on a tiled copy)
    auto kernels = [](const fair::DevCSR &M, int prec) {
        const int g = M.sirt_groups[prec];
        return (g == 9 || g == 10 || g == 14) && M.tl.built() ? 2 : 1;
    };
    *launches = (h->prec != FAIR_PREC_F64 ? 1 : 0) +
                (int64_t)(kernels(h->A, h->prec) + kernels(h->AT, h->prec)) * K;
    return FAIR_OK;
}

int fair_csr_packed_info(fair_csr h, int32_t which, int32_t *has, int64_t *ngroups,
                         int64_t *nesc, int32_t *stride, int32_t *low_bits) {
    if (!h || !has || !ngroups || !nesc || !stride || !low_bits) return FAIR_ERR_NULL;
    if (which != 0 && which != 1) { set_detail("which must be 0 (A) or 1 (A')"); return FAIR_ERR_ARG; }
    const DevCSR &M = which == 0 ? h->A : h->AT;
    const bool ok = M.haspk && (which == 0 || h->at_valid);
    *has = ok ? 1 : 0;
    *ngroups = ok ? M.ngroups : 0;
    *nesc = ok ? M.nesc : 0;
    *stride = ok ? M.pk_S : 0;
    *low_bits = ok ? M.pk_L : 0;
    return FAIR_OK;
}

int fair_csr_sliced_info(fair_csr h, int32_t which, int32_t *has, int64_t *nslots) {
    if (!h || !has || !nslots) return FAIR_ERR_NULL;
    if (which != 0 && which != 1) { set_detail("which must be 0 (A) or 1 (A')"); return FAIR_ERR_ARG; }
    const DevCSR &M = which == 0 ? h->A : h->AT;
    const bool ok = M.hassl && (which == 0 || h->at_valid);
    *has = ok ? 1 : 0;
    *nslots = ok ? M.nslots : 0;
    return FAIR_OK;
}

int fair_sirt_set_tiles(fair_csr h, const int32_t *shape) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!shape) return FAIR_ERR_NULL;
    auto in = [](int32_t v, int lo, int hi) { return v == 0 || (v >= lo && v <= hi); };
    if (!in(shape[0], 16, 128) || !in(shape[1], 8, 64) || !in(shape[2], 1024, 16384)) {
        set_detail("tile shape: side of A's tiles 16-128, pixel tiles of A' 8-64, cells 1024-16384 (0: default)");
        return FAIR_ERR_ARG;
    }
    FAIR_CUDA(cudaStreamSynchronize(h->stream));
    h->A.tile_req[0] = shape[0];
    h->A.tile_req[1] = 0;
    FAIR_TRY(ensure_transpose(h));
    h->AT.tile_req[0] = shape[1];
    h->AT.tile_req[1] = shape[2];
    return FAIR_OK;  // the tiled copies are rebuilt with these shapes when a pass next reads them
}

int fair_csr_tiled_info(fair_csr h, int32_t which, int32_t *shape) {
    if (!h || !shape) return FAIR_ERR_NULL;
    if (which != 0 && which != 1) { set_detail("which must be 0 (A) or 1 (A')"); return FAIR_ERR_ARG; }
    const DevCSR &M = which == 0 ? h->A : h->AT;
    const DevCSR::Tiled &t = M.tl;
    const bool ok = t.built() && (which == 0 || h->at_valid);
    const int32_t v[8] = {ok ? 1 : 0, ok ? t.T : 0, ok ? t.ntr : 0, ok ? t.NA : 0,
                          ok ? t.nab : 0, ok ? t.W : 0, ok ? t.nunits : 0, ok ? t.kind : 0};
    for (int i = 0; i < 8; ++i) shape[i] = v[i];
    return FAIR_OK;
}

int fair_spmv_device(fair_csr h, int32_t trans, const void *d_x, void *d_y) {
    ENTER(h);
    NEED_MATRIX(h);
    if (!d_x || !d_y) return FAIR_ERR_NULL;
    if (trans) FAIR_TRY(ensure_transpose(h));
    return spmv(trans ? h->AT : h->A, h->prec, d_x, d_y, h->stream, h->w_sched.as<unsigned>());
}

}  // extern "C"
