// fair_internal.cuh -- shared declarations of the GB300 AIR hot-path library.
//
// Device layout of one matrix (DevCSR): 64-bit row offsets (m+1), 0-based
// int32 column indices, FP64 master values plus optional FP32/FP16 copies
// derived from them. The transposed matrix (CSR of A') is a second DevCSR,
// built on the GPU by a stable counting sort and cached in the handle.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "fair_gpu.h"

namespace fair {

// ---- error plumbing -------------------------------------------------------
void set_detail(const std::string &s);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define FAIR_CUDA(call)                                                          \
    do {                                                                         \
        cudaError_t e__ = (call);                                                \
        if (e__ != cudaSuccess) return ::fair::cuda_fail(e__, #call, __FILE__, __LINE__); \
    } while (0)

#define FAIR_TRY(call)                    \
    do {                                  \
        int s__ = (call);                 \
        if (s__ != FAIR_OK) return s__;   \
    } while (0)

// ---- device buffers ---------------------------------------------------------
// A growable device allocation; grow() keeps nothing of the old contents.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    int grow(size_t need);
    void release();
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

// A scratch allocation released when it goes out of scope.
struct TmpBuf : DevBuf {
    TmpBuf() = default;
    TmpBuf(const TmpBuf &) = delete;
    TmpBuf &operator=(const TmpBuf &) = delete;
    ~TmpBuf() { release(); }
};

// Spare entries after every column/value array: the 16-byte-aligned load
// window of the row engine (rows.cuh) may read up to 3 entries past the end.
constexpr int64_t kEntryPad = 4;

struct DevCSR {
    int32_t m = 0, n = 0;
    int64_t nnz = 0;
    int32_t max_row = 0;        // longest row (nonzeros)
    int lanes_per_row = 8;      // G of the row engine (4, 8, 16 or 32)
    int sirt_lanes[4] = {8, 8, 8, 8};  // G of the SIRT passes per form (autotuned)
    // layout of the SIRT passes per form: 0 the CSR; 1, 2 the packed stream with
    // that many groups per lane and step; 3, 4 the fused records (2-byte forms);
    // 5, 6 the sliced copy with 2 or 4 steps in flight; 7, 8 the same with
    // the gathers one step ahead
    int sirt_groups[4] = {0, 1, 1, 1};
    // requested shape of the tiled copy (0: the defaults): [0] the tile side
    // (A, pass 1: T x T pixels) or the pixel-tile side (A', pass 2); [1] (A')
    // the most residual cells a tile's shared copy holds (angles per block x
    // bins per angle)
    int tile_req[2] = {0, 0};
    // allocate col and v64 for nnz entries plus the pad (pad zeroed)
    int alloc_entries(int64_t nnz_, cudaStream_t s);
    DevBuf rowptr;        // int64 [m+1]
    DevBuf col;           // int32 [nnz], 0-based
    DevBuf v64;           // double [nnz]
    DevBuf v32;           // float [nnz] (derived, valid if has32)
    DevBuf v16;           // __half [nnz] (derived, valid if has16)
    DevBuf vq;            // uint16/int16 [nnz] fixed point (derived, valid if hasq)
    bool has32 = false, has16 = false, hasq = false;
    bool qsigned = false;  // vq holds int16 (some value negative) instead of uint16
    double qscale = 1.0;   // value = qscale * vq
    // Packed index stream of the reduced-precision SIRT passes (csr_make_packed):
    // rows padded to whole groups of 4 entries, one PkGroup word per group,
    // padded value copies with 4 values per group.
    int32_t stride_hint = 0;   // column step across the image (N for a ray matrix)
    int32_t tstride_hint = 0;  // the same for the transpose (bins per angle)
    bool pk_tried = false, haspk = false;
    int pk_S = 0, pk_L = 7;    // step code: delta = lo + hi * S, lo the low L bits
    int64_t ngroups = 0, nesc = 0;
    DevBuf prow;               // int64 [m+1] group offsets
    DevBuf gidx;               // uint2 [ngroups]
    DevBuf gside;              // int4 [nesc] columns of groups without a step code
    DevBuf pv64, pv32, pv16, pvq;  // padded double / float / half / 16-bit values
    bool hasp64 = false, hasp32 = false, hasp16 = false, haspq = false;
    DevBuf pf16, pfq;          // fused 16-byte records {index word, 4 values} (2-byte forms)
    bool hasf16 = false, hasfq = false;
    // Sliced copies of the packed stream (rows.cuh): slices of 32/sl_G rows
    // with sl_G lanes per row, each chunk of 32 rows one run of slots.
    DevBuf soff;               // int64 [chunks+1] slot offsets
    int64_t nslots = 0;
    int sl_G = 0;              // lanes per row of the built copy
    bool hassl = false;        // soff built
    DevBuf sidx;               // uint2 [nslots] index words (FP32 and FP64 forms)
    DevBuf sv64, sv32;         // 4 values per slot
    DevBuf sf16, sfq;          // fused records per slot (2-byte forms)
    bool hassidx = false, hassv64 = false, hassv32 = false, hassf16 = false, hassfq = false;
    // Tiled copy (tiled.cu): rows cut into segments by tiles whose part of the
    // gathered vector fits in shared memory, segments stored per tile (one
    // lane per segment, sliced by chunks of 32 segments), column indices local
    // to the tile's copy.
    struct Tiled {
        int T = 0, N = 0, ntr = 0;      // tile side, image side, tiles per image column
        // kind 0: tiles of the columns (A: pixels); kind 1: tiles of the rows
        // (A': pixels) times blocks of NA angles of the columns (rays a*p + b),
        // each with a window of W bins per angle starting at bmin
        int kind = 0, p = 0, nth = 0, NA = 1, nab = 1, W = 0;
        int cells_cap = 0;  // kind 1: the residual cells per tile it was built for
        DevBuf bmin;      // int32 [ntr*ntr*nth] (kind 1)
        DevBuf srow;      // int32 [nseg] row of each segment (value fills)
        int64_t nseg = 0, nchunks = 0, nslots = 0;
        int32_t nunits = 0;
        DevBuf segbase;   // int64 [m+1] first segment (partial slot) of each row
        DevBuf soff;      // int64 [nchunks+1] slot offsets of the chunks
        DevBuf pslot;     // int32 [nchunks*32] segment of each chunk lane (-1: none)
        DevBuf units;     // int4 [nunits] {tile, first chunk, end chunk, 0}
        DevBuf idx;       // uint2 [nslots] four local indices (FP32, FP64 forms)
        DevBuf v64, v32;  // values per slot
        DevBuf r16, rq;   // fused records {local indices, 2-byte values} (f16, q16)
        DevBuf sstart, send;  // int64 [nseg] entry range of each segment (value fills)
        // the 6-entry step records of the 2-byte forms (layout code 14): per slot
        // {six 5-bit steps of the tile-local index, six 2-byte values}, the
        // segment's first local index in anc6 [nchunks*32]
        int S6 = 0, L6 = 5;
        int64_t nslots6 = 0, nesc6 = 0;
        bool tried6 = false, built6 = false;
        DevBuf soff6, anc6, code6, side6, r6_16, r6_q;
        bool has6_16 = false, has6_q = false;
        bool has_idx = false, has_v64 = false, has_v32 = false, has_r16 = false, has_rq = false;
        DevBuf part;      // partial sums [nseg] (8 bytes each)
        bool built() const { return T > 0; }
        void release();
    } tl;
    // Delta copies (sirt_delta.cu): the sliced layout with one lane per row
    // whose slots carry column steps from the row's previous entry instead of
    // columns (the row's first column is its anchor). dl[0]: 4 entries per
    // slot, a word of four 7-bit steps beside the values (FP32, FP64 forms);
    // dl[1]: 6 entries per slot in one 16-byte record {six 5-bit steps, six
    // 2-byte values} (f16, q16).
    // Matrices held in FP32 only (fair_paralleltomo_f32): no FP64 values; the
    // rows' 1- and 2-norms, computed in FP64 from the traced FP64 values, are
    // kept for the SIRT weights and the norm queries.
    bool f32_only = false;
    DevBuf rn1, rn2;   // double [m]
    struct Delta {
        int E = 4, bits = 7;      // entries per slot, bits per step code
        int S = 0, L = 7;         // step code: delta = lo + hi * S, lo the low L bits
        int64_t nslots = 0, nesc = 0;
        bool tried = false, built = false;
        DevBuf soff;              // int64 [chunks+1]
        DevBuf anchor;            // int32 [m] first column of each row (0 if empty)
        DevBuf code;              // uint32 [nslots] step words
        DevBuf side;              // int4 [nesc*(E+3)/4] the columns of a slot without codes
        DevBuf v64, v32;          // 4 values per slot (E = 4)
        DevBuf r16, rq;           // records {word, six 2-byte values} (E = 6)
        bool has_v64 = false, has_v32 = false, has_r16 = false, has_rq = false;
        void release();
    } dl[2];
    void drop_sliced();
    void release();
    bool empty() const { return rowptr.p == nullptr; }
};

// ---- geometry (geometry.cu) -------------------------------------------------
struct GeomTables {
    int kind = 0;  // 0 = parallel beam, 1 = fan beam
    int N = 0, nth = 0, p = 0;
    // host-computed tables (libm trig, no fused multiply-add), uploaded
    DevBuf grid;                 // N+1 grid-line coordinates (x == y)
    DevBuf cth, sth;             // parallel: cos/sin per angle
    DevBuf bx0, by0;             // parallel: detector start points per bin
    DevBuf ax0th, ay0th, aath, abth;  // fan: rotated source and direction per angle
    DevBuf com, som;             // fan: cos/sin of the ray angle per bin
    void release();
};
int build_geometry(const GeomTables &G, DevCSR &A, cudaStream_t s);
// Nonzeros the tables' rays produce (the count pass of build_geometry only).
int geometry_nnz(const GeomTables &T, int64_t *nnz, cudaStream_t s);
// linspace, system_generation.f90:17-35: x(i) = c*i + d (host).
void linspace_host(double a, double b, int n, double *x);

// ---- scans / sparse kernels (sparse.cu) -----------------------------------------
// Exclusive scan of counts[0..m) into out[0..m] (out[m] = total).
int scan_counts(const int32_t *counts, int64_t m, int64_t *out, cudaStream_t s);
int csr_max_row(DevCSR &A, cudaStream_t s);
int csr_build_transpose(const DevCSR &A, DevCSR &AT, cudaStream_t s);
// After an upload of 1-based JA: convert to 0-based, validate, find max row.
int csr_check_upload(DevCSR &A, cudaStream_t s);
int csr_make_lowprec(DevCSR &A, int prec, cudaStream_t s);
// Packed index stream plus padded values for `prec` (f32/f16/q16); leaves
// haspk false when too many groups need the escape table. Set
// FAIR_PACKED=0 to disable.
int csr_make_packed(DevCSR &A, int prec, cudaStream_t s);
bool packed_enabled();
// Fused 16-byte records of the packed stream for a 2-byte form (f16, q16).
int csr_make_fused(DevCSR &A, int prec, cudaStream_t s);
// Sliced copy of the packed stream with G lanes per row (1, 2, 4 or 8;
// rows.cuh) for `prec`, rebuilt when G changes (needs the packed stream; does
// nothing without it or when a chunk would exceed 2^31 slots).
int csr_make_sliced(DevCSR &A, int prec, int G, cudaStream_t s);
// Reduced-precision copies, packed streams and sliced copies of A and A' for
// SIRT (solvers.cu): every layout with `all`, else the ones the passes are
// set to read; no sliced copies with sliced = false.
int sirt_make_forms(DevCSR &A, DevCSR &AT, int prec, cudaStream_t s, bool all = false,
                    bool sliced = true);
int csr_scale(DevCSR &A, double c, cudaStream_t s);
int csr_row_norms(const DevCSR &A, int p, double *d_out, cudaStream_t s);
int csr_row_dot(const DevCSR &A, int32_t row, const double *d_x, double *d_out, cudaStream_t s);
int csr_add_mult_row(const DevCSR &A, int32_t row, double c, double *d_w, int bmode,
                     double lb, double ub, cudaStream_t s);

// y = A x in the requested precision (FP64 vectors for F64; FP32 for F32/F16).
// `sched`: two zeroed counters for dynamic chunk scheduling (rows.cuh), or null.
int spmv(const DevCSR &A, int prec, const void *d_x, void *d_y, cudaStream_t s,
         unsigned *sched = nullptr);

// ---- fused solvers (solvers.cu) -----------------------------------------------
struct SirtDev {
    int prec = FAIR_PREC_F64;
    int32_t m = 0, n = 0;
    const DevCSR *A = nullptr, *AT = nullptr;
    const double *b = nullptr;   // m
    const double *Minv = nullptr;  // m: 1/M, reciprocal row weights (FP64)
    const double *D = nullptr;   // n: 1/D, reciprocal column weights (FP64; nullptr: D = 1)
    double *x = nullptr;         // n, FP64 master iterate
    float *x32 = nullptr;        // n, FP32 shadow (F32/F16)
    void *r = nullptr;           // m residual (double or float)
    double omg = 1.0;
    int bmode = 0;  // bit0 = upper bound, bit1 = lower bound
    double lb = 0.0, ub = 0.0;
    unsigned *sched = nullptr;   // chunk-scheduling counters (rows.cuh)
};
int sirt_weights(const DevCSR &A, const DevCSR &AT, bool sart, double *d_M, double *d_D,
                 cudaStream_t s);
// The same weights stored as reciprocals 1/M, 1/D: what the SIRT epilogues
// (sirt_epi.cuh) multiply by.
int sirt_weights_recip(const DevCSR &A, const DevCSR &AT, bool sart, double *d_Mi, double *d_Di,
                       cudaStream_t s);
// v = 1/v elementwise (IEEE: 1/0 = Inf, 1/Inf = 0).
int vec_reciprocal(double *v, int64_t n, cudaStream_t s);
int sirt_iterations(const SirtDev &S, int K, cudaStream_t s);
// One SIRT pass (1: residual over A, 2: update over A') with the forms
// already made; enqueues one kernel.
void sirt_pass(const SirtDev &S, int pass, cudaStream_t s);
// Tiled copy of a matrix (tiled.cu) for SIRT pass `pass`: pass 1 reads A,
// whose columns must be an N x N image; pass 2 reads A', whose rows must be
// an N x N image and whose columns rays of p bins per angle (p = its stride
// hint). Does nothing for other matrices.
int csr_make_tiled(DevCSR &A, int prec, int pass, cudaStream_t s);
// The tile shape csr_make_tiled uses for M in `pass` (the request or the
// default): tile side and (pass 2) residual cells per tile.
void tiled_shape(const DevCSR &M, int pass, int *side, int *cells);
// A SIRT pass on the tiled copy (layout codes 9, 10, 14; two kernels); false
// when the matrix has no tiled copy of the form.
bool sirt_pass_tiled(const SirtDev &S, const DevCSR &M, int pass, int code, cudaStream_t s);

// Tiled passes of many problems at once (batches, tiled.cu): one launch of
// partial sums over the work units of every problem, one of row sums and
// epilogues. TlBatchProb describes one problem's pass; TlBatch holds the
// device tables built from them.
struct TlBatchProb {
    const DevCSR *M;          // A (pass 1) or A' (pass 2), its tiled copy built
    const void *xin;          // the gathered vector: x32 or x (pass 1), r (pass 2)
    const double *b, *Minv;   // pass 1: r = (b - A x) / M, Minv = 1/M
    void *r;
    const double *D;          // pass 2: x = P(x + omega A'r / D), D here 1/D; null: D = 1
    double *x;
    float *x32;
};
struct TlBatch {
    DevBuf desc, uoff, roff;  // per-problem descriptors, unit and row offsets
    int np = 0;
    int64_t units = 0, rows = 0;
    size_t smem = 0;          // shared memory of the largest tile
    void release() {
        desc.release(); uoff.release(); roff.release();
        np = 0; units = rows = 0; smem = 0;
    }
};
// True when M's tiled copy holds what a batched pass in `prec` reads.
bool tl_batch_ready(const DevCSR &M, int prec);
// Frees the parts of M's tiled copy that only its builders read.
void tl_drop_build(DevCSR &M);
int tl_batch_bind(TlBatch &T, int prec, const std::vector<TlBatchProb> &probs);
// dry: only the kernel attributes and grids (outside a graph capture).
int tl_batch_launch(const TlBatch &T, int prec, int pass, double omg, double lb, double ub, int bmode,
                    unsigned *ctr, cudaStream_t s, bool dry);
// Delta copy of the form (sirt_delta.cu): does nothing when too many groups
// would need the side table.
int csr_make_delta(DevCSR &A, int prec, cudaStream_t s);
// A SIRT pass over the delta copy (layout codes 11, 12); false without one.
bool sirt_pass_delta(const SirtDev &S, const DevCSR &M, int pass, int code, cudaStream_t s);
// One SIRT pass over the sliced copy (layout codes 5-8, sirt_sliced.cu);
// false when the matrix has no sliced copy of the form.
bool sirt_pass_sliced(const SirtDev &S, const DevCSR &M, int pass, int code, cudaStream_t s);
// Same with CUDA events around each pass; summed pass durations in ms.
int sirt_iterations_timed(const SirtDev &S, int K, cudaStream_t s, float *ms1, float *ms2);
// Times each SIRT pass for every lanes-per-row choice and keeps the fastest
// in A.sirt_lanes[prec] / AT.sirt_lanes[prec] (x and r are overwritten).
int sirt_autotune(const SirtDev &S, DevCSR &A, DevCSR &AT, int reps, cudaStream_t s,
                  float *ms_best);
int sirt_prepare_shadow(const SirtDev &S, cudaStream_t s);

// Gradient descent and power method pieces (solvers.cu).
struct GdDev {
    const DevCSR *A = nullptr, *AT = nullptr;
    const double *b = nullptr;
    double *x = nullptr, *xn = nullptr, *r = nullptr;
    double *partials = nullptr;  // reduction scratch
    int *flag = nullptr;         // [0] = done, [1] = accepted iterations
    double step = 0.0;           // rho / sigma^2
    double tol = 0.0;
    int bmode = 0;
    double lb = 0.0, ub = 0.0;
};
int gd_run(const GdDev &G, int maxiter, cudaStream_t s);
int normest_run(const DevCSR &A, const DevCSR &AT, double *d_v, double *d_vn, double *d_w,
                double *d_partials, int *d_flag, double tol, int maxit, double *sigma,
                cudaStream_t s);
int fill_uniform(double *d_v, int64_t n, uint64_t seed, uint64_t ctr, cudaStream_t s);

// Adjoint of unrolled SIRT (adjoint.cu); the handle must hold A and A'.
int sirt_adjoint(fair_csr h, bool sart, int nrhs, const double *b, const double *x0, int K,
                 const double *lam, int bmode, double lb, double ub, const double *gx,
                 double *xK, double *gb, double *gx0, double *glam);

// Kaczmarz sweep (kaczmarz.cu).
// Buffers of the Kaczmarz sweeps (kaczmarz.cu), kept by the handle between the
// sweeps of one call and released at its end.
struct SweepWork {
    DevBuf steps;                      // schedule of one sweep
    // level set-up: step lengths and entry offsets, grouped columns, window
    // rows, longest paths within the windows, levels, per-level counts, the
    // column level table (large images), the fallback flag, the blocks' stamp
    // tables
    DevBuf lens, eoff, idx, rec, dpath, lvl, cnt, lvtab, err, tabs;
    DevBuf gsync;                      // grid barrier of the cooperative sweep {count, generation, error}
    int32_t tab_n = 0, tab_blocks = 0;
    uint64_t uid = 0;                  // next window stamp (the tables hold older ones)
    bool err_valid = false;            // err holds the set-up's repeated-column flag
    // level schedules of the last order per direction (forward, backward)
    struct Levels {
        uint64_t key = 0;              // the order they were built for (0: none)
        int32_t nord = 0, nlev = 0;    // steps, levels
        int64_t entries = 0;           // entries of all steps
        bool use = false;              // enough steps per level to run the levels
        DevBuf sched, lptr, dnlev;     // steps in level order, level pointers, level count
    } lev[2];
    void release();
};

struct SweepDev {
    SweepWork *work = nullptr;
    // identifies the step order of a sweep (the same key: the same rows in the
    // same order); 0 for orders drawn anew in each sweep
    uint64_t order_key = 0;
    const DevCSR *A = nullptr;
    const double *b = nullptr, *nrA = nullptr, *cumul = nullptr;
    double *x = nullptr;
    const int32_t *ord = nullptr;  // 1-based rows
    int32_t nord = 0;
    bool rand_rowprob = false;
    uint64_t seed = 0, ctr = 0;
    double omg = 1.0;
    int bmode = 0;  // bit0 = upper bound, bit1 = lower bound (add_mult_row)
    double lb = 0.0, ub = 0.0;
};
int kaczmarz_sweep(const SweepDev &S, int dir, cudaStream_t s);

// Elementwise vector ops (solvers.cu): op 0: out = a - b; 1: out = a + c*b;
// 2: out = a / c; 3: out = .5*(a + b). Every operation separately rounded.
enum { VEC_SUB = 0, VEC_AXPY = 1, VEC_DIV = 2, VEC_MEAN = 3 };
int vec_op(int op, double *out, const double *a, const double *b, double c, int64_t n,
           cudaStream_t s);
int vec_to_f32(const double *a, int64_t n, float *o, cudaStream_t s);
int vec_to_f64(const float *a, int64_t n, double *o, cudaStream_t s);

// Deterministic reductions (solvers.cu).
int dev_sumsq_diff(const double *a, const double *b, int64_t n, double *d_partials,
                   double *d_out, cudaStream_t s);
int dev_dot(const double *a, const double *b, int64_t n, double *d_partials, double *d_out,
            cudaStream_t s);

// ---- launch helpers -----------------------------------------------------------
int sm_count();
constexpr int kReduceBlocks = 4096;  // partial-sum slots used by reductions (>= any grid)

// Grid of a chunk kernel (rows.cuh, 256 threads = 8 warps per block): the
// blocks that stay resident on every SM, no more than the chunks of 32 rows
// need, and never more than the partial-sum slots.
template <class K>
int chunk_grid(K kernel, int64_t m) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, 0);
    if (occ < 1) occ = 1;
    const int64_t need = (((int64_t)m + 31) / 32 + 7) / 8;
    int64_t g = (int64_t)sm_count() * occ;
    if (g > need) g = need;
    if (g < 1) g = 1;
    return (int)(g < kReduceBlocks ? g : kReduceBlocks);
}

// ---- project random stream ---------------------------------------------------------
// Reserve `count` draws of the library stream (fair_host.cu): seed and first counter.
void rng_take(uint64_t count, uint64_t *seed, uint64_t *ctr);
__host__ __device__ inline uint64_t splitmix64(uint64_t seed, uint64_t k) {
    uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__host__ __device__ inline double uniform01(uint64_t seed, uint64_t k) {
    return (double)(splitmix64(seed, k) >> 11) * 0x1.0p-53;
}

// gfortran MAX/MIN semantics: the non-NaN argument wins.
__host__ __device__ inline double fmax_f(double a, double b) { return (b > a || a != a) ? b : a; }
__host__ __device__ inline double fmin_f(double a, double b) { return (b < a || a != a) ? b : a; }

}  // namespace fair

// The opaque handle behind fair_csr.
struct fair_csr_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int prec = FAIR_PREC_F64;
    fair::DevCSR A;   // the matrix
    fair::DevCSR AT;  // cached transpose
    bool at_valid = false;
    // work buffers reused across calls
    fair::DevBuf w_in, w_out, w_b, w_x, w_x32, w_r, w_M, w_D, w_xn, w_tmp, w_part, w_flag;
    fair::DevBuf w_ord, w_cumul, w_nrA, w_y;
    fair::DevBuf w_sched;  // two zeroed counters for dynamic chunk scheduling
    fair::SweepWork w_sweep;  // Kaczmarz sweep buffers (released after each call)
    // state of fair_sirt_prepare (device-resident SIRT)
    bool sirt_ready = false, sirt_sart = false;
    int sirt_prec = FAIR_PREC_F64;
    double sirt_omg = 1.0, sirt_lb = 0.0, sirt_ub = 0.0;
    int sirt_bmode = 0;
    fair::DevBuf s_M, s_D, s_r, s_x32;
};
