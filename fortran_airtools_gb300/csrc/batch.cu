// batch.cu -- many independent SIRT/SART problems advanced together
// (include/fair_batch.h).
//
// Each pass of an iteration is ONE launch for the whole batch: the chunks of
// 32 rows of every problem are numbered consecutively (problem p owns chunks
// chunk0[p]..chunk0[p+1]-1), warps claim chunks from one atomic counter, find
// the owning problem by binary search over chunk0 and run the same row engine
// and epilogue as the single-problem passes (rows.cuh, sirt_epi.cuh), so a
// batched iteration computes, problem by problem, the numbers of the
// single-problem path with the same lanes per row and groups per lane. The
// K iterations (plus the FP32 shadow of x) are captured once in a CUDA graph
// and replayed. Small problems no longer cost a launch (and a tail) each.
//
// Memory per problem: reduced forms keep the packed index streams and padded
// values of A and A' (16-24 bytes per 4 nonzeros each) and the FP64 weights;
// the FP64 form keeps the CSR of A and A'. The FP64 master values are
// dropped after the weights are computed.
#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <vector>

#include "fair_batch.h"
#include "fair_internal.cuh"
#include "rows.cuh"
#include "sirt_epi.cuh"

namespace fair {

namespace {

// One pass of one problem.
struct BPass {
    const int64_t *ptr;  // packed group offsets, or CSR row pointers (FP64 form)
    const void *idx;     // packed index words (uint2), or int32 columns
    const int4 *gside;
    const void *val;     // padded values, or FP64 values
    int32_t rows;
    int S, L;
    double scale;        // fixed-point scale of 16-bit codes (else 1)
    const void *xin;     // gathered vector: x32 / x (pass 1), r (pass 2)
    const double *b, *M; // pass 1: r = (b - A x) / M
    void *r;
    const double *D;     // pass 2: x = P(x + omg A'r / D)
    double *x;
    float *x32;
};

struct BOpts {
    double omg, lb, ub;
    int bmode;
};

// last p in [0, np) with chunk0[p] <= ch (chunk0[0] = 0 <= ch < chunk0[np])
__device__ __forceinline__ int owner(const int64_t *__restrict__ chunk0, int np, int64_t ch) {
    int lo = 0, hi = np;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(chunk0 + mid) <= ch) lo = mid; else hi = mid;
    }
    return lo;
}

template <typename VT, int G, int NG, int PASS>
__global__ void __launch_bounds__(256) k_batch_pk(const BPass *__restrict__ P,
                                                  const int64_t *__restrict__ chunk0, int np,
                                                  BOpts o, unsigned *sched) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = __ldg(chunk0 + np);
    for (int64_t ch = next_chunk(sched, 0, nwarps, lane); ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int p = owner(chunk0, np, ch);
        const BPass &d = P[p];
        const int64_t base = (ch - __ldg(chunk0 + p)) << 5;
        const float mine = pk_chunk_sums<VT, float, float, G, NG>(
            d.ptr, d.rows, (const uint2 *)d.idx, d.gside, d.S, d.L, (const VT *)d.val,
            (const float *)d.xin, base);
        const int64_t row = base + lane;
        if (row < d.rows) {
            if (PASS == 1) {
                EpiResidLP e{d.b, d.M, (float *)d.r, d.scale};
                e(row, mine);
            } else {
                EpiUpdateLP e{d.D, d.x, d.x32, o.omg, o.lb, o.ub, o.bmode, d.scale};
                e(row, mine);
            }
        }
    }
    finish_chunks(sched, nwarps, lane);
}

template <int G, int PASS>
__global__ void __launch_bounds__(256) k_batch_f64(const BPass *__restrict__ P,
                                                   const int64_t *__restrict__ chunk0, int np,
                                                   BOpts o, unsigned *sched) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = __ldg(chunk0 + np);
    for (int64_t ch = next_chunk(sched, 0, nwarps, lane); ch < nchunks;
         ch = next_chunk(sched, ch, nwarps, lane)) {
        const int p = owner(chunk0, np, ch);
        const BPass &d = P[p];
        const int64_t base = (ch - __ldg(chunk0 + p)) << 5;
        const double mine = csr_chunk_sums<double, double, double, G>(
            d.ptr, d.rows, (const int32_t *)d.idx, (const double *)d.val,
            (const double *)d.xin, base);
        const int64_t row = base + lane;
        if (row < d.rows) {
            if (PASS == 1) {
                EpiResidF64 e{d.b, d.M, (double *)d.r};
                e(row, mine);
            } else {
                EpiUpdateF64 e{d.D, d.x, o.omg, o.lb, o.ub, o.bmode};
                e(row, mine);
            }
        }
    }
    finish_chunks(sched, nwarps, lane);
}

// Resident blocks of a 256-thread kernel on every SM, looked up once per
// kernel and device (so no occupancy query runs while a graph is captured:
// fair_batch_run_device primes the table before capturing).
template <class K>
int resident_grid(K kernel) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> table;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair((const void *)kernel, dev);
    auto it = table.find(key);
    if (it != table.end()) return it->second;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, 0);
    const int g = std::max(1, occ) * sm_count();
    table[key] = g;
    return g;
}

#define FAIR_BATCH_G(G, CALL)                            \
    switch (G) {                                         \
        case 4: { constexpr int g_ = 4; CALL; } break;   \
        case 16: { constexpr int g_ = 16; CALL; } break; \
        case 32: { constexpr int g_ = 32; CALL; } break; \
        default: { constexpr int g_ = 8; CALL; } break;  \
    }

// Launch one batched pass (dry: only look up its grid).
template <class K>
void launch(K kernel, bool dry, const BPass *P, const int64_t *c0, int np, const BOpts &o,
            unsigned *sched, cudaStream_t s) {
    const int grid = resident_grid(kernel);
    if (!dry) kernel<<<grid, 256, 0, s>>>(P, c0, np, o, sched);
}

template <typename VT, int PASS>
void launch_pk(int G, int NG, bool dry, const BPass *P, const int64_t *c0, int np,
               const BOpts &o, unsigned *sched, cudaStream_t s) {
    if (NG == 2)
        FAIR_BATCH_G(G, launch(k_batch_pk<VT, g_, 2, PASS>, dry, P, c0, np, o, sched, s))
    else
        FAIR_BATCH_G(G, launch(k_batch_pk<VT, g_, 1, PASS>, dry, P, c0, np, o, sched, s))
}

template <int PASS>
void launch_f64(int G, bool dry, const BPass *P, const int64_t *c0, int np, const BOpts &o,
                unsigned *sched, cudaStream_t s) {
    FAIR_BATCH_G(G, launch(k_batch_f64<g_, PASS>, dry, P, c0, np, o, sched, s))
}

}  // namespace

// The layout the "auto" batch (layout 2) chose for a class of problems (the
// same image side and bins per angle): tiled copies with their tile shape, or
// the packed streams (the CSR in FP64), and the pass times that decided it.
struct ClassChoice {
    bool tiled = false;
    int tile[3] = {0, 0, 0};  // A's tile side, A''s pixel-tile side and cells
    float ms_tiled[2] = {-1.f, -1.f}, ms_packed[2] = {-1.f, -1.f};
};

// One problem of a batch.
struct BatchProb {
    DevCSR A, AT;
    DevBuf M_sart, M_cim, D;  // FP64 reciprocal weights: 1/row 1-norms, 1/(m*|a_i|^2), 1/column 1-norms
    bool tiled = false;       // passes on the tiled copies of A and A' (else packed / CSR)
    void release() {
        A.release(); AT.release();
        M_sart.release(); M_cim.release(); D.release();
    }
};

}  // namespace fair

using fair::BatchProb;
using fair::BPass;
using fair::DevBuf;
using fair::DevCSR;

struct fair_batch_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int prec = FAIR_PREC_F32;
    std::vector<BatchProb *> probs;
    std::vector<int64_t> row_off{0}, col_off{0};
    int64_t nnz = 0;
    int cfg[4] = {8, 8, 1, 1};  // lanes A, lanes A', groups A, groups A'
    int layout = 0;             // 0: packed streams (CSR in FP64); 1: tiled copies where they
                                // build; 2: per class of problems, the faster of the two, the
                                // tiled copies with the fastest tile shape
    std::map<std::pair<int64_t, int64_t>, fair::ClassChoice> classes;  // layout 2, by (n, bins)
    int ntiled = 0;             // problems on their tiled copies
    fair::TlBatch tb1, tb2;     // device tables of the tiled problems' passes
    // prepared state
    bool ready = false, sart = false;
    fair::BOpts opts{1.0, 0.0, 0.0, 0};
    // device tables and work vectors
    DevBuf desc1, desc2, c0_1, c0_2, sched, x32, r, w_b, w_x;
    const double *bound_b = nullptr;
    double *bound_x = nullptr;
    // captured iterations
    cudaGraphExec_t gexec = nullptr;
    int g_K = -1, g_cfg[4] = {0, 0, 0, 0};
    const double *g_x = nullptr;  // the shadow conversion of x is a graph node
    std::mutex mu;
};

namespace fair {
namespace {

int64_t device_bytes(const fair_batch_s *B) {
    int64_t t = 0;
    auto add = [&](const DevBuf &d) { t += (int64_t)d.bytes; };
    for (const BatchProb *p : B->probs) {
        for (const DevCSR *M : {&p->A, &p->AT}) {
            add(M->rowptr); add(M->col); add(M->v64); add(M->v32); add(M->v16); add(M->vq);
            add(M->prow); add(M->gidx); add(M->gside); add(M->pv32); add(M->pv16); add(M->pvq);
            const DevCSR::Tiled &tl = M->tl;
            for (const DevBuf *d : {&tl.bmin, &tl.segbase, &tl.soff, &tl.pslot, &tl.units, &tl.idx, &tl.v64,
                                    &tl.v32, &tl.r16, &tl.rq, &tl.part})
                add(*d);
        }
        add(p->M_sart); add(p->M_cim); add(p->D);
    }
    for (const DevBuf *d : {&B->desc1, &B->desc2, &B->c0_1, &B->c0_2, &B->sched, &B->x32,
                            &B->r, &B->w_b, &B->w_x})
        add(*d);
    return t;
}

void drop_graph(fair_batch_s *B) {
    if (B->gexec) cudaGraphExecDestroy(B->gexec);
    B->gexec = nullptr;
    B->g_K = -1;
}

// Descriptor tables of the two passes for vectors d_b, d_x.
int bind_vectors(fair_batch_s *B, const double *d_b, double *d_x) {
    const int np = (int)B->probs.size();
    const bool red = B->prec != FAIR_PREC_F64;
    std::vector<BPass> t1(np), t2(np);
    std::vector<int64_t> c1(np + 1, 0), c2(np + 1, 0);
    std::vector<TlBatchProb> l1, l2;
    const size_t sx = red ? sizeof(float) : sizeof(double);
    for (int p = 0; p < np; ++p) {
        BatchProb &q = *B->probs[p];
        const int64_t ro = B->row_off[p], co = B->col_off[p];
        char *r = (char *)B->r.p + sx * ro;
        const void *xin = red ? (const void *)(B->x32.as<float>() + co) : (const void *)(d_x + co);
        if (q.tiled) {  // no chunks in the packed / CSR launch
            c1[p + 1] = c1[p];
            c2[p + 1] = c2[p];
            l1.push_back(TlBatchProb{&q.A, xin, d_b + ro, B->sart ? q.M_sart.as<double>() : q.M_cim.as<double>(),
                                     r, nullptr, nullptr, nullptr});
            l2.push_back(TlBatchProb{&q.AT, r, nullptr, nullptr, nullptr, B->sart ? q.D.as<double>() : nullptr,
                                     d_x + co, red ? B->x32.as<float>() + co : nullptr});
            continue;
        }
        for (int pass = 1; pass <= 2; ++pass) {
            const DevCSR &M = pass == 1 ? q.A : q.AT;
            BPass d{};
            if (red) {
                d.ptr = M.prow.as<int64_t>();
                d.idx = M.gidx.p;
                d.gside = M.gside.as<int4>();
                d.val = B->prec == FAIR_PREC_F32 ? M.pv32.p : B->prec == FAIR_PREC_F16 ? M.pv16.p : M.pvq.p;
                d.S = M.pk_S;
                d.L = M.pk_L;
                d.scale = B->prec == FAIR_PREC_Q16 ? M.qscale : 1.0;
            } else {
                d.ptr = M.rowptr.as<int64_t>();
                d.idx = M.col.p;
                d.val = M.v64.p;
                d.S = 0;
                d.L = 7;
                d.scale = 1.0;
            }
            d.rows = M.m;
            if (pass == 1) {
                d.xin = xin;
                d.b = d_b + ro;
                d.M = B->sart ? q.M_sart.as<double>() : q.M_cim.as<double>();
                d.r = r;
                t1[p] = d;
                c1[p + 1] = c1[p] + ((int64_t)M.m + 31) / 32;
            } else {
                d.xin = r;
                d.D = B->sart ? q.D.as<double>() : nullptr;
                d.x = d_x + co;
                d.x32 = red ? B->x32.as<float>() + co : nullptr;
                t2[p] = d;
                c2[p + 1] = c2[p] + ((int64_t)M.m + 31) / 32;
            }
        }
    }
    cudaStream_t s = B->stream;
    FAIR_TRY(B->desc1.grow(sizeof(BPass) * std::max(np, 1)));
    FAIR_TRY(B->desc2.grow(sizeof(BPass) * std::max(np, 1)));
    FAIR_TRY(B->c0_1.grow(sizeof(int64_t) * (np + 1)));
    FAIR_TRY(B->c0_2.grow(sizeof(int64_t) * (np + 1)));
    // synchronous copies: the host tables go out of scope on return
    FAIR_CUDA(cudaStreamSynchronize(s));
    FAIR_CUDA(cudaMemcpy(B->desc1.p, t1.data(), sizeof(BPass) * np, cudaMemcpyHostToDevice));
    FAIR_CUDA(cudaMemcpy(B->desc2.p, t2.data(), sizeof(BPass) * np, cudaMemcpyHostToDevice));
    FAIR_CUDA(cudaMemcpy(B->c0_1.p, c1.data(), sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice));
    FAIR_CUDA(cudaMemcpy(B->c0_2.p, c2.data(), sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice));
    FAIR_TRY(tl_batch_bind(B->tb1, B->prec, l1));
    FAIR_TRY(tl_batch_bind(B->tb2, B->prec, l2));
    B->bound_b = d_b;
    B->bound_x = d_x;
    return FAIR_OK;
}

// One batched pass (dry: only the kernel attributes and grids, outside a
// graph capture); launch errors are left for the caller's cudaGetLastError.
int batch_pass(fair_batch_s *B, int pass, cudaStream_t s, bool dry = false) {
    const int np = (int)B->probs.size();
    const BOpts &ot = B->opts;
    if (B->ntiled > 0)
        FAIR_TRY(tl_batch_launch(pass == 1 ? B->tb1 : B->tb2, B->prec, pass, ot.omg, ot.lb, ot.ub, ot.bmode,
                                 B->sched.as<unsigned>(), s, dry));
    if (B->ntiled == np) return FAIR_OK;  // no problem on the packed streams / CSR
    const BPass *P = (pass == 1 ? B->desc1 : B->desc2).as<BPass>();
    const int64_t *c0 = (pass == 1 ? B->c0_1 : B->c0_2).as<int64_t>();
    unsigned *sched = B->sched.as<unsigned>();
    const int G = B->cfg[pass - 1], NG = B->cfg[pass + 1];
    const BOpts &o = B->opts;
    switch (B->prec) {
        case FAIR_PREC_F64:
            if (pass == 1) launch_f64<1>(G, dry, P, c0, np, o, sched, s);
            else launch_f64<2>(G, dry, P, c0, np, o, sched, s);
            break;
        case FAIR_PREC_F32:
            if (pass == 1) launch_pk<float, 1>(G, NG, dry, P, c0, np, o, sched, s);
            else launch_pk<float, 2>(G, NG, dry, P, c0, np, o, sched, s);
            break;
        case FAIR_PREC_F16:
            if (pass == 1) launch_pk<__half, 1>(G, NG, dry, P, c0, np, o, sched, s);
            else launch_pk<__half, 2>(G, NG, dry, P, c0, np, o, sched, s);
            break;
        default:
            if (pass == 1) launch_pk<uint16_t, 1>(G, NG, dry, P, c0, np, o, sched, s);
            else launch_pk<uint16_t, 2>(G, NG, dry, P, c0, np, o, sched, s);
            break;
    }
    return FAIR_OK;
}

int enqueue_iterations(fair_batch_s *B, int K, cudaStream_t s) {
    if (B->prec != FAIR_PREC_F64 && B->col_off.back() > 0)
        FAIR_TRY(vec_to_f32(B->bound_x, B->col_off.back(), B->x32.as<float>(), s));
    for (int it = 0; it < K; ++it) {
        FAIR_TRY(batch_pass(B, 1, s));
        FAIR_TRY(batch_pass(B, 2, s));
    }
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

// Keep of a problem's matrices only what the batch's passes read.
void compact(DevCSR &M, int prec, bool tiled) {
    M.drop_sliced();
    M.dl[0].release();
    M.dl[1].release();
    M.v32.release(); M.v16.release(); M.vq.release();
    M.has32 = M.has16 = M.hasq = false;
    if (tiled) {  // the tiled copy is all the passes read
        tl_drop_build(M);
        M.rowptr.release(); M.col.release(); M.v64.release();
        M.prow.release(); M.gidx.release(); M.gside.release();
        M.pv64.release(); M.pv32.release(); M.pv16.release(); M.pvq.release();
        M.pf16.release(); M.pfq.release();
        M.haspk = M.hasp64 = M.hasp32 = M.hasp16 = M.haspq = M.hasf16 = M.hasfq = false;
        return;
    }
    M.tl.release();
    if (prec == FAIR_PREC_F64) {
        M.prow.release(); M.gidx.release(); M.gside.release();
        M.pv64.release(); M.pv32.release(); M.pv16.release(); M.pvq.release();
        M.pf16.release(); M.pfq.release();
        M.haspk = M.hasp64 = M.hasp32 = M.hasp16 = M.haspq = M.hasf16 = M.hasfq = false;
    } else {
        M.rowptr.release(); M.col.release(); M.v64.release();
        M.pv64.release(); M.pf16.release(); M.pfq.release();
        M.hasp64 = M.hasf16 = M.hasfq = false;
        if (prec != FAIR_PREC_F32) { M.pv32.release(); M.hasp32 = false; }
        if (prec != FAIR_PREC_F16) { M.pv16.release(); M.hasp16 = false; }
        if (prec != FAIR_PREC_Q16) { M.pvq.release(); M.haspq = false; }
    }
}

int copy_csr(const DevCSR &src, DevCSR &dst, cudaStream_t s) {
    dst.release();
    dst.m = src.m;
    dst.n = src.n;
    dst.nnz = src.nnz;
    dst.max_row = src.max_row;
    dst.stride_hint = src.stride_hint;
    dst.tstride_hint = src.tstride_hint;
    FAIR_TRY(dst.rowptr.grow(sizeof(int64_t) * ((size_t)src.m + 1)));
    FAIR_TRY(dst.alloc_entries(src.nnz, s));
    FAIR_CUDA(cudaMemcpyAsync(dst.rowptr.p, src.rowptr.p, sizeof(int64_t) * ((size_t)src.m + 1),
                              cudaMemcpyDeviceToDevice, s));
    if (src.nnz > 0) {
        FAIR_CUDA(cudaMemcpyAsync(dst.col.p, src.col.p, sizeof(int32_t) * (size_t)src.nnz,
                                  cudaMemcpyDeviceToDevice, s));
        FAIR_CUDA(cudaMemcpyAsync(dst.v64.p, src.v64.p, sizeof(double) * (size_t)src.nnz,
                                  cudaMemcpyDeviceToDevice, s));
    }
    return FAIR_OK;
}

// Layout 2: times one problem's passes (alone, on scratch vectors) on the
// packed streams (the CSR in FP64) and on its tiled copies with each candidate
// tile shape, and keeps the faster layout, with the fastest shape per pass.
// The problem's weights and transpose are in place.
int tune_class(fair_batch_s *B, BatchProb &q, ClassChoice &c) {
    cudaStream_t s = B->stream;
    const int prec = B->prec;
    const bool red = prec != FAIR_PREC_F64;
    const int64_t m = q.A.m, n = q.A.n;
    TmpBuf b, x, x32, r, sched;
    FAIR_TRY(b.grow(sizeof(double) * (size_t)(m + 1)));
    FAIR_TRY(x.grow(sizeof(double) * (size_t)(n + 1)));
    FAIR_TRY(x32.grow(sizeof(float) * (size_t)(n + 1)));
    FAIR_TRY(r.grow(sizeof(double) * (size_t)(m + 1)));
    FAIR_TRY(sched.grow(4 * sizeof(unsigned)));
    FAIR_CUDA(cudaMemsetAsync(b.p, 0, sizeof(double) * (size_t)(m + 1), s));
    FAIR_CUDA(cudaMemsetAsync(x.p, 0, sizeof(double) * (size_t)(n + 1), s));
    FAIR_CUDA(cudaMemsetAsync(x32.p, 0, sizeof(float) * (size_t)(n + 1), s));
    FAIR_CUDA(cudaMemsetAsync(sched.p, 0, 4 * sizeof(unsigned), s));
    SirtDev S;
    S.prec = prec;
    S.m = (int32_t)m;
    S.n = (int32_t)n;
    S.A = &q.A;
    S.AT = &q.AT;
    S.b = b.as<double>();
    S.Minv = q.M_sart.as<double>();
    S.D = q.D.as<double>();
    S.x = x.as<double>();
    S.x32 = x32.as<float>();
    S.r = r.p;
    S.sched = sched.as<unsigned>();
    cudaEvent_t ev[2];
    for (auto &e : ev) FAIR_CUDA(cudaEventCreate(&e));
    struct EvScope {
        cudaEvent_t *e;
        ~EvScope() { cudaEventDestroy(e[0]); cudaEventDestroy(e[1]); }
    } evs{ev};
    // time of one pass on the layout M is set to (best of two rounds of 5)
    auto timed = [&](int pass, float *out) -> int {
        *out = -1.f;
        for (int round = 0; round < 2; ++round) {
            sirt_pass(S, pass, s);  // warm-up
            cudaEventRecord(ev[0], s);
            for (int k = 0; k < 5; ++k) sirt_pass(S, pass, s);
            cudaEventRecord(ev[1], s);
            FAIR_CUDA(cudaEventSynchronize(ev[1]));
            FAIR_CUDA(cudaGetLastError());  // a launch that failed times as nothing
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[0], ev[1]);
            ms /= 5;
            *out = round == 0 ? ms : std::min(*out, ms);
        }
        return FAIR_OK;
    };
    DevCSR *mats[2] = {&q.A, &q.AT};
    // the packed streams (reduced forms; groups of 4, 8 lanes) or the CSR (FP64)
    bool pk = !red;
    if (red) {
        FAIR_TRY(sirt_make_forms(q.A, q.AT, prec, s, false, false));
        pk = q.A.haspk && q.AT.haspk && !(prec == FAIR_PREC_Q16 && (q.A.qsigned || q.AT.qsigned));
    }
    if (pk)
        for (int pass = 1; pass <= 2; ++pass) {
            mats[pass - 1]->sirt_lanes[prec] = 8;
            mats[pass - 1]->sirt_groups[prec] = red ? 1 : 0;
            FAIR_TRY(timed(pass, &c.ms_packed[pass - 1]));
        }
    // the tiled copies, each candidate shape
    static const int shapes[2][4][2] = {{{96, 0}, {64, 0}, {128, 0}, {0, 0}},
                                        {{32, 13000}, {32, 6500}, {16, 6500}, {48, 13000}}};
    bool tl_ok = true;
    for (int pass = 1; pass <= 2 && tl_ok; ++pass) {
        DevCSR &M = *mats[pass - 1];
        float best = -1.f;
        int bk = -1;
        for (int k = 0; k < 4; ++k) {
            if (shapes[pass - 1][k][0] == 0) continue;
            M.tile_req[0] = shapes[pass - 1][k][0];
            M.tile_req[1] = shapes[pass - 1][k][1];
            FAIR_TRY(csr_make_tiled(M, prec, pass, s));
            if (!tl_batch_ready(M, prec)) continue;
            M.sirt_lanes[prec] = 8;
            M.sirt_groups[prec] = 9;
            float t = -1.f;
            FAIR_TRY(timed(pass, &t));
            if (best < 0.f || t < best) {
                best = t;
                bk = k;
            }
        }
        if (bk < 0) {
            tl_ok = false;
            break;
        }
        M.tile_req[0] = shapes[pass - 1][bk][0];
        M.tile_req[1] = shapes[pass - 1][bk][1];
        c.ms_tiled[pass - 1] = best;
    }
    for (DevCSR *M : mats) {  // the batch sets the passes' layouts itself
        M->sirt_lanes[prec] = 8;
        M->sirt_groups[prec] = red ? 1 : 0;
    }
    c.tiled = tl_ok && (!pk || c.ms_tiled[0] + c.ms_tiled[1] < c.ms_packed[0] + c.ms_packed[1]);
    c.tile[0] = q.A.tile_req[0];
    c.tile[1] = q.AT.tile_req[0];
    c.tile[2] = q.AT.tile_req[1];
    if (!c.tiled) {
        q.A.tl.release();
        q.AT.tl.release();
    }
    FAIR_CUDA(cudaStreamSynchronize(s));
    return FAIR_OK;
}

// Weights, transpose and forms of a new problem whose A is in place.
int finish_problem(fair_batch_s *B, BatchProb &q) {
    cudaStream_t s = B->stream;
    FAIR_TRY(csr_build_transpose(q.A, q.AT, s));
    FAIR_TRY(q.M_sart.grow(sizeof(double) * ((size_t)q.A.m + 1)));
    FAIR_TRY(q.M_cim.grow(sizeof(double) * ((size_t)q.A.m + 1)));
    FAIR_TRY(q.D.grow(sizeof(double) * ((size_t)q.A.n + 1)));
    FAIR_TRY(sirt_weights_recip(q.A, q.AT, true, q.M_sart.as<double>(), q.D.as<double>(), s));
    FAIR_TRY(sirt_weights_recip(q.A, q.AT, false, q.M_cim.as<double>(), nullptr, s));
    bool want_tiled = B->layout == 1;
    if (B->layout == 2) {  // the class's choice, timed on its first problem
        const std::pair<int64_t, int64_t> key{q.A.n, q.A.tstride_hint};
        auto it = B->classes.find(key);
        if (it == B->classes.end()) {
            ClassChoice c;
            FAIR_TRY(tune_class(B, q, c));
            it = B->classes.emplace(key, c).first;
        }
        const ClassChoice &c = it->second;
        want_tiled = c.tiled;
        if (c.tiled) {
            q.A.tile_req[0] = c.tile[0];
            q.A.tile_req[1] = 0;
            q.AT.tile_req[0] = c.tile[1];
            q.AT.tile_req[1] = c.tile[2];
        }
    }
    if (want_tiled) {  // tiled copies of A (pass 1) and A' (pass 2) where both build
        FAIR_TRY(csr_make_tiled(q.A, B->prec, 1, s));
        FAIR_TRY(csr_make_tiled(q.AT, B->prec, 2, s));
        FAIR_CUDA(cudaStreamSynchronize(s));
        q.tiled = tl_batch_ready(q.A, B->prec) && tl_batch_ready(q.AT, B->prec);
        if (!q.tiled) {
            q.A.tl.release();
            q.AT.tl.release();
        }
    } else {
        q.A.tl.release();
        q.AT.tl.release();
    }
    if (B->prec != FAIR_PREC_F64 && !q.tiled) {
        FAIR_TRY(sirt_make_forms(q.A, q.AT, B->prec, s, false, false));
        FAIR_CUDA(cudaStreamSynchronize(s));
        if (q.A.nnz > 0 && (!q.A.haspk || !q.AT.haspk)) {
            set_detail("a reduced-precision batch needs matrices with a packed index stream");
            return FAIR_ERR_ARG;
        }
        if (B->prec == FAIR_PREC_Q16 && (q.A.qsigned || q.AT.qsigned)) {
            set_detail("a q16 batch needs nonnegative matrix values");
            return FAIR_ERR_ARG;
        }
    }
    FAIR_CUDA(cudaStreamSynchronize(s));
    compact(q.A, B->prec, q.tiled);
    compact(q.AT, B->prec, q.tiled);
    return FAIR_OK;
}

bool config_ok(const int32_t *c) {
    auto lanes = [](int32_t g) { return g == 4 || g == 8 || g == 16 || g == 32; };
    return lanes(c[0]) && lanes(c[1]) && (c[2] == 1 || c[2] == 2) && (c[3] == 1 || c[3] == 2);
}

}  // namespace
}  // namespace fair

#define BENTER(B)                                                  \
    do {                                                           \
        if (!(B)) { fair::set_detail("null batch"); return FAIR_ERR_NULL; } \
        FAIR_CUDA(cudaSetDevice((B)->device));                     \
    } while (0)

extern "C" {

int fair_batch_create(fair_batch *out, int32_t prec) {
    if (!out) return FAIR_ERR_NULL;
    *out = nullptr;
    if (prec < FAIR_PREC_F64 || prec > FAIR_PREC_Q16) {
        fair::set_detail("unknown precision");
        return FAIR_ERR_ARG;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        fair::set_detail(e != cudaSuccess ? cudaGetErrorString(e) : "no CUDA device");
        return FAIR_ERR_NOGPU;
    }
    fair_batch B = new (std::nothrow) fair_batch_s();
    if (!B) return FAIR_ERR_ALLOC;
    cudaGetDevice(&B->device);
    B->prec = prec;
    e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete B;
        return fair::cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    B->own_stream = true;
    if (B->sched.grow(4 * sizeof(unsigned)) != FAIR_OK ||
        cudaMemset(B->sched.p, 0, 4 * sizeof(unsigned)) != cudaSuccess) {
        fair_batch_destroy(B);
        return FAIR_ERR_ALLOC;
    }
    *out = B;
    return FAIR_OK;
}

int fair_batch_destroy(fair_batch B) {
    if (!B) return FAIR_OK;
    cudaSetDevice(B->device);
    cudaStreamSynchronize(B->stream);
    fair::drop_graph(B);
    for (BatchProb *p : B->probs) {
        p->release();
        delete p;
    }
    for (DevBuf *d : {&B->desc1, &B->desc2, &B->c0_1, &B->c0_2, &B->sched, &B->x32, &B->r,
                      &B->w_b, &B->w_x})
        d->release();
    B->tb1.release();
    B->tb2.release();
    if (B->own_stream) cudaStreamDestroy(B->stream);
    delete B;
    return FAIR_OK;
}

int fair_batch_set_stream(fair_batch B, void *cuda_stream) {
    BENTER(B);
    std::lock_guard<std::mutex> lk(B->mu);
    FAIR_CUDA(cudaStreamSynchronize(B->stream));
    if (B->own_stream) cudaStreamDestroy(B->stream);
    if (cuda_stream) {
        B->stream = (cudaStream_t)cuda_stream;
        B->own_stream = false;
    } else {
        FAIR_CUDA(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
        B->own_stream = true;
    }
    fair::drop_graph(B);
    return FAIR_OK;
}

int fair_batch_set_layout(fair_batch B, int32_t layout) {
    BENTER(B);
    if (layout != 0 && layout != 1 && layout != 2) {
        fair::set_detail("layout must be 0 (packed streams), 1 (tiled copies) or 2 (chosen per class)");
        return FAIR_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(B->mu);
    if (!B->probs.empty()) {
        fair::set_detail("the layout is chosen before the first problem is added");
        return FAIR_ERR_STATE;
    }
    B->layout = layout;
    return FAIR_OK;
}

int fair_batch_add(fair_batch B, fair_csr h, int32_t take) {
    BENTER(B);
    if (!h) return FAIR_ERR_NULL;
    if (h->device != B->device) {
        fair::set_detail("the handle lives on another device");
        return FAIR_ERR_ARG;
    }
    if (h->A.empty()) {
        fair::set_detail("handle holds no matrix");
        return FAIR_ERR_STATE;
    }
    if (h->A.f32_only) {  // the batch derives its forms and weights from FP64 values
        fair::set_detail("the matrix is held in FP32 only (fair_paralleltomo_f32)");
        return FAIR_ERR_STATE;
    }
    std::lock_guard<std::mutex> lk(B->mu);
    FAIR_CUDA(cudaStreamSynchronize(h->stream));
    BatchProb *q = new (std::nothrow) BatchProb();
    if (!q) return FAIR_ERR_ALLOC;
    int st = FAIR_OK;
    if (take) {
        q->A = h->A;  // the buffers move to the batch
        h->A = DevCSR();
        h->AT.release();
        h->at_valid = false;
        h->sirt_ready = false;
    } else {
        st = fair::copy_csr(h->A, q->A, B->stream);
    }
    if (st == FAIR_OK) st = fair::finish_problem(B, *q);
    if (st != FAIR_OK) {
        cudaStreamSynchronize(B->stream);
        q->release();
        delete q;
        return st;
    }
    B->probs.push_back(q);
    B->ntiled += q->tiled ? 1 : 0;
    B->row_off.push_back(B->row_off.back() + q->A.m);
    B->col_off.push_back(B->col_off.back() + q->A.n);
    B->nnz += q->A.nnz;
    B->ready = false;
    fair::drop_graph(B);
    return FAIR_OK;
}

int fair_batch_problem_layout(fair_batch B, int32_t p, int32_t *layout) {
    if (!B || !layout) return FAIR_ERR_NULL;
    std::lock_guard<std::mutex> lk(B->mu);
    if (p < 0 || p >= (int32_t)B->probs.size()) {
        fair::set_detail("problem index outside 0..problems-1");
        return FAIR_ERR_ARG;
    }
    const BatchProb &q = *B->probs[p];
    layout[0] = q.tiled ? 1 : 0;
    layout[1] = q.tiled ? q.A.tl.T : 0;
    layout[2] = q.tiled ? q.AT.tl.T : 0;
    layout[3] = q.tiled ? q.AT.tl.cells_cap : 0;
    return FAIR_OK;
}

int fair_batch_info(fair_batch B, int32_t *nprob, int64_t *rows, int64_t *cols, int64_t *nnz,
                    int64_t *device_bytes) {
    if (!B) return FAIR_ERR_NULL;
    if (nprob) *nprob = (int32_t)B->probs.size();
    if (rows) *rows = B->row_off.back();
    if (cols) *cols = B->col_off.back();
    if (nnz) *nnz = B->nnz;
    if (device_bytes) *device_bytes = fair::device_bytes(B);
    return FAIR_OK;
}

int fair_batch_pass_bytes(fair_batch B, int32_t sart, int64_t *pass1, int64_t *pass2) {
    if (!B || !pass1 || !pass2) return FAIR_ERR_NULL;
    const bool red = B->prec != FAIR_PREC_F64;
    const int64_t sv = B->prec == FAIR_PREC_F64 ? 8 : B->prec == FAIR_PREC_F32 ? 4 : 2;
    const int64_t sx = red ? 4 : 8;
    auto matrix = [&](const DevCSR &M, bool tiled) -> int64_t {
        // tiled copies: per 4 entries 8 bytes of local indices and 4 values, or
        // one 16-byte record (2-byte forms); row ends as a row pointer
        if (tiled) return M.nnz * (sv == 2 ? 4 : 2 + sv) + ((int64_t)M.m + 1) * 8;
        if (!red) return M.nnz * 12 + ((int64_t)M.m + 1) * 8;
        return M.ngroups * (8 + 4 * sv) + M.nesc * 16 + ((int64_t)M.m + 1) * 8;
    };
    int64_t p1 = 0, p2 = 0;
    for (const BatchProb *q : B->probs) {
        const int64_t m = q->A.m, n = q->A.n;
        p1 += matrix(q->A, q->tiled) + n * sx + m * 8 + m * 8 + m * sx;  // x, b, M, r
        p2 += matrix(q->AT, q->tiled) + m * sx + 2 * n * 8 + (sart ? n * 8 : 0) + (red ? n * 4 : 0);
    }
    *pass1 = p1;
    *pass2 = p2;
    return FAIR_OK;
}

int fair_batch_offsets(fair_batch B, int64_t *row_off, int64_t *col_off) {
    if (!B || !row_off || !col_off) return FAIR_ERR_NULL;
    std::copy(B->row_off.begin(), B->row_off.end(), row_off);
    std::copy(B->col_off.begin(), B->col_off.end(), col_off);
    return FAIR_OK;
}

int fair_batch_prepare(fair_batch B, const char *sirt_method, const fair_opts *options) {
    BENTER(B);
    if (!sirt_method) return FAIR_ERR_NULL;
    bool sart;
    if (!strcmp(sirt_method, "cimmino")) sart = false;
    else if (!strcmp(sirt_method, "sart")) sart = true;
    else { fair::set_detail("Not a recognised SIRT method."); return FAIR_ERR_METHOD; }
    if (B->probs.empty()) { fair::set_detail("empty batch"); return FAIR_ERR_STATE; }
    std::lock_guard<std::mutex> lk(B->mu);
    fair_opts o;
    if (options) o = *options;
    else FAIR_TRY(fair_opts_initialise(&o));
    B->sart = sart;
    B->opts = fair::BOpts{o.relaxpar, o.lbound, o.ubound,
                          (o.upb ? 1 : 0) | (o.lwrb ? 2 : 0)};
    const bool red = B->prec != FAIR_PREC_F64;
    const size_t sx = red ? sizeof(float) : sizeof(double);
    FAIR_TRY(B->r.grow(sx * ((size_t)B->row_off.back() + 1)));
    if (red) FAIR_TRY(B->x32.grow(sizeof(float) * ((size_t)B->col_off.back() + 1)));
    B->bound_b = nullptr;
    B->bound_x = nullptr;
    B->ready = true;
    return FAIR_OK;
}

static int batch_bind(fair_batch B, const double *d_b, double *d_x) {
    if (!B->ready) {
        fair::set_detail("call fair_batch_prepare first (after adding problems)");
        return FAIR_ERR_STATE;
    }
    if (!d_b || !d_x) return FAIR_ERR_NULL;
    // descriptors hold the method's weights and the vector pointers
    return fair::bind_vectors(B, d_b, d_x);
}

int fair_batch_run_device(fair_batch B, const double *d_b, double *d_x, int32_t K) {
    BENTER(B);
    if (K < 0) { fair::set_detail("K >= 0 required"); return FAIR_ERR_ARG; }
    std::lock_guard<std::mutex> lk(B->mu);
    FAIR_TRY(batch_bind(B, d_b, d_x));
    if (K == 0) return FAIR_OK;
    if (!B->gexec || B->g_K != K || B->g_x != d_x || memcmp(B->g_cfg, B->cfg, sizeof(B->cfg)) != 0) {
        fair::drop_graph(B);
        FAIR_TRY(fair::batch_pass(B, 1, B->stream, true));  // grids looked up outside the capture
        FAIR_TRY(fair::batch_pass(B, 2, B->stream, true));
        fair::sm_count();
        cudaGraph_t g = nullptr;
        FAIR_CUDA(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
        int st = fair::enqueue_iterations(B, K, B->stream);
        cudaError_t e = cudaStreamEndCapture(B->stream, &g);
        if (st != FAIR_OK) { if (g) cudaGraphDestroy(g); return st; }
        FAIR_CUDA(e);
        e = cudaGraphInstantiate(&B->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { B->gexec = nullptr; return fair::cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__); }
        B->g_K = K;
        B->g_x = d_x;
        memcpy(B->g_cfg, B->cfg, sizeof(B->cfg));
    }
    FAIR_CUDA(cudaGraphLaunch(B->gexec, B->stream));
    return FAIR_OK;
}

int fair_batch_run_device_unbatched(fair_batch B, const double *d_b, double *d_x, int32_t K) {
    BENTER(B);
    if (K < 0) { fair::set_detail("K >= 0 required"); return FAIR_ERR_ARG; }
    std::lock_guard<std::mutex> lk(B->mu);
    FAIR_TRY(batch_bind(B, d_b, d_x));
    const bool red = B->prec != FAIR_PREC_F64;
    cudaStream_t s = B->stream;
    if (red && B->col_off.back() > 0)
        FAIR_TRY(fair::vec_to_f32(d_x, B->col_off.back(), B->x32.as<float>(), s));
    const size_t sx = red ? sizeof(float) : sizeof(double);
    std::vector<fair::SirtDev> S(B->probs.size());
    for (size_t p = 0; p < B->probs.size(); ++p) {
        BatchProb &q = *B->probs[p];
        for (DevCSR *M : {&q.A, &q.AT}) {
            M->sirt_lanes[B->prec] = B->cfg[M == &q.A ? 0 : 1];
            M->sirt_groups[B->prec] = q.tiled ? 9 : B->cfg[M == &q.A ? 2 : 3];
        }
        fair::SirtDev &d = S[p];
        d.prec = B->prec;
        d.m = q.A.m;
        d.n = q.A.n;
        d.A = &q.A;
        d.AT = &q.AT;
        d.b = d_b + B->row_off[p];
        d.Minv = B->sart ? q.M_sart.as<double>() : q.M_cim.as<double>();
        d.D = B->sart ? q.D.as<double>() : nullptr;
        d.x = d_x + B->col_off[p];
        d.x32 = red ? B->x32.as<float>() + B->col_off[p] : nullptr;
        d.r = (char *)B->r.p + sx * B->row_off[p];
        d.omg = B->opts.omg;
        d.bmode = B->opts.bmode;
        d.lb = B->opts.lb;
        d.ub = B->opts.ub;
        d.sched = B->sched.as<unsigned>();
    }
    for (int it = 0; it < K; ++it)
        for (const fair::SirtDev &d : S) {
            fair::sirt_pass(d, 1, s);
            fair::sirt_pass(d, 2, s);
        }
    FAIR_CUDA(cudaGetLastError());
    return FAIR_OK;
}

int fair_batch_launches(fair_batch B, int32_t K, int64_t *launches) {
    if (!B || !launches) return FAIR_ERR_NULL;
    // per pass: one packed / CSR launch, and partials + row sums for the tiled problems
    const int64_t per_pass = (B->ntiled < (int)B->probs.size() ? 1 : 0) + (B->ntiled > 0 ? 2 : 0);
    *launches = (B->prec != FAIR_PREC_F64 ? 1 : 0) + 2 * per_pass * (int64_t)K;
    return FAIR_OK;
}

int fair_batch_sirt(fair_batch B, const char *sirt_method, const double *b_all, int32_t K,
                    const double *x0_all, const fair_opts *options, double *x_all) {
    BENTER(B);
    if (!b_all || !x_all) return FAIR_ERR_NULL;
    FAIR_TRY(fair_batch_prepare(B, sirt_method, options));
    const int64_t m = B->row_off.back(), n = B->col_off.back();
    {
        std::lock_guard<std::mutex> lk(B->mu);
        FAIR_TRY(B->w_b.grow(sizeof(double) * ((size_t)m + 1)));
        FAIR_TRY(B->w_x.grow(sizeof(double) * ((size_t)n + 1)));
        FAIR_CUDA(cudaMemcpyAsync(B->w_b.p, b_all, sizeof(double) * m, cudaMemcpyHostToDevice, B->stream));
        if (x0_all)
            FAIR_CUDA(cudaMemcpyAsync(B->w_x.p, x0_all, sizeof(double) * n, cudaMemcpyHostToDevice, B->stream));
        else
            FAIR_CUDA(cudaMemsetAsync(B->w_x.p, 0, sizeof(double) * n, B->stream));
    }
    FAIR_TRY(fair_batch_run_device(B, B->w_b.as<double>(), B->w_x.as<double>(), K));
    FAIR_CUDA(cudaMemcpyAsync(x_all, B->w_x.p, sizeof(double) * n, cudaMemcpyDeviceToHost, B->stream));
    FAIR_CUDA(cudaStreamSynchronize(B->stream));
    return FAIR_OK;
}

int fair_batch_set_config(fair_batch B, const int32_t *config) {
    BENTER(B);
    if (!config) return FAIR_ERR_NULL;
    if (!fair::config_ok(config)) {
        fair::set_detail("lanes per row must be 4, 8, 16 or 32 and groups per lane 1 or 2");
        return FAIR_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(B->mu);
    for (int i = 0; i < 4; ++i) B->cfg[i] = config[i];
    return FAIR_OK;
}

int fair_batch_autotune(fair_batch B, const double *d_b, double *d_x, int32_t reps,
                        int32_t *config) {
    BENTER(B);
    if (reps < 1) { fair::set_detail("reps >= 1 required"); return FAIR_ERR_ARG; }
    std::lock_guard<std::mutex> lk(B->mu);
    FAIR_TRY(batch_bind(B, d_b, d_x));
    if (B->ntiled == (int)B->probs.size()) {  // every problem on its tiled copies: nothing to tune
        if (config)
            for (int i = 0; i < 4; ++i) config[i] = B->cfg[i];
        return FAIR_OK;
    }
    cudaStream_t s = B->stream;
    if (B->prec != FAIR_PREC_F64 && B->col_off.back() > 0)
        FAIR_TRY(fair::vec_to_f32(d_x, B->col_off.back(), B->x32.as<float>(), s));
    static const int lanes[4] = {4, 8, 16, 32};
    const int ngmax = B->prec != FAIR_PREC_F64 ? 2 : 1;
    cudaEvent_t ev[2];
    for (auto &e : ev) FAIR_CUDA(cudaEventCreate(&e));
    int st = FAIR_OK;
    for (int pass = 1; pass <= 2 && st == FAIR_OK; ++pass) {
        float t[2][4];
        float best_ms = -1.f;
        int best_g = B->cfg[pass - 1], best_ng = B->cfg[pass + 1];
        for (int round = 0; round < 2 && st == FAIR_OK; ++round)
            for (int ng = 1; ng <= ngmax && st == FAIR_OK; ++ng)
                for (int c = 0; c < 4 && st == FAIR_OK; ++c) {
                    B->cfg[pass - 1] = lanes[c];
                    B->cfg[pass + 1] = ng;
                    st = fair::batch_pass(B, pass, s);  // warm-up
                    if (st != FAIR_OK) break;
                    cudaEventRecord(ev[0], s);
                    for (int r = 0; r < reps && st == FAIR_OK; ++r) st = fair::batch_pass(B, pass, s);
                    if (st != FAIR_OK) break;
                    cudaEventRecord(ev[1], s);
                    cudaError_t e = cudaEventSynchronize(ev[1]);
                    if (e != cudaSuccess) { st = fair::cuda_fail(e, "autotune", __FILE__, __LINE__); break; }
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, ev[0], ev[1]);
                    ms /= reps;
                    float &tc = t[ng - 1][c];
                    tc = round == 0 ? ms : std::min(tc, ms);
                    if (round == 1 && (best_ms < 0.f || tc < best_ms)) {
                        best_ms = tc;
                        best_g = lanes[c];
                        best_ng = ng;
                    }
                }
        B->cfg[pass - 1] = best_g;
        B->cfg[pass + 1] = best_ng;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (st == FAIR_OK && config)
        for (int i = 0; i < 4; ++i) config[i] = B->cfg[i];
    return st;
}

}  // extern "C"
