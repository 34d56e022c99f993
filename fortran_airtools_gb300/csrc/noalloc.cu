// noalloc.cu -- fair_matvecmul_noalloc: the product w = A*v for callers that
// must not allocate GPU memory.
//
// fair_matvecmul stages the caller's host vectors in device buffers that the
// handle grows on demand (cudaMalloc). Some callers cannot allow that during
// their run: a program that reserves the whole GPU memory up front for its own
// pool (so a later cudaMalloc fails), a real-time loop that cannot take the
// implicit device synchronisation of cudaMalloc/cudaFree, or a host program
// that hands the library a GPU shared with others under a fixed memory budget.
// This entry point stages both vectors in one fixed device array defined in
// this file instead, and keeps the two chunk-scheduling counters of the
// product kernel in a second one. Both arrays exist on every GPU that loads
// the library, for as long as the process lives.
//
// Limits and rules:
//   * n + m must not exceed FAIR_NOALLOC_MAX_ENTRIES (4,194,304 doubles,
//     32 MiB); larger problems are rejected with FAIR_ERR_ARG.
//   * The product is computed in FP64 whatever precision the handle is set to.
//   * Every call looks up the arrays' device addresses (cudaGetSymbolAddress)
//     with the handle's device current, so an address is never reused after
//     the device's context was reset and the module loaded again; the first
//     call on a device also loads the arrays, so make it before any stream
//     capture.
//   * Every call shares the arrays and leaves its vectors in them: two calls
//     whose work overlaps on the GPU (different streams or handles at once)
//     race and corrupt each other's results. The counters are cleared by
//     every call before the product runs.
//   * Nothing here calls cudaMalloc, cudaFree or an allocating library routine;
//     the matrix itself must already be on the GPU (built or uploaded earlier).
#include "fair_gpu_ext.h"
#include "fair_internal.cuh"

namespace fair {
namespace {

__device__ __align__(256) double g_noalloc_vectors[FAIR_NOALLOC_MAX_ENTRIES];
__device__ __align__(256) unsigned g_noalloc_sched[4];

struct NoAllocAddrs {
    double *vectors = nullptr;
    unsigned *sched = nullptr;
};

// Device addresses of the two arrays on the current device, looked up on every
// call (a cheap host query; a cached address would go stale after a context
// reset reloads the module).
int noalloc_addresses(NoAllocAddrs &out) {
    void *pv = nullptr, *ps = nullptr;
    FAIR_CUDA(cudaGetSymbolAddress(&pv, g_noalloc_vectors));
    FAIR_CUDA(cudaGetSymbolAddress(&ps, g_noalloc_sched));
    out.vectors = static_cast<double *>(pv);
    out.sched = static_cast<unsigned *>(ps);
    return FAIR_OK;
}

}  // namespace
}  // namespace fair

using namespace fair;

extern "C" int fair_matvecmul_noalloc(fair_csr h, const double *v, int64_t size_v, double *w) {
    if (!h) return FAIR_ERR_NULL;
    if (!v || !w) return FAIR_ERR_NULL;
    FAIR_CUDA(cudaSetDevice(h->device));
    if (h->A.empty()) {
        set_detail("handle holds no matrix");
        return FAIR_ERR_STATE;
    }
    if (h->A.f32_only) {  // the product here reads the FP64 values
        set_detail("the matrix is held in FP32 only (fair_paralleltomo_f32)");
        return FAIR_ERR_STATE;
    }
    const int64_t m = h->A.m, n = h->A.n;
    if (size_v != n) return FAIR_ERR_SIZE;  // "Vector input size incorrect."
    if (n + m > (int64_t)FAIR_NOALLOC_MAX_ENTRIES) {
        set_detail("fair_matvecmul_noalloc: n + m exceeds FAIR_NOALLOC_MAX_ENTRIES (4194304)");
        return FAIR_ERR_ARG;
    }
    NoAllocAddrs a;
    FAIR_TRY(noalloc_addresses(a));
    cudaStream_t s = h->stream;
    double *d_v = a.vectors, *d_w = a.vectors + n;
    if (n) FAIR_CUDA(cudaMemcpyAsync(d_v, v, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    FAIR_CUDA(cudaMemsetAsync(a.sched, 0, 4 * sizeof(unsigned), s));
    FAIR_TRY(spmv(h->A, FAIR_PREC_F64, d_v, d_w, s, a.sched));
    if (m) FAIR_CUDA(cudaMemcpyAsync(w, d_w, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
    FAIR_CUDA(cudaStreamSynchronize(s));
    return FAIR_OK;
}
