// sirt_sliced.cu -- the two SIRT passes (AIRMs.f90:1089-1110) over the sliced
// copy of the packed stream (rows.cuh, chunk_rows_sliced): layout codes 5-8
// (2 or 4 steps of 32 slots in flight per warp; 7 and 8 also gather x one
// step ahead), with the lanes per row of each chunk read from the copy. The epilogues are those of the other
// layouts (sirt_epi.cuh), so every layout computes the same per-row
// arithmetic and differs only in the order of the FP32 (or FP64) sums.
#include <type_traits>

#include "fair_internal.cuh"
#include "rows.cuh"
#include "sirt_epi.cuh"

namespace fair {

namespace {

struct SlArgs {
    const int64_t *prow, *soff;
    const int4 *gside;
    int S, L;
};

template <class LD, int D, int GF, int PF, typename XT, typename ACC, class Epi>
__global__ void __launch_bounds__(256) k_sirt_resid_sl(SlArgs P, int32_t m, LD ldr, const XT *x,
                                                       Epi epi, unsigned *sched) {
    __shared__ int lut[256];
    pk_lut_fill(lut, P.S, P.L);
    chunk_rows_sliced<XT, ACC, D, GF, PF>(P.prow, P.soff, m, ldr, P.gside, lut, x, epi, sched);
}
template <class LD, int D, int GF, int PF, typename XT, typename ACC, class Epi>
__global__ void __launch_bounds__(256) k_sirt_update_sl(SlArgs P, int32_t m, LD ldr, const XT *r,
                                                        Epi epi, unsigned *sched) {
    __shared__ int lut[256];
    pk_lut_fill(lut, P.S, P.L);
    chunk_rows_sliced<XT, ACC, D, GF, PF>(P.prow, P.soff, m, ldr, P.gside, lut, r, epi, sched);
}

template <int PASS, int D, int GF, int PF, class LD, typename XT, typename ACC, class Epi>
void launch(const SlArgs &P, int32_t m, const LD &ldr, const XT *x, const Epi &e, unsigned *sched,
            cudaStream_t s) {
    if constexpr (PASS == 1) {
        auto k = k_sirt_resid_sl<LD, D, GF, PF, XT, ACC, Epi>;
        k<<<chunk_grid(k, m), 256, 0, s>>>(P, m, ldr, x, e, sched);
    } else {
        auto k = k_sirt_update_sl<LD, D, GF, PF, XT, ACC, Epi>;
        k<<<chunk_grid(k, m), 256, 0, s>>>(P, m, ldr, x, e, sched);
    }
}

template <int PASS, int D, int PF, class LD, typename XT, typename ACC, class Epi>
void launch_g(bool g1, const SlArgs &P, int32_t m, const LD &ldr, const XT *x, const Epi &e,
              unsigned *sched, cudaStream_t s) {
    if (g1) launch<PASS, D, 1, PF, LD, XT, ACC>(P, m, ldr, x, e, sched, s);
    else launch<PASS, D, 0, PF, LD, XT, ACC>(P, m, ldr, x, e, sched, s);
}

// Code 5, 6: 2 or 4 steps in flight; 7, 8: the same with the gathers one
// step ahead. The G = 1 copy runs on its own kernels.
template <int PASS, class LD, typename XT, typename ACC, class Epi>
void dispatch(int code, bool g1, const SlArgs &P, int32_t m, const LD &ldr, const XT *x,
              const Epi &e, unsigned *sched, cudaStream_t s) {
    switch (code) {
        case 6: launch_g<PASS, 4, 0, LD, XT, ACC>(g1, P, m, ldr, x, e, sched, s); break;
        case 7: launch_g<PASS, 2, 1, LD, XT, ACC>(g1, P, m, ldr, x, e, sched, s); break;
        case 8: launch_g<PASS, 4, 1, LD, XT, ACC>(g1, P, m, ldr, x, e, sched, s); break;
        default: launch_g<PASS, 2, 0, LD, XT, ACC>(g1, P, m, ldr, x, e, sched, s); break;
    }
}

template <class LD, typename XT, typename ACC, class EpiR, class EpiU>
void pass_lp(const SirtDev &S, const DevCSR &M, int pass, int code, const LD &ldr, const EpiR &er,
             const EpiU &eu, const XT *x, const XT *r, cudaStream_t s) {
    const SlArgs P{M.prow.as<int64_t>(), M.soff.as<int64_t>(), M.gside.as<int4>(), M.pk_S, M.pk_L};
    if (pass == 1)
        dispatch<1, LD, XT, ACC>(code, M.sl_G == 1, P, M.m, ldr, x, er, S.sched, s);
    else
        dispatch<2, LD, XT, ACC>(code, M.sl_G == 1, P, M.m, ldr, r, eu, S.sched, s);
}

}  // namespace

bool sirt_pass_sliced(const SirtDev &S, const DevCSR &M, int pass, int code, cudaStream_t s) {
    if (!M.hassl || !M.haspk || !packed_enabled()) return false;
    if (S.prec == FAIR_PREC_F64) {
        if (!M.hassidx || !M.hassv64) return false;
        const SplitRec<double> ld{M.sidx.as<uint2>(), M.sv64.as<double>()};
        pass_lp<SplitRec<double>, double, double>(
            S, M, pass, code, ld, EpiResidF64{S.b, S.Minv, (double *)S.r},
            EpiUpdateF64{S.D, S.x, S.omg, S.lb, S.ub, S.bmode}, S.x, (const double *)S.r, s);
        return true;
    }
    const double scale = S.prec == FAIR_PREC_Q16 ? M.qscale : 1.0;
    const EpiResidLP er{S.b, S.Minv, (float *)S.r, scale};
    const EpiUpdateLP eu{S.D, S.x, S.x32, S.omg, S.lb, S.ub, S.bmode, scale};
    const float *x = S.x32, *r = (const float *)S.r;
    switch (S.prec) {
        case FAIR_PREC_F32:
            if (!M.hassidx || !M.hassv32) return false;
            pass_lp<SplitRec<float>, float, float>(S, M, pass, code,
                                                   SplitRec<float>{M.sidx.as<uint2>(), M.sv32.as<float>()},
                                                   er, eu, x, r, s);
            return true;
        case FAIR_PREC_F16:
            if (!M.hassf16) return false;
            pass_lp<FusedRec<__half>, float, float>(S, M, pass, code, FusedRec<__half>{M.sf16.as<uint4>()},
                                                    er, eu, x, r, s);
            return true;
        default:
            if (!M.hassfq) return false;
            if (M.qsigned)
                pass_lp<FusedRec<int16_t>, float, float>(S, M, pass, code,
                                                         FusedRec<int16_t>{M.sfq.as<uint4>()}, er, eu, x, r, s);
            else
                pass_lp<FusedRec<uint16_t>, float, float>(S, M, pass, code,
                                                          FusedRec<uint16_t>{M.sfq.as<uint4>()}, er, eu, x, r, s);
            return true;
    }
}

}  // namespace fair
