// Launch layer of the reduced-precision voxel kernels (operator_mixed.cuh), templated on the
// LUT type: compartment tables, occupancy-tuned launches of A and A' pass 1.  Instantiated
// once per LUT format by operator_mixed_{bf16,fp16,f32}.cu (separate units so the three
// compile in parallel).
#pragma once
#include "operator_launch.cuh"
#include "operator_mixed.cuh"

namespace cgb {
namespace mixed_launch {
using namespace detail;

// nSp and FP16 lengths: the BF16 / FP16 copies use their own row stride and FP16 lengths,
// the F32 path the float-float kernels' padded FP32 rows and FP32 lengths
template <class LT, int ARITH>
CompsM<LT> comps(const cgb_op *op) {
    constexpr bool kF32 = ARITH == CGB_ARITH_F32;
    CompsM<LT> C;
    C.n = 0;
    C.nSp = kF32 ? op->nSp : op->nSp_r;
    const uint32_t ndirs = (uint32_t)op->ndirs, nSp = (uint32_t)C.nSp;
    const LT *ic = (const LT *)op->lut_r_ic(ARITH);
    const LT *ec = (const LT *)op->lut_r_ec(ARITH);
    const LT *iso = (const LT *)op->lut_r_iso(ARITH);
    const bool l16 = !kF32;
    if (op->nIC > 0)
        C.c[C.n++] = CompM<LT>{op->vox_ptr, op->seg_f, op->seg_o, l16 ? nullptr : op->seg_l, l16 ? op->seg_l16 : nullptr,
                               op->len16_inv_scale, op->eval, ic, 0, op->nF, ndirs * nSp, op->nIC, 1};
    if (op->nEC > 0 && op->nE > 0)
        C.c[C.n++] = CompM<LT>{op->ec_ptr, op->ec_col, op->ec_o, nullptr, nullptr, 1.f, nullptr, ec,
                               (int64_t)op->nF * op->nIC, op->nE, ndirs * nSp, op->nEC, 0};
    if (op->nISO > 0 && op->nISOv > 0)
        C.c[C.n++] = CompM<LT>{op->iso_ptr, op->iso_col, nullptr, nullptr, nullptr, 1.f, nullptr, iso,
                               (int64_t)op->nF * op->nIC + (int64_t)op->nE * op->nEC, op->nISOv, nSp, op->nISO, 0};
    return C;
}

template <class LT, int ARITH>
struct FwdMix {
    cgb_op *op;
    const double *x;
    float *y, *ax;
    const float *yobs, *sqw;
    double *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N, int MINB>
    int launch() {
        auto kern = k_forward_mix<LT, L, N, MINB>;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, 0, st>>>(op->nV, op->nS, comps<LT, ARITH>(op), x, y, ax, yobs, sqw, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
    template <int L, int N>
    int run() {
        return occ_launch(op, kOccFwdMix + (ARITH - CGB_ARITH_BF16), st, [&] { return launch<L, N, 5>(); },
                          [&] { return launch<L, N, 6>(); });
    }
};

template <class LT, int ARITH>
struct AdjMix {
    cgb_op *op;
    const float *yin;
    int in_mode;
    const double *x;
    const float *yobs, *sqw, *ax_a, *ax_b;
    float ca, cb;
    double *xout, *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N, int MINB, bool FUSED>
    int launch() {
        auto kern = k_adjoint_mix<LT, L, N, MINB, FUSED>;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, 0, st>>>(op->vr1 > 0 ? op->vr0 : 0, op->vr1 > 0 ? op->vr1 : op->nV, op->nS, op->n, comps<LT, ARITH>(op),
                                   yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, op->scratch32, xout, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
    template <int L, int N>
    int run() {
        // the fused-forward build (in_mode 1) holds the forward row as well
        if (in_mode == 1)
            return occ_launch(op, kOccAdjMixFused + (ARITH - CGB_ARITH_BF16), st,
                              [&] { return launch<L, N, 3, true>(); }, [&] { return launch<L, N, 4, true>(); });
        return occ_launch(op, kOccAdjMix + (ARITH - CGB_ARITH_BF16), st, [&] { return launch<L, N, 4, false>(); },
                          [&] { return launch<L, N, 5, false>(); });
    }
};

template <class LT, int ARITH>
int forward(cgb_op *op, const double *x, float *y, float *ax, const float *yobs, const float *sqw, double *partials,
            cudaStream_t st, int *grid) {
    FwdMix<LT, ARITH> L{op, x, y, ax, yobs, sqw, partials, st, grid};
    return dispatch_pair_shape(pick_pair_shape(op->nS), L);
}

template <class LT, int ARITH>
int adjoint(cgb_op *op, const float *yin, int in_mode, const double *x, const float *yobs, const float *sqw,
            const float *ax_a, const float *ax_b, float ca, float cb, double *xout, double *partials, cudaStream_t st,
            int *grid) {
    AdjMix<LT, ARITH> L{op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid};
    return dispatch_pair_shape(pick_pair_shape(op->nS), L);
}

}  // namespace mixed_launch
}  // namespace cgb
