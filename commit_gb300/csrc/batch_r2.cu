// Instantiation of the multi-right-hand-side BF16-LUT kernels for R = 2 vectors per pass.
#include "batch.cuh"
#include "operator_launch.cuh"

namespace cgb {
namespace {
using namespace detail;
using LT = __nv_bfloat16;

CompsM<LT> comps_bf16(const cgb_op *op) {
    CompsM<LT> C;
    C.n = 0;
    C.nSp = op->nSp_r;
    const uint32_t ndirs = (uint32_t)op->ndirs, nSp = (uint32_t)op->nSp_r;
    const LT *ic = (const LT *)op->lut_r_ic(CGB_ARITH_BF16);
    const LT *ec = (const LT *)op->lut_r_ec(CGB_ARITH_BF16);
    const LT *iso = (const LT *)op->lut_r_iso(CGB_ARITH_BF16);
    if (op->nIC > 0)
        C.c[C.n++] = CompM<LT>{op->vox_ptr, op->seg_f, op->seg_o, nullptr, op->seg_l16, op->len16_inv_scale, op->eval,
                               ic, 0, op->nF, ndirs * nSp, op->nIC, 1};
    if (op->nEC > 0 && op->nE > 0)
        C.c[C.n++] = CompM<LT>{op->ec_ptr, op->ec_col, op->ec_o, nullptr, nullptr, 1.f, nullptr, ec,
                               (int64_t)op->nF * op->nIC, op->nE, ndirs * nSp, op->nEC, 0};
    if (op->nISO > 0 && op->nISOv > 0)
        C.c[C.n++] = CompM<LT>{op->iso_ptr, op->iso_col, nullptr, nullptr, nullptr, 1.f, nullptr, iso,
                               (int64_t)op->nF * op->nIC + (int64_t)op->nE * op->nEC, op->nISOv, nSp, op->nISO, 0};
    return C;
}

struct FwdR {
    cgb_op *op;
    const RhsPtrs *V;
    const float *yobs, *sqw;
    double *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N>
    int run() {
        auto kern = k_forward_R<LT, L, N, 2>;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, 0, st>>>(op->nV, op->nS, comps_bf16(op), *V, yobs, sqw, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
};

struct AdjR {
    cgb_op *op;
    const RhsPtrs *V;
    int in_mode;
    const float *yobs, *sqw;
    double *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N, int MINB, bool FUSED>
    int launch() {
        auto kern = k_adjoint_R<LT, L, N, 2, MINB, FUSED>;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, 0, st>>>(op->vr1 > 0 ? op->vr0 : 0, op->vr1 > 0 ? op->vr1 : op->nV, op->nS, op->n,
                                   comps_bf16(op), *V, in_mode, yobs, sqw, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
    template <int L, int N>
    int run() {
        if (in_mode == 1)
            return occ_launch(op, kOccAdjR2Fused, st, [&] { return launch<L, N, 1, true>(); },
                              [&] { return launch<L, N, 3, true>(); });
        return occ_launch(op, kOccAdjR2, st, [&] { return launch<L, N, 2, false>(); },
                          [&] { return launch<L, N, 3, false>(); });
    }
};

}  // namespace

int forward_R2(cgb_op *op, const RhsPtrs &V, const float *yobs, const float *sqw, double *partials,
                cudaStream_t st, int *grid) {
    FwdR L{op, &V, yobs, sqw, partials, st, grid};
    return dispatch_pair_shape(op->batch_lpv == 2 ? wide_pair_shape(op->nS) : pick_pair_shape(op->nS), L);
}

int adjoint_R2(cgb_op *op, const RhsPtrs &V, int in_mode, const float *yobs, const float *sqw,
                double *partials, cudaStream_t st, int *grid) {
    AdjR L{op, &V, in_mode, yobs, sqw, partials, st, grid};
    return dispatch_pair_shape(op->batch_lpv == 2 ? wide_pair_shape(op->nS) : pick_pair_shape(op->nS), L);
}

}  // namespace cgb
