// Instantiation of the reduced-precision voxel kernels with a fp16 LUT.
#include "operator_launch.cuh"
#include "operator_mixed.cuh"

namespace cgb {
namespace {
using namespace detail;
using LT = __half;

MixLut<LT> mixlut(const cgb_op *op) {
    MixLut<LT> T;
    T.ic = (const LT *)op->lut_r_ic(CGB_ARITH_FP16);
    T.ec = (const LT *)op->lut_r_ec(CGB_ARITH_FP16);
    T.iso = op->lutISO_p;
    T.nSp = op->nSp;
    T.len16 = op->seg_l16;
    T.len_inv_scale = op->len16_inv_scale;
    return T;
}

struct FwdMix {
    cgb_op *op;
    const double *x;
    float *y, *ax;
    const float *yobs, *sqw;
    double *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N>
    int run() {
        auto kern = k_forward_mix<LT, L, N>;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, 0, st>>>(op->dev(), mixlut(op), x, y, ax, yobs, sqw, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
};

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
    template <int L, int N>
    int run() {
        auto kern = k_adjoint_mix<LT, L, N>;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, 0, st>>>(op->dev(), mixlut(op), yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb,
                                   op->scratch32, xout, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
};

}  // namespace

int forward_mix_fp16(cgb_op *op, const double *x, float *y, float *ax, const float *yobs, const float *sqw,
                    double *partials, cudaStream_t st, int *grid) {
    FwdMix L{op, x, y, ax, yobs, sqw, partials, st, grid};
    return dispatch_pair_shape(pick_pair_shape(op->nS), L);
}

int adjoint_mix_fp16(cgb_op *op, const float *yin, int in_mode, const double *x, const float *yobs,
                    const float *sqw, const float *ax_a, const float *ax_b, float ca, float cb, double *xout,
                    double *partials, cudaStream_t st, int *grid) {
    AdjMix L{op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid};
    return dispatch_pair_shape(pick_pair_shape(op->nS), L);
}

}  // namespace cgb
