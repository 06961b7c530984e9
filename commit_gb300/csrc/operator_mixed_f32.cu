// The reduced-precision voxel kernels with a f32 LUT (operator_mixed_launch.cuh).
#include "operator_mixed_launch.cuh"

namespace cgb {

int forward_mix_f32(cgb_op *op, const double *x, float *y, float *ax, const float *yobs, const float *sqw,
                      double *partials, cudaStream_t st, int *grid) {
    return mixed_launch::forward<float, CGB_ARITH_F32>(op, x, y, ax, yobs, sqw, partials, st, grid);
}

int adjoint_mix_f32(cgb_op *op, const float *yin, int in_mode, const double *x, const float *yobs,
                      const float *sqw, const float *ax_a, const float *ax_b, float ca, float cb, double *xout,
                      double *partials, cudaStream_t st, int *grid) {
    return mixed_launch::adjoint<float, CGB_ARITH_F32>(op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st,
                                                grid);
}

}  // namespace cgb
