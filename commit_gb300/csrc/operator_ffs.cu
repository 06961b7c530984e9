// Instantiation of the scalar-sample voxel kernels for the float-float policy.
#include "operator_kernels.cuh"
#include "operator_launch.cuh"

namespace cgb {
int forward_ffs(cgb_op *op, const double *x, double *y, double *ax, const double *yobs, const double *sqw,
                double *partials, cudaStream_t st, int *grid) {
    detail::FwdLaunch<detail::ArFF> L{op, x, y, ax, yobs, sqw, partials, st, grid};
    return detail::dispatch_shape(detail::pick_shape(op->nS), L);
}
int adjoint_ffs(cgb_op *op, const double *yin, int in_mode, const double *x, const double *yobs,
                const double *sqw, const double *ax_a, const double *ax_b, double ca, double cb, double *xout,
                double *partials, cudaStream_t st, int *grid) {
    detail::AdjLaunch<detail::ArFF> L{op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid};
    return detail::dispatch_shape(detail::pick_shape(op->nS), L);
}
}  // namespace cgb
