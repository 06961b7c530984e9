// Float-float operator launches: the packed-pair kernels of operator_pair.cuh.
#include "operator_launch.cuh"
#include "operator_pair.cuh"

namespace cgb {
namespace {

using namespace detail;

struct FwdPair {
    cgb_op *op;
    const double *x;
    double *y, *ax;
    const double *yobs, *sqw;
    double *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N, int MINB>
    int launch() {
        OpDev P = op->dev();
        if (op->vr1 > 0) {
            P.v0 = op->vr0;
            P.nV = op->vr1;
        }
        const Comps C = make_comps(op);
        auto kern = k_forward_p<L, N, MINB>;
        int g = 0;  // sized for all voxels, so every range launch has the same grid
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        const int vec_ok = ((uintptr_t)y % 16 == 0) && ((uintptr_t)ax % 16 == 0);
        kern<<<g, kBlock, 0, st>>>(P, C, x, y, ax, yobs, sqw, partials, vec_ok);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
    template <int L, int N>
    int run() {
        return occ_launch(op, kOccFwdFF, st, [&] { return launch<L, N, 3>(); }, [&] { return launch<L, N, 4>(); });
    }
};

struct AdjPair {
    cgb_op *op;
    const double *yin;
    int in_mode;
    const double *x, *yobs, *sqw, *ax_a, *ax_b;
    double ca, cb;
    double *xout, *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N, int MINB, bool FUSED>
    int launch() {
        OpDev P = op->dev();
        if (op->vr1 > 0) {
            P.v0 = op->vr0;
            P.nV = op->vr1;
        }
        const Comps C = make_comps(op);
        auto kern = k_adjoint_p<L, N, MINB, FUSED>;
        int g = 0;  // sized for all voxels, so every range launch has the same grid
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, 0, st>>>(P, C, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, op->scratch, xout, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
    template <int L, int N>
    int run() {
        // the fused-forward build (in_mode 1) holds the forward row as well
        if (in_mode == 1)
            return occ_launch(op, kOccAdjFFFused, st, [&] { return launch<L, N, 1, true>(); },
                              [&] { return launch<L, N, 2, true>(); });
        return occ_launch(op, kOccAdjFF, st, [&] { return launch<L, N, 2, false>(); },
                          [&] { return launch<L, N, 3, false>(); });
    }
};

}  // namespace

int forward_ff(cgb_op *op, const double *x, double *y, double *ax, const double *yobs, const double *sqw,
               double *partials, cudaStream_t st, int *grid) {
    FwdPair L{op, x, y, ax, yobs, sqw, partials, st, grid};
    return dispatch_pair_shape(pick_pair_shape(op->nS), L);
}

int adjoint_ff(cgb_op *op, const double *yin, int in_mode, const double *x, const double *yobs, const double *sqw,
               const double *ax_a, const double *ax_b, double ca, double cb, double *xout, double *partials,
               cudaStream_t st, int *grid) {
    AdjPair L{op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid};
    return dispatch_pair_shape(pick_pair_shape(op->nS), L);
}

}  // namespace cgb
