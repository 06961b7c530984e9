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
        const int slot = L == 32 && L != pick_pair_shape(op->nS).lpv ? kOccFwdFFWide : kOccFwdFF;
        return occ_launch(op, slot, st, [&] { return launch<L, N, 3>(); }, [&] { return launch<L, N, 4>(); });
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
        const bool wide = L == 32 && L != pick_pair_shape(op->nS).lpv;
        // the fused-forward build (in_mode 1) holds the forward row as well
        if (in_mode == 1)
            return occ_launch(op, wide ? kOccAdjFFWideFused : kOccAdjFFFused, st,
                              [&] { return launch<L, N, 1, true>(); }, [&] { return launch<L, N, 2, true>(); });
        return occ_launch(op, wide ? kOccAdjFFWide : kOccAdjFF, st, [&] { return launch<L, N, 2, false>(); },
                          [&] { return launch<L, N, 3, false>(); });
    }
};

}  // namespace

// Voxel shape of the pair kernels: the single-vector default (fewest padded samples) or a
// warp per voxel (half the samples per lane, fewer registers).  On the first call outside
// stream capture both are run with their occupancy builds tuned, and the faster shape is
// kept on the handle (ff_shape[0] for A, [1] for A').
template <class Fn>
static int shaped(cgb_op *op, int which, int slot_default, int slot_wide, cudaStream_t st, Fn &L) {
    const PairShape d = pick_pair_shape(op->nS), w = wide_pair_shape(op->nS);
    int &choice = op->ff_shape[which];
    if (choice == 0 && w.lpv != d.lpv) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CGB_CUDA(cudaStreamIsCapturing(st, &cs));
        if (cs == cudaStreamCaptureStatusNone) {
            CGB_TRY(dispatch_pair_shape(d, L));
            CGB_TRY(dispatch_pair_shape(w, L));
            const float td = fminf(op->occ_ms[slot_default][0], op->occ_ms[slot_default][1]);
            const float tw = fminf(op->occ_ms[slot_wide][0], op->occ_ms[slot_wide][1]);
            choice = tw < td ? 2 : 1;
        }
    }
    return dispatch_pair_shape(choice == 2 && w.lpv != d.lpv ? w : d, L);
}

int forward_ff(cgb_op *op, const double *x, double *y, double *ax, const double *yobs, const double *sqw,
               double *partials, cudaStream_t st, int *grid) {
    FwdPair L{op, x, y, ax, yobs, sqw, partials, st, grid};
    return shaped(op, 0, kOccFwdFF, kOccFwdFFWide, st, L);
}

int adjoint_ff(cgb_op *op, const double *yin, int in_mode, const double *x, const double *yobs, const double *sqw,
               const double *ax_a, const double *ax_b, double ca, double cb, double *xout, double *partials,
               cudaStream_t st, int *grid) {
    AdjPair L{op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid};
    // the first A' call of any input mode chooses the shape, so a solve whose first A' is the
    // fused gradient does not change shape (and summation order) at its second
    if (in_mode == 1) return shaped(op, 1, kOccAdjFFFused, kOccAdjFFWideFused, st, L);
    return shaped(op, 1, kOccAdjFF, kOccAdjFFWide, st, L);
}

}  // namespace cgb
