// Shape selection and launch of the templated voxel kernels (operator_kernels.cuh).
#pragma once
#include "operator_kernels.cuh"

namespace cgb {
namespace detail {

struct Shape {
    int lpv, nch;  // lanes per voxel, samples per lane
};

// (LPV, NCH) pairs that have kernels; the shape with the fewest padded sample slots
// (LPV*NCH >= nS) wins, ties going to wider groups
constexpr Shape kShapes[] = {{1, 1},  {2, 1},  {4, 1},  {4, 2},  {8, 1},  {8, 2},   {8, 3},   {8, 4},  {8, 6},
                             {8, 9},  {16, 1}, {16, 2}, {32, 1}, {32, 2}, {32, 3},  {32, 4},  {32, 6}, {32, 9},
                             {32, 12}, {32, 16}};

inline Shape pick_shape(int nS) {
    Shape best = {32, kMaxChunks};
    int best_slots = 1 << 30;
    for (const Shape &s : kShapes) {
        const int slots = s.lpv * s.nch;
        if (slots < nS) continue;
        if (slots < best_slots || (slots == best_slots && s.lpv > best.lpv)) {
            best = s;
            best_slots = slots;
        }
    }
    return best;
}

template <class Fn>
int dispatch_shape(Shape s, Fn &fn) {
#define CGB_SHAPE(L, N) \
    if (s.lpv == L && s.nch == N) return fn.template run<L, N>();
    CGB_SHAPE(1, 1) CGB_SHAPE(2, 1) CGB_SHAPE(4, 1) CGB_SHAPE(4, 2) CGB_SHAPE(8, 1) CGB_SHAPE(8, 2) CGB_SHAPE(8, 3)
    CGB_SHAPE(8, 4) CGB_SHAPE(8, 6) CGB_SHAPE(8, 9) CGB_SHAPE(16, 1) CGB_SHAPE(16, 2) CGB_SHAPE(32, 1)
    CGB_SHAPE(32, 2) CGB_SHAPE(32, 3) CGB_SHAPE(32, 4) CGB_SHAPE(32, 6) CGB_SHAPE(32, 9) CGB_SHAPE(32, 12)
    CGB_SHAPE(32, 16)
#undef CGB_SHAPE
    return fail(CGB_ERR_UNSUPPORTED, "no kernel shape for this number of samples");
}

template <class K>
int grid_for_kernel(K kernel, size_t smem, int nsm, int work_groups, int gpb, int *grid) {
    int per_sm = 0;
    CGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem));
    if (per_sm < 1) per_sm = 1;
    int g = nsm * per_sm;
    const int need = (work_groups + gpb - 1) / gpb;
    if (need < g) g = need;
    if (g < 1) g = 1;
    *grid = g;
    return CGB_OK;
}

template <class AR>
struct FwdLaunch {
    cgb_op *op;
    const double *x;
    double *y, *ax;
    const double *yobs, *sqw;
    double *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N>
    int run() {
        const OpDev P = op->dev();
        auto kern = k_forward<L, N, AR>;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, 0, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, 0, st>>>(P, x, y, ax, yobs, sqw, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
};

template <class AR>
struct AdjLaunch {
    cgb_op *op;
    const double *yin;
    int in_mode;
    const double *x, *yobs, *sqw, *ax_a, *ax_b;
    double ca, cb;
    double *xout, *partials;
    cudaStream_t st;
    int *grid_out;
    template <int L, int N>
    int run() {
        const OpDev P = op->dev();
        auto kern = k_adjoint<L, N, AR>;
        const size_t smem = 0;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, smem, op->nsm, op->nV, kBlock / L, &g));
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        kern<<<g, kBlock, smem, st>>>(P, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, op->scratch, xout, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
};

}  // namespace detail
}  // namespace cgb
