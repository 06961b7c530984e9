// Launch layer of the FP64-accurate operator: chooses the arithmetic policy, runs the
// LUT-free kernels (setup_operator.py:713-915) and the per-fibre second pass of A'.
#include "operator_kernels.cuh"

#include <math.h>
#include <string.h>

namespace cgb {

int forward_f64(cgb_op *op, const double *x, double *y, double *ax, const double *yobs, const double *sqw,
                double *partials, cudaStream_t st, int *grid);
int adjoint_f64(cgb_op *op, const double *yin, int in_mode, const double *x, const double *yobs,
                const double *sqw, const double *ax_a, const double *ax_b, double ca, double cb, double *xout,
                double *partials, cudaStream_t st, int *grid);
int forward_ffs(cgb_op *op, const double *x, double *y, double *ax, const double *yobs, const double *sqw,
                double *partials, cudaStream_t st, int *grid);
int adjoint_ffs(cgb_op *op, const double *yin, int in_mode, const double *x, const double *yobs,
                const double *sqw, const double *ax_a, const double *ax_b, double ca, double cb, double *xout,
                double *partials, cudaStream_t st, int *grid);
int forward_ff(cgb_op *op, const double *x, double *y, double *ax, const double *yobs, const double *sqw,
               double *partials, cudaStream_t st, int *grid);
int adjoint_ff(cgb_op *op, const double *yin, int in_mode, const double *x, const double *yobs,
               const double *sqw, const double *ax_a, const double *ax_b, double ca, double cb, double *xout,
               double *partials, cudaStream_t st, int *grid);

namespace detail {
// second A' pass: per-fibre sums of the voxel-ordered segment terms, fibres in the order
// of their first segment (fib_order)
__global__ void k_fibre_sum(const OpDev P, const double *__restrict__ scratch, double *__restrict__ xout) {
    const int64_t total = (int64_t)P.nF * P.nIC;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / P.nF);
        const uint32_t f = P.fib_order[q - (int64_t)i * P.nF];
        const uint32_t beg = P.fib_ptr[f], end = P.fib_ptr[f + 1];
        const double s = fibre_gather_sum(P.fib_perm, scratch + (size_t)i * P.n, beg, end, 0.0);
        const int64_t c = (int64_t)i * P.nF + f;
        xout[c] = s * (double)P.eval[c];
    }
}

// ------------------------------------------------------------------ LUT-free operator (nS == 1)
__global__ void k_forward_nolut(const OpDev P, const double *__restrict__ x, double *__restrict__ yout,
                                double *__restrict__ axout, const double *__restrict__ yobs,
                                const double *__restrict__ sqw, double *__restrict__ partials) {
    double nrm = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < P.nV; v += gridDim.x * blockDim.x) {
        double a = 0.0;
        if (P.nIC > 0)
            for (uint32_t j = P.vox_ptr[v]; j < P.vox_ptr[v + 1]; ++j) {
                const uint32_t f = P.seg_f[j];
                const double x0 = x[f] * (double)P.eval[f];
                if (x0 != 0) a += (double)P.seg_l[j] * x0;
            }
        if (P.nISO > 0)
            for (uint32_t j = P.iso_ptr[v]; j < P.iso_ptr[v + 1]; ++j) {
                const double x0 = x[P.iso_base + P.iso_col[j]];
                if (x0 != 0) a += x0;
            }
        if (yout) yout[v] = a;
        if (axout) axout[v] = a;
        if (partials) {
            double r = yobs ? a - yobs[v] : a;
            if (sqw) r *= sqw[v];
            nrm = fma(r, r, nrm);
        }
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

__global__ void k_adjoint_nolut(const OpDev P, const double *__restrict__ yin, int in_mode,
                                const double *__restrict__ x, const double *__restrict__ yobs,
                                const double *__restrict__ sqw, const double *__restrict__ ax_a,
                                const double *__restrict__ ax_b, double ca, double cb, double *__restrict__ scratch,
                                double *__restrict__ xout, double *__restrict__ partials) {
    double nrm = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < P.nV; v += gridDim.x * blockDim.x) {
        double z;
        if (in_mode == 0) {
            z = yin[v];
        } else {
            double a = 0.0;
            if (in_mode == 1) {
                if (P.nIC > 0)
                    for (uint32_t j = P.vox_ptr[v]; j < P.vox_ptr[v + 1]; ++j) {
                        const uint32_t f = P.seg_f[j];
                        const double x0 = x[f] * (double)P.eval[f];
                        if (x0 != 0) a += (double)P.seg_l[j] * x0;
                    }
                if (P.nISO > 0)
                    for (uint32_t j = P.iso_ptr[v]; j < P.iso_ptr[v + 1]; ++j) {
                        const double x0 = x[P.iso_base + P.iso_col[j]];
                        if (x0 != 0) a += x0;
                    }
            } else {
                a = ax_combine(ca, ax_a[v], cb, ax_b[v]);
            }
            double r = a - yobs[v];
            if (sqw) r *= sqw[v];
            nrm = fma(r, r, nrm);
            z = sqw ? sqw[v] * r : r;
        }
        if (P.nIC > 0)
            for (uint32_t j = P.vox_ptr[v]; j < P.vox_ptr[v + 1]; ++j) scratch[j] = (double)P.seg_l[j] * z;
        if (P.nISO > 0)
            for (uint32_t j = P.iso_ptr[v]; j < P.iso_ptr[v + 1]; ++j) xout[P.iso_base + P.iso_col[j]] = z;
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

// fibre pass of slab s, fibres in pass order (fib_order): the running sums continue from
// acc (slab 0 starts at 0), terms in the fibre's position order, so the sums are those of
// k_fibre_sum; the last slab applies eval and writes the fibre's column
__global__ void k_fibre_sum_slab(const OpDev P, const double *__restrict__ scratch, double *__restrict__ xout,
                                 const uint32_t *__restrict__ fib_slab, double *__restrict__ accb, int s, int S) {
    const int64_t total = (int64_t)P.nF * P.nIC;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / P.nF);
        const int64_t fq = q - (int64_t)i * P.nF;
        const uint32_t beg = fib_slab[(size_t)s * P.nF + fq], end = fib_slab[(size_t)(s + 1) * P.nF + fq];
        if (s > 0 && s < S - 1 && beg == end) continue;
        const double acc = fibre_gather_sum(P.fib_perm, scratch + (size_t)i * P.n, beg, end, s == 0 ? 0.0 : accb[q]);
        if (s == S - 1) {
            const int64_t c = (int64_t)i * P.nF + P.fib_order[fq];
            xout[c] = acc * (double)P.eval[c];
        } else {
            accb[q] = acc;
        }
    }
}

// largest finite magnitude (as bits: non-negative floats order like their bit patterns)
__global__ void k_absmax_f64(const double *__restrict__ a, int64_t n, unsigned long long *__restrict__ out) {
    unsigned long long m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(a[i]) & 0x7fffffffffffffffull;
        if (b < 0x7ff0000000000000ull && b > m) m = b;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

__global__ void k_absmax_f32(const float *__restrict__ a, int64_t n, unsigned *__restrict__ out) {
    unsigned m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned b = __float_as_uint(a[i]) & 0x7fffffffu;
        if (b < 0x7f800000u && b > m) m = b;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

}  // namespace detail

using namespace detail;

int measure_input(cgb_op *op, const double *x, int64_t n, cudaStream_t st) {
    CGB_CUDA(cudaMemsetAsync(op->d_xmax, 0, sizeof(unsigned long long), st));
    if (n <= 0) return CGB_OK;
    int g = (int)((n + 255) / 256);
    if (g > op->nsm * 8) g = op->nsm * 8;
    k_absmax_f64<<<g, 256, 0, st>>>(x, n, op->d_xmax);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

int update_lut_exponents(cgb_op *op) {
    // [0] max |LUT| over IC, EC and ISO, [1] max |IC length| (bits of non-negative floats)
    unsigned *m = reinterpret_cast<unsigned *>(op->d_xmax);
    CGB_CUDA(cudaMemset(m, 0, 2 * sizeof(unsigned)));
    const struct {
        const float *p;
        int64_t n;
        int slot;
    } parts[4] = {{op->lutIC, (int64_t)op->nIC * op->ndirs * op->nS, 0},
                  {op->lutEC, (int64_t)op->nEC * op->ndirs * op->nS, 0},
                  {op->lutISO, (int64_t)op->nISO * op->nS, 0},
                  {op->seg_l, op->nIC > 0 ? op->n : 0, 1}};
    for (const auto &q : parts) {
        if (!q.p || q.n <= 0) continue;
        int g = (int)((q.n + 255) / 256);
        if (g > op->nsm * 8) g = op->nsm * 8;
        k_absmax_f32<<<g, 256>>>(q.p, q.n, m + q.slot);
        CGB_CUDA(cudaGetLastError());
    }
    unsigned h[2] = {0, 0};
    CGB_CUDA(cudaMemcpy(h, m, sizeof(h), cudaMemcpyDeviceToHost));
    float lut, len;
    memcpy(&lut, &h[0], 4);
    memcpy(&len, &h[1], 4);
    op->lut_exp_adj = lut > 0.f ? ilogbf(lut) : 0;
    op->lut_exp_fwd = op->lut_exp_adj + (len > 1.f ? ilogbf(len) : 0);
    return CGB_OK;
}

int fibre_sum_slab(cgb_op *op, double *xout, int s, cudaStream_t st) {
    if (op->nIC > 0 && op->nF > 0) {
        const OpDev P = op->dev();
        const int64_t total = (int64_t)op->nF * op->nIC;
        int gb = (int)((total + 255) / 256);
        if (gb > op->nsm * 16) gb = op->nsm * 16;
        k_fibre_sum_slab<<<gb, 256, 0, st>>>(P, op->scratch, xout, op->fib_slab, op->fib_acc, s, op->nslab);
        CGB_CUDA(cudaGetLastError());
    }
    return CGB_OK;
}

int fibre_sum(cgb_op *op, double *xout, cudaStream_t st) {
    if (op->nIC > 0 && op->nF > 0) {
        const OpDev P = op->dev();
        const int64_t total = (int64_t)op->nF * op->nIC;
        int gb = (int)((total + 255) / 256);
        if (gb > op->nsm * 16) gb = op->nsm * 16;
        k_fibre_sum<<<gb, 256, 0, st>>>(P, op->scratch, xout);
        CGB_CUDA(cudaGetLastError());
    }
    return CGB_OK;
}

static int run_forward(cgb_op *op, const double *x, double *y, double *ax, const double *yobs, const double *sqw,
                       double *partials, cudaStream_t st, int arith, int *grid_out) {
    if (grid_out) *grid_out = 0;
    if (op->nV == 0) return CGB_OK;
    if (op->nolut) {
        const OpDev P = op->dev();
        int g = (op->nV + kBlock - 1) / kBlock;
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        k_forward_nolut<<<g, kBlock, 0, st>>>(P, x, y, ax, yobs, sqw, partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
        return CGB_OK;
    }
    CGB_TRY(measure_input(op, x, op->ncols, st));
    XScale guard(op);
    if (arith == CGB_ARITH_F64) return forward_f64(op, x, y, ax, yobs, sqw, partials, st, grid_out);
    if (op->ff_variant == 0) return forward_ffs(op, x, y, ax, yobs, sqw, partials, st, grid_out);
    return forward_ff(op, x, y, ax, yobs, sqw, partials, st, grid_out);
}

static int run_adjoint(cgb_op *op, const double *yin, int in_mode, const double *x, const double *yobs,
                       const double *sqw, const double *ax_a, const double *ax_b, double ca, double cb, double *xout,
                       double *partials, cudaStream_t st, int arith, int *grid_out) {
    if (grid_out) *grid_out = 0;
    if (op->nV == 0) {
        if (op->ncols > 0) CGB_CUDA(cudaMemsetAsync(xout, 0, op->ncols * sizeof(double), st));
        return CGB_OK;
    }
    // the fused gradient pass recomputes A x: measure x for the range guard
    const bool mx = in_mode == 1 && !op->nolut;
    if (mx) CGB_TRY(measure_input(op, x, op->ncols, st));
    XScale guard(op, mx);
    if (op->nolut) {
        const OpDev P = op->dev();
        int g = (op->nV + kBlock - 1) / kBlock;
        if (g > reduction_blocks(op)) g = reduction_blocks(op);
        k_adjoint_nolut<<<g, kBlock, 0, st>>>(P, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, op->scratch, xout,
                                              partials);
        CGB_CUDA(cudaGetLastError());
        if (grid_out) *grid_out = g;
    } else if (arith == CGB_ARITH_F64) {
        CGB_TRY(adjoint_f64(op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid_out));
    } else if (op->ff_variant == 0) {
        CGB_TRY(adjoint_ffs(op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid_out));
    } else if (op->nslab > 1) {
        // slab by slab: voxel pass, then the fibre pass while the slab's terms are in L2;
        // slab s writes its norm partials after the s * grid blocks of the earlier slabs
        int g = 0;
        CGB_TRY(slab_schedule(
            op, st,
            [&](int sl, cudaStream_t q) {
                VoxelRange vr(op, op->slab_v[sl], op->slab_v[sl + 1]);
                int gs = 0;
                const int rc = adjoint_ff(op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout,
                                          partials ? partials + (size_t)sl * g * kRedSlots : nullptr, q, &gs);
                if (sl == 0) g = gs;
                return rc;
            },
            [&](int sl, cudaStream_t q) { return fibre_sum_slab(op, xout, sl, q); }));
        if (grid_out) *grid_out = g * op->nslab;
        return CGB_OK;
    } else {
        CGB_TRY(adjoint_ff(op, yin, in_mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid_out));
    }
    return fibre_sum(op, xout, st);
}

int launch_forward(cgb_op *op, const double *x, double *y, cudaStream_t st, int arith) {
    return run_forward(op, x, y, nullptr, nullptr, nullptr, nullptr, st, arith, nullptr);
}

int launch_adjoint(cgb_op *op, const double *y, double *x, cudaStream_t st, int arith) {
    return run_adjoint(op, y, 0, nullptr, nullptr, nullptr, nullptr, nullptr, 0.0, 0.0, x, nullptr, st, arith,
                       nullptr);
}

int launch_resnorm_grid(cgb_op *op, const double *x, const double *y, const double *sqw, double *partials,
                        double *ax_out, cudaStream_t st, int arith, int *grid) {
    return run_forward(op, x, nullptr, ax_out, y, sqw, partials, st, arith, grid);
}

int launch_gradient_grid(cgb_op *op, const double *x, const double *y, const double *sqw, double *grad,
                         double *partials, const double *ax_a, const double *ax_b, double ca, double cb,
                         cudaStream_t st, int arith, int *grid) {
    const int mode = ax_a ? 2 : 1;
    return run_adjoint(op, nullptr, mode, x, y, sqw, ax_a, ax_b, ca, cb, grad, partials, st, arith, grid);
}

}  // namespace cgb
