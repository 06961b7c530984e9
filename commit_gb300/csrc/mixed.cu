// Reduced-precision operator path: on-demand BF16/FP16 LUT copies and FP16 lengths, launch
// of the mixed kernels (operator_mixed_*.cu) and the per-fibre FP64 sum of FP32 terms.
#include <math.h>

#include <type_traits>

#include "cgb_internal.cuh"
#include "operator_pair.cuh"

namespace cgb {

int forward_mix_bf16(cgb_op *, const double *, float *, float *, const float *, const float *, double *,
                     cudaStream_t, int *);
int forward_mix_fp16(cgb_op *, const double *, float *, float *, const float *, const float *, double *,
                     cudaStream_t, int *);
int forward_mix_f32(cgb_op *, const double *, float *, float *, const float *, const float *, double *,
                    cudaStream_t, int *);
int adjoint_mix_bf16(cgb_op *, const float *, int, const double *, const float *, const float *, const float *,
                     const float *, float, float, double *, double *, cudaStream_t, int *);
int adjoint_mix_fp16(cgb_op *, const float *, int, const double *, const float *, const float *, const float *,
                     const float *, float, float, double *, double *, cudaStream_t, int *);
int adjoint_mix_f32(cgb_op *, const float *, int, const double *, const float *, const float *, const float *,
                    const float *, float, float, double *, double *, cudaStream_t, int *);

namespace {

// rows of `w` entries at stride `sin` -> rows at stride `sout` (sout >= sin), zero beyond w
template <class T>
__global__ void k_to_reduced(const float *__restrict__ in, T *__restrict__ out, size_t rows, int sin, int sout) {
    const size_t n = rows * (size_t)sout;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / sout;
        const int k = (int)(i - r * sout);
        const float v = k < sin ? in[r * sin + k] : 0.f;
        if constexpr (sizeof(T) == 2 && std::is_same<T, __nv_bfloat16>::value) out[i] = __float2bfloat16_rn(v);
        else out[i] = __float2half_rn(v);
    }
}

__global__ void k_to_bf16(const float *in, __nv_bfloat16 *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(in[i]);
}

__global__ void k_to_fp16(const float *in, __half *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __float2half_rn(in[i]);
}

__global__ void k_len16(const float *in, __half *out, size_t n, float scale) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __float2half_rn(in[i] * scale);
}

__global__ void k_maxabs(const float *in, size_t n, unsigned int *out) {
    float m = 0.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(in[i]));
    // non-negative floats order like their bit patterns
    atomicMax(out, __float_as_uint(m));
}

__global__ void k_f64_to_f32(const double *in, float *out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

__global__ void k_f32_to_f64(const float *in, double *out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

__global__ void k_fibre_sum32(const OpDev P, const float *__restrict__ scr, double *__restrict__ xout) {
    const int64_t total = (int64_t)P.nF * P.nIC;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / P.nF);
        const uint32_t f = P.fib_order[q - (int64_t)i * P.nF];
        const double s = fibre_gather_sum(P.fib_perm, scr + (size_t)i * P.n, P.fib_ptr[f], P.fib_ptr[f + 1], 0.0);
        const int64_t c = (int64_t)i * P.nF + f;
        xout[c] = s * (double)P.eval[c];
    }
}

int grid_n(size_t n) {
    size_t g = (n + 255) / 256;
    if (g > 4096) g = 4096;
    if (g < 1) g = 1;
    return (int)g;
}

int fibre_sum32(cgb_op *op, double *xout, cudaStream_t st) {
    if (op->nIC > 0 && op->nF > 0) {
        const int64_t total = (int64_t)op->nF * op->nIC;
        int gb = (int)((total + 255) / 256);
        if (gb > op->nsm * 16) gb = op->nsm * 16;
        k_fibre_sum32<<<gb, 256, 0, st>>>(op->dev(), op->scratch32, xout);
        CGB_CUDA(cudaGetLastError());
    }
    return CGB_OK;
}

}  // namespace

__global__ void k_fibre_sum32_slab(const OpDev P, const float *__restrict__ scr, double *__restrict__ xout,
                                   const uint32_t *__restrict__ fib_slab, double *__restrict__ accb, int s, int S) {
    const int64_t total = (int64_t)P.nF * P.nIC;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / P.nF);
        const int64_t fq = q - (int64_t)i * P.nF;
        const uint32_t beg = fib_slab[(size_t)s * P.nF + fq], end = fib_slab[(size_t)(s + 1) * P.nF + fq];
        if (s > 0 && s < S - 1 && beg == end) continue;
        const double acc = fibre_gather_sum(P.fib_perm, scr + (size_t)i * P.n, beg, end, s == 0 ? 0.0 : accb[q]);
        if (s == S - 1) {
            const int64_t c = (int64_t)i * P.nF + P.fib_order[fq];
            xout[c] = acc * (double)P.eval[c];
        } else {
            accb[q] = acc;
        }
    }
}

int fibre_sum32_slab(cgb_op *op, const float *scr, double *xout, int s, cudaStream_t st, int slot) {
    if (op->nIC > 0 && op->nF > 0) {
        const int64_t total = (int64_t)op->nF * op->nIC;
        if (slot >= op->fib_acc_slots) return fail(CGB_ERR_INVALID, "fibre pass: no accumulator for this vector");
        int gb = (int)((total + 255) / 256);
        if (gb > op->nsm * 16) gb = op->nsm * 16;
        k_fibre_sum32_slab<<<gb, 256, 0, st>>>(op->dev(), scr, xout, op->fib_slab, op->fib_acc + (size_t)slot * total,
                                                s, op->nslab);
        CGB_CUDA(cudaGetLastError());
    }
    return CGB_OK;
}

int fibre_sum32_from(cgb_op *op, const float *scr, double *xout, cudaStream_t st) {
    if (op->nIC > 0 && op->nF > 0) {
        const int64_t total = (int64_t)op->nF * op->nIC;
        int gb = (int)((total + 255) / 256);
        if (gb > op->nsm * 16) gb = op->nsm * 16;
        k_fibre_sum32<<<gb, 256, 0, st>>>(op->dev(), scr, xout);
        CGB_CUDA(cudaGetLastError());
    }
    return CGB_OK;
}

int forward_R2(cgb_op *, const RhsPtrs &, const float *, const float *, double *, cudaStream_t, int *);
int forward_R4(cgb_op *, const RhsPtrs &, const float *, const float *, double *, cudaStream_t, int *);
int adjoint_R2(cgb_op *, const RhsPtrs &, int, const float *, const float *, double *, cudaStream_t, int *);
int adjoint_R4(cgb_op *, const RhsPtrs &, int, const float *, const float *, double *, cudaStream_t, int *);

int launch_forward_R(cgb_op *op, int R, const RhsPtrs &V, const float *yobs, const float *sqw, double *partials,
                     cudaStream_t st, int *grid) {
    CGB_TRY(ensure_reduced(op, CGB_ARITH_BF16));
    if (grid) *grid = 0;
    if (op->nV == 0) return CGB_OK;
    if (R == 2) return forward_R2(op, V, yobs, sqw, partials, st, grid);
    if (R == 4) return forward_R4(op, V, yobs, sqw, partials, st, grid);
    return fail(CGB_ERR_UNSUPPORTED, "vectors per pass must be 2 or 4");
}

int launch_adjoint_R(cgb_op *op, int R, const RhsPtrs &V, int in_mode, const float *yobs, const float *sqw,
                     double *partials, cudaStream_t st, int *grid) {
    CGB_TRY(ensure_reduced(op, CGB_ARITH_BF16));
    if (grid) *grid = 0;
    if (op->nV == 0) return CGB_OK;
    if (R == 2) return adjoint_R2(op, V, in_mode, yobs, sqw, partials, st, grid);
    if (R == 4) return adjoint_R4(op, V, in_mode, yobs, sqw, partials, st, grid);
    return fail(CGB_ERR_UNSUPPORTED, "vectors per pass must be 2 or 4");
}

int convert_f64_to_f32(const double *in, float *out, int64_t n, cudaStream_t st) {
    if (n <= 0) return CGB_OK;
    k_f64_to_f32<<<grid_n(n), 256, 0, st>>>(in, out, n);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

int convert_f32_to_f64(const float *in, double *out, int64_t n, cudaStream_t st) {
    if (n <= 0) return CGB_OK;
    k_f32_to_f64<<<grid_n(n), 256, 0, st>>>(in, out, n);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

int ensure_reduced(cgb_op *op, int arith) {
    if (arith != CGB_ARITH_BF16 && arith != CGB_ARITH_FP16 && arith != CGB_ARITH_F32)
        return fail(CGB_ERR_INVALID, "reduced-precision arith must be BF16, FP16 or F32");
    if (op->nolut) return fail(CGB_ERR_UNSUPPORTED, "the reduced-precision path needs a LUT operator");
    if (!op->scratch32) {
        CGB_CUDA(cudaMalloc((void **)&op->scratch32, (size_t)(op->n > 0 ? op->n : 1) * (op->nIC > 0 ? op->nIC : 1) *
                                                         sizeof(float)));
        op->bytes += (size_t)op->n * op->nIC * sizeof(float);
    }
    if (arith == CGB_ARITH_F32) return CGB_OK;
    if (op->lut_r_kind != arith) {
        if (op->lutIC_r) cudaFree(op->lutIC_r);
        if (op->lutEC_r) cudaFree(op->lutEC_r);
        if (op->lutISO_r) cudaFree(op->lutISO_r);
        op->lutIC_r = op->lutEC_r = op->lutISO_r = nullptr;
        // rows at a stride with room for the 32-lane shape of the multi-vector kernels
        const int wide = 2 * detail::wide_pair_shape(op->nS).lpv * detail::wide_pair_shape(op->nS).np;
        op->nSp_r = wide > op->nSp ? wide : op->nSp;
        const size_t ric = (size_t)op->nIC * op->ndirs, rec = (size_t)op->nEC * op->ndirs, riso = (size_t)op->nISO;
        const size_t nic = ric * op->nSp_r, nec = rec * op->nSp_r, niso = riso * op->nSp_r;
        CGB_CUDA(cudaMalloc(&op->lutIC_r, (nic ? nic : 1) * 2));
        CGB_CUDA(cudaMalloc(&op->lutEC_r, (nec ? nec : 1) * 2));
        CGB_CUDA(cudaMalloc(&op->lutISO_r, (niso ? niso : 1) * 2));
        if (arith == CGB_ARITH_BF16) {
            if (nic) k_to_reduced<<<grid_n(nic), 256>>>(op->lutIC_p, (__nv_bfloat16 *)op->lutIC_r, ric, op->nSp, op->nSp_r);
            if (nec) k_to_reduced<<<grid_n(nec), 256>>>(op->lutEC_p, (__nv_bfloat16 *)op->lutEC_r, rec, op->nSp, op->nSp_r);
            if (niso)
                k_to_reduced<<<grid_n(niso), 256>>>(op->lutISO_p, (__nv_bfloat16 *)op->lutISO_r, riso, op->nSp, op->nSp_r);
        } else {
            if (nic) k_to_reduced<<<grid_n(nic), 256>>>(op->lutIC_p, (__half *)op->lutIC_r, ric, op->nSp, op->nSp_r);
            if (nec) k_to_reduced<<<grid_n(nec), 256>>>(op->lutEC_p, (__half *)op->lutEC_r, rec, op->nSp, op->nSp_r);
            if (niso) k_to_reduced<<<grid_n(niso), 256>>>(op->lutISO_p, (__half *)op->lutISO_r, riso, op->nSp, op->nSp_r);
        }
        CGB_CUDA(cudaGetLastError());
        op->lut_r_kind = arith;
    }
    if (!op->seg_l16 && op->n > 0) {
        // lengths as FP16 of l * 2^k, with the largest length just below 2^15
        unsigned int *dmax;
        CGB_CUDA(cudaMalloc((void **)&dmax, sizeof(unsigned int)));
        CGB_CUDA(cudaMemset(dmax, 0, sizeof(unsigned int)));
        k_maxabs<<<grid_n(op->n), 256>>>(op->seg_l, op->n, dmax);
        unsigned int hb = 0;
        cudaError_t e = cudaMemcpy(&hb, dmax, sizeof(hb), cudaMemcpyDeviceToHost);
        cudaFree(dmax);
        CGB_CUDA(e);
        float mx;
        memcpy(&mx, &hb, 4);
        int k = 0;
        if (mx > 0.f && isfinite(mx)) k = (int)floor(log2(32768.0 / mx));
        if (k > 60) k = 60;
        if (k < -60) k = -60;
        CGB_CUDA(cudaMalloc((void **)&op->seg_l16, (size_t)op->n * sizeof(__half)));
        op->bytes += (size_t)op->n * sizeof(__half);
        k_len16<<<grid_n(op->n), 256>>>(op->seg_l, op->seg_l16, op->n, ldexpf(1.f, k));
        CGB_CUDA(cudaGetLastError());
        op->len16_inv_scale = ldexpf(1.f, -k);
    }
    CGB_CUDA(cudaDeviceSynchronize());
    return CGB_OK;
}

static int fwd_mix(cgb_op *op, int arith, const double *x, float *y, float *ax, const float *yobs, const float *sqw,
                   double *partials, cudaStream_t st, int *grid) {
    if (arith == CGB_ARITH_BF16 && tc_forward_enabled(op)) return forward_tc(op, x, y, ax, yobs, sqw, partials, st, grid);
    if (arith == CGB_ARITH_BF16) return forward_mix_bf16(op, x, y, ax, yobs, sqw, partials, st, grid);
    if (arith == CGB_ARITH_FP16) return forward_mix_fp16(op, x, y, ax, yobs, sqw, partials, st, grid);
    return forward_mix_f32(op, x, y, ax, yobs, sqw, partials, st, grid);
}

static int adj_mix(cgb_op *op, int arith, const float *yin, int mode, const double *x, const float *yobs,
                   const float *sqw, const float *ax_a, const float *ax_b, float ca, float cb, double *xout,
                   double *partials, cudaStream_t st, int *grid) {
    if (arith == CGB_ARITH_BF16)
        return adjoint_mix_bf16(op, yin, mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid);
    if (arith == CGB_ARITH_FP16)
        return adjoint_mix_fp16(op, yin, mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid);
    return adjoint_mix_f32(op, yin, mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid);
}

// A' in reduced precision: voxel pass and fibre pass, slab by slab when the handle has
// slabs (the fibre pass then gathers each slab's terms from L2)
static int adj_mix_slabs(cgb_op *op, int arith, const float *yin, int mode, const double *x, const float *yobs,
                         const float *sqw, const float *ax_a, const float *ax_b, float ca, float cb, double *xout,
                         double *partials, cudaStream_t st, int *grid) {
    if (op->nslab <= 1) {
        CGB_TRY(adj_mix(op, arith, yin, mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout, partials, st, grid));
        return fibre_sum32(op, xout, st);
    }
    int g = 0;
    CGB_TRY(slab_schedule(
        op, st,
        [&](int sl, cudaStream_t q) {
            VoxelRange vr(op, op->slab_v[sl], op->slab_v[sl + 1]);
            int gs = 0;
            const int rc = adj_mix(op, arith, yin, mode, x, yobs, sqw, ax_a, ax_b, ca, cb, xout,
                                   partials ? partials + (size_t)sl * g * kRedSlots : nullptr, q, &gs);
            if (sl == 0) g = gs;
            return rc;
        },
        [&](int sl, cudaStream_t q) { return fibre_sum32_slab(op, op->scratch32, xout, sl, q); }));
    if (grid) *grid = g * op->nslab;
    return CGB_OK;
}

int launch_resnorm_mix(cgb_op *op, const double *x, const float *y, const float *sqw, double *partials,
                       float *ax_out, float *yout, cudaStream_t st, int arith, int *grid) {
    if (grid) *grid = 0;
    CGB_TRY(ensure_reduced(op, arith));
    if (op->nV == 0) return CGB_OK;
    return fwd_mix(op, arith, x, yout, ax_out, y, sqw, partials, st, grid);
}

int launch_gradient_mix(cgb_op *op, const double *x, const float *y, const float *sqw, double *grad,
                        double *partials, const float *ax_a, const float *ax_b, float ca, float cb,
                        cudaStream_t st, int arith, int *grid) {
    if (grid) *grid = 0;
    CGB_TRY(ensure_reduced(op, arith));
    if (op->nV == 0) {
        if (op->ncols > 0) CGB_CUDA(cudaMemsetAsync(grad, 0, op->ncols * sizeof(double), st));
        return CGB_OK;
    }
    if (arith == CGB_ARITH_BF16 && tc_forward_enabled(op)) {
        // tensor cores: A x into a row buffer first when it is not given, then A' of the residual
        if (!ax_a) {
            if (!op->tc_ax) {
                CGB_CUDA(cudaMalloc((void **)&op->tc_ax, (size_t)op->nrows * sizeof(float)));
                op->bytes += (size_t)op->nrows * sizeof(float);
            }
            CGB_TRY(forward_tc(op, x, nullptr, op->tc_ax, nullptr, nullptr, nullptr, st, nullptr));
            return adjoint_tc(op, 2, nullptr, op->tc_ax, nullptr, 1.f, 0.f, y, sqw, grad, partials, st, grid);
        }
        return adjoint_tc(op, 2, nullptr, ax_a, ax_b, ca, cb, y, sqw, grad, partials, st, grid);
    }
    return adj_mix_slabs(op, arith, nullptr, ax_a ? 2 : 1, x, y, sqw, ax_a, ax_b, ca, cb, grad, partials, st, grid);
}

int launch_adjoint_mix(cgb_op *op, const float *yin, double *xout, cudaStream_t st, int arith) {
    CGB_TRY(ensure_reduced(op, arith));
    if (op->nV == 0) {
        if (op->ncols > 0) CGB_CUDA(cudaMemsetAsync(xout, 0, op->ncols * sizeof(double), st));
        return CGB_OK;
    }
    if (arith == CGB_ARITH_BF16 && tc_forward_enabled(op))
        return adjoint_tc(op, 0, yin, nullptr, nullptr, 0.f, 0.f, nullptr, nullptr, xout, nullptr, st, nullptr);
    return adj_mix_slabs(op, arith, yin, 0, nullptr, nullptr, nullptr, nullptr, nullptr, 0.f, 0.f, xout, nullptr, st,
                         nullptr);
}

}  // namespace cgb
