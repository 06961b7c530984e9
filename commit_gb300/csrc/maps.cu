// Voxelwise maps of a fit, as Evaluation.save_results computes them (commit/core.pyx:1614-1740):
// fitting errors per voxel (RMSE, NRMSE, and their confidence-weighted forms) from the
// estimated signal A x, and the compartment maps (IC: sum over the voxel's segments of
// length * the streamline's weight summed over its responses, EC / ISO: sum of the voxel's
// coefficients).  All are segmented reductions over the voxel-ordered streams the operator
// already holds: one warp per voxel, no atomics, FP64 sums.
#include "cgb_internal.cuh"

namespace cgb {
namespace {

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// core.pyx:1662-1705 (no debias mask): y_est and y_mea are compared as FP32 values, as the
// reference casts both with astype(np.float32); sums are FP64 here (numpy sums FP32).
__global__ void k_voxel_errors(int nV, int nS, const double *__restrict__ yest, const double *__restrict__ ymea,
                               const double *__restrict__ conf, double *__restrict__ rmse, double *__restrict__ nrmse,
                               double *__restrict__ rmse_c, double *__restrict__ nrmse_c) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = warp; v < nV; v += nw) {
        double se = 0.0, sy = 0.0, sc = 0.0, sce = 0.0, scy = 0.0;
        for (int s = lane; s < nS; s += 32) {
            const size_t i = (size_t)v * nS + s;
            const float a = (float)ymea[i], b = (float)yest[i];
            const double d = (double)(a - b);
            se += d * d;
            sy += (double)a * (double)a;
            if (conf) {
                const double c = (double)(float)conf[i];
                sc += c;
                sce += c * d * d;
                scy += c * (double)a * (double)a;
            }
        }
        se = wsum(se);
        sy = wsum(sy);
        if (conf) {
            sc = wsum(sc);
            sce = wsum(sce);
            scy = wsum(scy);
        }
        if (lane == 0) {
            if (rmse) rmse[v] = sqrt(se / nS);
            if (nrmse) nrmse[v] = sy < 1e-12 ? 0.0 : sqrt(se / sy);
            if (conf && rmse_c) rmse_c[v] = sc < 1e-12 ? 0.0 : sqrt(sce / sc);
            if (conf && nrmse_c) nrmse_c[v] = scy < 1e-12 ? 0.0 : sqrt(sce / scy);
        }
    }
}

// core.pyx:1717-1750: IC[v] = sum_j len_j * sum_i x[i*nF + f_j] * w[i*nF + f_j] (w = norm_fib
// or 1); EC[v] = sum over the voxel's peaks e of sum_i x[ec_base + i*nE + e]; ISO likewise.
__global__ void k_compartment_maps(const OpDev P, const double *__restrict__ x, const double *__restrict__ wfib,
                                   double *__restrict__ ic, double *__restrict__ ec, double *__restrict__ iso) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = warp; v < P.nV; v += nw) {
        if (ic) {
            double a = 0.0;
            if (P.nIC > 0 && P.n > 0) {
                for (uint32_t j = P.vox_ptr[v] + lane; j < P.vox_ptr[v + 1]; j += 32) {
                    const uint32_t f = P.seg_f[j];
                    double t = 0.0;
                    for (int i = 0; i < P.nIC; ++i) {
                        const int64_t q = (int64_t)i * P.nF + f;
                        t += wfib ? x[q] * wfib[q] : x[q];
                    }
                    a += t * (double)P.seg_l[j];
                }
            }
            a = wsum(a);
            if (lane == 0) ic[v] = a;
        }
        if (ec) {
            double a = 0.0;
            if (P.nEC > 0 && P.nE > 0) {
                for (uint32_t j = P.ec_ptr[v] + lane; j < P.ec_ptr[v + 1]; j += 32) {
                    const uint32_t e = P.ec_col[j];
                    for (int i = 0; i < P.nEC; ++i) a += x[P.ec_base + (int64_t)i * P.nE + e];
                }
            }
            a = wsum(a);
            if (lane == 0) ec[v] = a;
        }
        if (iso) {
            double a = 0.0;
            if (P.nISO > 0 && P.nISOv > 0) {
                for (uint32_t j = P.iso_ptr[v] + lane; j < P.iso_ptr[v + 1]; j += 32) {
                    const uint32_t c = P.iso_col[j];
                    for (int i = 0; i < P.nISO; ++i) a += x[P.iso_base + (int64_t)i * P.nISOv + c];
                }
            }
            a = wsum(a);
            if (lane == 0) iso[v] = a;
        }
    }
}

int warp_grid(const cgb_op *op, int64_t items) {
    int64_t g = (items * 32 + 255) / 256;
    const int64_t cap = (int64_t)op->nsm * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace
}  // namespace cgb

using namespace cgb;

extern "C" int cgb_op_voxel_maps(cgb_op *op, const double *x, const double *y_mea, const double *conf,
                                 const double *norm_fib, double *ic, double *ec, double *iso, double *rmse,
                                 double *nrmse, double *rmse_conf, double *nrmse_conf, void *stream) {
    if (!op || !x) return fail(CGB_ERR_INVALID, "null argument");
    if (conf && !y_mea) return fail(CGB_ERR_INVALID, "a confidence map needs the measured signal");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != op->device) cudaSetDevice(op->device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = CGB_OK;
    double *yest = nullptr;
    if (op->nV > 0) {
        if (ic || ec || iso) {
            k_compartment_maps<<<warp_grid(op, op->nV), 256, 0, st>>>(op->dev(), x, norm_fib, ic, ec, iso);
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) rc = cuda_fail(e, "k_compartment_maps");
        }
        if (rc == CGB_OK && y_mea && (rmse || nrmse || rmse_conf || nrmse_conf)) {
            cudaError_t e = cudaMalloc((void **)&yest, (size_t)op->nrows * sizeof(double));
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc");
            if (rc == CGB_OK) rc = launch_forward(op, x, yest, st, op->arith);
            if (rc == CGB_OK) {
                k_voxel_errors<<<warp_grid(op, op->nV), 256, 0, st>>>(op->nV, op->nS, yest, y_mea, conf, rmse, nrmse,
                                                                     rmse_conf, nrmse_conf);
                e = cudaGetLastError();
                if (e != cudaSuccess) rc = cuda_fail(e, "k_voxel_errors");
            }
            if (yest) {
                cudaStreamSynchronize(st);
                cudaFree(yest);
            }
        }
    }
    if (prev >= 0 && prev != op->device) cudaSetDevice(prev);
    return rc;
}
