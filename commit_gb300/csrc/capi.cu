// Operator application entry points of the C ABI (LinearOperator.dot, operator.pyx:114-184).
#include "cgb_internal.cuh"

using namespace cgb;

namespace {
struct DevGuard {
    int prev = -1;
    explicit DevGuard(int d) {
        cudaGetDevice(&prev);
        if (prev != d) cudaSetDevice(d);
    }
    ~DevGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int check_lengths(const cgb_op *op, int adjoint, int64_t in_len, int64_t out_len) {
    const int64_t want_in = adjoint ? op->nrows : op->ncols;
    const int64_t want_out = adjoint ? op->ncols : op->nrows;
    if (in_len != want_in || out_len != want_out) return fail(CGB_ERR_DIMENSION, "A.dot(): dimensions do not match");
    return CGB_OK;
}
}  // namespace

extern "C" {

int cgb_op_apply(cgb_op *op, int adjoint, const void *in, int64_t in_len, void *out, int64_t out_len, int dtype,
                 int arith, void *stream) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    CGB_TRY(check_lengths(op, adjoint, in_len, out_len));
    if ((in_len > 0 && !in) || (out_len > 0 && !out)) return fail(CGB_ERR_INVALID, "null vector");
    DevGuard g(op->device);
    cudaStream_t st = (cudaStream_t)stream;
    if (out_len == 0) return CGB_OK;
    if (dtype == CGB_DTYPE_F64) {
        const int ar = (arith == CGB_ARITH_F64 || arith == CGB_ARITH_FF) ? arith : op->arith;
        if (in_len == 0) {
            CGB_CUDA(cudaMemsetAsync(out, 0, out_len * sizeof(double), st));
            return CGB_OK;
        }
        if (adjoint) return launch_adjoint(op, (const double *)in, (double *)out, st, ar);
        return launch_forward(op, (const double *)in, (double *)out, st, ar);
    }
    if (dtype == CGB_DTYPE_F32) {
        if (arith != CGB_ARITH_BF16 && arith != CGB_ARITH_FP16 && arith != CGB_ARITH_F32)
            return fail(CGB_ERR_INVALID, "FP32 vectors need arith BF16, FP16 or F32");
        if (!op->d_x64) CGB_CUDA(cudaMalloc((void **)&op->d_x64, (op->ncols > 0 ? op->ncols : 1) * sizeof(double)));
        if (!adjoint) {
            CGB_TRY(convert_f32_to_f64((const float *)in, op->d_x64, op->ncols, st));
            return launch_resnorm_mix(op, op->d_x64, nullptr, nullptr, nullptr, nullptr, (float *)out, st, arith,
                                      nullptr);
        }
        CGB_TRY(launch_adjoint_mix(op, (const float *)in, op->d_x64, st, arith));
        return convert_f64_to_f32(op->d_x64, (float *)out, op->ncols, st);
    }
    return fail(CGB_ERR_UNSUPPORTED, "unsupported dtype / arithmetic combination");
}

int cgb_op_apply_host(cgb_op *op, int adjoint, const double *in, int64_t in_len, double *out, int64_t out_len) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    CGB_TRY(check_lengths(op, adjoint, in_len, out_len));
    if ((in_len > 0 && !in) || (out_len > 0 && !out)) return fail(CGB_ERR_INVALID, "null vector");
    DevGuard g(op->device);
    if (out_len == 0) return CGB_OK;
    // staging buffers sized for the larger of the two vector lengths, kept on the handle
    const int64_t need = op->nrows > op->ncols ? op->nrows : op->ncols;
    if (op->d_in_len < need) {
        if (op->d_in) cudaFree(op->d_in);
        if (op->d_out) cudaFree(op->d_out);
        op->d_in = op->d_out = nullptr;
        op->d_in_len = op->d_out_len = 0;
        CGB_CUDA(cudaMalloc((void **)&op->d_in, need * sizeof(double)));
        CGB_CUDA(cudaMalloc((void **)&op->d_out, need * sizeof(double)));
        op->d_in_len = op->d_out_len = need;
    }
    cudaStream_t st = nullptr;
    if (in_len > 0) CGB_CUDA(cudaMemcpyAsync(op->d_in, in, in_len * sizeof(double), cudaMemcpyHostToDevice, st));
    CGB_TRY(cgb_op_apply(op, adjoint, op->d_in, in_len, op->d_out, out_len, CGB_DTYPE_F64, op->arith, st));
    CGB_CUDA(cudaMemcpyAsync(out, op->d_out, out_len * sizeof(double), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    return CGB_OK;
}

}  // extern "C"

extern "C" int cgb_op_occupancy(cgb_op *op, int slot, int set, int *choice, float *ms_a, float *ms_b) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (slot < 0 || slot >= kOccSlots) return fail(CGB_ERR_INVALID, "slot out of range");
    if (set >= 0) {
        if (set > 2) return fail(CGB_ERR_INVALID, "choice must be 0 (retune), 1 or 2");
        op->occ_choice[slot] = set;
    }
    if (choice) *choice = op->occ_choice[slot];
    if (ms_a) *ms_a = op->occ_ms[slot][0];
    if (ms_b) *ms_b = op->occ_ms[slot][1];
    return CGB_OK;
}
