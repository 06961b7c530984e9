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

// Host-buffer pipeline for the float-float operator on large problems: the voxels are cut
// into kPipe ranges; A writes the rows of range k while the rows of range k-1 are copied to
// the host on a second stream, and A' copies the rows of range k+1 in while pass 1 runs on
// range k (pass 2 follows once all ranges are in).  The copies of the row vector (the
// large one) hide behind the computation.  Results are those of the one-shot path (the
// same per-voxel computation).
static constexpr int kPipe = 8;

// Direct row access: when the caller's row vector (y, the large one) is in page-locked host
// memory, the voxel kernels read or write it in place through its device mapping (on
// GB300 the host memory sits behind NVLink-C2C), so no row-sized copy or staging buffer is
// needed; the column vector (gathered at random by A) is still copied.  Used when the
// handle's host mode is automatic (0) or direct (2).
static bool direct_rows(const cgb_op *op, const double *rows) {
    if (op->host_mode == 1 || op->nolut || op->nrows < ((int64_t)1 << 20)) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, rows) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost && a.devicePointer != nullptr;
}

static int apply_host_direct(cgb_op *op, int adjoint, const double *in, int64_t in_len, double *out,
                             int64_t out_len) {
    cudaStream_t st = nullptr;
    cudaPointerAttributes a;
    if (!adjoint) {
        CGB_CUDA(cudaPointerGetAttributes(&a, out));
        double *yd = (double *)a.devicePointer;
        CGB_CUDA(cudaMemcpyAsync(op->d_in, in, in_len * sizeof(double), cudaMemcpyHostToDevice, st));
        CGB_TRY(cgb_op_apply(op, 0, op->d_in, in_len, yd, out_len, CGB_DTYPE_F64, op->arith, st));
    } else {
        CGB_CUDA(cudaPointerGetAttributes(&a, in));
        const double *yd = (const double *)a.devicePointer;
        CGB_TRY(cgb_op_apply(op, 1, yd, in_len, op->d_out, out_len, CGB_DTYPE_F64, op->arith, st));
        CGB_CUDA(cudaMemcpyAsync(out, op->d_out, out_len * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    CGB_CUDA(cudaStreamSynchronize(st));
    return CGB_OK;
}

static bool pipelined(const cgb_op *op) {
    return op->arith == CGB_ARITH_FF && op->ff_variant != 0 && !op->nolut && op->nV >= 4 * kPipe &&
           op->nrows >= ((int64_t)1 << 22);
}

namespace cgb {
int forward_ff(cgb_op *op, const double *x, double *y, double *ax, const double *yobs, const double *sqw,
               double *partials, cudaStream_t st, int *grid);
int adjoint_ff(cgb_op *op, const double *yin, int in_mode, const double *x, const double *yobs, const double *sqw,
               const double *ax_a, const double *ax_b, double ca, double cb, double *xout, double *partials,
               cudaStream_t st, int *grid);
}  // namespace cgb

static int apply_host_pipelined(cgb_op *op, int adjoint, const double *in, int64_t in_len, double *out,
                                int64_t out_len) {
    if (!op->pipe_st[0]) {
        for (int i = 0; i < 2; ++i) CGB_CUDA(cudaStreamCreateWithFlags(&op->pipe_st[i], cudaStreamNonBlocking));
        for (int k = 0; k < kPipe; ++k) CGB_CUDA(cudaEventCreateWithFlags(&op->pipe_ev[k], cudaEventDisableTiming));
    }
    cudaStream_t sc = op->pipe_st[0], sx = op->pipe_st[1];
    const int nS = op->nS;
    // ranges: the adjoint slabs when the handle has them (the fibre pass of a range then
    // runs right after its voxel pass), else kPipe equal voxel ranges
    const bool slabs = adjoint && op->nslab > 1;
    const int K = slabs ? op->nslab : kPipe;
    auto vb = [&](int k) { return slabs ? op->slab_v[k] : (int)((int64_t)op->nV * k / kPipe); };
    if (!adjoint) {
        CGB_CUDA(cudaMemcpyAsync(op->d_in, in, in_len * sizeof(double), cudaMemcpyHostToDevice, sc));
        CGB_TRY(measure_input(op, op->d_in, in_len, sc));
        XScale guard(op);
        for (int k = 0; k < K; ++k) {
            const int v0 = vb(k), v1 = vb(k + 1);
            if (v1 > v0) {
                VoxelRange vr(op, v0, v1);
                CGB_TRY(forward_ff(op, op->d_in, op->d_out, nullptr, nullptr, nullptr, nullptr, sc, nullptr));
            }
            CGB_CUDA(cudaEventRecord(op->pipe_ev[k % kPipe], sc));
            CGB_CUDA(cudaStreamWaitEvent(sx, op->pipe_ev[k % kPipe], 0));
            const size_t r0 = (size_t)v0 * nS, nr = (size_t)(v1 - v0) * nS;
            if (nr) CGB_CUDA(cudaMemcpyAsync(out + r0, op->d_out + r0, nr * sizeof(double), cudaMemcpyDeviceToHost, sx));
        }
        CGB_CUDA(cudaStreamSynchronize(sx));
        CGB_CUDA(cudaStreamSynchronize(sc));
        return CGB_OK;
    }
    for (int k = 0; k < K; ++k) {
        const int v0 = vb(k), v1 = vb(k + 1);
        const size_t r0 = (size_t)v0 * nS, nr = (size_t)(v1 - v0) * nS;
        if (nr) CGB_CUDA(cudaMemcpyAsync(op->d_in + r0, in + r0, nr * sizeof(double), cudaMemcpyHostToDevice, sx));
        CGB_CUDA(cudaEventRecord(op->pipe_ev[k % kPipe], sx));
        CGB_CUDA(cudaStreamWaitEvent(sc, op->pipe_ev[k % kPipe], 0));
        if (v1 > v0) {
            VoxelRange vr(op, v0, v1);
            CGB_TRY(adjoint_ff(op, op->d_in, 0, nullptr, nullptr, nullptr, nullptr, nullptr, 0.0, 0.0, op->d_out,
                               nullptr, sc, nullptr));
        }
        if (slabs) CGB_TRY(fibre_sum_slab(op, op->d_out, k, sc));
    }
    if (!slabs) CGB_TRY(fibre_sum(op, op->d_out, sc));
    CGB_CUDA(cudaMemcpyAsync(out, op->d_out, out_len * sizeof(double), cudaMemcpyDeviceToHost, sc));
    CGB_CUDA(cudaStreamSynchronize(sc));
    return CGB_OK;
}

extern "C" {

int cgb_op_apply(cgb_op *op, int adjoint, const void *in, int64_t in_len, void *out, int64_t out_len, int dtype,
                 int arith, void *stream) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    CGB_TRY(check_lengths(op, adjoint, in_len, out_len));
    if ((in_len > 0 && !in) || (out_len > 0 && !out)) return fail(CGB_ERR_INVALID, "null vector");
    NvtxRange nv(adjoint ? "cgb_op_apply A'" : "cgb_op_apply A");
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
    NvtxRange nv(adjoint ? "cgb_op_apply_host A'" : "cgb_op_apply_host A");
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
    if (in_len > 0 && direct_rows(op, adjoint ? in : out))
        return apply_host_direct(op, adjoint, in, in_len, out, out_len);
    if (in_len > 0 && pipelined(op)) return apply_host_pipelined(op, adjoint, in, in_len, out, out_len);
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
    if (slot < 0 || slot >= kOccSlots) return fail(CGB_ERR_INVALID, "slot out of range");  // kOccSlots = 24
    if (set >= 0) {
        if (set > 2) return fail(CGB_ERR_INVALID, "choice must be 0 (retune), 1 or 2");
        op->occ_choice[slot] = set;
    }
    if (choice) *choice = op->occ_choice[slot];
    if (ms_a) *ms_a = op->occ_ms[slot][0];
    if (ms_b) *ms_b = op->occ_ms[slot][1];
    return CGB_OK;
}

extern "C" int cgb_op_host_mode(cgb_op *op, int mode, int *out) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (mode > 2) return fail(CGB_ERR_INVALID, "host mode must be 0 (automatic), 1 (staged) or 2 (direct)");
    if (mode >= 0) op->host_mode = mode;
    if (out) *out = op->host_mode;
    return CGB_OK;
}
