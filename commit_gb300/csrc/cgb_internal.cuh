// Internal declarations shared by the commit_gb300 CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stdio.h>

#include <nvtx3/nvToolsExt.h>

#include <string>

#include "../../include/commit_gb300.h"

namespace cgb {

// ------------------------------------------------------------------ errors
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define CGB_CUDA(call)                                                  \
    do {                                                                \
        cudaError_t e__ = (call);                                       \
        if (e__ != cudaSuccess) return ::cgb::cuda_fail(e__, #call);    \
    } while (0)

#define CGB_TRY(call)                         \
    do {                                      \
        int rc__ = (call);                    \
        if (rc__ != CGB_OK) return rc__;      \
    } while (0)

// ------------------------------------------------------------------ tracing
// NVTX range over a scope (an entry point, a FISTA iteration); a no-op unless a profiler
// (Nsight Systems / Compute) is attached
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// ------------------------------------------------------------------ sizes
constexpr int kMaxChunks = 16;       // samples per lane: nS <= 32 * kMaxChunks
constexpr int kMaxSamples = 32 * kMaxChunks;
constexpr int kBlock = 256;          // threads per block of the voxel kernels
constexpr int kRedSlots = 16;        // doubles reduced per block in the FISTA partial sums

// ------------------------------------------------------------------ device view of a handle
// a + sum of terms[perm[k]] for k in [beg, end), added in k order (the fibre passes' column
// sums); eight gathers in flight per step
template <class T>
__device__ __forceinline__ double fibre_gather_sum(const uint32_t *__restrict__ perm, const T *__restrict__ terms,
                                                   uint32_t beg, uint32_t end, double a) {
    uint32_t k = beg;
    for (; k + 8 <= end; k += 8) {
        uint32_t i[8];
        T t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) i[u] = __ldg(perm + k + u);
#pragma unroll
        for (int u = 0; u < 8; ++u) t[u] = __ldg(terms + i[u]);
#pragma unroll
        for (int u = 0; u < 8; ++u) a += (double)t[u];
    }
    for (; k < end; ++k) a += (double)__ldg(terms + __ldg(perm + k));
    return a;
}

struct OpDev {
    int nS, ndirs, nF, nE, nV, nISOv, nIC, nEC, nISO;
    int v0;                         // first voxel of the launch (voxels v0 .. nV-1; 0 for a full pass)
    int64_t n;
    int64_t ec_base, iso_base;      // first EC / ISO column
    const float *lutIC, *lutEC, *lutISO;          // float32 LUTs
    const void *lutIC_r, *lutEC_r;                // reduced-precision LUT copies (bf16/fp16) or null
    const uint32_t *vox_ptr;        // [nV+1] IC segments of voxel v: [vox_ptr[v], vox_ptr[v+1])
    const uint32_t *seg_f;          // [n] voxel-ordered fibre index
    const uint16_t *seg_o;          // [n] voxel-ordered orientation
    const float *seg_l;             // [n] voxel-ordered length
    const __half *seg_l16;          // [n] FP16 lengths (reduced path) or null
    const uint32_t *eval;           // [nF*nIC]
    const uint32_t *fib_ptr;        // [nF+1] fibre f owns fib_perm[fib_ptr[f] .. fib_ptr[f+1])
    const uint32_t *fib_perm;       // [n] voxel-order positions grouped by fibre
    const uint32_t *fib_order;      // [nF] fibres by their first position (fibre-pass order)
    const uint32_t *ec_ptr;         // [nV+1]
    const uint32_t *ec_col;         // [nE] EC element (column) of each voxel-ordered entry
    const uint16_t *ec_o;           // [nE]
    const uint32_t *iso_ptr;        // [nV+1]
    const uint32_t *iso_col;        // [nISOv]
    // float-float range guard (operator_kernels.cuh ff_exp_hi): magnitude bits of max|x| of
    // the forward input (null: not measured, no scaling) and the exponents of the largest
    // LUT value times the largest length (forward) and of the largest LUT value (adjoint)
    const unsigned long long *xmax;
    int lut_exp_fwd, lut_exp_adj;
};

// vectors of a multi-right-hand-side pass (batch.cuh)
constexpr int kMaxRhs = 16;
struct RhsPtrs {
    const double *x[kMaxRhs];       // column vectors (forward input / gradient point)
    float *y[kMaxRhs];              // row outputs (forward), may be null
    float *ax[kMaxRhs];             // A x outputs (momentum reuse), may be null
    const float *yin[kMaxRhs];      // adjoint inputs (in_mode 0)
    const float *axa[kMaxRhs];      // momentum reuse inputs (in_mode 2)
    const float *axb[kMaxRhs];
    float ca[kMaxRhs], cb[kMaxRhs];
    double *xout[kMaxRhs];          // adjoint outputs (EC / ISO columns; IC via scratch)
    float *scr[kMaxRhs];            // per-segment terms
    int active[kMaxRhs];            // 0: skip this vector (outputs untouched)
};

}  // namespace cgb

struct cgb_op {
    int device;
    int nS, ndirs, nF, nE, nV, nISOv, nIC, nEC, nISO, nolut;
    int64_t n, nrows, ncols;
    int arith;
    int ff_variant;                 // float-float kernels: 0 scalar samples, 1 packed pairs
    int lpv;                        // lanes per voxel (1..32)
    // device buffers (owned)
    float *lutIC, *lutEC, *lutISO;
    float *lutIC_p, *lutEC_p, *lutISO_p;  // zero-padded rows of stride nSp (paired kernels)
    int nSp;
    void *lutIC_r, *lutEC_r, *lutISO_r;  // reduced-precision LUT copies (padded pair layout)
    int lut_r_kind;                 // CGB_ARITH_BF16 / CGB_ARITH_FP16 / 0
    int nSp_r;                      // row stride of the BF16 / FP16 copies: room for the 16- and 32-lane shapes
    int ff_shape[2];                // float-float A / A' voxel shape: 0 not tuned, 1 default, 2 a warp per voxel
    int batch_lpv;                  // voxel shape of the multi-vector kernels: 0 not tuned, 1 default, 2 a warp per voxel
    __half *seg_l16;                // FP16 lengths scaled by 2^k (reduced path)
    float len16_inv_scale;          // 2^-k
    double *d_x64;                  // [ncols] staging for FP32 applies
    void *gstate;                   // LUT-gradient streams (lutgrad.cu), built on first use
    int batch_rhs;                  // vectors per multi-right-hand-side pass (0: not tuned)
    int batch_reuse;                // batched FISTA momentum reuse chosen by timing (0: not tuned, 1 off, 2 on)
    int occ_choice[24];             // occupancy build per tuned kernel (0: not tuned, 1 or 2), see occ_launch
    float occ_ms[24][2];            // the two builds' times measured by the tuning
    uint32_t *vox_ptr, *seg_f, *eval, *fib_ptr, *fib_perm, *fib_order, *ec_ptr, *ec_col, *iso_ptr, *iso_col;
    uint16_t *seg_o, *ec_o;
    float *seg_l;
    double *scratch;                // [nIC*n] per-segment adjoint terms (FP64 path)
    float *scratch32;               // [nIC*n] per-segment adjoint terms (FP32 path), on demand
    double *partials;               // block partial sums
    double *dscal;                  // device scalars
    unsigned long long *d_xmax;     // max |x| (magnitude bits) of the current forward input
    int xmax_on;                    // 1 while d_xmax holds the input of the launches being issued
    int lut_exp_fwd, lut_exp_adj;   // exponents of max|LUT| * max(length, 1) and of max|LUT|
    double *h_scal;                 // pinned host scalars
    double *d_in, *d_out;           // staging for cgb_op_apply_host
    int64_t d_in_len, d_out_len;
    cudaStream_t pipe_st[2];        // host-buffer pipeline: compute and copy streams (created on first use)
    int vr0, vr1;                   // voxel range [vr0, vr1) of the next voxel-kernel launches (vr1 0: all)
    int host_mode;                  // host-buffer products: 0 automatic, 1 staged copies, 2 direct row access
    // adjoint slabs: voxel ranges whose per-segment terms fit in L2, so the fibre pass of a
    // slab gathers them from L2 right after the voxel pass wrote them (see run_adjoint)
    int nslab;                      // 1: no slabs
    int *slab_v;                    // host [nslab+1] voxel boundaries
    uint32_t *fib_slab;             // device [(nslab+1) * nF]: where slab s starts in the position list of
                                    // the fibre at pass position fq (fib_order[fq])
    double *fib_acc;                // device [fib_acc_slots * nF * nIC]: running fibre sums between slabs,
    int fib_acc_slots;              // pass order, one accumulator per vector of a pass
    cudaStream_t slab_st[3];        // slab schedule streams (created on first use)
    cudaEvent_t slab_ev[68];
    cudaEvent_t pipe_ev[8];
    // tensor-core BF16 forward (tc_forward.cu), laid out on first use
    int tc_mode;                    // 0 automatic, 1 CUDA cores only, 2 tensor cores
    int tc_ready;                   // entries and LUT images built
    int tc_np, tc_nkb, tc_ntiles;   // padded samples, IC K-blocks of 64 LUT rows, tiles of 128 voxels
    float tc_lscale;                // 2^-k of the FP16 lengths
    uint32_t *tc_ptr, *tc_co;       // entry offsets per (tile, K-block, voxel); column | row << 26
    __half *tc_l;                   // entry lengths (FP16, scaled by 2^k)
    uint8_t *tc_vl;                 // entry voxel within its tile
    __nv_bfloat16 *tc_bimg;         // LUT K-block images (swizzled BF16)
    float *tc_xe;                   // x * eval as FP32, per forward
    int *tc_err;                    // device status word of the bounded waits
    int tc_kbs, tc_rounds;          // adjoint: sample K-blocks of 64, rounds of 256 LUT rows
    int64_t tc_nent;                // entries
    uint32_t *tc_fptr, *tc_fperm;   // adjoint: CSR offsets per IC column; entry positions grouped by column
                                    // (layout only)
    uint32_t *tc_fpos;              // adjoint: column-sorted position of every IC entry (where its term goes)
    uint32_t *tc_ford;              // adjoint: IC columns by their first entry position (fibre-pass order)
    __nv_bfloat16 *tc_abimg;        // adjoint LUT images
    float *tc_terms;                // adjoint IC terms in entry order
    float *tc_ax;                   // A x rows for the gradient (FISTA), on demand
    __nv_bfloat16 *tc_rows16;       // EC rows (nEC * ndirs) then ISO rows (nISO) as BF16, stride tc_np
    size_t bytes;
    int nsm;
    cgb::OpDev dev() const;
    // reduced-precision LUT rows (padded pair layout) for CGB_ARITH_BF16 / FP16 / F32
    const void *lut_r_ic(int kind) const { return kind == CGB_ARITH_F32 ? (const void *)lutIC_p : lutIC_r; }
    const void *lut_r_ec(int kind) const { return kind == CGB_ARITH_F32 ? (const void *)lutEC_p : lutEC_r; }
    const void *lut_r_iso(int kind) const { return kind == CGB_ARITH_F32 ? (const void *)lutISO_p : lutISO_r; }
};

namespace cgb {
// operator launches (operator.cu); `grid` returns the number of blocks that wrote partials
int launch_forward(cgb_op *op, const double *x, double *y, cudaStream_t st, int arith);
int launch_adjoint(cgb_op *op, const double *y, double *x, cudaStream_t st, int arith);
// |sqw*(A x - y)|^2 partial sums (y, sqw may be null); ax_out (optional) receives A x
int launch_resnorm_grid(cgb_op *op, const double *x, const double *y, const double *sqw, double *partials,
                        double *ax_out, cudaStream_t st, int arith, int *grid);
// grad = A'(sqw * r), r = sqw*(A x - y), |r|^2 partial sums; with ax_a non-null, A x is
// taken as ca*ax_a + cb*ax_b instead of being recomputed
int launch_gradient_grid(cgb_op *op, const double *x, const double *y, const double *sqw, double *grad,
                         double *partials, const double *ax_a, const double *ax_b, double ca, double cb,
                         cudaStream_t st, int arith, int *grid);
int reduction_blocks(const cgb_op *op);
void free_grad_state(cgb_op *op);
// reduced-precision path (mixed.cu): FP32 rows, FP64 columns
int ensure_reduced(cgb_op *op, int arith);
int launch_resnorm_mix(cgb_op *op, const double *x, const float *y, const float *sqw, double *partials,
                       float *ax_out, float *yout, cudaStream_t st, int arith, int *grid);
int launch_gradient_mix(cgb_op *op, const double *x, const float *y, const float *sqw, double *grad,
                        double *partials, const float *ax_a, const float *ax_b, float ca, float cb,
                        cudaStream_t st, int arith, int *grid);
int launch_adjoint_mix(cgb_op *op, const float *yin, double *xout, cudaStream_t st, int arith);
int convert_f64_to_f32(const double *in, float *out, int64_t n, cudaStream_t st);
// multi-right-hand-side BF16 path (batch_r*.cu, mixed.cu)
int launch_forward_R(cgb_op *op, int R, const RhsPtrs &V, const float *yobs, const float *sqw, double *partials,
                     cudaStream_t st, int *grid);
int launch_adjoint_R(cgb_op *op, int R, const RhsPtrs &V, int in_mode, const float *yobs, const float *sqw,
                     double *partials, cudaStream_t st, int *grid);
int fibre_sum32_from(cgb_op *op, const float *scr, double *xout, cudaStream_t st);
// tensor-core BF16 forward (tc_forward.cu)
bool tc_forward_enabled(const cgb_op *op);
bool tc_supported(const cgb_op *op);
int ensure_tc(cgb_op *op);
// tensor-core BF16 A' (tc_adjoint.cu): mode 0 z = yin; 2 z = sqw*r, r = sqw*(ca*axa + cb*axb - yobs)
int adjoint_tc(cgb_op *op, int mode, const float *yin, const float *axa, const float *axb, float ca, float cb,
               const float *yobs, const float *sqw, double *xout, double *partials, cudaStream_t st, int *grid);
int forward_tc(cgb_op *op, const double *x, float *y, float *ax, const float *yobs, const float *sqw,
               double *partials, cudaStream_t st, int *grid);
// float-float packed kernels over the voxel range [v0, v1) (host-buffer pipeline); A' pass 1
// only (the fibre pass follows once all ranges are done)
int fibre_sum(cgb_op *op, double *xout, cudaStream_t st);
// fibre pass of one adjoint slab (sums continue across slabs in fibre order; the last slab
// applies eval), FP64 / FP32 terms
// fibre pass of slab s; the running sums between slabs live in accumulator `slot` of
// op->fib_acc (one per vector of a multi-vector pass: ensure_fib_acc)
int fibre_sum_slab(cgb_op *op, double *xout, int s, cudaStream_t st);
int fibre_sum32_slab(cgb_op *op, const float *scr, double *xout, int s, cudaStream_t st, int slot = 0);
int ensure_fib_acc(cgb_op *op, int slots);
// blocks of partial sums an adjoint may write (one grid per slab)
int partial_blocks(const cgb_op *op);

// Slab schedule of an adjoint: the voxel passes of consecutive slabs alternate between two
// streams (they touch disjoint voxels, rows and terms, so they overlap and hide each
// other's tail), the fibre passes run in slab order on a third stream, each after its
// slab's voxel pass.  The three streams fork from `st` and join back into it.  Inside a
// stream capture the same steps run in order on `st`.  pass1(s, stream) / pass2(s, stream)
// return a status.
template <class P1, class P2>
int slab_schedule(cgb_op *op, cudaStream_t st, P1 &&pass1, P2 &&pass2) {
    const int S = op->nslab;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CGB_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone || S + 4 > 68) {
        for (int s = 0; s < S; ++s) {
            CGB_TRY(pass1(s, st));
            CGB_TRY(pass2(s, st));
        }
        return CGB_OK;
    }
    if (!op->slab_st[0]) {
        for (auto &q : op->slab_st) CGB_CUDA(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
        for (auto &e : op->slab_ev) CGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    cudaEvent_t fork = op->slab_ev[64], *join = op->slab_ev + 65;
    CGB_CUDA(cudaEventRecord(fork, st));
    for (auto &q : op->slab_st) CGB_CUDA(cudaStreamWaitEvent(q, fork, 0));
    int rc = CGB_OK;
    for (int s = 0; s < S && rc == CGB_OK; ++s) {
        cudaStream_t a = op->slab_st[s & 1];
        rc = pass1(s, a);
        if (rc != CGB_OK) break;
        CGB_CUDA(cudaEventRecord(op->slab_ev[s], a));
        CGB_CUDA(cudaStreamWaitEvent(op->slab_st[2], op->slab_ev[s], 0));
        rc = pass2(s, op->slab_st[2]);
    }
    for (int i = 0; i < 3; ++i) {
        cudaEventRecord(join[i], op->slab_st[i]);
        cudaStreamWaitEvent(st, join[i], 0);
    }
    return rc;
}

// restricts the voxel kernels launched while it lives to voxels [v0, v1)
struct VoxelRange {
    cgb_op *op;
    VoxelRange(cgb_op *o, int v0, int v1) : op(o) {
        op->vr0 = v0;
        op->vr1 = v1;
    }
    ~VoxelRange() {
        op->vr0 = 0;
        op->vr1 = 0;
    }
};
int convert_f32_to_f64(const float *in, double *out, int64_t n, cudaStream_t st);

// Float-float range guard of the forward input: enqueues max|x| into op->d_xmax; while an
// XScale lives, the FP64-path voxel kernels scale x by the exact power of two that keeps
// their FP32 words in range (no scaling, bitwise unchanged results, for ordinary ranges).
int measure_input(cgb_op *op, const double *x, int64_t n, cudaStream_t st);
struct XScale {
    cgb_op *op;
    explicit XScale(cgb_op *o, bool on = true) : op(o) { op->xmax_on = on ? 1 : 0; }
    ~XScale() { op->xmax_on = 0; }
};
// exponents of the LUT bounds used by the range guard, from the device LUTs and lengths
int update_lut_exponents(cgb_op *op);

// ------------------------------------------------------------------ occupancy autotuning
// A tuned kernel has two builds with different __launch_bounds__ min-blocks (register caps:
// fewer registers give more resident warps at the price of a few spills; the pairs were
// picked from measurements: float-float A 3 / 4, float-float A' 2 / 3 (1 / 2 for the build
// with the fused forward), reduced A 5 / 6, reduced A' 4 / 5 (3 / 4 fused), two-vector A'
// 2 / 3 (1 / 3 fused), four-vector A' 1 / 2).  On the first call for a handle, outside stream capture, both builds run twice
// on the call's own arguments (every output is overwritten by the real launch that
// follows) and the faster build of the second round is kept on the handle.  Both builds
// do the same arithmetic in the same order, so results do not depend on the choice.
enum OccSlot {
    kOccFwdFF = 0,
    kOccAdjFF = 1,
    kOccAdjMix = 2,  // + arith - BF16
    kOccAdjR2 = 5,
    kOccFwdMix = 6,  // + arith - BF16
    kOccAdjFFFused = 9,
    kOccAdjMixFused = 10,  // + arith - BF16
    kOccAdjR2Fused = 13,
    kOccAdjR4 = 14,
    kOccFwdFFWide = 16,
    kOccAdjFFWide = 17,
    kOccAdjFFWideFused = 18,
    kOccSlots = 24
};

template <class FA, class FB>
int occ_launch(cgb_op *op, int slot, cudaStream_t st, FA &&a, FB &&b) {
    int &c = op->occ_choice[slot];
    if (c == 0) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CGB_CUDA(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone) return a();
        cudaEvent_t e[3];
        for (auto &ev : e) CGB_CUDA(cudaEventCreate(&ev));
        float ta = 0.f, tb = 0.f;
        int rc = CGB_OK;
        for (int rep = 0; rep < 2 && rc == CGB_OK; ++rep) {
            cudaEventRecord(e[0], st);
            rc = a();
            cudaEventRecord(e[1], st);
            if (rc == CGB_OK) rc = b();
            cudaEventRecord(e[2], st);
            cudaEventSynchronize(e[2]);
            cudaEventElapsedTime(&ta, e[0], e[1]);
            cudaEventElapsedTime(&tb, e[1], e[2]);
        }
        for (auto &ev : e) cudaEventDestroy(ev);
        CGB_TRY(rc);
        op->occ_ms[slot][0] = ta;
        op->occ_ms[slot][1] = tb;
        c = tb < ta ? 2 : 1;
    }
    return c == 2 ? b() : a();
}

}  // namespace cgb
