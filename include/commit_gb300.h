/*
 * commit_gb300 -- C ABI of the GB300 (sm_103a) implementation of COMMIT's implicit
 * dictionary operator A / A' and of its FISTA solver.
 *
 * Every entry point returns a status code (CGB_OK on success); the message of the last
 * failure on the calling thread is available from cgb_last_error().  Handles are
 * independent: calls on different handles may run concurrently from different host
 * threads.  A handle owns the device copy of the dictionary (re-laid-out once at
 * creation) and its work buffers; callers own the vectors they pass in and out.
 *
 * Reference interfaces replaced (file:line within the reference project):
 *   LinearOperator.__init__     commit/operator/operator.pyx:40-94     -> cgb_op_create
 *   LinearOperator.dot (A, A')  commit/operator/operator.pyx:114-184   -> cgb_op_apply_host / cgb_op_apply
 *   COMMIT_A / COMMIT_At        setup_operator.py:245-365, 591-710     -> cgb_op_apply(adjoint = 0 / 1)
 *   COMMIT_A_nolut / _At_nolut  setup_operator.py:776-811, 877-915     -> same, on a handle created with nolut = 1
 *   Evaluation.set_threads      commit/core.pyx:586-724                -> (no counterpart: the device re-layout in
 *                                                                         cgb_op_create replaces the CPU partitions)
 *   solvers.fista / solve       commit/solvers.py:218-391              -> cgb_fista_run
 *   proximals.pyx               commit/proximals.pyx:13-186            -> cgb_prox_* / cgb_omega_*
 */
#ifndef COMMIT_GB300_H
#define COMMIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define CGB_OK 0
#define CGB_ERR_INVALID 1     /* bad argument or dictionary content (index out of range, ...)   */
#define CGB_ERR_CUDA 2        /* a CUDA runtime call failed                                        */
#define CGB_ERR_NOMEM 3       /* device allocation failed                                          */
#define CGB_ERR_UNSUPPORTED 4 /* shape outside what the kernels handle (e.g. nS > 1024)            */
#define CGB_ERR_DIMENSION 5   /* vector length does not match the operator ("dimensions do not match") */
#define CGB_ERR_BACKTRACK 6   /* FISTA: one iteration's backtracking reached its cap (max_backtracks) */

/* arithmetic of the FP64 operator path */
#define CGB_ARITH_F64 0 /* native FP64 FMA, the reference's own arithmetic                             */
#define CGB_ARITH_FF 1  /* float-float (two FP32 words, ~48-bit significand) products and sums, FP64    */
                        /* inputs/outputs; error well below 1e-10 relative at a fraction of FP64 cost  */
/* reduced-precision operator path (FP32 vectors, FP32 accumulation) */
#define CGB_ARITH_BF16 2 /* LUT in bfloat16, segment lengths in FP16                                   */
#define CGB_ARITH_FP16 3 /* LUT in FP16, segment lengths in FP16                                       */
#define CGB_ARITH_F32 4  /* LUT and lengths in FP32, FP32 accumulation                                  */

/* vector element types for cgb_op_apply */
#define CGB_DTYPE_F64 0
#define CGB_DTYPE_F32 1

typedef struct cgb_op cgb_op; /* opaque operator handle */

/* Human-readable message of the last failing call on this thread ("" if none). */
const char *cgb_last_error(void);

/* Library version string. */
const char *cgb_version(void);

/*
 * Create an operator on device `device` from the dictionary and LUT arrays (host or device
 * pointers, layout of LinearOperator.__init__, operator.pyx:40-94):
 *   IC: ICf[n] fibre (column) index, ICv[n] voxel, ICo[n] orientation, ICl[n] length,
 *       ICeval[nF*nIC] per-column 0/1 mask;
 *   EC: ECv[nE], ECo[nE];  ISO: ISOv[nISOv];
 *   LUTs: lutIC[nIC*ndirs*nS], lutEC[nEC*ndirs*nS], lutISO[nISO*nS] (float32, C order).
 * nV is the number of voxels (rows = nV*nS).  Columns: nF*nIC + nE*nEC + nISOv*nISO.
 * The arrays need not be sorted; they are copied, validated and re-laid-out on the
 * device (voxel-ordered stream for A, fibre-ordered index for A').  With nolut = 1 the
 * operator is the LUT-free scalar operator of setup_operator.py:713-915 (nS must be 1,
 * IC uses one response, ISO at most one).  `arith` selects the default arithmetic
 * (CGB_ARITH_F64 or CGB_ARITH_FF); reduced-precision copies are made on demand.
 */
int cgb_op_create(int device, int nS, int ndirs, int nF, int64_t n, int nE, int nV, int nISOv,
                  const uint32_t *ICf, const uint32_t *ICeval, const uint32_t *ICv, const uint16_t *ICo,
                  const float *ICl, const uint32_t *ECv, const uint16_t *ECo, const uint32_t *ISOv,
                  const float *lutIC, const float *lutEC, const float *lutISO, int nIC, int nEC, int nISO,
                  int nolut, int arith, cgb_op **out);

/*
 * Evaluation.load_dictionary's re-layout (commit/core.pyx:493-580) on DEVICE arrays, in
 * place: the raw arrays of the dictionary_*.dict files (voxel ids as linear grid indices
 * x + X*(y + Y*z), IC lengths in mm) are sorted by voxel (stable, as numpy's argsort), IC
 * lengths are divided by trk_norm[ICf] (FP32) when `normalize` is set, and voxel ids become
 * indices among the mask voxels in the same linear order (mask: ngrid bytes in that order;
 * ids outside the mask map to 0, as the reference's zero-filled table does).  *nV_out
 * receives the number of mask voxels.  ICo / ECo may be NULL.  Synchronises `stream`.
 * The results can be passed to cgb_op_create directly (it accepts device pointers).
 */
int cgb_dict_relayout(const uint8_t *mask, int64_t ngrid, int64_t n, int nF, uint32_t *ICf, uint32_t *ICv,
                      uint16_t *ICo, float *ICl, const float *trk_norm, int normalize, int64_t nE, uint32_t *ECv,
                      uint16_t *ECo, int64_t nISOv, uint32_t *ISOv, int64_t *nV_out, void *stream);

/* Release the handle and every device buffer it owns. */
int cgb_op_destroy(cgb_op *op);

/* nROWS and nCOLS of A (operator.pyx:69-70). */
int cgb_op_shape(const cgb_op *op, int64_t *nrows, int64_t *ncols);

/* Device bytes held by the handle. */
int cgb_op_device_bytes(const cgb_op *op, size_t *bytes);

/*
 * Replace the LUT values (same shapes as at creation; host or device pointers, NULL leaves
 * that compartment unchanged).  Used when the LUT itself is being fitted.  No counterpart
 * in the reference, whose LUTs are fixed after load_kernels (commit/core.pyx:364-433).
 */
int cgb_op_set_lut(cgb_op *op, const float *lutIC, const float *lutEC, const float *lutISO);

/*
 * Gradient of a loss with respect to the LUTs given dLoss/dy = g (DEVICE, nrows doubles)
 * at the point x (DEVICE, ncols doubles): g_ic[nIC*ndirs*nS], g_ec[nEC*ndirs*nS],
 * g_iso[nISO*nS] (DEVICE doubles; NULL skips that compartment).  Deterministic: items are
 * reduced per orientation in a fixed order.  No counterpart in the reference.
 */
int cgb_op_lut_grad(cgb_op *op, const double *x, const double *g, double *g_ic, double *g_ec, double *g_iso,
                    void *stream);

/*
 * Voxel shape of the float-float pair kernels: 1 the default (fewest padded samples), 2 a
 * warp per voxel, 0 = timed on the next call (the default at creation); set < 0 only reads.
 * *fwd / *adj (may be NULL) receive the shapes of A and A'.  Results agree to ~1e-16.
 */
int cgb_op_ff_shape(cgb_op *op, int set, int *fwd, int *adj);

/*
 * Float-float kernel family: 1 (default) packed f32x2 pairs of samples on padded LUT rows,
 * 0 one sample per lane; a negative value only reads.  Same arithmetic to ~1e-15.
 */
int cgb_op_ff_kernels(cgb_op *op, int variant, int *out);

/*
 * Adjoint slabs: A' runs its voxel pass and fibre pass slab by slab (voxel ranges whose
 * per-segment terms fit in L2, so the fibre pass gathers them from L2).  nslab 0 chooses
 * the count from the problem size (the default at creation), 1 turns slabs off, 2..64
 * fixes it, a negative value only reads; *out (may be NULL) receives the count in use.  The sums are the same in every
 * case (each fibre's terms are added in the same order).
 */
int cgb_op_set_slabs(cgb_op *op, int nslab, int *out);

/*
 * Host-buffer products (cgb_op_apply_host): mode 0 (default) reads / writes a page-locked
 * row vector in place through its device mapping and copies only the column vector, else
 * stages both through device buffers with the copies pipelined against the kernels; 1
 * always stages; 2 is the same as 0.  A negative mode only reads; *out (may be NULL)
 * receives the mode.  Results are identical in every mode.
 */
int cgb_op_host_mode(cgb_op *op, int mode, int *out);

/* Select the arithmetic used by later FP64 applies (CGB_ARITH_F64 / CGB_ARITH_FF). */
int cgb_op_set_arith(cgb_op *op, int arith);

/*
 * out = A*in (adjoint = 0) or out = A'*in (adjoint = 1) on DEVICE vectors, enqueued on
 * `stream` (a cudaStream_t; NULL = legacy default stream).  `out` is fully written (no
 * pre-zeroing needed).  dtype CGB_DTYPE_F64 uses the handle's FP64 arithmetic;
 * CGB_DTYPE_F32 uses the reduced-precision path `arith` (CGB_ARITH_BF16/FP16/F32).
 * in_len/out_len are checked against the operator shape (CGB_ERR_DIMENSION).  FP64 inputs
 * may have any finite magnitude: the float-float kernels scale operands whose products
 * with the LUT would leave FP32's exponent range by an exact power of two (the forward
 * input as a whole, the adjoint input per voxel row) and scale the results back in FP64.
 */
int cgb_op_apply(cgb_op *op, int adjoint, const void *in, int64_t in_len, void *out, int64_t out_len, int dtype,
                 int arith, void *stream);

/*
 * The LinearOperator.dot contract on HOST float64 buffers: copies `in` to the device,
 * applies A or A', copies the result to `out` and synchronises.  Replaces COMMIT_A /
 * COMMIT_At called from operator.pyx:136-182.
 */
int cgb_op_apply_host(cgb_op *op, int adjoint, const double *in, int64_t in_len, double *out, int64_t out_len);

/*
 * A'*y that allocates no device memory.  No counterpart in the reference.
 *
 * For callers that cannot let a library call cudaMalloc: an application that reserves
 * the GPU's memory up front in its own pool (a plug-in's cudaMalloc would fail or
 * fragment that pool), or one that issues work on a latency-critical stream and cannot
 * accept cudaMalloc's implicit device-wide synchronisation.  Every input and output is a
 * DEVICE buffer owned by the caller, in the reference's layout: IC segments, EC and ISO
 * elements sorted by voxel (as load_dictionary leaves them, commit/core.pyx:508-562),
 * the eval mask and the f32 LUTs, plus a fibre index computed once by the caller:
 * fib_perm[n] lists segment indices grouped by fibre and fib_ptr[nF+1] gives each
 * fibre's range (a stable argsort of ICf and its counts).  ICf itself is not read (the
 * fibre index replaces it) and may be NULL.  x (nF*nIC + nE*nEC + nISOv*nISO doubles) is
 * fully written.  Float-float arithmetic with the range guard of cgb_op_apply.
 *
 * Working memory is a static device array of CGB_NOALLOC_MAX_TERMS doubles (8 MiB) in
 * this library's module; calls with n*nIC > CGB_NOALLOC_MAX_TERMS return
 * CGB_ERR_UNSUPPORTED.  Under CUDA's lazy module loading (the default since CUDA 12.2) a
 * module's static memory is allocated, and its kernels' code loaded, on first use, so
 * the FIRST call on each device does that set-up, with the device current: it looks up
 * the array's address (cudaGetSymbolAddress) and loads every kernel this entry point
 * uses.  That first call may therefore allocate and synchronise: make it before
 * reserving the device's memory and before any stream capture (or run with
 * CUDA_MODULE_LOADING=EAGER).  A call with nS = 1, ndirs = 1, every other size 0 and any
 * non-null y does only this set-up.  Later calls allocate and load nothing; the array
 * then stays allocated on that device until the process exits.  The address is cached
 * per device: after cudaDeviceReset on a device, do not call this entry point there.
 * All calls share the array: calls whose work overlaps on the GPU (different streams, or
 * different host threads) race and must be serialised by the caller.  Enqueued on
 * `stream`; returns without synchronising.
 */
#define CGB_NOALLOC_MAX_TERMS (1 << 20)
int cgb_op_adjoint_noalloc(int nS, int ndirs, int nF, int64_t n, int nE, int nV, int nISOv, const double *y,
                           double *x, const uint32_t *ICf, const uint32_t *ICeval, const uint32_t *ICv,
                           const uint16_t *ICo, const float *ICl, const uint32_t *ECv, const uint16_t *ECo,
                           const uint32_t *ISOv, const float *lutIC, const float *lutEC, const float *lutISO,
                           int nIC, int nEC, int nISO, const uint32_t *fib_ptr, const uint32_t *fib_perm,
                           void *stream);

/*
 * Reduced-precision A*x and A'*y with a BF16 LUT on the tensor cores (tcgen05): per tile
 * of 128 voxels the IC part is a dense product of the voxel-by-LUT-row coefficients (A) or
 * of the input rows (A') with the BF16 LUT, FP32 accumulation in tensor memory; the EC and
 * ISO items run on the CUDA cores in the same kernels.  mode 0 (the default) uses it when
 * the shape allows it (an IC compartment, nS <= 320, fewer than 2^26 columns) and the IC
 * segments are dense enough for the dense product to pay, at least 32 per voxel on
 * average (measured on GB300: 1.5x faster than the CUDA-core kernels at 62 per voxel,
 * 1.9x at 212, slower at 21); 1 keeps the CUDA-core kernels; 2 requires it
 * (CGB_ERR_UNSUPPORTED when the shape does not allow it); a negative mode only reads.
 * *out (may be NULL) receives 1 when the tensor-core kernels are in use.  The first use on
 * a handle builds its tile-ordered entry stream and LUT images (about 6 bytes per
 * segment).  No counterpart in the reference (setup_operator.py:50-218 and 591-710 are its
 * CPU A and A').
 */
int cgb_op_tensor_cores(cgb_op *op, int mode, int *out);

/*
 * Synchronises the handle's device and reports whether a tensor-core kernel gave up a
 * bounded wait since the last check (CGB_ERR_CUDA; the kernel then returned early and its
 * output is incomplete).  No counterpart in the reference.
 */
int cgb_op_device_status(cgb_op *op);

/* ------------------------------------------------------------------ regularisation */
#define CGB_REG_NONE 0
#define CGB_REG_LASSO 1
#define CGB_REG_GROUP_LASSO 2
#define CGB_REG_SPARSE_GROUP_LASSO 3

/*
 * Regulariser of commit/solvers.py:16-206, per compartment.  Ranges are column ranges of
 * x.  All pointers are DEVICE pointers (may be NULL when unused).
 */
typedef struct {
    int64_t start_ic, size_ic, start_ec, size_ec, start_iso, size_iso;
    int reg_ic, reg_ec, reg_iso; /* CGB_REG_* (EC/ISO: NONE or LASSO)                      */
    int nn_ic, nn_ec, nn_iso;    /* non-negativity per compartment                        */
    double lambda_ic, lambda_ic_group; /* lasso / l1 part and group part (sparse group lasso) */
    double lambda_ec, lambda_iso;
    const double *coeff_weights; /* all_coeff_weights[ncols] (solvers.py:38-46) or NULL   */
    int weighted_ic, weighted_iso; /* use coeff_weights in the IC / ISO l1 terms            */
    /* groups (IC): concatenated indices, CSR offsets [ngroups+1], weights [ngroups] */
    const int32_t *group_idx;
    const int64_t *group_ptr;
    const double *group_w;
    int64_t ngroups;
    /* level schedule: groups [level_ptr[k], level_ptr[k+1]) are pairwise disjoint and are
       processed together; levels run in order (reproduces the sequential loop of
       proximals.pyx:103-134 for overlapping, hierarchical groups).  HOST pointer. */
    const int64_t *level_ptr;
    int64_t nlevels;
} cgb_reg;

typedef struct {
    double tol_fun, tol_x;
    int max_iter;
    int verbose;          /* 0: quiet                                                    */
    int arith;            /* CGB_ARITH_F64 / CGB_ARITH_FF                                 */
    int momentum_reuse;   /* 1: A*xhat from A*x and A*prev_x (exact in exact arithmetic);   */
                          /* 2 (cgb_fista_batch_run only): on or off as timed on first use */
    /* optional convergence trace: with x_ref (DEVICE, ncols) and trace (HOST, 2*trace_len
       doubles) set, accepted iteration k (k < trace_len) records trace[2k] = seconds since
       the call started and trace[2k+1] = |x_k - x_ref| / |x_ref| */
    const double *x_ref;
    double *trace;
    int trace_len;
    int graph;            /* 1: the iteration loop runs as one CUDA graph launch with device-side */
                          /* decisions (conditional nodes); no trace, verbose output or restart */
    int max_backtracks;   /* step reductions allowed per iteration (0: 1000, negative: none);    */
                          /* one more ends the solve with CGB_ERR_BACKTRACK (the reference's    */
                          /* loop has no cap, commit/solvers.py:322-333)                        */
    int restart;          /* 1: reset the momentum (t = 1) after an iteration whose objective     */
                          /* rose (function-value restart, O'Donoghue & Candes 2015); 0 is the   */
                          /* reference's FISTA.  Host-driven loop only.                          */
    int trace_cost;       /* 1: the trace holds 3 doubles per iteration (3*trace_len), the third  */
                          /* the cost function of accepted iteration k                           */
} cgb_fista_params;

typedef struct {
    double residual, regterm, cost_function, abs_cost, rel_cost, abs_x, rel_x;
    int iterations;
    int stopping_criterion; /* 0 abs obj, 1 rel obj, 2 abs x, 3 rel x, 4 max iter          */
    int backtracks;
    int operator_calls;     /* number of A and A' products                                  */
    int anchors;            /* with momentum reuse: iterations whose qfval was evaluated    */
                            /* again directly after the test failed (f(x_hat) from the      */
                            /* stored rows rounds differently from the evaluation of x)     */
} cgb_fista_result;

/*
 * FISTA with backtracking (solvers.py:244-391) on device vectors: y[nrows], optional
 * sqrt_w[nrows] (square root of the confidence map, or NULL), x[ncols] holds x0 on
 * entry and the solution on return.  Enqueued on `stream`; returns after the solve.
 */
int cgb_fista_run(cgb_op *op, const double *y, const double *sqrt_w, const cgb_reg *reg,
                  const cgb_fista_params *params, double *x, cgb_fista_result *result, void *stream);

/*
 * Batched FISTA: nprob problems that share the operator, y and sqrt_w and differ in their
 * regulariser regs[p] (a regularisation path over lambda).  Each problem follows the same
 * iteration as cgb_fista_run (own step size, momentum, backtracking, stopping test) with the
 * operator in BF16-LUT arithmetic (params->arith must be CGB_ARITH_BF16); the A / A' passes of
 * all problems that need one at the same point run as multi-right-hand-side passes that load
 * each LUT row once for 2 or 4 vectors.  The vectors per pass are chosen on first use by
 * timing both widths on the operator (kept on the handle).  x[p] (device pointers) hold x0 on
 * entry and the solutions on return; results[p] per problem (operator_calls: the batch total
 * in results[0], 0 elsewhere).  The reference has no batched solver: commit/solvers.py:218-243
 * solves one problem per call.
 */
int cgb_fista_batch_run(cgb_op *op, const double *y, const double *sqrt_w, const cgb_reg *regs, int nprob,
                        const cgb_fista_params *params, double *const *x, cgb_fista_result *results, void *stream);

/*
 * A or A' of nvec vectors in one multi-right-hand-side pass per 2 or 4 vectors (BF16 LUT,
 * FP32 accumulation): forward in[r] = double x[ncols] -> out[r] = float y[nrows]; adjoint
 * in[r] = float y[nrows] -> out[r] = double x[ncols].  Device pointers, enqueued on `stream`
 * (the adjoint's per-segment scratch is allocated and freed stream-ordered on `stream`).
 * No reference counterpart: commit/operator/operator.pyx:118-184 applies one vector per call.
 */
int cgb_op_apply_batch(cgb_op *op, int adjoint, int nvec, const void *const *in, void *const *out, void *stream);

/*
 * Occupancy autotuning of the voxel kernels.  Slots: 0 float-float A, 1 float-float A' pass
 * 1, 2 / 3 / 4 reduced-precision A' pass 1 (BF16 / FP16 / F32), 5 two-vector BF16 A',
 * 6 / 7 / 8 reduced-precision A (BF16 / FP16 / F32), 9 float-float fused A x + A' pass 1,
 * 10 / 11 / 12 reduced-precision fused A x + A' pass 1, 13 two-vector fused, 14 four-vector A',
 * 16 / 17 / 18 float-float A / A' / fused A' in the warp-per-voxel shape.
 * Each tuned kernel has two builds with different register caps (2: the tighter cap, more
 * resident warps); the first call on a handle times both on its own arguments and keeps the
 * faster.
 * set >= 0 stores a choice (0 = tune again on the next call, 1 or 2 = fixed), set < 0 only
 * reads; choice / ms_a / ms_b (may be NULL) receive the choice and the two measured times.
 * Both builds compute the same operations in the same order: results are identical.
 */
int cgb_op_occupancy(cgb_op *op, int slot, int set, int *choice, float *ms_a, float *ms_b);

/* Vectors per multi-right-hand-side pass: set >= 0 stores it (0 = time both widths on the next
 * batched solve of >= 4 problems, 2 or 4 = fixed), set < 0 only reads; *width (may be NULL)
 * receives the current value (0 while untuned). */
int cgb_op_batch_width(cgb_op *op, int set, int *width);

/* Voxel shape of the multi-right-hand-side kernels: 1 the single-vector kernels' lanes per
 * voxel, 2 a warp per voxel (half the samples per lane, fewer registers per vector), 0 =
 * chosen by timing on the next batched solve; set < 0 only reads. */
int cgb_op_batch_shape(cgb_op *op, int set, int *shape);

/* ------------------------------------------------------------------ voxelwise maps */
/*
 * The maps of Evaluation.save_results (commit/core.pyx:1614-1750) for a fitted x (device
 * f64[ncols]); every output is a device f64[nV] (mask voxel order) or NULL to skip it.
 *   ic / ec / iso: compartment maps (core.pyx:1717-1750).  IC sums len * (sum over the
 *     streamline's responses of x * norm_fib) over the voxel's segments; norm_fib is
 *     f64[nF*nIC] or NULL for ones.  EC / ISO sum the voxel's coefficients.
 *   rmse / nrmse (core.pyx:1662-1680) and rmse_conf / nrmse_conf (core.pyx:1682-1705, need
 *     conf f64[nrows]) compare y_mea (f64[nrows]) with A x, both rounded to FP32 as the
 *     reference does; sums are FP64.  A x is formed in a temporary device buffer.
 */
int cgb_op_voxel_maps(cgb_op *op, const double *x, const double *y_mea, const double *conf, const double *norm_fib,
                      double *ic, double *ec, double *iso, double *rmse, double *nrmse, double *rmse_conf,
                      double *nrmse_conf, void *stream);

/* ------------------------------------------------------------------ trk2dictionary */
/*
 * Streamline voxelisation (commit/trk2dictionary/trk2dictionary_c.cpp:111-440) on the device.
 * All arrays are DEVICE pointers.  Streamline f has the points pts[3*offsets[f] ..
 * 3*offsets[f+1]) (x, y, z in mm of the image grid, i.e. the .trk "voxmm" space).  The
 * grids (mask, iso_mask: u8, peaks: f32 [.. , n_peaks, 3], tdi: f64) are C-order arrays over
 * (x, y, z) as the reference reads them; mask / iso_mask / peaks / blur_apply may be NULL.
 * hash: the 181 x 181 table from (colatitude, longitude) in whole degrees to a direction
 * index.  Outputs are allocated on the device by the call and released by
 * cgb_trk2dict_free; they are the arrays of the dictionary_*.dict files (IC_f counts kept
 * streamlines, voxel ids x + X*(y + Y*z)).  Geometry in FP64 without fused multiply-adds
 * and FP32 per-key sums, as the reference.
 */
typedef struct {
    int dim[3];
    float pixdim[3];
    float fiber_shift[3];          /* in voxels, as the reference's fiber_shift */
    float min_seg_len, min_fiber_len, max_fiber_len;
    int do_intersect;
    int n_replicas;                /* blur replicas (1: none); rho / angle / weights on the device */
    const double *blur_rho, *blur_angle, *blur_weights;
    int n_peaks;                   /* EC: peaks per voxel, relative threshold, axis flips, affine */
    float vf_thr;
    int flip[3];
    double peaks_affine[9];
} cgb_t2d_params;

typedef struct {
    int64_t n_fibers, n_kept, n_segments, n_ec, n_iso;
    uint32_t *ic_f, *ic_v;
    uint16_t *ic_o;
    float *ic_len;
    float *trk_norm, *trk_len, *trk_lentot; /* per kept streamline */
    uint8_t *trk_kept;                      /* per input streamline */
    uint32_t *ec_v;
    uint16_t *ec_o;
    uint32_t *iso_v;
    double *tdi;                            /* track density (sum of segment lengths), C order */
} cgb_t2d_result;

int cgb_trk2dict(const cgb_t2d_params *prm, const float *pts, const int64_t *offsets, int64_t nfib,
                 const uint8_t *blur_apply, const int16_t *hash, const uint8_t *mask, const float *peaks,
                 const uint8_t *iso_mask, cgb_t2d_result *out, void *stream);
int cgb_trk2dict_free(cgb_t2d_result *res);

/* ------------------------------------------------------------------ proximal maps */
/* In-place proximal maps on a DEVICE float64 vector (proximals.pyx:13-77). */
int cgb_prox_non_negativity(double *x, int64_t start, int64_t size, void *stream);
int cgb_prox_soft_thresholding(double *x, double lam, int64_t start, int64_t size, void *stream);
int cgb_prox_w_soft_thresholding(double *x, const double *w, double lam, int64_t start, int64_t size,
                                 void *stream);
int cgb_prox_projection_onto_l2_ball(double *x, double lam, int64_t start, int64_t size, void *stream);
/* prox_group_lasso (proximals.pyx:103-134): groups as CSR (device), level schedule (host);
   nx = length of x (group indices outside [0, nx) are ignored). */
int cgb_prox_group_lasso(double *x, int64_t nx, const int32_t *group_idx, const int64_t *group_ptr, const double *group_w,
                         int64_t ngroups, const int64_t *level_ptr, int64_t nlevels, double lam, void *stream);
/* penalties (proximals.pyx:80-99, 138-186); result written to *out (host), synchronous. */
int cgb_omega_group_lasso(const double *x, int64_t nx, const int32_t *group_idx, const int64_t *group_ptr,
                          const double *group_w, int64_t ngroups, double lam, double *out, void *stream);
int cgb_omega_sparse_group_lasso(const double *x, int64_t nx, const double *w, const int32_t *group_idx,
                                 const int64_t *group_ptr, const double *group_w, int64_t ngroups, double lam1,
                                 double lam2, double *out, void *stream);
/* weighted / plain l1 over [start, start+size): lam * sum |w_i x_i| (w may be NULL). */
int cgb_omega_l1(const double *x, const double *w, int64_t start, int64_t size, double lam, double *out,
                 void *stream);

#ifdef __cplusplus
}
#endif
#endif /* COMMIT_GB300_H */
