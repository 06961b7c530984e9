// Operator handle: upload, validation and one-time device re-layout of the dictionary.
//
// The reference keeps the dictionary in the order load_dictionary leaves it (segments
// stable-sorted by voxel, commit/core.pyx:508-514) and splits the work over CPU threads
// with per-thread ranges (core.pyx:586-724).  Here the arrays are copied once to the
// device and re-laid-out there:
//   * IC segments are radix-sorted by (voxel, orientation) -> a voxel CSR stream
//     (vox_ptr, seg_f, seg_o, seg_l) read by the voxel kernels of A and A';
//   * a stable sort of the voxel-ordered positions by fibre gives fib_ptr/fib_perm, the
//     fibre-ordered index of the second A' pass (per-fibre sums, no atomics);
//   * EC and ISO elements get voxel CSR offsets plus their original column index.
#include <cub/cub.cuh>

#include <mutex>
#include <vector>

#include <algorithm>
#include <vector>

#include "cgb_internal.cuh"
#include "operator_pair.cuh"

namespace cgb {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? CGB_ERR_NOMEM : CGB_ERR_CUDA;
}

namespace {

__global__ void k_validate(const uint32_t *ICf, const uint32_t *ICv, const uint16_t *ICo, int64_t n,
                           const uint32_t *ECv, const uint16_t *ECo, int nE, const uint32_t *ISOv, int nISOv,
                           int nF, int nV, int ndirs, int check_o, unsigned int *flags) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned int bad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        if (ICf[i] >= (uint32_t)nF) bad |= 1u;
        if (ICv[i] >= (uint32_t)nV) bad |= 2u;
        if (check_o && ICo[i] >= (uint32_t)ndirs) bad |= 4u;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nE; i += stride) {
        if (ECv[i] >= (uint32_t)nV) bad |= 8u;
        if (check_o && ECo[i] >= (uint32_t)ndirs) bad |= 16u;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nISOv; i += stride)
        if (ISOv[i] >= (uint32_t)nV) bad |= 32u;
    if (bad) atomicOr(flags, bad);
}

__global__ void k_iota(uint32_t *a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (uint32_t)i;
}

__global__ void k_key_vo(const uint32_t *v, const uint16_t *o, int64_t n, uint32_t ndirs, uint64_t *key) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        key[i] = (uint64_t)v[i] * ndirs + (o ? o[i] : 0);
}

__global__ void k_hist(const uint32_t *key, int64_t n, uint32_t *count) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&count[key[i]], 1u);
}

__global__ void k_gather_ic(const uint32_t *perm, int64_t n, const uint32_t *f, const uint16_t *o, const float *l,
                            uint32_t *fo, uint16_t *oo, float *lo) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = perm[i];
        fo[i] = f[p];
        if (o) oo[i] = o[p];
        lo[i] = l[p];
    }
}

__global__ void k_gather_u16(const uint32_t *perm, int64_t n, const uint16_t *src, uint16_t *dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}

template <class T>
int dalloc(cgb_op *op, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    op->bytes += count * sizeof(T);
    return CGB_OK;
}

template <class T>
int upload(T *dst, const T *src, size_t count) {
    if (count == 0 || src == nullptr) return CGB_OK;
    CGB_CUDA(cudaMemcpy(dst, src, count * sizeof(T), cudaMemcpyDefault));  // host or device source
    return CGB_OK;
}

struct Temp {
    std::vector<void *> ptrs;
    ~Temp() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T>
    int alloc(T **p, size_t count) {
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (temporary)");
        ptrs.push_back(*p);
        return CGB_OK;
    }
};

int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g < 1) g = 1;
    if (g > 4096) g = 4096;
    return (int)g;
}

// CSR offsets [nkeys+1] of a key array (keys < nkeys) by histogram + exclusive scan.
int csr_offsets(const uint32_t *keys, int64_t n, int nkeys, uint32_t *ptr, Temp &tmp) {
    uint32_t *count;
    CGB_TRY(tmp.alloc(&count, (size_t)nkeys + 1));
    CGB_CUDA(cudaMemset(count, 0, ((size_t)nkeys + 1) * sizeof(uint32_t)));
    if (n > 0) k_hist<<<grid_for(n), 256>>>(keys, n, count);
    size_t bytes = 0;
    CGB_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, count, ptr, nkeys + 1));
    void *t;
    CGB_TRY(tmp.alloc((char **)&t, bytes));
    CGB_CUDA(cub::DeviceScan::ExclusiveSum(t, bytes, count, ptr, nkeys + 1));
    return CGB_OK;
}

// stable sort of (key, iota) pairs; returns the permutation in perm_out.
// first voxel-order position of each fibre's segments (n for a fibre without segments)
__global__ void k_fib_first(const uint32_t *__restrict__ fib_ptr, const uint32_t *__restrict__ fib_perm, int nF,
                            uint32_t n, uint32_t *__restrict__ key) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f < nF) key[f] = fib_ptr[f] < fib_ptr[f + 1] ? fib_perm[fib_ptr[f]] : n;
}

template <class K>
int sort_perm(const K *keys, int64_t n, int end_bit, uint32_t *perm_out, Temp &tmp) {
    if (n == 0) return CGB_OK;
    K *keys_out;
    uint32_t *vals_in;
    CGB_TRY(tmp.alloc(&keys_out, n));
    CGB_TRY(tmp.alloc(&vals_in, n));
    k_iota<<<grid_for(n), 256>>>(vals_in, n);
    size_t bytes = 0;
    CGB_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys, keys_out, vals_in, perm_out, (int)n, 0, end_bit));
    void *t;
    CGB_TRY(tmp.alloc((char **)&t, bytes));
    CGB_CUDA(cub::DeviceRadixSort::SortPairs(t, bytes, keys, keys_out, vals_in, perm_out, (int)n, 0, end_bit));
    return CGB_OK;
}

int bits_for(uint64_t maxval) {
    int b = 1;
    while (b < 64 && (maxval >> b) != 0) b++;
    return b;
}

}  // namespace

int reduction_blocks(const cgb_op *op) { return op->nsm * 8; }
int partial_blocks(const cgb_op *op) { return reduction_blocks(op) * (op->nslab > 1 ? op->nslab : 1); }

}  // namespace cgb

cgb::OpDev cgb_op::dev() const {
    cgb::OpDev d;
    d.nS = nS; d.ndirs = ndirs; d.nF = nF; d.nE = nE; d.nV = nV; d.nISOv = nISOv; d.v0 = 0;
    d.nIC = nIC; d.nEC = nEC; d.nISO = nISO; d.n = n;
    d.ec_base = (int64_t)nF * nIC;
    d.iso_base = d.ec_base + (int64_t)nE * nEC;
    d.lutIC = lutIC; d.lutEC = lutEC; d.lutISO = lutISO;
    d.lutIC_r = lutIC_r; d.lutEC_r = lutEC_r;
    d.vox_ptr = vox_ptr; d.seg_f = seg_f; d.seg_o = seg_o; d.seg_l = seg_l; d.seg_l16 = seg_l16;
    d.eval = eval; d.fib_ptr = fib_ptr; d.fib_perm = fib_perm; d.fib_order = fib_order;
    d.ec_ptr = ec_ptr; d.ec_col = ec_col; d.ec_o = ec_o;
    d.iso_ptr = iso_ptr; d.iso_col = iso_col;
    d.xmax = xmax_on ? d_xmax : nullptr;
    d.lut_exp_fwd = lut_exp_fwd; d.lut_exp_adj = lut_exp_adj;
    return d;
}

using namespace cgb;

// Adjoint slabs.  The voxel pass writes one term per segment in voxel order and the fibre
// pass gathers them in fibre order: a gather over the whole term stream (≈ 1 GB for 1M
// streamlines) misses L2 on almost every access (ncu: 15.6 GB of DRAM reads for a 1.5 GB
// pass).  Cutting the voxels into slabs of about kSlabTermBytes of FP64 terms and running
// the fibre pass of each slab right after its voxel pass (overlapped, see slab_schedule)
// keeps most gathers in L2.  fib_slab[s*nF + f] is the first entry of fibre f's
// (ascending) position list that lies in slab s, for the fibre f = fib_order[fq] at pass
// position fq (fib_slab[s*nF + fq]), so the passes read it, and their running sums in
// fib_acc, in order.
constexpr double kSlabTermBytes = 128.0 * (1 << 20);  // measured best band: 8-12 slabs at 1M streamlines

__global__ void k_fib_slabs(const uint32_t *__restrict__ fib_ptr, const uint32_t *__restrict__ fib_perm,
                            const uint32_t *__restrict__ fib_order, int nF, int S,
                            const uint32_t *__restrict__ slab_pos, uint32_t *__restrict__ fib_slab) {
    const int64_t fq = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (fq >= nF) return;
    const uint32_t f = fib_order[fq];
    uint32_t k = fib_ptr[f];
    const uint32_t end = fib_ptr[f + 1];
    for (int s = 0; s <= S; ++s) {
        while (k < end && fib_perm[k] < slab_pos[s]) ++k;
        fib_slab[(size_t)s * nF + fq] = k;
    }
}

static int build_slabs(cgb_op *op, int want = 0) {
    op->nslab = 1;
    delete[] op->slab_v;
    op->slab_v = new int[2]{0, op->nV};
    if (op->fib_slab) {
        cudaFree(op->fib_slab);
        op->fib_slab = nullptr;
    }
    if (op->fib_acc) {
        cudaFree(op->fib_acc);
        op->fib_acc = nullptr;
    }
    op->fib_acc_slots = 0;
    const double bytes = (double)op->n * (op->nIC > 0 ? op->nIC : 1) * sizeof(double);
    int S = want > 0 ? want : (int)(bytes / kSlabTermBytes + 0.5);
    if (S > 64) S = 64;
    if (S < 2 || op->nV < 2 * S || op->nF == 0 || op->nolut) return CGB_OK;
    std::vector<uint32_t> vp((size_t)op->nV + 1);
    CGB_CUDA(cudaMemcpy(vp.data(), op->vox_ptr, vp.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    std::vector<int> sv(S + 1);
    std::vector<uint32_t> pos(S + 1);
    for (int s = 0; s <= S; ++s) {
        const uint64_t target = (uint64_t)op->n * s / S;
        sv[s] = s == S ? op->nV : (int)(std::lower_bound(vp.begin(), vp.end(), (uint32_t)target) - vp.begin());
        if (s > 0 && sv[s] < sv[s - 1]) sv[s] = sv[s - 1];
        pos[s] = vp[sv[s]];
    }
    uint32_t *dpos = nullptr;
    CGB_CUDA(cudaMalloc((void **)&dpos, pos.size() * sizeof(uint32_t)));
    CGB_CUDA(cudaMemcpy(dpos, pos.data(), pos.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    cudaError_t e = cudaMalloc((void **)&op->fib_slab, (size_t)(S + 1) * op->nF * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&op->fib_acc, (size_t)op->nF * (op->nIC > 0 ? op->nIC : 1) * sizeof(double));
    op->fib_acc_slots = e == cudaSuccess ? 1 : 0;
    if (e != cudaSuccess) {
        cudaFree(dpos);
        cudaFree(op->fib_slab);
        op->fib_slab = nullptr;
        op->fib_acc = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    k_fib_slabs<<<(op->nF + 255) / 256, 256>>>(op->fib_ptr, op->fib_perm, op->fib_order, op->nF, S, dpos,
                                                op->fib_slab);
    const cudaError_t e2 = cudaGetLastError();
    cudaDeviceSynchronize();
    cudaFree(dpos);
    if (e2 != cudaSuccess) return cuda_fail(e2, "k_fib_slabs");
    delete[] op->slab_v;
    op->slab_v = new int[S + 1];
    for (int s = 0; s <= S; ++s) op->slab_v[s] = sv[s];
    op->nslab = S;
    return CGB_OK;
}

// room for `slots` running-sum accumulators of the slab fibre passes (one per vector of a
// multi-vector pass); grows outside stream capture only
int cgb::ensure_fib_acc(cgb_op *op, int slots) {
    if (op->nslab <= 1 || slots <= op->fib_acc_slots) return CGB_OK;
    CGB_CUDA(cudaDeviceSynchronize());
    if (op->fib_acc) cudaFree(op->fib_acc);
    op->fib_acc = nullptr;
    op->fib_acc_slots = 0;
    CGB_CUDA(cudaMalloc((void **)&op->fib_acc, (size_t)slots * op->nF * (op->nIC > 0 ? op->nIC : 1) * sizeof(double)));
    op->fib_acc_slots = slots;
    return CGB_OK;
}

static void free_op(cgb_op *op) {
    if (!op) return;
    free_grad_state(op);
    void *ptrs[] = {op->lutIC, op->lutEC, op->lutISO, op->lutIC_p, op->lutEC_p, op->lutISO_p, op->lutIC_r, op->lutEC_r, op->lutISO_r, op->seg_l16, op->vox_ptr,
                    op->seg_f, op->eval, op->fib_ptr, op->fib_perm, op->fib_order, op->ec_ptr, op->ec_col, op->iso_ptr,
                    op->iso_col, op->seg_o, op->ec_o, op->seg_l, op->scratch, op->scratch32, op->partials,
                    op->dscal, op->d_in, op->d_out, op->d_x64, op->fib_slab, op->fib_acc, op->d_xmax,
                    op->tc_ptr, op->tc_co, op->tc_l, op->tc_vl, op->tc_bimg, op->tc_xe, op->tc_err,
                    op->tc_fptr, op->tc_fperm, op->tc_abimg, op->tc_terms, op->tc_ax, op->tc_rows16, op->tc_ford, op->tc_fpos};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (op->h_scal) cudaFreeHost(op->h_scal);
    for (cudaStream_t s : op->pipe_st)
        if (s) cudaStreamDestroy(s);
    for (cudaStream_t s : op->slab_st)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : op->slab_ev)
        if (e) cudaEventDestroy(e);
    delete[] op->slab_v;
    for (cudaEvent_t e : op->pipe_ev)
        if (e) cudaEventDestroy(e);
    delete op;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

static int create_impl(int device, int nS, int ndirs, int nF, int64_t n, int nE, int nV, int nISOv,
                       const uint32_t *ICf, const uint32_t *ICeval, const uint32_t *ICv, const uint16_t *ICo,
                       const float *ICl, const uint32_t *ECv, const uint16_t *ECo, const uint32_t *ISOv,
                       const float *lutIC, const float *lutEC, const float *lutISO, int nIC, int nEC, int nISO,
                       int nolut, int arith, cgb_op *op) {
    if (nS < 1) return fail(CGB_ERR_INVALID, "nS must be >= 1");
    if (nolut && nS != 1) return fail(CGB_ERR_INVALID, "the LUT-free operator needs nS == 1");
    if (nS > kMaxSamples) return fail(CGB_ERR_UNSUPPORTED, "nS > 512 is not supported");
    if (nF < 0 || n < 0 || nE < 0 || nV < 0 || nISOv < 0) return fail(CGB_ERR_INVALID, "negative size");
    if (n >= (int64_t)0x7fffffff) return fail(CGB_ERR_UNSUPPORTED, "more than 2^31-1 IC segments");
    if (nIC < 0 || nEC < 0 || nISO < 0 || nIC > 32 || nEC > 32 || nISO > 32)
        return fail(CGB_ERR_INVALID, "number of response functions per compartment must be in [0, 32]");
    if (!nolut && (nIC > 0 || nEC > 0) && ndirs < 1) return fail(CGB_ERR_INVALID, "ndirs must be >= 1");
    if (nolut) {
        nEC = 0;
        nIC = nIC > 0 ? 1 : 0;
        nISO = nISO > 0 ? 1 : 0;
    }
    if (arith != CGB_ARITH_F64 && arith != CGB_ARITH_FF) return fail(CGB_ERR_INVALID, "arith must be F64 or FF");
    if ((n > 0 && (!ICf || !ICv || !ICl || (!nolut && !ICo))) || (nE > 0 && (!ECv || (!nolut && !ECo))) ||
        (nISOv > 0 && !ISOv))
        return fail(CGB_ERR_INVALID, "null dictionary array");

    op->device = device;
    op->nS = nS; op->ndirs = ndirs < 1 ? 1 : ndirs; op->nF = nF; op->nE = nE; op->nV = nV; op->nISOv = nISOv;
    op->nIC = nIC; op->nEC = nEC; op->nISO = nISO; op->nolut = nolut; op->n = n;
    op->nrows = (int64_t)nV * nS;
    op->ncols = (int64_t)nF * nIC + (int64_t)nE * nEC + (int64_t)nISOv * nISO;
    op->arith = arith;
    op->ff_variant = 1;  // float-float kernel family: packed pairs (cgb_op_ff_kernels selects the other)
    CGB_CUDA(cudaDeviceGetAttribute(&op->nsm, cudaDevAttrMultiProcessorCount, device));
    // lanes per voxel: whole warps for long sample vectors, sub-warps for short ones
    if (nS >= 96) op->lpv = 32;
    else if (nS > 16) op->lpv = (nS <= 48) ? 16 : 32;
    else if (nS > 8) op->lpv = 16;
    else if (nS > 4) op->lpv = 8;
    else if (nS > 1) op->lpv = 4;
    else op->lpv = 1;
    if (nS == 66) op->lpv = 8;

    const size_t lutIC_n = (size_t)nIC * op->ndirs * nS, lutEC_n = (size_t)nEC * op->ndirs * nS,
                 lutISO_n = (size_t)nISO * nS;
    Temp tmp;
    // raw uploads
    uint32_t *rf, *rv, *recv, *risov;
    uint16_t *ro = nullptr, *reco = nullptr;
    float *rl;
    CGB_TRY(tmp.alloc(&rf, n)); CGB_TRY(tmp.alloc(&rv, n)); CGB_TRY(tmp.alloc(&rl, n));
    CGB_TRY(upload(rf, ICf, n)); CGB_TRY(upload(rv, ICv, n)); CGB_TRY(upload(rl, ICl, n));
    if (!nolut) { CGB_TRY(tmp.alloc(&ro, n)); CGB_TRY(upload(ro, ICo, n)); }
    CGB_TRY(tmp.alloc(&recv, nE)); CGB_TRY(upload(recv, ECv, nE));
    if (!nolut) { CGB_TRY(tmp.alloc(&reco, nE)); CGB_TRY(upload(reco, ECo, nE)); }
    CGB_TRY(tmp.alloc(&risov, nISOv)); CGB_TRY(upload(risov, ISOv, nISOv));

    // validation
    unsigned int *dflag;
    CGB_TRY(tmp.alloc(&dflag, 1));
    CGB_CUDA(cudaMemset(dflag, 0, sizeof(unsigned int)));
    int64_t vmax = n > nE ? n : nE;
    if (nISOv > vmax) vmax = nISOv;
    if (vmax > 0)
        k_validate<<<grid_for(vmax), 256>>>(rf, rv, ro, n, recv, reco, nEC > 0 ? nE : 0, risov,
                                            nISO > 0 ? nISOv : 0, nF, nV, op->ndirs, !nolut, dflag);
    unsigned int hflag = 0;
    CGB_CUDA(cudaMemcpy(&hflag, dflag, sizeof(hflag), cudaMemcpyDeviceToHost));
    if (hflag) {
        std::string m = "invalid dictionary:";
        if (hflag & 1) m += " IC fibre index >= nF;";
        if (hflag & 2) m += " IC voxel index >= nV;";
        if (hflag & 4) m += " IC orientation >= ndirs;";
        if (hflag & 8) m += " EC voxel index >= nV;";
        if (hflag & 16) m += " EC orientation >= ndirs;";
        if (hflag & 32) m += " ISO voxel index >= nV;";
        return fail(CGB_ERR_INVALID, m);
    }

    // LUTs and eval
    CGB_TRY(dalloc(op, &op->lutIC, lutIC_n)); CGB_TRY(upload(op->lutIC, lutIC, nolut ? 0 : lutIC_n));
    CGB_TRY(dalloc(op, &op->lutEC, lutEC_n)); CGB_TRY(upload(op->lutEC, lutEC, nolut ? 0 : lutEC_n));
    CGB_TRY(dalloc(op, &op->lutISO, lutISO_n)); CGB_TRY(upload(op->lutISO, lutISO, nolut ? 0 : lutISO_n));
    // zero-padded copies with row stride nSp for the paired float-float kernels
    {
        // rows padded for both voxel shapes of the pair kernels (the tuner may pick either)
        const detail::PairShape ps = detail::pick_pair_shape(nS), pw = detail::wide_pair_shape(nS);
        op->nSp = 2 * ps.lpv * ps.np > 2 * pw.lpv * pw.np ? 2 * ps.lpv * ps.np : 2 * pw.lpv * pw.np;
        const size_t sp = (size_t)op->nSp;
        CGB_TRY(dalloc(op, &op->lutIC_p, (size_t)nIC * op->ndirs * sp));
        CGB_TRY(dalloc(op, &op->lutEC_p, (size_t)nEC * op->ndirs * sp));
        CGB_TRY(dalloc(op, &op->lutISO_p, (size_t)nISO * sp));
        auto padded = [&](size_t rows) { return (rows * sp > 0 ? rows * sp : 1) * sizeof(float); };
        CGB_CUDA(cudaMemset(op->lutIC_p, 0, padded((size_t)nIC * op->ndirs)));
        CGB_CUDA(cudaMemset(op->lutEC_p, 0, padded((size_t)nEC * op->ndirs)));
        CGB_CUDA(cudaMemset(op->lutISO_p, 0, padded((size_t)nISO)));
        if (!nolut) {
            if (lutIC_n) CGB_CUDA(cudaMemcpy2D(op->lutIC_p, sp * sizeof(float), lutIC, nS * sizeof(float),
                                               nS * sizeof(float), (size_t)nIC * op->ndirs, cudaMemcpyDefault));
            if (lutEC_n) CGB_CUDA(cudaMemcpy2D(op->lutEC_p, sp * sizeof(float), lutEC, nS * sizeof(float),
                                               nS * sizeof(float), (size_t)nEC * op->ndirs, cudaMemcpyDefault));
            if (lutISO_n) CGB_CUDA(cudaMemcpy2D(op->lutISO_p, sp * sizeof(float), lutISO, nS * sizeof(float),
                                                nS * sizeof(float), (size_t)nISO, cudaMemcpyDefault));
        }
    }
    CGB_TRY(dalloc(op, &op->eval, (size_t)nF * (nIC > 0 ? nIC : 1)));
    if (ICeval) {
        CGB_TRY(upload(op->eval, ICeval, (size_t)nF * nIC));
    } else {
        std::vector<uint32_t> ones((size_t)nF * nIC, 1u);
        CGB_TRY(upload(op->eval, ones.data(), ones.size()));
    }

    // IC: sort by (voxel, orientation)
    CGB_TRY(dalloc(op, &op->seg_f, n)); CGB_TRY(dalloc(op, &op->seg_o, n)); CGB_TRY(dalloc(op, &op->seg_l, n));
    CGB_TRY(dalloc(op, &op->vox_ptr, (size_t)nV + 1));
    if (n > 0) {
        uint32_t *perm;
        CGB_TRY(tmp.alloc(&perm, n));
        const uint64_t maxkey = (uint64_t)(nV > 0 ? nV : 1) * (nolut ? 1 : op->ndirs);
        uint64_t *key;
        CGB_TRY(tmp.alloc(&key, n));
        k_key_vo<<<grid_for(n), 256>>>(rv, nolut ? nullptr : ro, n, nolut ? 1u : (uint32_t)op->ndirs, key);
        CGB_TRY(sort_perm(key, n, bits_for(maxkey), perm, tmp));
        k_gather_ic<<<grid_for(n), 256>>>(perm, n, rf, ro, rl, op->seg_f, op->seg_o, op->seg_l);
        // vox_ptr from the (unsorted) voxel ids: counts do not depend on order
        CGB_TRY(csr_offsets(rv, n, nV, op->vox_ptr, tmp));
        // fibre order over voxel-ordered positions
        CGB_TRY(dalloc(op, &op->fib_perm, n));
        CGB_TRY(sort_perm(op->seg_f, n, bits_for((uint64_t)(nF > 0 ? nF : 1)), op->fib_perm, tmp));
    } else {
        CGB_CUDA(cudaMemset(op->vox_ptr, 0, ((size_t)nV + 1) * sizeof(uint32_t)));
        CGB_TRY(dalloc(op, &op->fib_perm, 1));
    }
    CGB_TRY(dalloc(op, &op->fib_ptr, (size_t)nF + 1));
    if (n > 0) {
        CGB_TRY(csr_offsets(op->seg_f, n, nF, op->fib_ptr, tmp));
    } else {
        CGB_CUDA(cudaMemset(op->fib_ptr, 0, ((size_t)nF + 1) * sizeof(uint32_t)));
    }
    // the fibres in the order of their first segment's voxel-order position: threads of the
    // fibre passes that are neighbours gather terms that are neighbours
    CGB_TRY(dalloc(op, &op->fib_order, (size_t)nF));
    if (nF > 0) {
        uint32_t *fkey;
        CGB_TRY(tmp.alloc(&fkey, (size_t)nF));
        k_fib_first<<<grid_for(nF), 256>>>(op->fib_ptr, op->fib_perm, nF, (uint32_t)n, fkey);
        CGB_TRY(sort_perm(fkey, nF, bits_for((uint64_t)n + 1), op->fib_order, tmp));
    }

    // EC / ISO voxel CSR with original column indices
    CGB_TRY(dalloc(op, &op->ec_ptr, (size_t)nV + 1));
    CGB_TRY(dalloc(op, &op->ec_col, nE));
    CGB_TRY(dalloc(op, &op->ec_o, nE));
    if (nE > 0 && nEC > 0) {
        CGB_TRY(sort_perm(recv, nE, bits_for((uint64_t)(nV > 0 ? nV : 1)), op->ec_col, tmp));
        if (!nolut) k_gather_u16<<<grid_for(nE), 256>>>(op->ec_col, nE, reco, op->ec_o);
        CGB_TRY(csr_offsets(recv, nE, nV, op->ec_ptr, tmp));
    } else {
        CGB_CUDA(cudaMemset(op->ec_ptr, 0, ((size_t)nV + 1) * sizeof(uint32_t)));
    }
    CGB_TRY(dalloc(op, &op->iso_ptr, (size_t)nV + 1));
    CGB_TRY(dalloc(op, &op->iso_col, nISOv));
    if (nISOv > 0 && nISO > 0) {
        CGB_TRY(sort_perm(risov, nISOv, bits_for((uint64_t)(nV > 0 ? nV : 1)), op->iso_col, tmp));
        CGB_TRY(csr_offsets(risov, nISOv, nV, op->iso_ptr, tmp));
    } else {
        CGB_CUDA(cudaMemset(op->iso_ptr, 0, ((size_t)nV + 1) * sizeof(uint32_t)));
    }

    CGB_TRY(build_slabs(op));

    // work buffers
    CGB_TRY(dalloc(op, &op->scratch, (size_t)n * (nIC > 0 ? nIC : 1)));
    CGB_TRY(dalloc(op, &op->partials, (size_t)partial_blocks(op) * kRedSlots));
    CGB_TRY(dalloc(op, &op->dscal, 64));
    CGB_TRY(dalloc(op, &op->d_xmax, 1));
    CGB_CUDA(cudaMallocHost((void **)&op->h_scal, 64 * sizeof(double)));
    if (!nolut) CGB_TRY(update_lut_exponents(op));
    CGB_CUDA(cudaDeviceSynchronize());
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

extern "C" {

const char *cgb_last_error(void) { return cgb::g_last_error.c_str(); }

const char *cgb_version(void) { return "commit_gb300 1.0 (sm_103a)"; }

int cgb_op_create(int device, int nS, int ndirs, int nF, int64_t n, int nE, int nV, int nISOv,
                  const uint32_t *ICf, const uint32_t *ICeval, const uint32_t *ICv, const uint16_t *ICo,
                  const float *ICl, const uint32_t *ECv, const uint16_t *ECo, const uint32_t *ISOv,
                  const float *lutIC, const float *lutEC, const float *lutISO, int nIC, int nEC, int nISO,
                  int nolut, int arith, cgb_op **out) {
    if (!out) return fail(CGB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    CGB_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(CGB_ERR_INVALID, "no such CUDA device");
    NvtxRange nv("cgb_op_create (device re-layout)");
    DeviceGuard g(device);
    cgb_op *op = new cgb_op();
    memset((void *)op, 0, sizeof(cgb_op));
    op->tc_mode = 0;  // tensor cores when dense enough (tc_forward_enabled)
    int rc = create_impl(device, nS, ndirs, nF, n, nE, nV, nISOv, ICf, ICeval, ICv, ICo, ICl, ECv, ECo, ISOv, lutIC,
                         lutEC, lutISO, nIC, nEC, nISO, nolut, arith, op);
    if (rc != CGB_OK) {
        std::string keep = cgb::g_last_error;
        free_op(op);
        cgb::g_last_error = keep;
        return rc;
    }
    *out = op;
    return CGB_OK;
}

int cgb_op_destroy(cgb_op *op) {
    if (!op) return CGB_OK;
    DeviceGuard g(op->device);
    cudaDeviceSynchronize();
    free_op(op);
    return CGB_OK;
}

int cgb_op_shape(const cgb_op *op, int64_t *nrows, int64_t *ncols) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (nrows) *nrows = op->nrows;
    if (ncols) *ncols = op->ncols;
    return CGB_OK;
}

int cgb_op_device_bytes(const cgb_op *op, size_t *bytes) {
    if (!op || !bytes) return fail(CGB_ERR_INVALID, "null argument");
    *bytes = op->bytes;
    return CGB_OK;
}

int cgb_op_set_lut(cgb_op *op, const float *lutIC, const float *lutEC, const float *lutISO) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (op->nolut) return fail(CGB_ERR_UNSUPPORTED, "the LUT-free operator has no LUT");
    DeviceGuard g(op->device);
    const size_t nS = op->nS, sp = op->nSp;
    struct Part {
        const float *src;
        float *dst, *dstp;
        size_t rows;
    } parts[3] = {{lutIC, op->lutIC, op->lutIC_p, (size_t)op->nIC * op->ndirs},
                  {lutEC, op->lutEC, op->lutEC_p, (size_t)op->nEC * op->ndirs},
                  {lutISO, op->lutISO, op->lutISO_p, (size_t)op->nISO}};
    for (const Part &p : parts) {
        if (!p.src || p.rows == 0) continue;
        CGB_CUDA(cudaMemcpy(p.dst, p.src, p.rows * nS * sizeof(float), cudaMemcpyDefault));
        CGB_CUDA(cudaMemcpy2D(p.dstp, sp * sizeof(float), p.src, nS * sizeof(float), nS * sizeof(float), p.rows,
                              cudaMemcpyDefault));
    }
    op->lut_r_kind = 0;  // reduced-precision copies are rebuilt on their next use
    return update_lut_exponents(op);
}

int cgb_op_ff_shape(cgb_op *op, int set, int *fwd, int *adj) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (set >= 0) {
        if (set > 2) return fail(CGB_ERR_INVALID, "shape must be 0 (tune), 1 (default) or 2 (a warp per voxel)");
        op->ff_shape[0] = op->ff_shape[1] = set;
    }
    if (fwd) *fwd = op->ff_shape[0];
    if (adj) *adj = op->ff_shape[1];
    return CGB_OK;
}

int cgb_op_ff_kernels(cgb_op *op, int variant, int *out) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (variant > 1) return fail(CGB_ERR_INVALID, "variant must be 0 (scalar samples) or 1 (packed pairs)");
    if (variant >= 0) op->ff_variant = variant;
    if (out) *out = op->ff_variant;
    return CGB_OK;
}

int cgb_op_set_slabs(cgb_op *op, int nslab, int *out) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (nslab < 0) {  // read only
        if (out) *out = op->nslab;
        return CGB_OK;
    }
    if (nslab > 64) return fail(CGB_ERR_INVALID, "nslab must be 0..64");
    DeviceGuard g(op->device);
    CGB_CUDA(cudaDeviceSynchronize());
    CGB_TRY(build_slabs(op, nslab == 0 ? 0 : nslab));
    if (nslab == 1) {
        // a single slab is the plain two-pass adjoint
        delete[] op->slab_v;
        op->slab_v = new int[2]{0, op->nV};
        if (op->fib_slab) cudaFree(op->fib_slab);
        if (op->fib_acc) cudaFree(op->fib_acc);
        op->fib_slab = nullptr;
        op->fib_acc = nullptr;
        op->fib_acc_slots = 0;
        op->nslab = 1;
    }
    if (op->partials) cudaFree(op->partials);
    op->partials = nullptr;
    CGB_CUDA(cudaMalloc((void **)&op->partials, (size_t)partial_blocks(op) * kRedSlots * sizeof(double)));
    if (out) *out = op->nslab;
    return CGB_OK;
}

int cgb_op_set_arith(cgb_op *op, int arith) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (arith != CGB_ARITH_F64 && arith != CGB_ARITH_FF) return fail(CGB_ERR_INVALID, "arith must be F64 or FF");
    op->arith = arith;
    return CGB_OK;
}

}  // extern "C"
