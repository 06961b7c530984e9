// A'*y without any device allocation (cgb_op_adjoint_noalloc).
//
// Some callers cannot let a library allocate GPU memory: an application that reserves
// the device's memory up front in its own pool (so a cudaMalloc from a plug-in fails or
// fragments that pool), or one issuing work on a latency-critical stream, where
// cudaMalloc's implicit device-wide synchronisation is not acceptable.  This entry point
// serves them: the caller passes every input and output as its own device buffer, and
// the only working memory -- the per-segment terms between the voxel pass and the fibre
// pass -- is a fixed array in the library's static device memory, reserved on every GPU
// that loads the library until the process exits.
//
// The kernels are variants of the operator's A' (operator_kernels.cuh) that read the
// reference's own array layout (segments, EC and ISO elements sorted by voxel, as
// load_dictionary leaves them) and find each voxel's range by binary search, so no
// re-laid-out copy of the dictionary is needed.  Like the operator's float-float A', each
// voxel row of y outside FP32's comfortable exponent range is scaled by an exact power of
// two (ff_exp_hi), using the LUT's largest magnitude measured on every call.
//
// Module loading.  Under CUDA's lazy module loading (the default since CUDA 12.2) the
// static array is allocated, and a kernel's code loaded, when the module or kernel is
// first used -- which would make the first call, and the first call for each kernel
// shape, allocate device memory.  The first call on a device therefore does all of that
// at once: it looks up the array's address and loads every kernel of this file
// (cudaFuncGetAttributes).  Later calls load and allocate nothing.  A call whose sizes are
// all zero (y may be any non-null pointer) does only this set-up.
#include <mutex>

#include "operator_launch.cuh"

namespace cgb {
namespace detail {

// 2^20 FP64 terms = 8 MiB of static device memory.
constexpr int64_t kNoAllocMaxTerms = CGB_NOALLOC_MAX_TERMS;
static __device__ __align__(256) double g_noalloc_terms[kNoAllocMaxTerms];

struct NoAllocArgs {
    int nS, ndirs, nF, nE, nV, nISOv, nIC, nEC, nISO;
    int64_t n;
    const double *y;
    double *x;
    const uint32_t *ICf, *ICeval, *ICv, *ECv, *ISOv, *fib_ptr, *fib_perm;
    const uint16_t *ICo, *ECo;
    const float *ICl, *lutIC, *lutEC, *lutISO;
};

__device__ __forceinline__ int64_t lower_bound_dev(const uint32_t *a, int64_t n, uint32_t key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// largest finite |LUT| of the three compartments, as float bits, into *out (zeroed)
__global__ void k_lut_absmax(const NoAllocArgs A, unsigned *__restrict__ out) {
    const float *L[3] = {A.lutIC, A.lutEC, A.lutISO};
    const int64_t n[3] = {(int64_t)A.nIC * A.ndirs * A.nS, (int64_t)A.nEC * A.ndirs * A.nS, (int64_t)A.nISO * A.nS};
    unsigned m = 0;
    for (int c = 0; c < 3; ++c)
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; L[c] && i < n[c];
             i += (int64_t)gridDim.x * blockDim.x) {
            const unsigned b = __float_as_uint(L[c][i]) & 0x7fffffffu;
            if (b < 0x7f800000u && b > m) m = b;
        }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

template <int LPV, int NCH>
__global__ void __launch_bounds__(kBlock) k_adjoint_noalloc(const NoAllocArgs A, double *__restrict__ terms,
                                                            const unsigned *__restrict__ lutmax) {
    using AR = ArFF;
    constexpr int B = LPV < 8 ? LPV : 8;
    constexpr int SPAN = LPV / B;
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    const int nS = A.nS;
    const int q_me = G.sub / SPAN;
    const bool writer = (G.sub % SPAN) == 0;
    const int64_t ec_base = (int64_t)A.nF * A.nIC;
    const int64_t iso_base = ec_base + (int64_t)A.nE * A.nEC;
    // exponent of the LUT's largest magnitude (0 when it was not measured)
    const unsigned lb = lutmax ? *lutmax : 0u;
    const int lut_exp = lb ? (int)((lb >> 23) & 0xffu) - 127 : 0;
    for (int v = blockIdx.x * gpb + (int)threadIdx.x / LPV; v < A.nV; v += ngroups) {
        typename AR::Coef z[NCH];
        unsigned zmax = 0;
#pragma unroll
        for (int k = 0; k < NCH; ++k) {
            const int s = G.sub + k * LPV;
            const double yv = s < nS ? A.y[(size_t)v * nS + s] : 0.0;
            const unsigned h = abs_hi(yv);
            zmax = h > zmax ? h : zmax;
            z[k] = AR::coef(yv);
        }
        const int ez = ff_exp_hi(group_max_u<LPV>(zmax, G.mask), lut_exp);
        if (ez) {
#pragma unroll
            for (int k = 0; k < NCH; ++k) {
                const int s = G.sub + k * LPV;
                z[k] = AR::coef((s < nS ? A.y[(size_t)v * nS + s] : 0.0) * pow2(-ez));
            }
        }
        if (A.nIC > 0) {
            const int64_t beg = lower_bound_dev(A.ICv, A.n, (uint32_t)v);
            const int64_t end = lower_bound_dev(A.ICv, A.n, (uint32_t)v + 1);
            for (int64_t b = beg; b < end; b += LPV) {
                const int64_t j = b + G.sub;
                const bool valid = j < end;
                uint32_t o = valid ? A.ICo[j] : 0;
                const bool o_ok = o < (uint32_t)A.ndirs;
                if (!o_ok) o = 0;
                const float l = (valid && o_ok) ? A.ICl[j] : 0.f;
                const int cntL = (int)((end - b) < LPV ? (end - b) : LPV);
                for (int i = 0; i < A.nIC; ++i) {
                    const uint32_t row = ((uint32_t)i * A.ndirs + o) * (uint32_t)nS;
                    for (int t0 = 0; t0 < cntL; t0 += B) {
                        const int cnt = min(B, cntL - t0);
                        auto rowf = [&](int q) { return __shfl_sync(G.mask, row, t0 + q, LPV); };
                        const AR::Acc tot = batch_dots<LPV, NCH, AR>(G, A.lutIC, rowf, cnt, nS, z);
                        const float lq = __shfl_sync(G.mask, l, t0 + q_me, LPV);
                        double tv = AR::val(tot);
                        if (ez) tv *= pow2(ez);
                        if (writer && q_me < cnt) terms[(size_t)i * A.n + b + t0 + q_me] = (double)lq * tv;
                    }
                }
            }
        }
        if (A.nEC > 0) {
            const int64_t beg = lower_bound_dev(A.ECv, A.nE, (uint32_t)v);
            const int64_t end = lower_bound_dev(A.ECv, A.nE, (uint32_t)v + 1);
            for (int64_t b = beg; b < end; b += LPV) {
                const int64_t j = b + G.sub;
                const bool valid = j < end;
                uint32_t o = valid ? A.ECo[j] : 0;
                const bool o_ok = o < (uint32_t)A.ndirs;
                if (!o_ok) o = 0;
                const int cntL = (int)((end - b) < LPV ? (end - b) : LPV);
                for (int i = 0; i < A.nEC; ++i) {
                    const uint32_t row = ((uint32_t)i * A.ndirs + o) * (uint32_t)nS;
                    for (int t0 = 0; t0 < cntL; t0 += B) {
                        const int cnt = min(B, cntL - t0);
                        auto rowf = [&](int q) { return __shfl_sync(G.mask, row, t0 + q, LPV); };
                        const AR::Acc tot = batch_dots<LPV, NCH, AR>(G, A.lutEC, rowf, cnt, nS, z);
                        const int okq = __shfl_sync(G.mask, (int)o_ok, t0 + q_me, LPV);
                        double tv = AR::val(tot);
                        if (ez) tv *= pow2(ez);
                        if (writer && q_me < cnt) A.x[ec_base + (size_t)i * A.nE + b + t0 + q_me] = okq ? tv : 0.0;
                    }
                }
            }
        }
        if (A.nISO > 0) {
            const int64_t beg = lower_bound_dev(A.ISOv, A.nISOv, (uint32_t)v);
            const int64_t end = lower_bound_dev(A.ISOv, A.nISOv, (uint32_t)v + 1);
            if (beg < end) {
                for (int t0 = 0; t0 < A.nISO; t0 += B) {
                    const int cnt = min(B, A.nISO - t0);
                    auto rowf = [&](int q) { return (uint32_t)((t0 + q) * nS); };
                    const AR::Acc tot = batch_dots<LPV, NCH, AR>(G, A.lutISO, rowf, cnt, nS, z);
                    if (writer && q_me < cnt) {
                        double d = AR::val(tot);
                        if (ez) d *= pow2(ez);
                        for (int64_t e = beg; e < end; ++e) A.x[iso_base + (size_t)(t0 + q_me) * A.nISOv + e] = d;
                    }
                }
            }
        }
    }
}

__global__ void k_fibre_sum_noalloc(const NoAllocArgs A, const double *__restrict__ terms) {
    const int64_t total = (int64_t)A.nF * A.nIC;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / A.nF);
        const uint32_t f = (uint32_t)(q - (int64_t)i * A.nF);
        uint32_t beg = A.fib_ptr[f], end = A.fib_ptr[f + 1];
        if (end > (uint32_t)A.n) end = (uint32_t)A.n;
        const double *S = terms + (size_t)i * A.n;
        double s = 0.0;
        for (uint32_t k = beg; k < end; ++k) {
            const uint32_t p = A.fib_perm[k];
            if (p < (uint32_t)A.n) s += S[p];
        }
        A.x[q] = s * (double)A.ICeval[q];
    }
}

struct NoAllocLaunch {
    NoAllocArgs args;
    double *terms;
    const unsigned *lutmax;
    int nsm;
    cudaStream_t st;
    template <int L, int N>
    int run() {
        auto kern = k_adjoint_noalloc<L, N>;
        int g = 0;
        CGB_TRY(grid_for_kernel(kern, 0, nsm, args.nV, kBlock / L, &g));
        kern<<<g, kBlock, 0, st>>>(args, terms, lutmax);
        CGB_CUDA(cudaGetLastError());
        return CGB_OK;
    }
};

// loads the code of one kernel shape (cudaFuncGetAttributes), so no later call does
struct NoAllocLoad {
    template <int L, int N>
    int run() {
        cudaFuncAttributes a;
        CGB_CUDA(cudaFuncGetAttributes(&a, k_adjoint_noalloc<L, N>));
        return CGB_OK;
    }
};

// Per-device set-up, done once with that device current: the static scratch's device
// address and the loading of every kernel of this file.  The cached address is that of
// the module loaded in the device's primary context: cudaDeviceReset invalidates it, so a
// process that resets a device must not call this entry point on it afterwards.
std::mutex g_noalloc_mutex;
double *g_noalloc_addr[64] = {nullptr};

int noalloc_terms(int dev, double **out) {
    if (dev < 0 || dev >= 64) return fail(CGB_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        CGB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_terms));
        NoAllocLoad ld;
        for (const Shape &s : kShapes) CGB_TRY(dispatch_shape(s, ld));
        cudaFuncAttributes a;
        CGB_CUDA(cudaFuncGetAttributes(&a, k_fibre_sum_noalloc));
        CGB_CUDA(cudaFuncGetAttributes(&a, k_lut_absmax));
        g_noalloc_addr[dev] = (double *)p;
    }
    *out = g_noalloc_addr[dev];
    return CGB_OK;
}

}  // namespace detail
}  // namespace cgb

using namespace cgb;
using namespace cgb::detail;

extern "C" int cgb_op_adjoint_noalloc(int nS, int ndirs, int nF, int64_t n, int nE, int nV, int nISOv,
                                      const double *y, double *x, const uint32_t *ICf, const uint32_t *ICeval,
                                      const uint32_t *ICv, const uint16_t *ICo, const float *ICl,
                                      const uint32_t *ECv, const uint16_t *ECo, const uint32_t *ISOv,
                                      const float *lutIC, const float *lutEC, const float *lutISO, int nIC,
                                      int nEC, int nISO, const uint32_t *fib_ptr, const uint32_t *fib_perm,
                                      void *stream) {
    if (nS < 1 || nS > kMaxSamples) return fail(CGB_ERR_UNSUPPORTED, "nS must be in [1, 512]");
    if (nF < 0 || n < 0 || nE < 0 || nV < 0 || nISOv < 0 || ndirs < 1)
        return fail(CGB_ERR_INVALID, "negative size or ndirs < 1");
    if (nIC < 0 || nEC < 0 || nISO < 0 || nIC > 32 || nEC > 32 || nISO > 32)
        return fail(CGB_ERR_INVALID, "number of response functions per compartment must be in [0, 32]");
    if (n * (int64_t)(nIC > 0 ? nIC : 0) > kNoAllocMaxTerms)
        return fail(CGB_ERR_UNSUPPORTED, "cgb_op_adjoint_noalloc: n*nIC = " + std::to_string(n * (int64_t)nIC) +
                                             " exceeds its static scratch of " + std::to_string(kNoAllocMaxTerms) +
                                             " terms; use cgb_op_create/cgb_op_apply");
    const int64_t ncols = (int64_t)nF * nIC + (int64_t)nE * nEC + (int64_t)nISOv * nISO;
    // ICf is not read: the fibre index (fib_ptr, fib_perm) replaces it
    if (!y || (ncols > 0 && !x) || (n > 0 && nIC > 0 && (!ICv || !ICo || !ICl || !fib_perm)) ||
        (nIC > 0 && (!ICeval || !fib_ptr || !lutIC)) || (nE > 0 && nEC > 0 && (!ECv || !ECo || !lutEC)) ||
        (nISOv > 0 && nISO > 0 && (!ISOv || !lutISO)))
        return fail(CGB_ERR_INVALID, "null array");
    int dev = 0;
    CGB_CUDA(cudaGetDevice(&dev));
    double *terms = nullptr;
    CGB_TRY(noalloc_terms(dev, &terms));
    int nsm = 0;
    CGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t st = (cudaStream_t)stream;
    // the terms of segments outside every voxel and the columns of elements outside every
    // voxel are never written by the passes below: start both from zero
    if (ncols > 0) CGB_CUDA(cudaMemsetAsync(x, 0, ncols * sizeof(double), st));
    // the LUT's largest magnitude goes to the slot after the terms (when there is one)
    const int64_t nterms = n * (nIC > 0 ? nIC : 0);
    unsigned *lutmax = nterms < kNoAllocMaxTerms ? reinterpret_cast<unsigned *>(terms + nterms) : nullptr;
    if (nV == 0 || ncols == 0) return CGB_OK;
    CGB_CUDA(cudaMemsetAsync(terms, 0, (nterms + (lutmax ? 1 : 0)) * sizeof(double), st));
    NoAllocArgs a;
    a.nS = nS; a.ndirs = ndirs; a.nF = nF; a.nE = nE; a.nV = nV; a.nISOv = nISOv;
    a.nIC = nIC; a.nEC = nE > 0 ? nEC : 0; a.nISO = nISOv > 0 ? nISO : 0; a.n = n;
    a.y = y; a.x = x; a.ICf = ICf; a.ICeval = ICeval; a.ICv = ICv; a.ECv = ECv; a.ISOv = ISOv;
    a.fib_ptr = fib_ptr; a.fib_perm = fib_perm; a.ICo = ICo; a.ECo = ECo; a.ICl = ICl;
    a.lutIC = lutIC; a.lutEC = lutEC; a.lutISO = lutISO;
    if (lutmax) {
        k_lut_absmax<<<nsm, 256, 0, st>>>(a, lutmax);
        CGB_CUDA(cudaGetLastError());
    }
    NoAllocLaunch L{a, terms, lutmax, nsm, st};
    CGB_TRY(dispatch_shape(pick_shape(nS), L));
    if (nIC > 0 && nF > 0) {
        const int64_t total = (int64_t)nF * nIC;
        int gb = (int)((total + 255) / 256);
        if (gb > nsm * 16) gb = nsm * 16;
        k_fibre_sum_noalloc<<<gb, 256, 0, st>>>(a, terms);
        CGB_CUDA(cudaGetLastError());
    }
    return CGB_OK;
}
