#pragma once
// A*x and A'*y kernels of the FP64-accurate path (templates; instantiated per arithmetic).
//
// Reference semantics: setup_operator.py:50-218 (A: COMMIT_A__block) and :370-563
// (A': COMMIT_At__block), :713-871 (LUT-free variants).  For a voxel v with IC segments
// (f, o, l), EC elements (o) and ISO elements:
//   y[v,s] = sum_seg l * sum_i x[i*nF+f]*eval[i*nF+f] * LUT_IC[i,o,s]
//          + sum_ec  sum_i x[ec_base + i*nE + e] * LUT_EC[i,o,s]
//          + sum_iso sum_i x[iso_base + i*nISO + j] * LUT_ISO[i,s]
//   x[i*nF+f] = eval[i*nF+f] * sum_{seg of f} l * <LUT_IC[i,o,:], y[v,:]>     (A')
//
// GB300 mapping.  A group of LPV lanes (a warp for long sample vectors) owns one voxel at
// a time and each lane owns NCH samples; segment metadata is loaded cooperatively
// (coalesced), the coefficient c = l*x*eval is formed once by the loading lane and
// broadcast with shuffles, and every lane streams its slice of the LUT row.  Output rows
// are written once, so A needs no zero fill and no atomics.  A' runs the same voxel pass:
// each lane accumulates partial dot products for a batch of 8 segments, a butterfly
// reduce-scatter across the group leaves each segment's total in one lane, and the
// per-segment terms l*<L,y> go to a scratch stream in voxel order; a second pass sums them per fibre through the
// fibre-ordered index (deterministic, no atomics).  EC/ISO outputs are owned by one voxel
// and are written directly by the first pass.
//
// Arithmetic.  GB300 issues FP64 FMAs at ~1/58 of the FP32 rate, so besides native FP64
// (ArF64) the kernels run a float-float policy (ArFF): FP64 inputs are split into two
// FP32 words, products are made exact with an FMA (two-product), sums are error-free
// (two-sum), giving ~48-bit significands -- far inside the 1e-10 parity bound -- on the
// FP32 pipe.  Reductions of residual norms stay in FP64.
#include "cgb_internal.cuh"

namespace cgb {
namespace detail {

// ------------------------------------------------------------------ arithmetic policies
struct ArF64 {
    using Acc = double;
    using Coef = double;
    __device__ static __forceinline__ void zero(Acc &a) { a = 0.0; }
    __device__ static __forceinline__ Coef coef(double c) { return c; }
    __device__ static __forceinline__ bool nz(const Coef &c) { return c != 0.0; }
    __device__ static __forceinline__ Coef shfl(unsigned m, const Coef &c, int src, int w) {
        return __shfl_sync(m, c, src, w);
    }
    __device__ static __forceinline__ Acc shfl_xor(unsigned m, const Acc &a, int lm, int w) {
        return __shfl_xor_sync(m, a, lm, w);
    }
    __device__ static __forceinline__ void fma_(Acc &a, const Coef &c, float L) { a = fma(c, (double)L, a); }
    __device__ static __forceinline__ void add(Acc &a, const Acc &b) { a += b; }
    __device__ static __forceinline__ double val(const Acc &a) { return a; }
};

struct ArFF {
    struct Acc {
        float s, e;
    };
    struct Coef {
        float h, l;
    };
    __device__ static __forceinline__ void zero(Acc &a) { a.s = 0.f; a.e = 0.f; }
    __device__ static __forceinline__ Coef coef(double c) {
        Coef r;
        r.h = __double2float_rn(c);
        r.l = __double2float_rn(c - (double)r.h);
        return r;
    }
    __device__ static __forceinline__ bool nz(const Coef &c) { return c.h != 0.f || c.l != 0.f; }
    __device__ static __forceinline__ Coef shfl(unsigned m, const Coef &c, int src, int w) {
        Coef r;
        r.h = __shfl_sync(m, c.h, src, w);
        r.l = __shfl_sync(m, c.l, src, w);
        return r;
    }
    __device__ static __forceinline__ Acc shfl_xor(unsigned m, const Acc &a, int lm, int w) {
        Acc r;
        r.s = __shfl_xor_sync(m, a.s, lm, w);
        r.e = __shfl_xor_sync(m, a.e, lm, w);
        return r;
    }
    // a += (c.h + c.l) * L with an exact two-product of the high word and a two-sum
    __device__ static __forceinline__ void fma_(Acc &a, const Coef &c, float L) {
        const float p = __fmul_rn(c.h, L);
        float e = __fmaf_rn(c.h, L, -p);
        e = __fmaf_rn(c.l, L, e);
        const float s = __fadd_rn(a.s, p);
        const float bb = __fsub_rn(s, a.s);
        const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(p, bb));
        a.s = s;
        a.e = __fadd_rn(a.e, __fadd_rn(err, e));
    }
    __device__ static __forceinline__ void add(Acc &a, const Acc &b) {
        const float s = __fadd_rn(a.s, b.s);
        const float bb = __fsub_rn(s, a.s);
        const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(b.s, bb));
        a.s = s;
        a.e = __fadd_rn(a.e, __fadd_rn(b.e, err));
    }
    __device__ static __forceinline__ double val(const Acc &a) { return (double)a.s + (double)a.e; }
};

template <int LPV>
struct Group {
    int sub;
    unsigned mask;
    __device__ __forceinline__ Group() {
        const int lane = threadIdx.x & 31;
        sub = lane & (LPV - 1);
        mask = (LPV == 32) ? 0xffffffffu : (((1u << LPV) - 1u) << (lane & ~(LPV - 1)));
    }
};

__device__ __forceinline__ void block_sum_store(double v, double *dst) {
    __shared__ double red[kBlock / 32];
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < kBlock / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) *dst = v;
    }
}

// ------------------------------------------------------------------ float-float range guard
// The float-float words are FP32: products and sums keep their ~48-bit significand only
// while they stay well inside FP32's exponent range, and FP64 operands can lie far outside
// it (the reference accumulates in FP64, setup_operator.py:92-96).  An operand is therefore
// scaled by an exact power of two 2^-e when the bound on its products with the LUT,
// 2^(exponent of its largest magnitude + lut_exp), leaves [2^-kFFRange, 2^kFFRange], and
// the results are scaled back by 2^e in FP64.  Inside that range e = 0: nothing is scaled
// and results are bitwise those of the unguarded kernels.  `hi` is the high word of the
// largest magnitude (exponent in bits 20..30); zero, infinities and NaN give e = 0.
constexpr int kFFRange = 60;
__device__ __forceinline__ int ff_exp_hi(unsigned hi, int lut_exp) {
    const int be = (int)(hi >> 20) & 0x7ff;
    if (hi == 0 || be == 0x7ff) return 0;
    const int e = (be == 0 ? -1022 : be - 1023) + lut_exp;
    if (e >= -kFFRange && e <= kFFRange) return 0;
    return e < -1000 ? -1000 : (e > 1000 ? 1000 : e);
}

// A x from stored rows (momentum reuse): ca*a + cb*b with one explicit rounding order, so
// that a separate pass forming the same row (the graph-captured FISTA) gives the same bits
__device__ __forceinline__ double ax_combine(double ca, double a, double cb, double b) {
    return __fma_rn(ca, a, __dmul_rn(cb, b));
}
__device__ __forceinline__ float ax_combine(float ca, float a, float cb, float b) {
    return __fmaf_rn(ca, a, __fmul_rn(cb, b));
}

// 2^e as a double for |e| <= 1000 (exponent field only)
__device__ __forceinline__ double pow2(int e) { return __hiloint2double((e + 1023) << 20, 0); }

// scaling exponent of the forward input x of this launch (0 when not measured)
__device__ __forceinline__ int ff_exp_x(const OpDev &P) {
    return P.xmax ? ff_exp_hi((unsigned)(*P.xmax >> 32), P.lut_exp_fwd) : 0;
}

// high word of |v| for finite v, 0 for infinities and NaN (they propagate unscaled)
__device__ __forceinline__ unsigned abs_hi(double v) {
    const unsigned h = (unsigned)__double2hiint(v) & 0x7fffffffu;
    return h < 0x7ff00000u ? h : 0u;
}

template <int LPV>
__device__ __forceinline__ unsigned group_max_u(unsigned m, unsigned mask) {
#pragma unroll
    for (int d = LPV / 2; d >= 1; d >>= 1) {
        const unsigned t = __shfl_xor_sync(mask, m, d, LPV);
        m = t > m ? t : m;
    }
    return m;
}

// ------------------------------------------------------------------ forward accumulation
// Accumulates row v of A*x into acc[NCH] (lane owns samples sub + k*LPV).
template <int LPV, int NCH, class AR>
__device__ __forceinline__ void forward_row(const OpDev &P, const Group<LPV> &G, int v, const double *__restrict__ x,
                                            typename AR::Acc (&acc)[NCH], int ex) {
    const int nS = P.nS;
#pragma unroll
    for (int k = 0; k < NCH; ++k) AR::zero(acc[k]);
    // IC segments
    if (P.nIC > 0) {
        const uint32_t beg = P.vox_ptr[v], end = P.vox_ptr[v + 1];
        for (uint32_t b = beg; b < end; b += LPV) {
            const uint32_t j = b + G.sub;
            const bool valid = j < end;
            uint32_t f = 0, o = 0;
            float l = 0.f;
            if (valid) {
                f = P.seg_f[j];
                o = P.seg_o[j];
                l = P.seg_l[j];
            }
            const int cnt = min((int)(end - b), LPV);
            for (int i = 0; i < P.nIC; ++i) {
                double c = 0.0;
                if (valid) {
                    const size_t col = (size_t)i * P.nF + f;
                    double xv = x[col];
                    if (ex) xv = xv * pow2(-ex);
                    c = (double)l * (xv * (double)P.eval[col]);
                }
                const typename AR::Coef cf = AR::coef(c);
                const uint32_t row = ((uint32_t)i * P.ndirs + o) * (uint32_t)nS;
                for (int t = 0; t < cnt; ++t) {
                    const typename AR::Coef ct = AR::shfl(G.mask, cf, t, LPV);
                    const uint32_t rt = __shfl_sync(G.mask, row, t, LPV);
                    if (AR::nz(ct)) {
                        const float *L = P.lutIC + rt;
#pragma unroll
                        for (int k = 0; k < NCH; ++k) {
                            const int s = G.sub + k * LPV;
                            if (s < nS) AR::fma_(acc[k], ct, __ldg(L + s));
                        }
                    }
                }
            }
        }
    }
    // EC elements
    if (P.nEC > 0) {
        const uint32_t beg = P.ec_ptr[v], end = P.ec_ptr[v + 1];
        for (uint32_t b = beg; b < end; b += LPV) {
            const uint32_t j = b + G.sub;
            const bool valid = j < end;
            uint32_t col = 0, o = 0;
            if (valid) {
                col = P.ec_col[j];
                o = P.ec_o[j];
            }
            const int cnt = min((int)(end - b), LPV);
            for (int i = 0; i < P.nEC; ++i) {
                double c = valid ? x[P.ec_base + (size_t)i * P.nE + col] : 0.0;
                if (ex) c = c * pow2(-ex);
                const typename AR::Coef cf = AR::coef(c);
                const uint32_t row = ((uint32_t)i * P.ndirs + o) * (uint32_t)nS;
                for (int t = 0; t < cnt; ++t) {
                    const typename AR::Coef ct = AR::shfl(G.mask, cf, t, LPV);
                    const uint32_t rt = __shfl_sync(G.mask, row, t, LPV);
                    if (AR::nz(ct)) {
                        const float *L = P.lutEC + rt;
#pragma unroll
                        for (int k = 0; k < NCH; ++k) {
                            const int s = G.sub + k * LPV;
                            if (s < nS) AR::fma_(acc[k], ct, __ldg(L + s));
                        }
                    }
                }
            }
        }
    }
    // ISO elements
    if (P.nISO > 0) {
        const uint32_t beg = P.iso_ptr[v], end = P.iso_ptr[v + 1];
        for (uint32_t b = beg; b < end; b += LPV) {
            const uint32_t j = b + G.sub;
            const bool valid = j < end;
            const uint32_t col = valid ? P.iso_col[j] : 0;
            const int cnt = min((int)(end - b), LPV);
            for (int i = 0; i < P.nISO; ++i) {
                double c = valid ? x[P.iso_base + (size_t)i * P.nISOv + col] : 0.0;
                if (ex) c = c * pow2(-ex);
                const typename AR::Coef cf = AR::coef(c);
                for (int t = 0; t < cnt; ++t) {
                    const typename AR::Coef ct = AR::shfl(G.mask, cf, t, LPV);
                    if (AR::nz(ct)) {
                        const float *L = P.lutISO + (size_t)i * nS;
#pragma unroll
                        for (int k = 0; k < NCH; ++k) {
                            const int s = G.sub + k * LPV;
                            if (s < nS) AR::fma_(acc[k], ct, __ldg(L + s));
                        }
                    }
                }
            }
        }
    }
}

// y = A x ; optionally ax_out = A x ; optionally partial sums of |sqw*(Ax - yobs)|^2
template <int LPV, int NCH, class AR>
__global__ void __launch_bounds__(kBlock) k_forward(const OpDev P, const double *__restrict__ x,
                                                    double *__restrict__ yout, double *__restrict__ axout,
                                                    const double *__restrict__ yobs, const double *__restrict__ sqw,
                                                    double *__restrict__ partials) {
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    double nrm = 0.0;
    const int ex = ff_exp_x(P);
    for (int v = blockIdx.x * gpb + (int)threadIdx.x / LPV; v < P.nV; v += ngroups) {
        typename AR::Acc acc[NCH];
        forward_row<LPV, NCH, AR>(P, G, v, x, acc, ex);
#pragma unroll
        for (int k = 0; k < NCH; ++k) {
            const int s = G.sub + k * LPV;
            if (s < P.nS) {
                const size_t idx = (size_t)v * P.nS + s;
                double a = AR::val(acc[k]);
                if (ex) a = a * pow2(ex);
                if (yout) yout[idx] = a;
                if (axout) axout[idx] = a;
                if (partials) {
                    double r = yobs ? a - yobs[idx] : a;
                    if (sqw) r *= sqw[idx];
                    nrm = fma(r, r, nrm);
                }
            }
        }
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

// ------------------------------------------------------------------ adjoint
// Dot products <LUT row of item q, z> for the B = min(8, LPV) items of a sub-batch
// (row(q) gives item q's LUT offset; only q < cnt are computed).  Each lane holds partial
// sums over its samples; a butterfly reduce-scatter across the group leaves the total of
// item q = sub / (LPV / B) in lane sub -- no shared memory, about two shuffles and one
// error-free add per item and lane.
template <int LPV, int NCH, class AR, class RowFn>
__device__ __forceinline__ typename AR::Acc batch_dots(const Group<LPV> &G, const float *__restrict__ lut,
                                                       RowFn row, int cnt, int nS,
                                                       const typename AR::Coef (&z)[NCH]) {
    constexpr int B = LPV < 8 ? LPV : 8;
    typename AR::Acc P[B];
#pragma unroll
    for (int q = 0; q < B; ++q) {
        AR::zero(P[q]);
        if (q < cnt) {
            const float *L = lut + row(q);
#pragma unroll
            for (int k = 0; k < NCH; ++k) {
                const int s = G.sub + k * LPV;
                if (s < nS) AR::fma_(P[q], z[k], __ldg(L + s));
            }
        }
    }
#pragma unroll
    for (int h = B / 2, m = LPV / 2; h >= 1; h /= 2, m /= 2) {
        const bool hi = (G.sub & m) != 0;
#pragma unroll
        for (int j = 0; j < h; ++j) {
            const typename AR::Acc send = hi ? P[j] : P[j + h];
            typename AR::Acc keep = hi ? P[j + h] : P[j];
            AR::add(keep, AR::shfl_xor(G.mask, send, m, LPV));
            P[j] = keep;
        }
    }
#pragma unroll
    for (int m = LPV / B / 2; m >= 1; m /= 2) AR::add(P[0], AR::shfl_xor(G.mask, P[0], m, LPV));
    return P[0];
}

// in_mode 0: z = yin[v,:]
// in_mode 1: z = sqw*r with r = sqw*(A x - yobs) (gradient of 1/2|sqw(Ax-y)|^2), |r|^2 partials
// in_mode 2: as 1 with A x replaced by ca*ax_a + cb*ax_b
template <int LPV, int NCH, class AR>
__global__ void __launch_bounds__(kBlock) k_adjoint(const OpDev P, const double *__restrict__ yin, int in_mode,
                                                    const double *__restrict__ x, const double *__restrict__ yobs,
                                                    const double *__restrict__ sqw, const double *__restrict__ ax_a,
                                                    const double *__restrict__ ax_b, double ca, double cb,
                                                    double *__restrict__ scratch, double *__restrict__ xout,
                                                    double *__restrict__ partials) {
    constexpr int B = LPV < 8 ? LPV : 8;
    constexpr int SPAN = LPV / B;  // lanes holding the same item after the reduce-scatter
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    const int nS = P.nS;
    const int q_me = G.sub / SPAN;
    const bool writer = (G.sub % SPAN) == 0;
    double nrm = 0.0;
    const int ex = in_mode == 1 ? ff_exp_x(P) : 0;
    for (int v = blockIdx.x * gpb + (int)threadIdx.x / LPV; v < P.nV; v += ngroups) {
        typename AR::Coef z[NCH];
        double a[NCH];
        if (in_mode == 1) {
            typename AR::Acc acc[NCH];
            forward_row<LPV, NCH, AR>(P, G, v, x, acc, ex);
#pragma unroll
            for (int k = 0; k < NCH; ++k) {
                a[k] = AR::val(acc[k]);
                if (ex) a[k] = a[k] * pow2(ex);
            }
        }
        // input row z (y, or the weighted residual); `first` adds the residual norm
        auto zval = [&](int k, bool first) -> double {
            const int s = G.sub + k * LPV;
            if (s >= nS) return 0.0;
            const size_t idx = (size_t)v * nS + s;
            if (in_mode == 0) return yin[idx];
            const double av = in_mode == 1 ? a[k] : ax_combine(ca, ax_a[idx], cb, ax_b[idx]);
            double r = av - yobs[idx];
            if (sqw) r *= sqw[idx];
            if (first) nrm = fma(r, r, nrm);
            return sqw ? sqw[idx] * r : r;
        };
        unsigned zmax = 0;
#pragma unroll
        for (int k = 0; k < NCH; ++k) {
            const double zz = zval(k, true);
            const unsigned h = abs_hi(zz);
            zmax = h > zmax ? h : zmax;
            z[k] = AR::coef(zz);
        }
        // range guard: a row outside float-float's range is split again, scaled (exact)
        const int ez = ff_exp_hi(group_max_u<LPV>(zmax, G.mask), P.lut_exp_adj);
        if (ez) {
#pragma unroll
            for (int k = 0; k < NCH; ++k) z[k] = AR::coef(zval(k, false) * pow2(-ez));
        }
        // IC segments -> per-segment terms l * <LUT, z> in voxel order
        if (P.nIC > 0) {
            const uint32_t beg = P.vox_ptr[v], end = P.vox_ptr[v + 1];
            for (uint32_t b = beg; b < end; b += LPV) {
                const uint32_t j = b + G.sub;
                const bool valid = j < end;
                const uint32_t o = valid ? P.seg_o[j] : 0;
                const float l = valid ? P.seg_l[j] : 0.f;
                const int cntL = min((int)(end - b), LPV);
                for (int i = 0; i < P.nIC; ++i) {
                    const uint32_t row = ((uint32_t)i * P.ndirs + o) * (uint32_t)nS;
                    for (int t0 = 0; t0 < cntL; t0 += B) {
                        const int cnt = min(B, cntL - t0);
                        auto rowf = [&](int q) { return __shfl_sync(G.mask, row, t0 + q, LPV); };
                        const typename AR::Acc tot = batch_dots<LPV, NCH, AR>(G, P.lutIC, rowf, cnt, nS, z);
                        const float lq = __shfl_sync(G.mask, l, t0 + q_me, LPV);
                        double tv = AR::val(tot);
                        if (ez) tv = tv * pow2(ez);
                        if (writer && q_me < cnt) scratch[(size_t)i * P.n + b + t0 + q_me] = (double)lq * tv;
                    }
                }
            }
        }
        if (P.nEC > 0) {
            const uint32_t beg = P.ec_ptr[v], end = P.ec_ptr[v + 1];
            for (uint32_t b = beg; b < end; b += LPV) {
                const uint32_t j = b + G.sub;
                const bool valid = j < end;
                const uint32_t o = valid ? P.ec_o[j] : 0;
                const uint32_t col = valid ? P.ec_col[j] : 0;
                const int cntL = min((int)(end - b), LPV);
                for (int i = 0; i < P.nEC; ++i) {
                    const uint32_t row = ((uint32_t)i * P.ndirs + o) * (uint32_t)nS;
                    for (int t0 = 0; t0 < cntL; t0 += B) {
                        const int cnt = min(B, cntL - t0);
                        auto rowf = [&](int q) { return __shfl_sync(G.mask, row, t0 + q, LPV); };
                        const typename AR::Acc tot = batch_dots<LPV, NCH, AR>(G, P.lutEC, rowf, cnt, nS, z);
                        const uint32_t cq = __shfl_sync(G.mask, col, t0 + q_me, LPV);
                        double tv = AR::val(tot);
                        if (ez) tv = tv * pow2(ez);
                        if (writer && q_me < cnt) xout[P.ec_base + (size_t)i * P.nE + cq] = tv;
                    }
                }
            }
        }
        if (P.nISO > 0) {
            // one dot product per ISO response, shared by the voxel's ISO elements
            const uint32_t beg = P.iso_ptr[v], end = P.iso_ptr[v + 1];
            if (beg < end) {
                for (int t0 = 0; t0 < P.nISO; t0 += B) {
                    const int cnt = min(B, P.nISO - t0);
                    auto rowf = [&](int q) { return (uint32_t)((t0 + q) * nS); };
                    const typename AR::Acc tot = batch_dots<LPV, NCH, AR>(G, P.lutISO, rowf, cnt, nS, z);
                    if (writer && q_me < cnt) {
                        double d = AR::val(tot);
                        if (ez) d = d * pow2(ez);
                        for (uint32_t e = beg; e < end; ++e)
                            xout[P.iso_base + (size_t)(t0 + q_me) * P.nISOv + P.iso_col[e]] = d;
                    }
                }
            }
        }
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

}  // namespace detail
}  // namespace cgb
