// Reduced-precision A*x and A'*y: LUT in BF16 or FP16 (or FP32), segment lengths in FP16,
// FP32 accumulation, FP32 row vectors (y, residual), FP64 column vectors (the FISTA state)
// and FP64 partial sums of the residual norm.
//
// Same voxel ownership and paired-sample layout as operator_pair.cuh: a lane owns sample
// pairs (2p, 2p+1), a pair of LUT entries is one 4-byte load (bf16x2 / half2), converted to
// two FP32 values, and one packed FMA updates both accumulators.  Segment lengths are
// stored as FP16 values of l * 2^k (k chosen at creation so the largest length is near
// 2^15), which keeps them in FP16's normal range; the exact power of two is undone in the
// coefficient.  The per-segment A' terms go to an FP32 scratch stream and are summed per
// fibre in FP64.
#pragma once
#include "operator_pair.cuh"

namespace cgb {
namespace detail {

template <class LT>
struct LutPair;

template <>
struct LutPair<__nv_bfloat16> {
    __device__ static __forceinline__ f2 ld(const __nv_bfloat16 *p) {
        const unsigned int u = __ldg(reinterpret_cast<const unsigned int *>(p));
        // bf16 -> f32 is a 16-bit left shift of each half
        return f2_pack(__uint_as_float(u << 16), __uint_as_float(u & 0xffff0000u));
    }
};

template <>
struct LutPair<__half> {
    __device__ static __forceinline__ f2 ld(const __half *p) {
        const unsigned int u = __ldg(reinterpret_cast<const unsigned int *>(p));
        __half2 h;
        memcpy(&h, &u, 4);
        const float2 f = __half22float2(h);
        return f2_pack(f.x, f.y);
    }
};

template <>
struct LutPair<float> {
    __device__ static __forceinline__ f2 ld(const float *p) { return f2_ldg(p); }
};

// One compartment for the reduced-precision kernels (see Comp in operator_pair.cuh); the
// LUT rows are of type LT and IC lengths may come as scaled FP16 values.
template <class LT>
struct CompM {
    const uint32_t *ptr, *col;
    const uint16_t *o;
    const float *l;          // FP32 lengths (or null)
    const __half *l16;       // FP16 lengths * 2^k (or null)
    float l16_scale;         // 2^-k
    const uint32_t *eval;
    const LT *lut;
    int64_t xbase, xstride;
    uint32_t rf_stride;
    int nrf;
    int to_scratch;
};

template <class LT>
struct CompsM {
    CompM<LT> c[3];
    int n;
    int nSp;
};

template <class LT, int LPV, int NP>
__device__ __forceinline__ void forward_row_mix(const CompsM<LT> &C, const Group<LPV> &G, int v,
                                                const double *__restrict__ x, f2 (&acc)[NP]) {
#pragma unroll
    for (int k = 0; k < NP; ++k) acc[k] = 0ull;
    const int base = 2 * G.sub;
#pragma unroll 1
    for (int ci = 0; ci < C.n; ++ci) {
        const CompM<LT> &cm = C.c[ci];
        const uint32_t beg = cm.ptr[v], end = cm.ptr[v + 1];
#pragma unroll 1
        for (uint32_t b = beg; b < end; b += LPV) {
            const uint32_t j = b + G.sub;
            const bool valid = j < end;
            uint32_t col = 0, o = 0;
            float l = 1.f;
            if (valid) {
                col = cm.col[j];
                if (cm.o) o = cm.o[j];
                if (cm.l16) l = __half2float(cm.l16[j]) * cm.l16_scale;
                else if (cm.l) l = cm.l[j];
            }
            const int cntL = min((int)(end - b), LPV);
            bool head, tail;
            run_flags<LPV>(G, valid, o, cntL, head, tail);
            const unsigned tails = group_bits<LPV>(__ballot_sync(G.mask, tail));
#pragma unroll 1
            for (int i = 0; i < cm.nrf; ++i) {
                float c = 0.f;
                if (valid) {
                    const int64_t q = (int64_t)i * cm.xstride + col;
                    c = l * (float)x[cm.xbase + q];
                    if (cm.eval) c *= (float)cm.eval[q];
                }
                int start = head;
#pragma unroll
                for (int d = 1; d < LPV; d <<= 1) {
                    const float u = __shfl_up_sync(G.mask, c, d, LPV);
                    const int us = __shfl_up_sync(G.mask, start, d, LPV);
                    if (G.sub >= d) {
                        if (!start) c += u;
                        start |= us;
                    }
                }
                const uint32_t row = (uint32_t)i * cm.rf_stride + o * (uint32_t)C.nSp;
                unsigned m = tails;
#pragma unroll 1
                while (m) {
                    const int t = __ffs(m) - 1;
                    m &= m - 1;
                    const float ct = __shfl_sync(G.mask, c, t, LPV);
                    const uint32_t rt = __shfl_sync(G.mask, row, t, LPV);
                    if (ct != 0.f) {
                        const f2 c2 = f2_pack(ct, ct);
                        const LT *L = cm.lut + rt + base;
#pragma unroll
                        for (int k = 0; k < NP; ++k) acc[k] = f2_fma(c2, LutPair<LT>::ld(L + 2 * LPV * k), acc[k]);
                    }
                }
            }
        }
    }
}

// y = A x (float rows); optional ax_out; optional FP64 partials of |sqw*(Ax - yobs)|^2
template <class LT, int LPV, int NP, int MINB = 1>
__global__ void __launch_bounds__(kBlock, MINB) k_forward_mix(const int nV, const int nS, const __grid_constant__ CompsM<LT> C,
                                                        const double *__restrict__ x, float *__restrict__ yout,
                                                        float *__restrict__ axout, const float *__restrict__ yobs,
                                                        const float *__restrict__ sqw, double *__restrict__ partials) {
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    double nrm = 0.0;
    for (int v = blockIdx.x * gpb + (int)threadIdx.x / LPV; v < nV; v += ngroups) {
        f2 acc[NP];
        forward_row_mix<LT, LPV, NP>(C, G, v, x, acc);
        float vn = 0.f;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            float a[2];
            f2_unpack(acc[k], a[0], a[1]);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int s = 2 * (G.sub + k * LPV) + u;
                if (s < nS) {
                    const size_t idx = (size_t)v * nS + s;
                    if (yout) yout[idx] = a[u];
                    if (axout) axout[idx] = a[u];
                    if (partials) {
                        float r = yobs ? a[u] - yobs[idx] : a[u];
                        if (sqw) r *= sqw[idx];
                        vn = fmaf(r, r, vn);
                    }
                }
            }
        }
        nrm += (double)vn;
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

template <int LPV, int NP, class LT, class RowFn>
__device__ __forceinline__ float batch_dots_mix(const Group<LPV> &G, const LT *__restrict__ lut, RowFn row, int cnt,
                                                const f2 (&z)[NP]) {
    constexpr int B = LPV < 8 ? LPV : 8;
    f2 Pq[B];
    const int base = 2 * G.sub;
#pragma unroll
    for (int q = 0; q < B; ++q) {
        Pq[q] = 0ull;
        if (q < cnt) {
            const LT *L = lut + row(q) + base;
#pragma unroll
            for (int k = 0; k < NP; ++k) Pq[q] = f2_fma(LutPair<LT>::ld(L + 2 * LPV * k), z[k], Pq[q]);
        }
    }
#pragma unroll
    for (int h = B / 2, m = LPV / 2; h >= 1; h /= 2, m /= 2) {
        const bool hi = (G.sub & m) != 0;
#pragma unroll
        for (int j = 0; j < h; ++j) {
            const f2 send = hi ? Pq[j] : Pq[j + h];
            const f2 keep = hi ? Pq[j + h] : Pq[j];
            Pq[j] = f2_add(keep, __shfl_xor_sync(G.mask, send, m, LPV));
        }
    }
#pragma unroll
    for (int m = LPV / B / 2; m >= 1; m /= 2) Pq[0] = f2_add(Pq[0], __shfl_xor_sync(G.mask, Pq[0], m, LPV));
    float a, b;
    f2_unpack(Pq[0], a, b);
    return a + b;
}

// A' pass 1.  in_mode 0: z = yin; 1: z = sqw*r, r = sqw*(A x - yobs) (FP64 norm partials);
// 2: as 1 with A x = ca*ax_a + cb*ax_b.  IC terms -> scr (FP32), EC/ISO -> xout (FP64).
template <class LT, int LPV, int NP, int MINB = 1, bool FUSED = true>
__global__ void __launch_bounds__(kBlock, MINB) k_adjoint_mix(const int v0, const int nV, const int nS, const int64_t n,
                                                        const __grid_constant__ CompsM<LT> C,
                                                        const float *__restrict__ yin, int in_mode,
                                                        const double *__restrict__ x, const float *__restrict__ yobs,
                                                        const float *__restrict__ sqw,
                                                        const float *__restrict__ ax_a, const float *__restrict__ ax_b,
                                                        float ca, float cb, float *__restrict__ scr,
                                                        double *__restrict__ xout, double *__restrict__ partials) {
    constexpr int B = LPV < 8 ? LPV : 8;
    constexpr int SPAN = LPV / B;
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    double nrm = 0.0;
    for (int v = v0 + blockIdx.x * gpb + (int)threadIdx.x / LPV; v < nV; v += ngroups) {
        f2 acc[NP];
        if (FUSED && in_mode == 1) forward_row_mix<LT, LPV, NP>(C, G, v, x, acc);
        f2 z[NP];
        float vn = 0.f;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            float a[2] = {0.f, 0.f}, zz[2] = {0.f, 0.f};
            if (in_mode == 1) f2_unpack(acc[k], a[0], a[1]);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int s = 2 * (G.sub + k * LPV) + u;
                if (s < nS) {
                    const size_t idx = (size_t)v * nS + s;
                    if (in_mode == 0) {
                        zz[u] = yin[idx];
                    } else {
                        const float av = in_mode == 1 ? a[u] : ax_combine(ca, ax_a[idx], cb, ax_b[idx]);
                        float r = av - yobs[idx];
                        if (sqw) r *= sqw[idx];
                        vn = fmaf(r, r, vn);
                        zz[u] = sqw ? sqw[idx] * r : r;
                    }
                }
            }
            z[k] = f2_pack(zz[0], zz[1]);
        }
        nrm += (double)vn;
#pragma unroll 1
        for (int ci = 0; ci < C.n; ++ci) {
            const CompM<LT> &cm = C.c[ci];
            const uint32_t beg = cm.ptr[v], end = cm.ptr[v + 1];
#pragma unroll 1
            for (uint32_t b = beg; b < end; b += LPV) {
                const uint32_t j = b + G.sub;
                const bool valid = j < end;
                uint32_t col = 0, o = 0;
                float l = 1.f;
                if (valid) {
                    col = cm.col[j];
                    if (cm.o) o = cm.o[j];
                    if (cm.l16) l = __half2float(cm.l16[j]) * cm.l16_scale;
                    else if (cm.l) l = cm.l[j];
                }
                const int cntL = min((int)(end - b), LPV);
                bool head, tail;
                run_flags<LPV>(G, valid, o, cntL, head, tail);
                const unsigned tails = group_bits<LPV>(__ballot_sync(G.mask, tail));
                const int K = __popc(tails);
                const unsigned at_or_after = tails & (0xffffffffu << G.sub);
                const int my_tail = __ffs(at_or_after) - 1;
                const int my_item = my_tail >= 0 ? __popc(tails & ((1u << my_tail) - 1u)) : -1;
#pragma unroll 1
                for (int i = 0; i < cm.nrf; ++i) {
                    const uint32_t row = (uint32_t)i * cm.rf_stride + o * (uint32_t)C.nSp;
                    unsigned rest = tails;
#pragma unroll 1
                    for (int u0 = 0; u0 < K; u0 += B) {
                        const int cnt = min(B, K - u0);
                        // lanes of items u0 .. u0+B-1: the lowest remaining tail bits
                        int src[B];
                        unsigned mrem = rest;
#pragma unroll
                        for (int q = 0; q < B; ++q) {
                            src[q] = mrem ? __ffs(mrem) - 1 : 0;
                            mrem &= mrem - 1;
                        }
                        rest = mrem;
                        auto rowf = [&](int q) { return __shfl_sync(G.mask, row, src[q], LPV); };
                        const float tot = batch_dots_mix<LPV, NP, LT>(G, cm.lut, rowf, cnt, z);
                        const int q = my_item - u0;
                        const bool mine = valid && q >= 0 && q < cnt;
                        const float t = __shfl_sync(G.mask, tot, mine ? q * SPAN : 0, LPV);
                        if (mine) {
                            if (cm.to_scratch) scr[(size_t)i * n + j] = l * t;
                            else xout[cm.xbase + (size_t)i * cm.xstride + col] = (double)t;
                        }
                    }
                }
            }
        }
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

}  // namespace detail
}  // namespace cgb
