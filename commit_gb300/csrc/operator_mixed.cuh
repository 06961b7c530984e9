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

template <class LT>
struct MixLut {
    const LT *ic, *ec;
    const float *iso;  // ISO rows stay FP32 (nISO x nSp floats)
    int nSp;
    const __half *len16;  // scaled FP16 lengths (null: use seg_l)
    float len_inv_scale;
};

template <class LT, int LPV, int NP>
__device__ __forceinline__ void forward_row_mix(const OpDev &P, const MixLut<LT> &T, const Group<LPV> &G, int v,
                                                const double *__restrict__ x, f2 (&acc)[NP]) {
#pragma unroll
    for (int k = 0; k < NP; ++k) acc[k] = 0ull;
    const int base = 2 * G.sub;
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
                l = T.len16 ? __half2float(T.len16[j]) * T.len_inv_scale : P.seg_l[j];
            }
            const int cnt = min((int)(end - b), LPV);
            for (int i = 0; i < P.nIC; ++i) {
                float c = 0.f;
                if (valid) {
                    const size_t col = (size_t)i * P.nF + f;
                    c = l * (float)x[col] * (float)P.eval[col];
                }
                const uint32_t row = ((uint32_t)i * P.ndirs + o) * (uint32_t)T.nSp;
                for (int t = 0; t < cnt; ++t) {
                    const float ct = __shfl_sync(G.mask, c, t, LPV);
                    const uint32_t rt = __shfl_sync(G.mask, row, t, LPV);
                    if (ct != 0.f) {
                        const f2 c2 = f2_pack(ct, ct);
                        const LT *L = T.ic + rt + base;
#pragma unroll
                        for (int k = 0; k < NP; ++k) acc[k] = f2_fma(c2, LutPair<LT>::ld(L + 2 * LPV * k), acc[k]);
                    }
                }
            }
        }
    }
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
                const float c = valid ? (float)x[P.ec_base + (size_t)i * P.nE + col] : 0.f;
                const uint32_t row = ((uint32_t)i * P.ndirs + o) * (uint32_t)T.nSp;
                for (int t = 0; t < cnt; ++t) {
                    const float ct = __shfl_sync(G.mask, c, t, LPV);
                    const uint32_t rt = __shfl_sync(G.mask, row, t, LPV);
                    if (ct != 0.f) {
                        const f2 c2 = f2_pack(ct, ct);
                        const LT *L = T.ec + rt + base;
#pragma unroll
                        for (int k = 0; k < NP; ++k) acc[k] = f2_fma(c2, LutPair<LT>::ld(L + 2 * LPV * k), acc[k]);
                    }
                }
            }
        }
    }
    if (P.nISO > 0) {
        const uint32_t beg = P.iso_ptr[v], end = P.iso_ptr[v + 1];
        for (uint32_t b = beg; b < end; b += LPV) {
            const uint32_t j = b + G.sub;
            const bool valid = j < end;
            const uint32_t col = valid ? P.iso_col[j] : 0;
            const int cnt = min((int)(end - b), LPV);
            for (int i = 0; i < P.nISO; ++i) {
                const float c = valid ? (float)x[P.iso_base + (size_t)i * P.nISOv + col] : 0.f;
                for (int t = 0; t < cnt; ++t) {
                    const float ct = __shfl_sync(G.mask, c, t, LPV);
                    if (ct != 0.f) {
                        const f2 c2 = f2_pack(ct, ct);
                        const float *L = T.iso + (size_t)i * T.nSp + base;
#pragma unroll
                        for (int k = 0; k < NP; ++k) acc[k] = f2_fma(c2, f2_ldg(L + 2 * LPV * k), acc[k]);
                    }
                }
            }
        }
    }
}

// y = A x (float rows); optional ax_out; optional FP64 partials of |sqw*(Ax - yobs)|^2
template <class LT, int LPV, int NP>
__global__ void __launch_bounds__(kBlock) k_forward_mix(const OpDev P, const MixLut<LT> T,
                                                        const double *__restrict__ x, float *__restrict__ yout,
                                                        float *__restrict__ axout, const float *__restrict__ yobs,
                                                        const float *__restrict__ sqw, double *__restrict__ partials) {
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    const int nS = P.nS;
    double nrm = 0.0;
    for (int v = blockIdx.x * gpb + (int)threadIdx.x / LPV; v < P.nV; v += ngroups) {
        f2 acc[NP];
        forward_row_mix<LT, LPV, NP>(P, T, G, v, x, acc);
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
template <class LT, int LPV, int NP>
__global__ void __launch_bounds__(kBlock) k_adjoint_mix(const OpDev P, const MixLut<LT> T,
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
    const int nS = P.nS;
    const int q_me = G.sub / SPAN;
    const bool writer = (G.sub % SPAN) == 0;
    double nrm = 0.0;
    for (int v = blockIdx.x * gpb + (int)threadIdx.x / LPV; v < P.nV; v += ngroups) {
        f2 acc[NP];
        if (in_mode == 1) forward_row_mix<LT, LPV, NP>(P, T, G, v, x, acc);
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
                        const float av = in_mode == 1 ? a[u] : ca * ax_a[idx] + cb * ax_b[idx];
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
        if (P.nIC > 0) {
            const uint32_t beg = P.vox_ptr[v], end = P.vox_ptr[v + 1];
            for (uint32_t b = beg; b < end; b += LPV) {
                const uint32_t j = b + G.sub;
                const bool valid = j < end;
                const uint32_t o = valid ? P.seg_o[j] : 0;
                const float l = valid ? (T.len16 ? __half2float(T.len16[j]) * T.len_inv_scale : P.seg_l[j]) : 0.f;
                const int cntL = min((int)(end - b), LPV);
                for (int i = 0; i < P.nIC; ++i) {
                    const uint32_t row = ((uint32_t)i * P.ndirs + o) * (uint32_t)T.nSp;
                    for (int t0 = 0; t0 < cntL; t0 += B) {
                        const int cnt = min(B, cntL - t0);
                        auto rowf = [&](int q) { return __shfl_sync(G.mask, row, t0 + q, LPV); };
                        const float tot = batch_dots_mix<LPV, NP, LT>(G, T.ic, rowf, cnt, z);
                        const float lq = __shfl_sync(G.mask, l, t0 + q_me, LPV);
                        if (writer && q_me < cnt) scr[(size_t)i * P.n + b + t0 + q_me] = lq * tot;
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
                    const uint32_t row = ((uint32_t)i * P.ndirs + o) * (uint32_t)T.nSp;
                    for (int t0 = 0; t0 < cntL; t0 += B) {
                        const int cnt = min(B, cntL - t0);
                        auto rowf = [&](int q) { return __shfl_sync(G.mask, row, t0 + q, LPV); };
                        const float tot = batch_dots_mix<LPV, NP, LT>(G, T.ec, rowf, cnt, z);
                        const uint32_t cq = __shfl_sync(G.mask, col, t0 + q_me, LPV);
                        if (writer && q_me < cnt) xout[P.ec_base + (size_t)i * P.nE + cq] = (double)tot;
                    }
                }
            }
        }
        if (P.nISO > 0) {
            const uint32_t beg = P.iso_ptr[v], end = P.iso_ptr[v + 1];
            if (beg < end) {
                for (int t0 = 0; t0 < P.nISO; t0 += B) {
                    const int cnt = min(B, P.nISO - t0);
                    auto rowf = [&](int q) { return (uint32_t)((t0 + q) * T.nSp); };
                    const float tot = batch_dots_mix<LPV, NP, float>(G, T.iso, rowf, cnt, z);
                    if (writer && q_me < cnt)
                        for (uint32_t e = beg; e < end; ++e)
                            xout[P.iso_base + (size_t)(t0 + q_me) * P.nISOv + P.iso_col[e]] = (double)tot;
                }
            }
        }
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

}  // namespace detail
}  // namespace cgb
