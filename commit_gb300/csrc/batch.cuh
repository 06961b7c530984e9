// Multi-right-hand-side reduced-precision operator: R column vectors through one dictionary
// pass.  Each segment's metadata and LUT row are loaded once and applied to R coefficients,
// so the LUT traffic per FMA drops R-fold (the single-vector reduced kernels are bound by
// those loads).  Vectors: X as R separate FP64 columns (the solvers' state), rows as R
// separate FP32 arrays; FP32 accumulation, FP64 partial sums of the residual norms (one
// slot per vector).
#pragma once
#include "operator_mixed.cuh"

namespace cgb {
namespace detail {

template <class LT, int LPV, int NP, int R>
__device__ __forceinline__ void forward_row_R(const CompsM<LT> &C, const Group<LPV> &G, int v, const RhsPtrs &V,
                                              f2 (&acc)[R][NP]) {
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int k = 0; k < NP; ++k) acc[r][k] = 0ull;
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
            const int cnt = min((int)(end - b), LPV);
#pragma unroll 1
            for (int i = 0; i < cm.nrf; ++i) {
                float c[R];
                const int64_t q = (int64_t)i * cm.xstride + col;
                const float ev = (valid && cm.eval) ? (float)cm.eval[q] : 1.f;
#pragma unroll
                for (int r = 0; r < R; ++r) c[r] = (valid && V.active[r]) ? l * (float)V.x[r][cm.xbase + q] * ev : 0.f;
                const uint32_t row = (uint32_t)i * cm.rf_stride + o * (uint32_t)C.nSp;
#pragma unroll 1
                for (int t = 0; t < cnt; ++t) {
                    float ct[R];
                    bool any = false;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        ct[r] = __shfl_sync(G.mask, c[r], t, LPV);
                        any |= ct[r] != 0.f;
                    }
                    const uint32_t rt = __shfl_sync(G.mask, row, t, LPV);
                    if (any) {
                        const LT *L = cm.lut + rt + base;
#pragma unroll
                        for (int k = 0; k < NP; ++k) {
                            const f2 l2 = LutPair<LT>::ld(L + 2 * LPV * k);
#pragma unroll
                            for (int r = 0; r < R; ++r) acc[r][k] = f2_fma(f2_pack(ct[r], ct[r]), l2, acc[r][k]);
                        }
                    }
                }
            }
        }
    }
}

// per-vector residual norms go to partials[block*kRedSlots + r]
template <int R>
__device__ __forceinline__ void block_sum_store_R(double (&v)[R], double *dst) {
    __shared__ double red[R][kBlock / 32];
#pragma unroll
    for (int r = 0; r < R; ++r) {
#pragma unroll
        for (int o = 16; o; o >>= 1) v[r] += __shfl_xor_sync(0xffffffffu, v[r], o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) red[r][threadIdx.x >> 5] = v[r];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            double t = threadIdx.x < kBlock / 32 ? red[r][threadIdx.x] : 0.0;
#pragma unroll
            for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) dst[r] = t;
        }
    }
}

template <class LT, int LPV, int NP, int R>
__global__ void __launch_bounds__(kBlock) k_forward_R(const int nV, const int nS, const __grid_constant__ CompsM<LT> C,
                                                      const __grid_constant__ RhsPtrs V, const float *__restrict__ yobs,
                                                      const float *__restrict__ sqw, double *__restrict__ partials) {
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    double nrm[R];
#pragma unroll
    for (int r = 0; r < R; ++r) nrm[r] = 0.0;
    for (int v = blockIdx.x * gpb + (int)threadIdx.x / LPV; v < nV; v += ngroups) {
        f2 acc[R][NP];
        forward_row_R<LT, LPV, NP, R>(C, G, v, V, acc);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (!V.active[r]) continue;
            float vn = 0.f;
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                float a[2];
                f2_unpack(acc[r][k], a[0], a[1]);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int s = 2 * (G.sub + k * LPV) + u;
                    if (s < nS) {
                        const size_t idx = (size_t)v * nS + s;
                        if (V.y[r]) V.y[r][idx] = a[u];
                        if (V.ax[r]) V.ax[r][idx] = a[u];
                        if (partials) {
                            float rr = yobs ? a[u] - yobs[idx] : a[u];
                            if (sqw) rr *= sqw[idx];
                            vn = fmaf(rr, rr, vn);
                        }
                    }
                }
            }
            nrm[r] += (double)vn;
        }
    }
    if (partials) block_sum_store_R<R>(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

// A' pass 1 for R vectors.  in_mode 0: z_r = yin_r; 1: z_r from the fused forward
// (r = sqw*(A x_r - yobs), FP64 norm partials per vector); 2: A x_r = ca_r*axa_r + cb_r*axb_r.
template <class LT, int LPV, int NP, int R, int MINB = 1, bool FUSED = true>
__global__ void __launch_bounds__(kBlock, MINB) k_adjoint_R(const int v0, const int nV, const int nS, const int64_t n,
                                                      const __grid_constant__ CompsM<LT> C,
                                                      const __grid_constant__ RhsPtrs V, int in_mode,
                                                      const float *__restrict__ yobs, const float *__restrict__ sqw,
                                                      double *__restrict__ partials) {
    constexpr int B = LPV < 4 ? LPV : 4;
    constexpr int SPAN = LPV / B;
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    const int q_me = G.sub / SPAN;
    const bool writer = (G.sub % SPAN) == 0;
    double nrm[R];
#pragma unroll
    for (int r = 0; r < R; ++r) nrm[r] = 0.0;
    for (int v = v0 + blockIdx.x * gpb + (int)threadIdx.x / LPV; v < nV; v += ngroups) {
        f2 z[R][NP];
        {
            f2 acc[R][NP];
            if (FUSED && in_mode == 1) forward_row_R<LT, LPV, NP, R>(C, G, v, V, acc);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                float vn = 0.f;
#pragma unroll
                for (int k = 0; k < NP; ++k) {
                    float a[2] = {0.f, 0.f}, zz[2] = {0.f, 0.f};
                    if (FUSED && in_mode == 1) f2_unpack(acc[r][k], a[0], a[1]);
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int s = 2 * (G.sub + k * LPV) + u;
                        if (s < nS && V.active[r]) {
                            const size_t idx = (size_t)v * nS + s;
                            if (in_mode == 0) {
                                zz[u] = V.yin[r][idx];
                            } else {
                                const float av = in_mode == 1 ? a[u] : V.ca[r] * V.axa[r][idx] + V.cb[r] * V.axb[r][idx];
                                float rr = av - yobs[idx];
                                if (sqw) rr *= sqw[idx];
                                vn = fmaf(rr, rr, vn);
                                zz[u] = sqw ? sqw[idx] * rr : rr;
                            }
                        }
                    }
                    z[r][k] = f2_pack(zz[0], zz[1]);
                }
                nrm[r] += (double)vn;
            }
        }
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
#pragma unroll 1
                for (int i = 0; i < cm.nrf; ++i) {
                    const uint32_t row = (uint32_t)i * cm.rf_stride + o * (uint32_t)C.nSp;
#pragma unroll 1
                    for (int t0 = 0; t0 < cntL; t0 += B) {
                        const int cnt = min(B, cntL - t0);
                        // partial dots of B items against R vectors
                        f2 Pq[B][R];
                        const int base = 2 * G.sub;
#pragma unroll
                        for (int q = 0; q < B; ++q) {
#pragma unroll
                            for (int r = 0; r < R; ++r) Pq[q][r] = 0ull;
                            if (q < cnt) {
                                const uint32_t rq = __shfl_sync(G.mask, row, t0 + q, LPV);
                                const LT *L = cm.lut + rq + base;
#pragma unroll
                                for (int k = 0; k < NP; ++k) {
                                    const f2 l2 = LutPair<LT>::ld(L + 2 * LPV * k);
#pragma unroll
                                    for (int r = 0; r < R; ++r) Pq[q][r] = f2_fma(l2, z[r][k], Pq[q][r]);
                                }
                            }
                        }
                        // reduce-scatter over the group, all R vectors together
#pragma unroll
                        for (int h = B / 2, m = LPV / 2; h >= 1; h /= 2, m /= 2) {
                            const bool hi = (G.sub & m) != 0;
#pragma unroll
                            for (int jj = 0; jj < h; ++jj)
#pragma unroll
                                for (int r = 0; r < R; ++r) {
                                    const f2 send = hi ? Pq[jj][r] : Pq[jj + h][r];
                                    const f2 keep = hi ? Pq[jj + h][r] : Pq[jj][r];
                                    Pq[jj][r] = f2_add(keep, __shfl_xor_sync(G.mask, send, m, LPV));
                                }
                        }
#pragma unroll
                        for (int m = SPAN / 2; m >= 1; m /= 2)
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                Pq[0][r] = f2_add(Pq[0][r], __shfl_xor_sync(G.mask, Pq[0][r], m, LPV));
                        const float lq = __shfl_sync(G.mask, l, t0 + q_me, LPV);
                        const uint32_t cq = __shfl_sync(G.mask, col, t0 + q_me, LPV);
                        if (writer && q_me < cnt) {
#pragma unroll
                            for (int r = 0; r < R; ++r) {
                                if (!V.active[r]) continue;
                                float a, bb;
                                f2_unpack(Pq[0][r], a, bb);
                                const float tot = a + bb;
                                if (cm.to_scratch) V.scr[r][(size_t)i * n + b + t0 + q_me] = lq * tot;
                                else V.xout[r][cm.xbase + (size_t)i * cm.xstride + cq] = (double)tot;
                            }
                        }
                    }
                }
            }
        }
    }
    if (partials) block_sum_store_R<R>(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

}  // namespace detail
}  // namespace cgb
