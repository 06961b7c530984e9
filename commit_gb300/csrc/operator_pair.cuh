// Float-float A*x and A'*y kernels on packed FP32 pairs (Blackwell f32x2 instructions).
//
// Same voxel ownership as operator_kernels.cuh, but each lane owns PAIRS of samples
// (2p, 2p+1) for p = sub + k*LPV, k < NP, and every float-float operation is issued as one
// f32x2 instruction acting on both samples.  The LUT rows used here are a zero-padded copy
// with row stride nSp = 2*LPV*NP >= nS, so loads are aligned 8-byte loads with no bounds
// guards and padded samples contribute zeros.  Per term the arithmetic is the exact
// two-product (FMA) and two-sum of the scalar float-float policy -- 11 FP32 operations --
// but issued as 5.5 instructions, which is what the FP32 pipes need to approach their
// throughput instead of being limited by instruction issue.
#pragma once
#include "operator_kernels.cuh"

namespace cgb {
namespace detail {

typedef unsigned long long f2;  // two packed FP32 words: low = even sample, high = odd

__device__ __forceinline__ f2 f2_pack(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2 f2_ldg(const float *p) {
    return __ldg(reinterpret_cast<const unsigned long long *>(p));
}

// float-float accumulator of two samples
struct DD2 {
    f2 s, e;
};

// coefficient c = h + l split in FP32, broadcast to both halves, with -h precomputed
struct Coef2 {
    f2 nh, h, l;
};

__device__ __forceinline__ Coef2 coef2(float h, float l) {
    Coef2 c;
    c.h = f2_pack(h, h);
    c.l = f2_pack(l, l);
    c.nh = f2_pack(-h, -h);
    return c;
}

// a += (c.h + c.l) * L on both halves: exact two-product of the high word (the product
// is formed negated so the FMA yields its rounding error directly) and a two-sum.
__device__ __forceinline__ void dd2_fma(DD2 &a, const Coef2 &c, f2 L) {
    const f2 pn = f2_mul(c.nh, L);
    f2 e = f2_fma(c.h, L, pn);
    e = f2_fma(c.l, L, e);
    const f2 s = f2_sub(a.s, pn);
    const f2 bb = f2_sub(s, a.s);
    const f2 t2 = f2_sub(a.s, f2_sub(s, bb));
    const f2 t3 = f2_add(pn, bb);
    const f2 err = f2_sub(t2, t3);
    a.e = f2_add(a.e, f2_add(err, e));
    a.s = s;
}

__device__ __forceinline__ void dd2_add(DD2 &a, const DD2 &b) {
    const f2 s = f2_add(a.s, b.s);
    const f2 bb = f2_sub(s, a.s);
    const f2 t2 = f2_sub(a.s, f2_sub(s, bb));
    const f2 t3 = f2_sub(b.s, bb);
    a.e = f2_add(f2_add(a.e, b.e), f2_add(t2, t3));
    a.s = s;
}

__device__ __forceinline__ void dd2_zero(DD2 &a) {
    a.s = 0ull;
    a.e = 0ull;
}

// the two halves as doubles
__device__ __forceinline__ void dd2_val(const DD2 &a, double &v0, double &v1) {
    float s0, s1, e0, e1;
    f2_unpack(a.s, s0, s1);
    f2_unpack(a.e, e0, e1);
    v0 = (double)s0 + (double)e0;
    v1 = (double)s1 + (double)e1;
}

// sum of the two halves (scalar float-float) as a double
__device__ __forceinline__ double dd2_hsum(const DD2 &a) {
    float s0, s1, e0, e1;
    f2_unpack(a.s, s0, s1);
    f2_unpack(a.e, e0, e1);
    ArFF::Acc x{s0, e0}, y{s1, e1};
    ArFF::add(x, y);
    return ArFF::val(x);
}

__device__ __forceinline__ DD2 dd2_shfl_xor(unsigned m, const DD2 &a, int lm, int w) {
    DD2 r;
    r.s = __shfl_xor_sync(m, a.s, lm, w);
    r.e = __shfl_xor_sync(m, a.e, lm, w);
    return r;
}

__device__ __forceinline__ void split2(double a, double b, f2 &h, f2 &l, f2 &nh) {
    const float ha = __double2float_rn(a), hb = __double2float_rn(b);
    const float la = __double2float_rn(a - (double)ha), lb = __double2float_rn(b - (double)hb);
    h = f2_pack(ha, hb);
    l = f2_pack(la, lb);
    nh = f2_pack(-ha, -hb);
}

// Padded-row view of the LUTs
struct PadLut {
    const float *ic, *ec, *iso;
    int nSp;
};

// One compartment's items as the voxel kernels see them.  Item j of voxel v is in
// [ptr[v], ptr[v+1]); its column for response i is xbase + i*xstride + col[j], its LUT row
// is lut + i*rf_stride + o[j]*nSp.  Null o / l / eval mean orientation 0, length 1, eval 1.
struct Comp {
    const uint32_t *ptr, *col;
    const uint16_t *o;
    const float *l;
    const uint32_t *eval;
    const float *lut;
    int64_t xbase, xstride;
    uint32_t rf_stride;
    int nrf;
    int to_scratch;  // A': per-segment terms l*<L,y> go to the scratch stream (IC)
};

struct Comps {
    Comp c[3];
    int n;
    int nSp;
};

__device__ __forceinline__ void ff_add(float &h, float &l, float bh, float bl) {
    const float s = __fadd_rn(h, bh);
    const float bb = __fsub_rn(s, h);
    const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    l = __fadd_rn(l, __fadd_rn(bl, err));
    h = s;
}

template <int LPV>
__device__ __forceinline__ unsigned group_bits(unsigned ballot) {
    const unsigned shift = (threadIdx.x & 31) & ~(LPV - 1);
    return LPV == 32 ? ballot : (ballot >> shift) & ((1u << LPV) - 1u);
}

// Items of a batch are sorted by orientation within the voxel, so equal rows are adjacent:
// head = first item of a run of equal orientation, tail = last one.
template <int LPV>
__device__ __forceinline__ void run_flags(const Group<LPV> &G, bool valid, uint32_t o, int cntL, bool &head,
                                          bool &tail) {
    const uint32_t o_prev = __shfl_up_sync(G.mask, o, 1, LPV);
    const uint32_t o_next = __shfl_down_sync(G.mask, o, 1, LPV);
    head = valid && (G.sub == 0 || o_prev != o);
    tail = valid && (G.sub == cntL - 1 || o_next != o);
}

// ex: range-guard exponent of x (ff_exp_x; 0 reads x unscaled, else x * 2^-ex)
template <int LPV, int NP>
__device__ __forceinline__ void forward_row_p(const Comps &C, const Group<LPV> &G, int v,
                                              const double *__restrict__ x, DD2 (&acc)[NP], int ex) {
#pragma unroll
    for (int k = 0; k < NP; ++k) dd2_zero(acc[k]);
    const int base = 2 * G.sub;
#pragma unroll 1
    for (int ci = 0; ci < C.n; ++ci) {
        const Comp &cm = C.c[ci];
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
                if (cm.l) l = cm.l[j];
            }
            const int cntL = min((int)(end - b), LPV);
            bool head, tail;
            run_flags<LPV>(G, valid, o, cntL, head, tail);
            const unsigned tails = group_bits<LPV>(__ballot_sync(G.mask, tail));
#pragma unroll 1
            for (int i = 0; i < cm.nrf; ++i) {
                float ch = 0.f, cl = 0.f;
                if (valid) {
                    const int64_t q = (int64_t)i * cm.xstride + col;
                    double xv = x[cm.xbase + q];
                    if (ex) xv = xv * pow2(-ex);
                    double c = (double)l * xv;
                    if (cm.eval) c *= (double)cm.eval[q];
                    ch = __double2float_rn(c);
                    cl = __double2float_rn(c - (double)ch);
                }
                // merged coefficient of each run (segmented inclusive scan, float-float)
                int start = head;
#pragma unroll
                for (int d = 1; d < LPV; d <<= 1) {
                    const float uh = __shfl_up_sync(G.mask, ch, d, LPV);
                    const float ul = __shfl_up_sync(G.mask, cl, d, LPV);
                    const int us = __shfl_up_sync(G.mask, start, d, LPV);
                    if (G.sub >= d) {
                        if (!start) ff_add(ch, cl, uh, ul);
                        start |= us;
                    }
                }
                const uint32_t row = (uint32_t)i * cm.rf_stride + o * (uint32_t)C.nSp;
                unsigned m = tails;
#pragma unroll 1
                while (m) {
                    const int t = __ffs(m) - 1;
                    m &= m - 1;
                    const float th = __shfl_sync(G.mask, ch, t, LPV);
                    const float tl = __shfl_sync(G.mask, cl, t, LPV);
                    const uint32_t rt = __shfl_sync(G.mask, row, t, LPV);
                    if (th != 0.f || tl != 0.f) {
                        const Coef2 cf = coef2(th, tl);
                        const float *L = cm.lut + rt + base;
#pragma unroll
                        for (int k = 0; k < NP; ++k) dd2_fma(acc[k], cf, f2_ldg(L + 2 * LPV * k));
                    }
                }
            }
        }
    }
}

template <int LPV, int NP, int MINB = 1>
__global__ void __launch_bounds__(kBlock, MINB) k_forward_p(const OpDev P, const __grid_constant__ Comps C,
                                                      const double *__restrict__ x,
                                                      double *__restrict__ yout, double *__restrict__ axout,
                                                      const double *__restrict__ yobs, const double *__restrict__ sqw,
                                                      double *__restrict__ partials, int vec_ok) {
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    const int nS = P.nS;
    // 16-byte row stores need an even row length and 16-byte aligned outputs
    const bool even = (nS & 1) == 0 && vec_ok;
    const int ex = ff_exp_x(P);
    double nrm = 0.0;
    for (int v = P.v0 + blockIdx.x * gpb + (int)threadIdx.x / LPV; v < P.nV; v += ngroups) {
        DD2 acc[NP];
        forward_row_p<LPV, NP>(C, G, v, x, acc, ex);
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            const int s = 2 * (G.sub + k * LPV);
            if (s < nS) {
                double a0, a1;
                dd2_val(acc[k], a0, a1);
                if (ex) {
                    a0 = a0 * pow2(ex);
                    a1 = a1 * pow2(ex);
                }
                const size_t idx = (size_t)v * nS + s;
                const bool two = s + 1 < nS;
                if (yout) {
                    if (two && even) *reinterpret_cast<double2 *>(yout + idx) = make_double2(a0, a1);
                    else { yout[idx] = a0; if (two) yout[idx + 1] = a1; }
                }
                if (axout) {
                    if (two && even) *reinterpret_cast<double2 *>(axout + idx) = make_double2(a0, a1);
                    else { axout[idx] = a0; if (two) axout[idx + 1] = a1; }
                }
                if (partials) {
                    double r0 = yobs ? a0 - yobs[idx] : a0;
                    if (sqw) r0 *= sqw[idx];
                    nrm = fma(r0, r0, nrm);
                    if (two) {
                        double r1 = yobs ? a1 - yobs[idx + 1] : a1;
                        if (sqw) r1 *= sqw[idx + 1];
                        nrm = fma(r1, r1, nrm);
                    }
                }
            }
        }
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

// items per reduce-scatter batch: 8, or 4 when the pair registers are many
template <int LPV, int NP>
struct PairBatch {
    static constexpr int B = LPV < (NP >= 5 ? 4 : 8) ? LPV : (NP >= 5 ? 4 : 8);
};

// <LUT row of item q, z> for the B items of a sub-batch (PairBatch); the total of item
// q = sub / (LPV/B) ends in lane sub (butterfly reduce-scatter on packed accumulators,
// halves combined at the end).
template <int LPV, int NP, class RowFn>
__device__ __forceinline__ double batch_dots_p(const Group<LPV> &G, const float *__restrict__ lut, RowFn row,
                                               int cnt, const f2 (&zh)[NP], const f2 (&zl)[NP]) {
    constexpr int B = PairBatch<LPV, NP>::B;
    DD2 Pq[B];
    const int base = 2 * G.sub;
#pragma unroll
    for (int q = 0; q < B; ++q) {
        dd2_zero(Pq[q]);
        if (q < cnt) {
            const float *L = lut + row(q) + base;
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                Coef2 zc;
                zc.h = zh[k];
                zc.l = zl[k];
                zc.nh = zh[k] ^ 0x8000000080000000ull;  // both halves negated
                dd2_fma(Pq[q], zc, f2_ldg(L + 2 * LPV * k));
            }
        }
    }
#pragma unroll
    for (int h = B / 2, m = LPV / 2; h >= 1; h /= 2, m /= 2) {
        const bool hi = (G.sub & m) != 0;
#pragma unroll
        for (int j = 0; j < h; ++j) {
            DD2 send, keep;
            send.s = hi ? Pq[j].s : Pq[j + h].s;
            send.e = hi ? Pq[j].e : Pq[j + h].e;
            keep.s = hi ? Pq[j + h].s : Pq[j].s;
            keep.e = hi ? Pq[j + h].e : Pq[j].e;
            dd2_add(keep, dd2_shfl_xor(G.mask, send, m, LPV));
            Pq[j] = keep;
        }
    }
#pragma unroll
    for (int m = LPV / PairBatch<LPV, NP>::B / 2; m >= 1; m /= 2) dd2_add(Pq[0], dd2_shfl_xor(G.mask, Pq[0], m, LPV));
    return dd2_hsum(Pq[0]);
}

// A' pass 1 over all compartments.  Per batch, one dot product per run of equal
// orientation; every item of the run takes that total: IC items write l*<L,z> to the
// per-segment scratch stream, EC / ISO items write their column of xout.
template <int LPV, int NP, int MINB = 1, bool FUSED = true>
__global__ void __launch_bounds__(kBlock, MINB) k_adjoint_p(const OpDev P, const __grid_constant__ Comps C,
                                                      const double *__restrict__ yin,
                                                      int in_mode, const double *__restrict__ x,
                                                      const double *__restrict__ yobs, const double *__restrict__ sqw,
                                                      const double *__restrict__ ax_a, const double *__restrict__ ax_b,
                                                      double ca, double cb, double *__restrict__ scratch,
                                                      double *__restrict__ xout, double *__restrict__ partials) {
    constexpr int B = PairBatch<LPV, NP>::B;
    constexpr int SPAN = LPV / B;
    const Group<LPV> G;
    const int gpb = kBlock / LPV;
    const int ngroups = gridDim.x * gpb;
    const int nS = P.nS;
    const int ex = FUSED && in_mode == 1 ? ff_exp_x(P) : 0;
    double nrm = 0.0;
    for (int v = P.v0 + blockIdx.x * gpb + (int)threadIdx.x / LPV; v < P.nV; v += ngroups) {
        double a[2 * NP];
        if (FUSED && in_mode == 1) {
            DD2 acc[NP];
            forward_row_p<LPV, NP>(C, G, v, x, acc, ex);
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                dd2_val(acc[k], a[2 * k], a[2 * k + 1]);
                if (ex) {
                    a[2 * k] = a[2 * k] * pow2(ex);
                    a[2 * k + 1] = a[2 * k + 1] * pow2(ex);
                }
            }
        }
        // element u of this lane's pair k of the input row z (y, or the weighted residual);
        // `first` adds the residual norm
        auto zval = [&](int k, int u, bool first) -> double {
            const int s = 2 * (G.sub + k * LPV) + u;
            if (s >= nS) return 0.0;
            const size_t idx = (size_t)v * nS + s;
            if (in_mode == 0) return yin[idx];
            const double av = FUSED && in_mode == 1 ? a[2 * k + u] : ax_combine(ca, ax_a[idx], cb, ax_b[idx]);
            double r = av - yobs[idx];
            if (sqw) r *= sqw[idx];
            if (first) nrm = fma(r, r, nrm);
            return sqw ? sqw[idx] * r : r;
        };
        f2 zh[NP], zl[NP];
        unsigned zmax = 0;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            const double z0 = zval(k, 0, true), z1 = zval(k, 1, true);
            const unsigned h0 = abs_hi(z0), h1 = abs_hi(z1);
            zmax = h0 > zmax ? h0 : zmax;
            zmax = h1 > zmax ? h1 : zmax;
            f2 unused;
            split2(z0, z1, zh[k], zl[k], unused);
        }
        // range guard: a row outside float-float's range is split again, scaled (exact)
        const int ez = ff_exp_hi(group_max_u<LPV>(zmax, G.mask), P.lut_exp_adj);
        if (ez) {
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                f2 unused;
                split2(zval(k, 0, false) * pow2(-ez), zval(k, 1, false) * pow2(-ez), zh[k], zl[k], unused);
            }
        }
#pragma unroll 1
        for (int ci = 0; ci < C.n; ++ci) {
            const Comp &cm = C.c[ci];
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
                    if (cm.l) l = cm.l[j];
                }
                const int cntL = min((int)(end - b), LPV);
                bool head, tail;
                run_flags<LPV>(G, valid, o, cntL, head, tail);
                const unsigned tails = group_bits<LPV>(__ballot_sync(G.mask, tail));
                const int K = __popc(tails);
                // run (item) index of this lane's segment
                const unsigned at_or_after = G.sub < 32 ? tails & (0xffffffffu << G.sub) : 0u;
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
                        const double tot = batch_dots_p<LPV, NP>(G, cm.lut, rowf, cnt, zh, zl);
                        const int q = my_item - u0;
                        const bool mine = valid && q >= 0 && q < cnt;
                        double t = __shfl_sync(G.mask, tot, mine ? q * SPAN : 0, LPV);
                        if (ez) t = t * pow2(ez);
                        if (mine) {
                            if (cm.to_scratch) scratch[(size_t)i * P.n + j] = (double)l * t;
                            else xout[cm.xbase + (size_t)i * cm.xstride + col] = t;
                        }
                    }
                }
            }
        }
    }
    if (partials) block_sum_store(nrm, partials + (size_t)blockIdx.x * kRedSlots);
}

// compartment table of a handle for the padded FP32 LUT rows
inline Comps make_comps(const cgb_op *op) {
    Comps C;
    C.n = 0;
    C.nSp = op->nSp;
    const uint32_t ndirs = (uint32_t)op->ndirs, nSp = (uint32_t)op->nSp;
    if (op->nIC > 0)
        C.c[C.n++] = Comp{op->vox_ptr, op->seg_f, op->seg_o, op->seg_l, op->eval, op->lutIC_p, 0, op->nF,
                          ndirs * nSp, op->nIC, 1};
    if (op->nEC > 0 && op->nE > 0)
        C.c[C.n++] = Comp{op->ec_ptr, op->ec_col, op->ec_o, nullptr, nullptr, op->lutEC_p,
                          (int64_t)op->nF * op->nIC, op->nE, ndirs * nSp, op->nEC, 0};
    if (op->nISO > 0 && op->nISOv > 0)
        C.c[C.n++] = Comp{op->iso_ptr, op->iso_col, nullptr, nullptr, nullptr, op->lutISO_p,
                          (int64_t)op->nF * op->nIC + (int64_t)op->nE * op->nEC, op->nISOv, nSp, op->nISO, 0};
    return C;
}

// (LPV, NP) pairs with kernels; 2*LPV*NP samples per voxel row
struct PairShape {
    int lpv, np;
};
constexpr PairShape kPairShapes[] = {{1, 1},  {2, 1},  {4, 1},  {4, 2},  {8, 1},  {8, 2},  {8, 3},  {8, 5},
                                     {16, 1}, {16, 2}, {16, 3}, {16, 5}, {16, 9}, {32, 1}, {32, 2}, {32, 3},
                                     {32, 5}, {32, 8}};

inline PairShape pick_pair_shape(int nS) {
    PairShape best = {32, 8};
    int best_slots = 1 << 30;
    for (const PairShape &s : kPairShapes) {
        const int slots = 2 * s.lpv * s.np;
        if (slots < nS) continue;
        if (slots < best_slots || (slots == best_slots && s.lpv > best.lpv)) {
            best = s;
            best_slots = slots;
        }
    }
    return best;
}

// the 32-lane shape for nS (a warp per voxel, half the samples per lane of the 16-lane
// shape): the smallest NP with 64 * NP >= nS that has kernels
inline PairShape wide_pair_shape(int nS) {
    PairShape best = {32, 8};
    for (const PairShape &s : kPairShapes)
        if (s.lpv == 32 && 2 * s.lpv * s.np >= nS && s.np < best.np) best = s;
    return best;
}

template <class Fn>
int dispatch_pair_shape(PairShape s, Fn &fn) {
#define CGB_PSHAPE(L, N) \
    if (s.lpv == L && s.np == N) return fn.template run<L, N>();
    CGB_PSHAPE(1, 1) CGB_PSHAPE(2, 1) CGB_PSHAPE(4, 1) CGB_PSHAPE(4, 2) CGB_PSHAPE(8, 1) CGB_PSHAPE(8, 2)
    CGB_PSHAPE(8, 3) CGB_PSHAPE(8, 5) CGB_PSHAPE(16, 1) CGB_PSHAPE(16, 2) CGB_PSHAPE(16, 3) CGB_PSHAPE(16, 5)
    CGB_PSHAPE(16, 9) CGB_PSHAPE(32, 1) CGB_PSHAPE(32, 2) CGB_PSHAPE(32, 3) CGB_PSHAPE(32, 5) CGB_PSHAPE(32, 8)
#undef CGB_PSHAPE
    return fail(CGB_ERR_UNSUPPORTED, "no paired kernel shape for this number of samples");
}

}  // namespace detail
}  // namespace cgb
