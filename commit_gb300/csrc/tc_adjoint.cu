// Reduced-precision A'*y voxel pass on the tensor cores (tcgen05, BF16 operands, FP32
// accumulation), followed by the per-fibre FP64 sums.
//
// The voxel pass of A' needs, for every item of voxel v, the dot product of its LUT row k
// with the voxel's input row z (setup_operator.py:591-710 forms one per segment).  For the
// IC compartment these are, over a tile of 128 voxels, the entries of the dense product
// G = Z * L^T (128 x every IC LUT row): the kernel loads the tile's rows of z (y, or the
// weighted residual of the FISTA gradient) once, splits them into BF16 high and low parts
// in shared memory (K-major, 64 samples per K-block), and multiplies them with the BF16
// LUT rows, 256 rows per round, into one half of tensor memory while the previous round's
// half is read back: for each IC item of the round's rows the drain warps form l * G[v, k]
// and write it to the term array at the item's column-sorted position (fpos: the items of
// a column are contiguous there, in entry order).  The IC columns are then the sums of
// their contiguous terms (deterministic, FP64 sums, as the CUDA-core path).  The EC and ISO items (one or two per voxel) are dot products of the
// same BF16 rows of z with their BF16 LUT rows on the CUDA cores, written straight to
// their column of x.
//
// Warp roles (256 threads, one CTA per SM): all threads load and split Z; warp 4's first
// lane fetches the LUT row images (bulk copies, 2 stages) and issues the MMAs; warps 0-3
// (one per TMEM lane quarter) drain the accumulators, 64 LUT rows (one K-block) at a time;
// warps 5-7 compute the EC / ISO dot products meanwhile.  Every wait is bounded
// (tc_ptx.cuh).
#include <cub/cub.cuh>

#include "operator_launch.cuh"
#include "tc_ptx.cuh"

namespace cgb {
namespace detail {
namespace {

constexpr int kAThreads = 256;
constexpr int kATile = 128;
constexpr int kARows = 256;         // LUT rows per round (one TMEM half)
constexpr int kANh = 128;           // LUT rows per MMA (N)
constexpr int kAMaxKBS = 5;         // sample K-blocks of 64: nS <= 320
constexpr int kADrainStride = 65;   // floats per drain staging row (64 columns + padding)
constexpr uint32_t kAColBits = 26;

struct TcAdjArgs {
    int nV, nS, KBS, R, NKB, ntiles, Np;
    // EC / ISO items (voxel-ordered arrays of the handle) and their BF16 LUT rows (stride Np)
    int nE, nEC, nISOv, nISO, ndirs;
    int64_t ec_base, iso_base;
    const uint32_t *ec_ptr, *ec_col, *iso_ptr, *iso_col;
    const uint16_t *ec_o;
    const __nv_bfloat16 *rows16;  // EC rows (nEC * ndirs) then ISO rows (nISO), BF16, stride Np
    const uint32_t *ent_ptr, *ent_co;
    const __half *ent_l;
    const uint32_t *ent_fpos;  // column-sorted position of each entry's term
    float l_scale;
    const __nv_bfloat16 *bimg;  // [R][KBS][2][128 x 64] swizzled
    int mode;                   // 0: z = yin; 2: r = sqw*(ca*axa + cb*axb - yobs), z = sqw*r, |r|^2 partials
    const float *yin, *axa, *axb, *yobs, *sqw;
    float ca, cb;
    float *terms;
    double *xout;
    double *partials;
    int *err;
};

__host__ __device__ constexpr size_t tca_smem_bytes(int KBS) {
    return 1024 + (size_t)KBS * 2 * 16384 + 2 * 16384 + 4 * 32 * kADrainStride * 4 + 128;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    float a[16], b[16];
    tc::tmem_ld16(taddr, a);
    tc::tmem_ld16(taddr + 16, b);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        v[i] = a[i];
        v[16 + i] = b[i];
    }
}

// dot products of row m of the tile's z (BF16 hi + lo, K-major swizzled in shared memory)
// with four BF16 LUT rows of stride Np (unused items point at a valid row and are ignored
// by the caller), FP32, samples in order, hi then lo per sample.  The chunk loop has no
// branches, so the row loads of the unrolled chunks are issued together.
__device__ __forceinline__ void z_dot_rows4(const uint8_t *a_hi, const uint8_t *a_lo, int m, int Np,
                                            const __nv_bfloat16 *const (&rp)[4], float (&acc)[4]) {
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] = 0.f;
    const uint32_t rbase = (uint32_t)(m >> 3) * 1024u + (uint32_t)(m & 7) * 128u, sw = (uint32_t)(m & 7);
    const int nch = Np >> 3;  // 8-sample chunks; Np is a multiple of 32
#pragma unroll 4
    for (int c = 0; c < nch; ++c) {
        const uint32_t off = (uint32_t)(c >> 3) * 16384u + rbase + (((uint32_t)(c & 7) ^ sw) << 4);
        const uint4 h = *reinterpret_cast<const uint4 *>(a_hi + off);
        const uint4 l = *reinterpret_cast<const uint4 *>(a_lo + off);
        uint4 w[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) w[u] = __ldg(reinterpret_cast<const uint4 *>(rp[u] + c * 8));
        const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t ww[4] = {w[u].x, w[u].y, w[u].z, w[u].w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float w0 = __uint_as_float(ww[e] << 16), w1 = __uint_as_float(ww[e] & 0xffff0000u);
                acc[u] = fmaf(__uint_as_float(hw[e] << 16), w0, acc[u]);
                acc[u] = fmaf(__uint_as_float(lw[e] << 16), w0, acc[u]);
                acc[u] = fmaf(__uint_as_float(hw[e] & 0xffff0000u), w1, acc[u]);
                acc[u] = fmaf(__uint_as_float(lw[e] & 0xffff0000u), w1, acc[u]);
            }
        }
    }
}

__global__ void __launch_bounds__(kAThreads, 1) k_adjoint_tc(const TcAdjArgs A) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t *a_hi = sm;                                  // KBS x 16384
    uint8_t *a_lo = sm + (size_t)A.KBS * 16384;          // KBS x 16384
    uint8_t *b_img = sm + (size_t)A.KBS * 2 * 16384;     // 2 x 16384
    float *dstage = reinterpret_cast<float *>(b_img + 2 * 16384);
    uint64_t *bars = reinterpret_cast<uint64_t *>(dstage + 4 * 32 * kADrainStride);
    uint64_t *bfull = bars, *bfree = bars + 2, *gfull = bars + 4, *drained = bars + 6;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 8);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&bfull[i], 1);
            tc::mbar_init(&bfree[i], 1);
            tc::mbar_init(&gfull[i], 1);
            tc::mbar_init(&drained[i], 128);
        }
        tc::mbar_init_fence();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, 512);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = tc::idesc_bf16(kATile, kANh);
    const int Q = A.R * A.KBS * 2;  // B items per tile
    constexpr uint32_t kNone = 0xffffffffu;
    // issuer state (warp 4, lane 0): items and rounds issued so far, last copy / commit per stage
    uint32_t gq = 0, rgi = 0;
    uint32_t last_b[2] = {kNone, kNone}, last_c[2] = {kNone, kNone};
    // drain state (warps 0-3): rounds drained so far, entry pipeline (see (3))
    uint32_t rgd = 0;
    uint32_t d_j0 = 0, d_j1 = 0, d_n0 = 0, d_n1 = 0;
    uint32_t d_co[8], d_fp[8];
    float d_l[8];
    bool d_primed = false;
    int bad = 0;
    double nrm = 0.0;
    // 8-sample items never straddle a row end and start 32-byte aligned when nS % 8 == 0
    auto al16 = [](const float *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    const bool vec8 = (A.nS & 7) == 0 && al16(A.yin) && al16(A.axa) && al16(A.axb) && al16(A.yobs) && al16(A.sqw);
    auto load8 = [](const float *p, size_t idx, float (&o)[8]) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(p + idx)), b = __ldg(reinterpret_cast<const float4 *>(p + idx) + 1);
        o[0] = a.x;
        o[1] = a.y;
        o[2] = a.z;
        o[3] = a.w;
        o[4] = b.x;
        o[5] = b.y;
        o[6] = b.z;
        o[7] = b.w;
    };

    for (int tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
        // (1) the tile's input rows -> BF16 hi / lo, K-major swizzled, one tile per K-block;
        // 8 samples per item, two 16-byte loads per input row when the rows allow it
        float vn = 0.f;
#pragma unroll 2
        for (int q = tid; q < A.KBS * kATile * 8; q += kAThreads) {
            const int kb = q >> 10, rem = q & 1023, m = rem >> 3, p = rem & 7, cl = p ^ (m & 7);
            const int v = tile * kATile + m;
            const int s0 = kb * 64 + cl * 8;
            float z[8];
            if (vec8 && v < A.nV && s0 < A.nS) {
                const size_t idx = (size_t)v * A.nS + s0;
                if (A.mode == 0) {
                    load8(A.yin, idx, z);
                } else {
                    float a[8], b[8], yo[8], w[8];
                    load8(A.axa, idx, a);
                    if (A.axb) load8(A.axb, idx, b);
                    load8(A.yobs, idx, yo);
                    if (A.sqw) load8(A.sqw, idx, w);
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const float av = A.axb ? ax_combine(A.ca, a[e], A.cb, b[e]) : __fmul_rn(A.ca, a[e]);
                        float r = av - yo[e];
                        if (A.sqw) r *= w[e];
                        vn = fmaf(r, r, vn);
                        z[e] = A.sqw ? w[e] * r : r;
                    }
                }
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int s = s0 + e;
                    float zz = 0.f;
                    if (v < A.nV && s < A.nS) {
                        const size_t idx = (size_t)v * A.nS + s;
                        if (A.mode == 0) {
                            zz = A.yin[idx];
                        } else {
                            const float av =
                                A.axb ? ax_combine(A.ca, A.axa[idx], A.cb, A.axb[idx]) : __fmul_rn(A.ca, A.axa[idx]);
                            float r = av - A.yobs[idx];
                            if (A.sqw) r *= A.sqw[idx];
                            vn = fmaf(r, r, vn);
                            zz = A.sqw ? A.sqw[idx] * r : r;
                        }
                    }
                    z[e] = zz;
                }
            }
            uint32_t hw[4], lw[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const __nv_bfloat162 h = __floats2bfloat162_rn(z[2 * e], z[2 * e + 1]);
                const float2 hf = __bfloat1622float2(h);
                const __nv_bfloat162 l = __floats2bfloat162_rn(z[2 * e] - hf.x, z[2 * e + 1] - hf.y);
                hw[e] = *reinterpret_cast<const uint32_t *>(&h);
                lw[e] = *reinterpret_cast<const uint32_t *>(&l);
            }
            const uint32_t off = (uint32_t)kb * 16384u + (uint32_t)(m >> 3) * 1024u + (uint32_t)(m & 7) * 128u +
                                 (uint32_t)p * 16u;
            *reinterpret_cast<uint4 *>(a_hi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4 *>(a_lo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        nrm += (double)vn;
        tc::fence_async_smem();
        __syncthreads();

        if (warp == 4) {
            // (2) issuer: LUT row images through 2 shared-memory stages, MMAs into TMEM half rg & 1
            if (lane == 0 && !bad) {
                auto issue = [&](int qi, uint32_t g) {
                    const int r = qi / (A.KBS * 2), kb = (qi / 2) % A.KBS, nh = qi & 1;
                    const uint32_t st = g & 1u;
                    tc::mbar_arrive_expect_tx(&bfull[st], 16384u);
                    tc::bulk_g2s(b_img + st * 16384, A.bimg + (((size_t)r * A.KBS + kb) * 2 + nh) * (kARows / 2 * 64),
                                 16384u, &bfull[st]);
                    last_b[st] = g;
                };
                bool ok = true;
                if (gq >= 2 && !tc::mbar_wait(&bfree[gq & 1u], ((gq >> 1) + 1u) & 1u)) ok = false;
                if (ok) issue(0, gq);
                for (int qi = 0; qi < Q && ok; ++qi) {
                    const uint32_t g = gq + (uint32_t)qi;
                    const int r = qi / (A.KBS * 2), kb = (qi / 2) % A.KBS, nh = qi & 1;
                    if (qi + 1 < Q) {
                        const uint32_t g1 = g + 1;
                        if (g1 >= 2 && !tc::mbar_wait(&bfree[g1 & 1u], ((g1 >> 1) + 1u) & 1u)) {
                            ok = false;
                            break;
                        }
                        issue(qi + 1, g1);
                    }
                    if (!tc::mbar_wait(&bfull[g & 1u], (g >> 1) & 1u)) {
                        ok = false;
                        break;
                    }
                    const uint32_t rg = rgi + (uint32_t)r;
                    if (kb == 0 && nh == 0 && rg >= 2 && !tc::mbar_wait(&drained[rg & 1u], ((rg >> 1) + 1u) & 1u)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t bb = tc::smem_u32(b_img + (g & 1u) * 16384);
                    const uint32_t ah = tc::smem_u32(a_hi + kb * 16384), al = tc::smem_u32(a_lo + kb * 16384);
                    const uint32_t d = tmem + (rg & 1u) * kARows + (uint32_t)nh * kANh;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const uint64_t db = tc::desc_sw128(bb + kk * 32);
                        tc::mma_bf16(d, tc::desc_sw128(ah + kk * 32), db, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
                        tc::mma_bf16(d, tc::desc_sw128(al + kk * 32), db, idesc, 1u);
                    }
                    tc::mma_commit(&bfree[g & 1u]);
                    last_c[g & 1u] = g;
                    if (kb == A.KBS - 1 && nh == 1) tc::mma_commit(&gfull[rg & 1u]);
                }
                if (!ok) {
                    bad = 1;
                    atomicExch(A.err, 11);
                }
                gq += (uint32_t)Q;
                rgi += (uint32_t)A.R;
            }
        } else if (warp < 4) {
            // (3) drain: each thread is one voxel (TMEM lane); items of the round's LUT rows.
            // Entry pipeline (carried across tiles): at the start of a K-block the first 8 of
            // its entries are in registers, the next K-block's first 8 start loading and the
            // offsets of the one after that too.
            const int vloc = warp * 32 + lane;
            float *row = dstage + (warp * 32 + lane) * kADrainStride;
            auto range_of = [&](int t, int k, uint32_t &b0, uint32_t &b1) {
                const size_t pb = ((size_t)t * A.NKB + k) * kATile + vloc;
                b0 = A.ent_ptr[pb];
                b1 = A.ent_ptr[pb + 1];
            };
            auto after = [&](int t, int k, int ahead, int &t2, int &k2) {
                k2 = k + ahead;
                t2 = t;
                while (k2 >= A.NKB) {
                    k2 -= A.NKB;
                    t2 += gridDim.x;
                }
                return t2 < A.ntiles;
            };
            auto load8 = [&](uint32_t j0, uint32_t j1, uint32_t (&co)[8], float (&l)[8], uint32_t (&fp)[8]) {
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    co[u] = 0xffffffffu;
                    l[u] = 0.f;
                    fp[u] = 0u;
                    if (j0 + u < j1) {
                        co[u] = __ldg(A.ent_co + j0 + u);
                        l[u] = __half2float(A.ent_l[j0 + u]);
                        fp[u] = __ldg(A.ent_fpos + j0 + u);
                    }
                }
            };
            if (!d_primed) {
                int t1, k1;
                range_of(tile, 0, d_j0, d_j1);
                load8(d_j0, d_j1, d_co, d_l, d_fp);
                d_n0 = d_n1 = 0;
                if (after(tile, 0, 1, t1, k1)) range_of(t1, k1, d_n0, d_n1);
                d_primed = true;
            }
            const float lsc = A.l_scale;
            for (int r = 0; r < A.R; ++r) {
                const uint32_t rg = rgd + (uint32_t)r;
                if (!bad && !tc::mbar_wait(&gfull[rg & 1u], (rg >> 1) & 1u)) {
                    bad = 1;
                    atomicExch(A.err, 12);
                }
                if (__any_sync(0xffffffffu, bad)) break;
                tc::tc_fence_after();
                for (int kbl = 0; kbl < kARows / 64; ++kbl) {
                    const int kbf = r * (kARows / 64) + kbl;
                    if (kbf >= A.NKB) break;
                    // next K-block's first entries and the offsets of the one after it
                    uint32_t nco[8], nfp[8];
                    float nl[8];
                    load8(d_n0, d_n1, nco, nl, nfp);
                    int t2, k2;
                    uint32_t q0 = 0, q1 = 0;
                    if (after(tile, kbf, 2, t2, k2)) range_of(t2, k2, q0, q1);
                    // the K-block's 64 columns of this voxel into its private row
                    __syncwarp();
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        float g[32];
                        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (rg & 1u) * kARows + (uint32_t)(kbl * 64 + c * 32),
                                  g);
#pragma unroll
                        for (int i = 0; i < 32; ++i) row[c * 32 + i] = g[i];
                    }
                    // the first 8 entries from registers, the rest four at a time
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const uint32_t o = d_co[u] >> kAColBits;
                        // o < 64 always holds for the layout's entries; never indexes outside the row
                        if (d_j0 + u < d_j1 && o < 64u) A.terms[d_fp[u]] = row[o] * (d_l[u] * lsc);
                    }
                    for (uint32_t j = d_j0 + 8; j < d_j1; j += 4) {
                        uint32_t co[4], fp[4];
                        float l[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            co[u] = 0xffffffffu;
                            l[u] = 0.f;
                            fp[u] = 0u;
                            if (j + u < d_j1) {
                                co[u] = __ldg(A.ent_co + j + u);
                                l[u] = __half2float(A.ent_l[j + u]);
                                fp[u] = __ldg(A.ent_fpos + j + u);
                            }
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const uint32_t o = co[u] >> kAColBits;
                            if (j + u < d_j1 && o < 64u) A.terms[fp[u]] = row[o] * (l[u] * lsc);
                        }
                    }
                    // shift the pipeline
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        d_co[u] = nco[u];
                        d_l[u] = nl[u];
                        d_fp[u] = nfp[u];
                    }
                    d_j0 = d_n0;
                    d_j1 = d_n1;
                    d_n0 = q0;
                    d_n1 = q1;
                }
                tc::tc_fence_before();
                tc::mbar_arrive(&drained[rg & 1u]);
            }
            rgd += (uint32_t)A.R;
        } else if (warp > 4) {
            // (4) EC / ISO items of the tile's voxels: dot products with the rows of z, four
            // items of a voxel at a time (their LUT rows loaded together, z read once)
            for (int m = tid - 5 * 32; m < kATile; m += kAThreads - 5 * 32) {
                const int v = tile * kATile + m;
                if (v >= A.nV) break;
                const uint32_t e0 = A.ec_ptr ? A.ec_ptr[v] : 0u, e1 = A.ec_ptr ? A.ec_ptr[v + 1] : 0u;
                const uint32_t i0 = A.iso_ptr ? A.iso_ptr[v] : 0u, i1 = A.iso_ptr ? A.iso_ptr[v + 1] : 0u;
                const int nec = (int)(e1 - e0) * A.nEC, n = nec + (int)(i1 - i0) * A.nISO;
                // item k: EC entry e0 + k / nEC and response k % nEC, then the ISO ones
                auto item = [&](int k, uint32_t &row, int64_t &col) {
                    if (k < nec) {
                        const uint32_t e = e0 + (uint32_t)(k / A.nEC);
                        const int i = k - (int)(e - e0) * A.nEC;
                        row = (uint32_t)i * (uint32_t)A.ndirs + A.ec_o[e];
                        col = A.ec_base + A.ec_col[e] + (int64_t)i * A.nE;
                    } else {
                        const int kk = k - nec;
                        const uint32_t e = i0 + (uint32_t)(kk / A.nISO);
                        const int i = kk - (int)(e - i0) * A.nISO;
                        row = (uint32_t)(A.nEC * A.ndirs + i);
                        col = A.iso_base + A.iso_col[e] + (int64_t)i * A.nISOv;
                    }
                };
                for (int k0 = 0; k0 < n; k0 += 4) {
                    const __nv_bfloat16 *rp[4];
                    int64_t col[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        uint32_t row = 0;
                        col[u] = -1;
                        if (k0 + u < n) item(k0 + u, row, col[u]);
                        rp[u] = A.rows16 + (size_t)row * A.Np;
                    }
                    float acc[4];
                    z_dot_rows4(a_hi, a_lo, m, A.Np, rp, acc);
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (k0 + u < n) A.xout[col[u]] = (double)acc[u];
                }
            }
        }
        if (__syncthreads_or(bad)) break;
    }
    // drain (a no-op after a normal exit) before TMEM is freed
    if (warp == 4 && lane == 0) {
        for (int st = 0; st < 2; ++st) {
            if (last_b[st] != kNone && !tc::mbar_wait(&bfull[st], (last_b[st] >> 1) & 1u)) atomicExch(A.err, 13);
            if (last_c[st] != kNone && !tc::mbar_wait(&bfree[st], (last_c[st] >> 1) & 1u)) atomicExch(A.err, 14);
        }
    }
    if (A.partials) block_sum_store(nrm, A.partials + (size_t)blockIdx.x * kRedSlots);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// x[c] = eval[c] * sum of IC column c's terms (stored contiguously, in entry order, at
// [fptr[c], fptr[c + 1])), FP64 sums; the columns in the order of their first entry (ford)
__global__ void k_fibre_sum_entries(const uint32_t *__restrict__ fptr, const uint32_t *__restrict__ ford,
                                    const float *__restrict__ terms, const uint32_t *__restrict__ eval, int64_t ncols,
                                    double *__restrict__ xout) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ncols;
         q += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = ford[q];
        const uint32_t e = fptr[c + 1];
        uint32_t k = fptr[c];
        double s = 0.0;
        for (; k + 8 <= e; k += 8) {
            float t[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) t[u] = __ldg(terms + k + u);
#pragma unroll
            for (int u = 0; u < 8; ++u) s += (double)t[u];
        }
        for (; k < e; ++k) s += (double)__ldg(terms + k);
        xout[c] = s * (double)eval[c];
    }
}

}  // namespace
}  // namespace detail

using namespace detail;

int adjoint_tc(cgb_op *op, int mode, const float *yin, const float *axa, const float *axb, float ca, float cb,
               const float *yobs, const float *sqw, double *xout, double *partials, cudaStream_t st, int *grid) {
    CGB_TRY(ensure_tc(op));
    if (grid) *grid = 0;
    static bool attr_set[64] = {false};
    if (op->device >= 0 && op->device < 64 && !attr_set[op->device]) {
        CGB_CUDA(cudaFuncSetAttribute(k_adjoint_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)tca_smem_bytes(kAMaxKBS)));
        attr_set[op->device] = true;
    }
    if (op->tc_kbs > kAMaxKBS) return fail(CGB_ERR_UNSUPPORTED, "tensor-core adjoint: nS > 320");
    TcAdjArgs A;
    A.nV = op->nV;
    A.nS = op->nS;
    A.KBS = op->tc_kbs;
    A.R = op->tc_rounds;
    A.NKB = op->tc_nkb;
    A.ntiles = op->tc_ntiles;
    A.Np = op->tc_np;
    const bool ec = op->nE > 0 && op->nEC > 0, iso = op->nISOv > 0 && op->nISO > 0;
    const OpDev P = op->dev();
    A.nE = op->nE;
    A.nEC = ec ? op->nEC : 0;
    A.nISOv = op->nISOv;
    A.nISO = iso ? op->nISO : 0;
    A.ndirs = op->ndirs;
    A.ec_base = P.ec_base;
    A.iso_base = P.iso_base;
    A.ec_ptr = ec ? op->ec_ptr : nullptr;
    A.ec_col = op->ec_col;
    A.ec_o = op->ec_o;
    A.iso_ptr = iso ? op->iso_ptr : nullptr;
    A.iso_col = op->iso_col;
    A.rows16 = op->tc_rows16;
    A.ent_ptr = op->tc_ptr;
    A.ent_co = op->tc_co;
    A.ent_l = op->tc_l;
    A.ent_fpos = op->tc_fpos;
    A.l_scale = op->tc_lscale;
    A.bimg = op->tc_abimg;
    A.mode = mode;
    A.yin = yin;
    A.axa = axa;
    A.axb = axb;
    A.yobs = yobs;
    A.sqw = sqw;
    A.ca = ca;
    A.cb = cb;
    A.terms = op->tc_terms;
    A.xout = xout;
    A.partials = partials;
    A.err = op->tc_err;
    int g = op->nsm < A.ntiles ? op->nsm : A.ntiles;
    if (g > reduction_blocks(op)) g = reduction_blocks(op);
    k_adjoint_tc<<<g, kAThreads, tca_smem_bytes(A.KBS), st>>>(A);
    CGB_CUDA(cudaGetLastError());
    const int64_t nic = (int64_t)op->nF * op->nIC;
    if (nic > 0) {
        int64_t gb = (nic + 255) / 256;
        if (gb > (int64_t)op->nsm * 16) gb = (int64_t)op->nsm * 16;
        k_fibre_sum_entries<<<(int)gb, 256, 0, st>>>(op->tc_fptr, op->tc_ford, op->tc_terms, op->eval, nic, xout);
        CGB_CUDA(cudaGetLastError());
    }
    if (grid) *grid = g;
    return CGB_OK;
}

}  // namespace cgb
