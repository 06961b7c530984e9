// Reduced-precision A*x on the tensor cores (tcgen05, BF16 operands, FP32 accumulation).
//
// A*x is, voxel by voxel, y[v, :] = sum_k C[v, k] * L[k, :] where k runs over the LUT rows
// of every compartment and C[v, k] is the sum of l * x * eval over the voxel's items that
// use row k (setup_operator.py:50-218 computes the same sums item by item).  For the IC
// compartment (many segments per voxel, spread over every orientation) this is, over a
// tile of 128 voxels, a dense product C[128 x K] * L[K x nS]: the kernel builds C in shared
// memory 64 LUT rows at a time, splits it into BF16 high and low parts (C = hi + lo to
// about 16 bits), and multiplies both with the BF16 LUT on the tensor cores into one FP32
// accumulator of 128 x nS in tensor memory.  The EC and ISO compartments have one or two
// items per voxel, which would leave their K-blocks nearly empty; the epilogue adds them
// on the CUDA cores (x * BF16 LUT row, FP32 FMAs in item order) to the accumulator rows it
// reads back.  The LUT is the only reduced-precision operand, as in the CUDA-core BF16
// path (operator_mixed.cuh).
//
// Data (built once per handle, ensure_tc):
//  - IC entries: every (segment, response) pair, ordered by (tile of 128 voxels, K-block
//    of 64 LUT rows, voxel) -- ent_co = column of x | row in the K-block << 26, ent_l =
//    FP16 length * 2^k -- and ent_ptr, the first entry of each (tile, K-block, voxel), so a
//    voxel's entries of one K-block are contiguous;
//  - B images: per K-block the LUT rows transposed to [Np samples x 64 rows] BF16 in the
//    K-major 128-byte-swizzled layout of tc_ptx.cuh, fetched whole by one bulk copy;
//  - the EC and ISO LUT rows as BF16 with row stride Np, EC first (read by the epilogue).
//
// Kernel: one CTA of 256 threads per SM (persistent over tiles), 2-stage pipeline over the
// K-blocks of a tile: while the tensor cores multiply K-block b, the threads build the C
// tile of block b+1 (two threads per voxel walk its entries into FP32 rows in shared
// memory, in order, so results are deterministic; the entry offsets of the next K-block
// are loaded one K-block ahead) and one thread fetches its B image.  The 128 x Np
// accumulator (two MMAs of N = Np/2 per 16-row K step) is read back by the 8 warps (lane
// quarter = warp % 4, column half = warp / 4), completed with the EC / ISO items and
// written to y, with the residual-norm epilogue of the CUDA-core kernel.
#include <cub/cub.cuh>

#include "operator_launch.cuh"
#include "tc_ptx.cuh"

namespace cgb {
namespace detail {
namespace {

constexpr int kTcThreads = 256;
constexpr int kTcTile = 128;           // voxels per tile (MMA M)
constexpr int kTcKB = 64;              // LUT rows per K-block
constexpr int kStageStride = 68;       // floats per FP32 staging row (64 + padding, 16-byte rows)
constexpr uint32_t kColBits = 26;      // ent_co: column in the low 26 bits
constexpr int kTcMaxNp = 320;          // padded samples the shared-memory budget allows

struct TcFwdArgs {
    int nV, nS, Np, NKB, ntiles;
    // EC / ISO items (voxel-ordered arrays of the handle) and their BF16 LUT rows
    int nE, nEC, nISOv, nISO, ndirs;
    int64_t ec_base, iso_base;
    const uint32_t *ec_ptr, *ec_col, *iso_ptr, *iso_col;
    const uint16_t *ec_o;
    const __nv_bfloat16 *rows16;  // EC rows (nEC * ndirs) then ISO rows (nISO), BF16, stride Np
    const uint32_t *ent_ptr;
    const uint32_t *ent_co;
    const __half *ent_l;
    const uint8_t *ent_vl;  // voxel of each entry within its tile
    float l_scale;
    const float *xe;
    const __nv_bfloat16 *bimg;
    float *yout, *axout;
    const float *yobs, *sqw;
    double *partials;
    int *err;
};

__host__ __device__ constexpr size_t tc_smem_bytes(int Np) {
    return 1024 /* alignment slack */ + 4 * 16384 /* A hi / lo x 2 stages */ + 2 * (size_t)Np * 128 /* B x 2 */ +
           kTcTile * kStageStride * 4 /* FP32 staging */ + 128 /* barriers, TMEM slot, flags */;
}

constexpr int kTcItems = 8;  // EC / ISO items of a voxel held in registers (more take a loop)
constexpr int kSlice = 8;    // entries of a K-block per thread and pass (kTcThreads * kSlice per pass)
constexpr int kWin = kSlice + 2;  // the entry before the slice, the slice, the entry after it

// A thread's window of entries for one pass over a K-block's range [b0, b1): entry s0 - 1,
// the slice [s0, s0 + kSlice) and entry s0 + kSlice; per entry its column | row (co) and
// its FP16 length | voxel-in-tile << 16 (lv); 0xffffffff marks an entry outside the range.
struct Window {
    uint32_t co[kWin], lv[kWin];
    __device__ __forceinline__ void load(const TcFwdArgs &A, uint32_t b0, uint32_t b1, uint32_t s0) {
#pragma unroll
        for (int i = 0; i < kWin; ++i) {
            const uint32_t j = s0 + (uint32_t)i - 1u;
            co[i] = 0xffffffffu;
            lv[i] = 0xffffffffu;
            if ((i > 0 || s0 > b0) && j < b1) {
                co[i] = __ldg(A.ent_co + j);
                lv[i] = (uint32_t)__half_as_ushort(A.ent_l[j]) | ((uint32_t)A.ent_vl[j] << 16);
            }
        }
    }
};

// cell of an entry: voxel in tile * 64 + row in the K-block (the staging index before padding)
__device__ __forceinline__ uint32_t cell_of(uint32_t co, uint32_t lv) { return ((lv >> 16) << 6) | (co >> kColBits); }

// r[0..15] += xv * the 16 BF16 values of w (two 16-byte words)
__device__ __forceinline__ void fma16(float (&r)[16], float xv, const uint4 &a, const uint4 &b) {
    const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        r[2 * i] = fmaf(xv, __uint_as_float(w[i] << 16), r[2 * i]);
        r[2 * i + 1] = fmaf(xv, __uint_as_float(w[i] & 0xffff0000u), r[2 * i + 1]);
    }
}

// The EC and ISO items of one voxel, in order (EC entries [e0, e1) x responses, then ISO
// entries [i0, i1) x responses): item k has BF16 row rows16[row(k)] and coefficient x(k).
struct VoxItems {
    uint32_t e0, e1, i0, i1;
    int n;  // items
    __device__ __forceinline__ int count(const TcFwdArgs &A) const {
        return (int)(e1 - e0) * A.nEC + (int)(i1 - i0) * A.nISO;
    }
    __device__ __forceinline__ void item(const TcFwdArgs &A, int k, uint32_t &row, float &xv) const {
        const int nec = (int)(e1 - e0) * A.nEC;
        if (k < nec) {
            const uint32_t e = e0 + (uint32_t)(k / A.nEC);
            const int i = k - (int)(e - e0) * A.nEC;
            row = (uint32_t)i * (uint32_t)A.ndirs + A.ec_o[e];
            xv = A.xe[A.ec_base + A.ec_col[e] + (int64_t)i * A.nE];
        } else {
            const int kk = k - nec;
            const uint32_t e = i0 + (uint32_t)(kk / A.nISO);
            const int i = kk - (int)(e - i0) * A.nISO;
            row = (uint32_t)(A.nEC * A.ndirs + i);
            xv = A.xe[A.iso_base + A.iso_col[e] + (int64_t)i * A.nISOv];
        }
    }
};

__global__ void __launch_bounds__(kTcThreads, 1) k_forward_tc(const TcFwdArgs A) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const uint32_t bbytes = (uint32_t)A.Np * 128u;
    uint8_t *a_hi = sm;                       // 2 x 16384
    uint8_t *a_lo = sm + 2 * 16384;           // 2 x 16384
    uint8_t *b_img = sm + 4 * 16384;          // 2 x bbytes
    float *stage = reinterpret_cast<float *>(b_img + 2 * bbytes);
    uint64_t *bars = reinterpret_cast<uint64_t *>(stage + kTcTile * kStageStride);  // bfull[2], mdone[2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 4);
    uint64_t *bfull = bars, *mdone = bars + 2;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        tc::mbar_init(&bfull[0], 1);
        tc::mbar_init(&bfull[1], 1);
        tc::mbar_init(&mdone[0], 1);
        tc::mbar_init(&mdone[1], 1);
        tc::mbar_init_fence();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, 512);
        tc::tmem_relinquish();
    }
    for (int i = tid; i < kTcTile * kStageStride; i += kTcThreads) stage[i] = 0.f;
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int half = A.Np / 2;
    const uint32_t idesc = tc::idesc_bf16(kTcTile, half);
    uint32_t it = 0;  // K-blocks processed by this CTA (pipeline stage = it & 1)
    // thread 0: iteration of the last bulk copy issued / MMA group committed per stage, for
    // draining on an early exit (kNone: none)
    constexpr uint32_t kNone = 0xffffffffu;
    uint32_t last_b[2] = {kNone, kNone}, last_c[2] = {kNone, kNone};
    const bool vec4 = (A.nS & 3) == 0 && (reinterpret_cast<uintptr_t>(A.yout) & 15) == 0 &&
                      (reinterpret_cast<uintptr_t>(A.axout) & 15) == 0;
    double nrm = 0.0;
    // a wait that ran out sets `bad` in its thread; every exit decision is taken on the OR
    // of all threads' flags at a barrier (__syncthreads_or), so all threads leave together
    int bad = 0;
    bool stop = false;

    // Entry walk.  A K-block's entries (one tile) form the range [b0, b1), sorted by cell
    // (voxel, LUT row), each cell's entries contiguous.  Each thread takes slices of
    // kSlice entries (pass p: s0 = b0 + (p * kTcThreads + tid) * kSlice) and sums, in entry
    // order, every cell whose first entry lies in its slice, reading past the slice to the
    // end of its last cell; each cell is stored once, by one thread, so the result does not
    // depend on the slicing.  Pipeline: while a K-block is walked, the x values of the next
    // one's first window and the entries of the window after that are loading.
    const uint32_t kColMask = (1u << kColBits) - 1u;
    // (tile, K-block) `ahead` blocks after (t, k) in this CTA's order; false past the end
    auto step = [&](int t, int k, int ahead, int &t2, int &k2) {
        k2 = k + ahead;
        t2 = t;
        while (k2 >= A.NKB) {
            k2 -= A.NKB;
            t2 += gridDim.x;
        }
        return t2 < A.ntiles;
    };
    auto range_of = [&](int t, int k, uint32_t &b0, uint32_t &b1) {
        const size_t pb = ((size_t)t * A.NKB + k) * kTcTile;
        b0 = A.ent_ptr[pb];
        b1 = A.ent_ptr[pb + kTcTile];
    };
    const uint32_t s_off = (uint32_t)tid * kSlice;
    Window cw, nw;  // current K-block's first window, next K-block's
    float cx[kWin];
    uint32_t cb0 = 0, cb1 = 0, nb0 = 0, nb1 = 0;
    auto load_x = [&](const Window &w, float (&x)[kWin]) {
#pragma unroll
        for (int i = 1; i < kWin; ++i) x[i] = w.co[i] != 0xffffffffu ? __ldg(A.xe + (w.co[i] & kColMask)) : 0.f;
        x[0] = 0.f;
    };
    if ((int)blockIdx.x < A.ntiles) {
        int t1, k1;
        range_of(blockIdx.x, 0, cb0, cb1);
        if (step(blockIdx.x, 0, 1, t1, k1)) range_of(t1, k1, nb0, nb1);
        cw.load(A, cb0, cb1, cb0 + s_off);
        nw.load(A, nb0, nb1, nb0 + s_off);
        load_x(cw, cx);
    }
    // the runs of one window: cells whose first entry is in the slice; returns with the
    // last one still open (cur, acc) when the slice ends inside it
    auto walk_window = [&](const Window &w, const float (&x)[kWin], uint32_t s0, uint32_t b0, uint32_t b1) {
        uint32_t cur = 0xffffffffu;
        float acc = 0.f;
        uint32_t prev = w.co[0] != 0xffffffffu ? cell_of(w.co[0], w.lv[0]) : 0xffffffffu;
#pragma unroll
        for (int i = 1; i <= kSlice; ++i) {
            if (w.co[i] == 0xffffffffu) break;
            const uint32_t c = cell_of(w.co[i], w.lv[i]);
            if (c != prev) {  // first entry of a cell
                if (cur != 0xffffffffu) stage[(cur >> 6) * kStageStride + (cur & 63u)] = acc;
                cur = c;
                acc = 0.f;
            }
            prev = c;
            if (cur != 0xffffffffu) acc += __half2float(__ushort_as_half((unsigned short)(w.lv[i] & 0xffffu))) * x[i];
        }
        if (cur == 0xffffffffu) return;
        // the open cell continues past the slice: the window's last entry, then loads
        uint32_t j = s0 + kSlice;
        if (w.co[kWin - 1] != 0xffffffffu && cell_of(w.co[kWin - 1], w.lv[kWin - 1]) == cur) {
            acc += __half2float(__ushort_as_half((unsigned short)(w.lv[kWin - 1] & 0xffffu))) * x[kWin - 1];
            for (j = s0 + kSlice + 1; j < b1; ++j) {
                const uint32_t co = __ldg(A.ent_co + j);
                if (cell_of(co, (uint32_t)A.ent_vl[j] << 16) != cur) break;
                acc += __half2float(A.ent_l[j]) * __ldg(A.xe + (co & kColMask));
            }
        }
        stage[(cur >> 6) * kStageStride + (cur & 63u)] = acc;
    };

    for (int tile = blockIdx.x; tile < A.ntiles && !stop; tile += gridDim.x) {
        // the epilogue's voxel: its EC / ISO items, the first kTcItems (row, x) loaded ahead
        // of the K-blocks
        const int ve = tile * kTcTile + (warp & 3) * 32 + lane;
        VoxItems V{0, 0, 0, 0, 0};
        if (ve < A.nV) {
            if (A.ec_ptr) {
                V.e0 = A.ec_ptr[ve];
                V.e1 = A.ec_ptr[ve + 1];
            }
            if (A.iso_ptr) {
                V.i0 = A.iso_ptr[ve];
                V.i1 = A.iso_ptr[ve + 1];
            }
        }
        V.n = V.count(A);
        uint32_t irow[kTcItems];
        float ix[kTcItems];
#pragma unroll
        for (int k = 0; k < kTcItems; ++k) {
            irow[k] = 0;
            ix[k] = 0.f;
            if (k < V.n) V.item(A, k, irow[k], ix[k]);
        }
        for (int kb = 0; kb < A.NKB; ++kb, ++it) {
            const uint32_t s = it & 1u;
            // stage s is free once the MMAs of its previous use (two K-blocks ago) completed
            if (it >= 2 && !tc::mbar_wait(&mdone[s], ((it >> 1) + 1u) & 1u)) {
                bad = 1;
                atomicExch(A.err, 1);
            }
            if (tid == 0 && !bad) {
                tc::mbar_arrive_expect_tx(&bfull[s], bbytes);
                tc::bulk_g2s(b_img + s * bbytes, A.bimg + (size_t)kb * A.Np * kTcKB, bbytes, &bfull[s]);
                last_b[s] = it;
            }
            // range of the block two ahead, loading during this block's walk
            int t2, k2;
            const bool has2 = step(tile, kb, 2, t2, k2);
            uint32_t qb0 = 0, qb1 = 0;
            if (has2) range_of(t2, k2, qb0, qb1);
            // C rows of this K-block: first pass from the prefetched window, further passes
            // (more than kTcThreads * kSlice entries) load their windows here
            walk_window(cw, cx, cb0 + s_off, cb0, cb1);
            for (uint32_t s0 = cb0 + s_off + kTcThreads * kSlice; s0 < cb1; s0 += kTcThreads * kSlice) {
                Window w;
                float x[kWin];
                w.load(A, cb0, cb1, s0);
                load_x(w, x);
                walk_window(w, x, s0, cb0, cb1);
            }
            // shift the pipeline: the next block's window (loaded a block ago) becomes current
            // and its x values start loading; the window of the block two ahead starts loading
            cw = nw;
            cb0 = nb0;
            cb1 = nb1;
            load_x(cw, cx);
            nb0 = qb0;
            nb1 = qb1;
            nw.load(A, nb0, nb1, nb0 + s_off);
            __syncthreads();
            // FP32 rows -> BF16 hi / lo in the swizzled layout; staging back to zero
            uint8_t *ah = a_hi + s * 16384, *al = a_lo + s * 16384;
            const float lsc = A.l_scale;
#pragma unroll
            for (int q = tid; q < kTcTile * 8; q += kTcThreads) {
                const int m = q >> 3, p = q & 7, cl = p ^ (m & 7);
                float4 *r0 = reinterpret_cast<float4 *>(stage + m * kStageStride + cl * 8);
                const float4 x0 = r0[0], x1 = r0[1];
                const float v[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float a = v[2 * e] * lsc, b = v[2 * e + 1] * lsc;
                    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
                    const float2 hf = __bfloat1622float2(h);
                    const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
                    hw[e] = *reinterpret_cast<const uint32_t *>(&h);
                    lw[e] = *reinterpret_cast<const uint32_t *>(&l);
                }
                const uint32_t off = (uint32_t)(m >> 3) * 1024u + (uint32_t)(m & 7) * 128u + (uint32_t)p * 16u;
                *reinterpret_cast<uint4 *>(ah + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(al + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
                const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
                r0[0] = z;
                r0[1] = z;
            }
            tc::fence_async_smem();
            if (__syncthreads_or(bad)) {
                stop = true;
                break;
            }
            if (tid == 0) {
                if (!tc::mbar_wait(&bfull[s], (it >> 1) & 1u)) {
                    bad = 1;
                    atomicExch(A.err, 2);
                } else {
                    tc::tc_fence_after();
                    const uint32_t ab_hi = tc::smem_u32(ah), ab_lo = tc::smem_u32(al);
                    const uint32_t bb = tc::smem_u32(b_img + s * bbytes);
#pragma unroll
                    for (int kk = 0; kk < kTcKB / 16; ++kk) {
                        const uint64_t dh = tc::desc_sw128(ab_hi + kk * 32), dl = tc::desc_sw128(ab_lo + kk * 32);
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const uint64_t db = tc::desc_sw128(bb + (uint32_t)h * (uint32_t)half * 128u + kk * 32);
                            const uint32_t d = tmem + (uint32_t)(h * half);
                            tc::mma_bf16(d, dh, db, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
                            tc::mma_bf16(d, dl, db, idesc, 1u);
                        }
                    }
                    tc::mma_commit(&mdone[s]);
                    last_c[s] = it;
                }
            }
        }
        if (stop) break;
        // epilogue: the accumulator is complete once the tile's last MMA group is
        const uint32_t last = it - 1;
        if (!tc::mbar_wait(&mdone[last & 1u], (last >> 1) & 1u)) {
            bad = 1;
            atomicExch(A.err, 3);
        }
        tc::tc_fence_after();
        if (__syncthreads_or(bad)) break;
        const int q = warp & 3, colh = warp >> 2;
        const int v = ve;
        float vn = 0.f;
        for (int c0 = colh * half; c0 < (colh + 1) * half; c0 += 16) {
            float r[16];
            tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
            // the voxel's EC / ISO items: all row loads of the chunk issued together
            {
                uint4 wa[kTcItems], wb[kTcItems];
#pragma unroll
                for (int k = 0; k < kTcItems; ++k) {
                    if (k < V.n) {
                        const uint4 *rp = reinterpret_cast<const uint4 *>(A.rows16 + (size_t)irow[k] * A.Np + c0);
                        wa[k] = __ldg(rp);
                        wb[k] = __ldg(rp + 1);
                    }
                }
#pragma unroll
                for (int k = 0; k < kTcItems; ++k)
                    if (k < V.n) fma16(r, ix[k], wa[k], wb[k]);
                for (int k = kTcItems; k < V.n; ++k) {
                    uint32_t row;
                    float xv;
                    V.item(A, k, row, xv);
                    const uint4 *rp = reinterpret_cast<const uint4 *>(A.rows16 + (size_t)row * A.Np + c0);
                    fma16(r, xv, __ldg(rp), __ldg(rp + 1));
                }
            }
            if (v < A.nV && vec4 && c0 + 16 <= A.nS && !A.partials) {
                const size_t idx = (size_t)v * A.nS + c0;
#pragma unroll
                for (int i = 0; i < 16; i += 4) {
                    const float4 w = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
                    if (A.yout) *reinterpret_cast<float4 *>(A.yout + idx + i) = w;
                    if (A.axout) *reinterpret_cast<float4 *>(A.axout + idx + i) = w;
                }
            } else if (v < A.nV) {
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int sidx = c0 + i;
                    if (sidx < A.nS) {
                        const size_t idx = (size_t)v * A.nS + sidx;
                        if (A.yout) A.yout[idx] = r[i];
                        if (A.axout) A.axout[idx] = r[i];
                        if (A.partials) {
                            float rr = A.yobs ? r[i] - A.yobs[idx] : r[i];
                            if (A.sqw) rr *= A.sqw[idx];
                            vn = fmaf(rr, rr, vn);
                        }
                    }
                }
            }
        }
        nrm += (double)vn;
        tc::tc_fence_before();
        __syncthreads();
    }
    // drain (a no-op after a normal exit): the last copy and MMA group of each stage have
    // completed before TMEM is freed; waits that run out are recorded
    __syncthreads();
    if (tid == 0) {
        for (int st = 0; st < 2; ++st) {
            if (last_b[st] != kNone && !tc::mbar_wait(&bfull[st], (last_b[st] >> 1) & 1u)) atomicExch(A.err, 4);
            if (last_c[st] != kNone && !tc::mbar_wait(&mdone[st], (last_c[st] >> 1) & 1u)) atomicExch(A.err, 5);
        }
    }
    if (A.partials) block_sum_store(nrm, A.partials + (size_t)blockIdx.x * kRedSlots);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------------------ one-time layout
__device__ __forceinline__ int owner_of(const uint32_t *ptr, int nV, uint32_t j) {
    // the voxel v with ptr[v] <= j < ptr[v+1]
    int lo = 0, hi = nV;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (ptr[mid] <= j) lo = mid;
        else hi = mid;
    }
    return lo;
}

struct TcLayoutArgs {
    const OpDev P;
    int NKB, nkbd;
};

// IC entries: key (tile, K-block, voxel in tile), value column | row << 26 | FP16 length << 32
__global__ void k_tc_entries(const TcLayoutArgs L, const __half *__restrict__ l16, uint32_t *__restrict__ key,
                             unsigned long long *__restrict__ val) {
    const OpDev &P = L.P;
    const int64_t nic = P.n * P.nIC;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nic;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / P.n);
        const uint32_t j = (uint32_t)(q - (int64_t)i * P.n);
        const int v = owner_of(P.vox_ptr, P.nV, j);
        const uint32_t o = P.seg_o[j];
        const int kb = i * L.nkbd + (int)(o >> 6);
        const uint32_t row = o & 63u;
        const uint32_t col = (uint32_t)i * (uint32_t)P.nF + P.seg_f[j];
        key[q] = ((uint32_t)(v >> 7) * (uint32_t)L.NKB + (uint32_t)kb) * (uint32_t)kTcTile + (uint32_t)(v & 127);
        val[q] = (unsigned long long)(col | (row << kColBits)) |
                 ((unsigned long long)__half_as_ushort(l16[j]) << 32);
    }
}

__global__ void k_tc_split(const unsigned long long *__restrict__ val, int64_t n, uint32_t *__restrict__ co,
                           __half *__restrict__ l, uint8_t *__restrict__ vl, const uint32_t *__restrict__ key,
                           uint32_t *__restrict__ count) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long w = val[q];
        co[q] = (uint32_t)w;
        l[q] = __ushort_as_half((unsigned short)(w >> 32));
        vl[q] = (uint8_t)(key[q] & (uint32_t)(kTcTile - 1));
        atomicAdd(count + key[q], 1u);
    }
}

// IC LUT rows of every K-block as [Np samples x 64 rows] BF16, K-major, 128-byte swizzle
__global__ void k_tc_bimg(const OpDev P, int Np, int NKB, int nkbd, __nv_bfloat16 *__restrict__ img) {
    const int64_t total = (int64_t)NKB * Np * kTcKB;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int kb = (int)(q / ((int64_t)Np * kTcKB));
        const int r = (int)(q - (int64_t)kb * Np * kTcKB);
        const int s = r / kTcKB, k = r - s * kTcKB;
        const int i = kb / nkbd, o = (kb - i * nkbd) * kTcKB + k;
        const float v = (s < P.nS && o < P.ndirs) ? P.lutIC[((size_t)i * P.ndirs + o) * P.nS + s] : 0.f;
        img[(size_t)kb * Np * kTcKB + tc::sw128_offset((uint32_t)s, (uint32_t)k) / 2] = __float2bfloat16_rn(v);
    }
}

// EC / ISO LUT rows as BF16 with row stride Np (zero padded)
__global__ void k_tc_rows16(const float *__restrict__ lut, int rows, int nS, int Np, __nv_bfloat16 *__restrict__ out) {
    const int64_t total = (int64_t)rows * Np;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = q / Np;
        const int s = (int)(q - r * Np);
        out[q] = __float2bfloat16_rn(s < nS ? lut[r * nS + s] : 0.f);
    }
}

// IC entries keyed by their column, for the entry-order fibre index
__global__ void k_tc_fib_keys(const uint32_t *__restrict__ co, int64_t n, uint32_t *__restrict__ ckey,
                              uint32_t *__restrict__ pos) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        ckey[q] = co[q] & ((1u << kColBits) - 1u);
        pos[q] = (uint32_t)q;
    }
}

// IC columns keyed by the entry position of their first term (nent without terms), for the
// fibre pass order
__global__ void k_tc_first(const uint32_t *__restrict__ fptr, const uint32_t *__restrict__ fperm, int64_t ncols,
                           uint32_t nent, uint32_t *__restrict__ key, uint32_t *__restrict__ col) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ncols;
         q += (int64_t)gridDim.x * blockDim.x) {
        key[q] = fptr[q] < fptr[q + 1] ? fperm[fptr[q]] : nent;
        col[q] = (uint32_t)q;
    }
}

// fpos = the inverse of fperm: the column-sorted position of every entry
__global__ void k_tc_inverse(const uint32_t *__restrict__ fperm, int64_t n, uint32_t *__restrict__ fpos) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        fpos[fperm[k]] = (uint32_t)k;
}

__global__ void k_tc_count(const uint32_t *__restrict__ ckey, int64_t n, uint32_t *__restrict__ count) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(count + ckey[q], 1u);
}

// IC LUT rows as the B operand of the adjoint: per round of 256 rows, sample K-block and
// half, [128 rows x 64 samples] BF16, K-major, 128-byte swizzle; row g is the forward's K
// index g
__global__ void k_tca_bimg(const OpDev P, int R, int KBS, int NKB, int nkbd, __nv_bfloat16 *__restrict__ img) {
    const int64_t total = (int64_t)R * KBS * 2 * 128 * 64;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = q / (128 * 64);
        const int rr = (int)(q - item * 128 * 64), row = rr / 64, k = rr - row * 64;
        const int nh = (int)(item & 1), kb = (int)((item >> 1) % KBS), r = (int)((item >> 1) / KBS);
        const int g = r * 256 + nh * 128 + row, s = kb * 64 + k;
        const int kbf = g / kTcKB, kk = g - kbf * kTcKB;
        float v = 0.f;
        if (s < P.nS && kbf < NKB) {
            const int i = kbf / nkbd, o = (kbf - i * nkbd) * kTcKB + kk;
            if (o < P.ndirs) v = P.lutIC[((size_t)i * P.ndirs + o) * P.nS + s];
        }
        img[item * 128 * 64 + tc::sw128_offset((uint32_t)row, (uint32_t)k) / 2] = __float2bfloat16_rn(v);
    }
}

__global__ void k_tc_xe(const double *__restrict__ x, const uint32_t *__restrict__ eval, int64_t nic, int64_t ncols,
                        float *__restrict__ xe) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ncols;
         q += (int64_t)gridDim.x * blockDim.x) {
        float v = (float)x[q];
        if (q < nic) v *= (float)eval[q];
        xe[q] = v;
    }
}

int grid_of(int64_t n, int nsm) {
    int64_t g = (n + 255) / 256;
    if (g > (int64_t)nsm * 16) g = (int64_t)nsm * 16;
    return g < 1 ? 1 : (int)g;
}

}  // namespace
}  // namespace detail

using namespace detail;

// Whether the tensor-core kernels handle this operator: an IC compartment with segments,
// padded samples within the shared-memory budget, columns within ent_co's 26 bits.
bool tc_supported(const cgb_op *op) {
    const int Np = (op->nS + 31) / 32 * 32;
    const int64_t nent = op->n * op->nIC;
    return !op->nolut && op->nV > 0 && Np <= kTcMaxNp && op->ncols < ((int64_t)1 << kColBits) && nent > 0 &&
           nent < ((int64_t)1 << 32);
}

// IC segments per voxel from which mode 0 takes the tensor cores: the dense product costs
// per (tile, K-block) whatever the segments, so sparse operators stay on the CUDA cores.
// Measured BF16 pairs/s, tensor cores vs CUDA cores (nS = 288): 318 vs 376 at 21 segments
// per voxel, 278 vs 184 at 62, 141 vs 73 at 212; the ratio crosses 1 near 32.
constexpr int64_t kTcMinSegmentsPerVoxel = 32;

bool tc_forward_enabled(const cgb_op *op) {
    if (op->tc_mode == 1 || !tc_supported(op)) return false;
    return op->tc_mode == 2 || op->n * op->nIC >= kTcMinSegmentsPerVoxel * (int64_t)op->nV;
}

// IC entries, their per-(tile, K-block, voxel) offsets, the B images and the BF16 EC / ISO
// rows; needs the FP16 lengths of ensure_reduced
int ensure_tc(cgb_op *op) {
    if (op->tc_ready) return CGB_OK;
    if (!tc_supported(op)) return fail(CGB_ERR_UNSUPPORTED, "tensor-core forward: operator shape not supported");
    const OpDev P = op->dev();
    const int nkbd = (op->ndirs + kTcKB - 1) / kTcKB;
    const int NKB = op->nIC * nkbd;
    const int Np = (op->nS + 31) / 32 * 32;
    const int ntiles = (op->nV + kTcTile - 1) / kTcTile;
    const int64_t nent = op->n * op->nIC;
    const int64_t nec_rows = (op->nE > 0 && op->nEC > 0) ? (int64_t)op->nEC * op->ndirs : 0;
    const int64_t niso_rows = (op->nISOv > 0 && op->nISO > 0) ? op->nISO : 0;
    const int64_t nkeys = (int64_t)ntiles * NKB * kTcTile;
    if (nkeys >= ((int64_t)1 << 32) - 1) return fail(CGB_ERR_UNSUPPORTED, "tensor-core forward: too many tiles");
    const int64_t ncount = nkeys + 1 > (int64_t)op->nF * op->nIC + 1 ? nkeys + 1 : (int64_t)op->nF * op->nIC + 1;
    const float lscale = op->len16_inv_scale > 0.f ? op->len16_inv_scale : 1.f;
    TcLayoutArgs L{P, NKB, nkbd};

    uint32_t *key = nullptr, *key2 = nullptr, *count = nullptr;
    unsigned long long *val = nullptr, *val2 = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    int rc = CGB_OK;
    auto cu = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && rc == CGB_OK) rc = cuda_fail(e, what);
        return rc == CGB_OK;
    };
    int bits = 1;
    while (bits < 32 && (((uint64_t)nkeys) >> bits) != 0) ++bits;
    cu(cudaMalloc((void **)&op->tc_co, nent * sizeof(uint32_t)), "cudaMalloc");
    cu(cudaMalloc((void **)&op->tc_l, nent * sizeof(__half)), "cudaMalloc");
    cu(cudaMalloc((void **)&op->tc_vl, nent * sizeof(uint8_t)), "cudaMalloc");
    cu(cudaMalloc((void **)&op->tc_ptr, (nkeys + 1) * sizeof(uint32_t)), "cudaMalloc");
    cu(cudaMalloc((void **)&op->tc_bimg, (size_t)(NKB > 0 ? NKB : 1) * Np * kTcKB * sizeof(__nv_bfloat16)),
       "cudaMalloc");
    cu(cudaMalloc((void **)&op->tc_xe, (size_t)(op->ncols > 0 ? op->ncols : 1) * sizeof(float)), "cudaMalloc");
    cu(cudaMalloc((void **)&op->tc_err, sizeof(int)), "cudaMalloc");
    cu(cudaMalloc((void **)&op->tc_rows16, (size_t)(nec_rows + niso_rows > 0 ? nec_rows + niso_rows : 1) * Np *
                                               sizeof(__nv_bfloat16)),
       "cudaMalloc");
    cu(cudaMalloc((void **)&key, nent * sizeof(uint32_t)), "cudaMalloc");
    cu(cudaMalloc((void **)&key2, nent * sizeof(uint32_t)), "cudaMalloc");
    cu(cudaMalloc((void **)&val, nent * sizeof(unsigned long long)), "cudaMalloc");
    cu(cudaMalloc((void **)&val2, nent * sizeof(unsigned long long)), "cudaMalloc");
    cu(cudaMalloc((void **)&count, ncount * sizeof(uint32_t)), "cudaMalloc");
    if (rc == CGB_OK) {
        cu(cudaMemset(op->tc_err, 0, sizeof(int)), "cudaMemset");
        cu(cudaMemset(count, 0, (nkeys + 1) * sizeof(uint32_t)), "cudaMemset");
        k_tc_entries<<<grid_of(nent, op->nsm), 256>>>(L, op->seg_l16, key, val);
        cu(cudaGetLastError(), "k_tc_entries");
        cu(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key, key2, val, val2, nent, 0, bits), "cub sort");
        size_t scan_bytes = 0;
        cu(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, count, op->tc_ptr, nkeys + 1), "cub scan");
        if (scan_bytes > tmp_bytes) tmp_bytes = scan_bytes;
        cu(cudaMalloc(&tmp, tmp_bytes), "cudaMalloc");
    }
    if (rc == CGB_OK) {
        cu(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, key, key2, val, val2, nent, 0, bits), "cub sort");
        k_tc_split<<<grid_of(nent, op->nsm), 256>>>(val2, nent, op->tc_co, op->tc_l, op->tc_vl, key2, count);
        cu(cudaGetLastError(), "k_tc_split");
        cu(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, count, op->tc_ptr, nkeys + 1), "cub scan");
        const int64_t nimg = (int64_t)NKB * Np * kTcKB;
        k_tc_bimg<<<grid_of(nimg, op->nsm), 256>>>(P, Np, NKB, nkbd, op->tc_bimg);
        cu(cudaGetLastError(), "k_tc_bimg");
        // EC rows (response, orientation) first, then the ISO rows
        if (nec_rows > 0) {
            k_tc_rows16<<<grid_of(nec_rows * Np, op->nsm), 256>>>(op->lutEC, (int)nec_rows, op->nS, Np, op->tc_rows16);
            cu(cudaGetLastError(), "k_tc_rows16");
        }
        if (niso_rows > 0) {
            k_tc_rows16<<<grid_of(niso_rows * Np, op->nsm), 256>>>(op->lutISO, (int)niso_rows, op->nS, Np,
                                                                   op->tc_rows16 + (size_t)nec_rows * Np);
            cu(cudaGetLastError(), "k_tc_rows16");
        }
        cu(cudaFuncSetAttribute(k_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes(Np)),
           "cudaFuncSetAttribute");
    }
    // adjoint: the IC entries' positions grouped by column (stable: ascending positions),
    // their CSR offsets per column, the LUT images of the adjoint and the term array
    const int KBS = (op->nS + 63) / 64;
    const int R = (NKB * kTcKB + 255) / 256;
    const int64_t nic_cols = (int64_t)op->nF * op->nIC;
    if (rc == CGB_OK) {
        // key / val buffers are reused: key <- column keys, (uint32 view of val) <- positions
        uint32_t *pos = reinterpret_cast<uint32_t *>(val), *pos2 = reinterpret_cast<uint32_t *>(val2);
        k_tc_fib_keys<<<grid_of(nent, op->nsm), 256>>>(op->tc_co, nent, key, pos);
        cu(cudaGetLastError(), "k_tc_fib_keys");
        const uint64_t hnic = (uint64_t)nent;
        int cbits = 1;
        while (cbits < 32 && (((uint64_t)nic_cols) >> cbits) != 0) ++cbits;
        size_t need = 0;
        cu(cub::DeviceRadixSort::SortPairs(nullptr, need, key, key2, pos, pos2, nent, 0, cbits), "cub sort");
        if (need > tmp_bytes) {
            cudaFree(tmp);
            tmp = nullptr;
            tmp_bytes = need;
            cu(cudaMalloc(&tmp, tmp_bytes), "cudaMalloc");
        }
        cu(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, key, key2, pos, pos2, nent, 0, cbits), "cub sort");
        cu(cudaMalloc((void **)&op->tc_fperm, (hnic > 0 ? hnic : 1) * sizeof(uint32_t)), "cudaMalloc");
        cu(cudaMalloc((void **)&op->tc_fptr, (nic_cols + 1) * sizeof(uint32_t)), "cudaMalloc");
        if (rc == CGB_OK && hnic > 0)
            cu(cudaMemcpy(op->tc_fperm, pos2, hnic * sizeof(uint32_t), cudaMemcpyDeviceToDevice), "cudaMemcpy");
        cu(cudaMemset(count, 0, (nic_cols + 1) * sizeof(uint32_t)), "cudaMemset");
        if (rc == CGB_OK && hnic > 0) {
            k_tc_count<<<grid_of((int64_t)hnic, op->nsm), 256>>>(key2, (int64_t)hnic, count);
            cu(cudaGetLastError(), "k_tc_count");
        }
        size_t scan_need = 0;
        cu(cub::DeviceScan::ExclusiveSum(nullptr, scan_need, count, op->tc_fptr, nic_cols + 1), "cub scan");
        if (scan_need > tmp_bytes) {
            cudaFree(tmp);
            tmp = nullptr;
            tmp_bytes = scan_need;
            cu(cudaMalloc(&tmp, tmp_bytes), "cudaMalloc");
        }
        cu(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, count, op->tc_fptr, nic_cols + 1), "cub scan");
        // columns in the order of their first entry, the fibre pass's thread order (measured:
        // 1.03 ms at 1M streamlines against 1.18 ms for a warp per column in column order)
        uint32_t *fk = nullptr, *fk2 = nullptr, *fc = nullptr;
        cu(cudaMalloc((void **)&fk, nic_cols * 2 * sizeof(uint32_t)), "cudaMalloc");
        cu(cudaMalloc((void **)&fc, nic_cols * sizeof(uint32_t)), "cudaMalloc");
        cu(cudaMalloc((void **)&op->tc_ford, nic_cols * sizeof(uint32_t)), "cudaMalloc");
        if (rc == CGB_OK) {
            fk2 = fk + nic_cols;
            k_tc_first<<<grid_of(nic_cols, op->nsm), 256>>>(op->tc_fptr, op->tc_fperm, nic_cols, (uint32_t)nent, fk, fc);
            cu(cudaGetLastError(), "k_tc_first");
            int ebits = 1;
            while (ebits < 32 && (((uint64_t)nent) >> ebits) != 0) ++ebits;
            size_t fneed = 0;
            cu(cub::DeviceRadixSort::SortPairs(nullptr, fneed, fk, fk2, fc, op->tc_ford, nic_cols, 0, ebits),
               "cub sort");
            if (fneed > tmp_bytes) {
                cudaFree(tmp);
                tmp = nullptr;
                tmp_bytes = fneed;
                cu(cudaMalloc(&tmp, tmp_bytes), "cudaMalloc");
            }
            cu(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, fk, fk2, fc, op->tc_ford, nic_cols, 0, ebits),
               "cub sort");
        }
        cu(cudaDeviceSynchronize(), "tensor-core layout");
        cudaFree(fk);
        cudaFree(fc);
        // the adjoint writes each term at its column-sorted position (fpos), so the fibre
        // pass reads every column's terms contiguously; fperm is not needed after this
        cu(cudaMalloc((void **)&op->tc_fpos, (size_t)nent * sizeof(uint32_t)), "cudaMalloc");
        if (rc == CGB_OK) {
            k_tc_inverse<<<grid_of(nent, op->nsm), 256>>>(op->tc_fperm, nent, op->tc_fpos);
            cu(cudaGetLastError(), "k_tc_inverse");
            cu(cudaDeviceSynchronize(), "tensor-core layout");
        }
        cudaFree(op->tc_fperm);
        op->tc_fperm = nullptr;
        cu(cudaMalloc((void **)&op->tc_abimg, (size_t)R * KBS * 2 * 128 * 64 * sizeof(__nv_bfloat16)), "cudaMalloc");
        if (rc == CGB_OK) {
            k_tca_bimg<<<grid_of((int64_t)R * KBS * 2 * 128 * 64, op->nsm), 256>>>(P, R, KBS, NKB, nkbd,
                                                                                   op->tc_abimg);
            cu(cudaGetLastError(), "k_tca_bimg");
        }
        cu(cudaMalloc((void **)&op->tc_terms, nent * sizeof(float)), "cudaMalloc");
        cu(cudaDeviceSynchronize(), "tensor-core layout");
    }
    cudaFree(key);
    cudaFree(key2);
    cudaFree(val);
    cudaFree(val2);
    cudaFree(count);
    cudaFree(tmp);
    if (rc != CGB_OK) return rc;
    op->tc_np = Np;
    op->tc_nkb = NKB;
    op->tc_ntiles = ntiles;
    op->tc_lscale = lscale;
    op->tc_kbs = KBS;
    op->tc_rounds = R;
    op->tc_nent = nent;
    op->bytes += nent * 7 + (nkeys + 1) * 4 + (size_t)NKB * Np * kTcKB * 2 + (size_t)op->ncols * 4 + nent * 8 +
                 (size_t)(nic_cols + 1) * 4 + (size_t)nic_cols * 4 + (size_t)R * KBS * 2 * 128 * 64 * 2 +
                 (size_t)(nec_rows + niso_rows) * Np * 2;
    op->tc_ready = 1;
    return CGB_OK;
}

int forward_tc(cgb_op *op, const double *x, float *y, float *ax, const float *yobs, const float *sqw,
               double *partials, cudaStream_t st, int *grid) {
    CGB_TRY(ensure_tc(op));
    if (grid) *grid = 0;
    if (op->ncols > 0) {
        k_tc_xe<<<grid_of(op->ncols, op->nsm), 256, 0, st>>>(x, op->eval, (int64_t)op->nF * op->nIC, op->ncols,
                                                                 op->tc_xe);
        CGB_CUDA(cudaGetLastError());
    }
    TcFwdArgs A;
    A.nV = op->nV;
    A.nS = op->nS;
    A.Np = op->tc_np;
    A.NKB = op->tc_nkb;
    A.ntiles = op->tc_ntiles;
    const bool ec = op->nE > 0 && op->nEC > 0, iso = op->nISOv > 0 && op->nISO > 0;
    A.nE = op->nE;
    A.nEC = ec ? op->nEC : 0;
    A.nISOv = op->nISOv;
    A.nISO = iso ? op->nISO : 0;
    A.ndirs = op->ndirs;
    const OpDev P = op->dev();
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
    A.ent_vl = op->tc_vl;
    A.l_scale = op->tc_lscale;
    A.xe = op->tc_xe;
    A.bimg = op->tc_bimg;
    A.yout = y;
    A.axout = ax;
    A.yobs = yobs;
    A.sqw = sqw;
    A.partials = partials;
    A.err = op->tc_err;
    int g = op->nsm < A.ntiles ? op->nsm : A.ntiles;
    if (g > reduction_blocks(op)) g = reduction_blocks(op);
    k_forward_tc<<<g, kTcThreads, tc_smem_bytes(A.Np), st>>>(A);
    CGB_CUDA(cudaGetLastError());
    if (grid) *grid = g;
    return CGB_OK;
}

}  // namespace cgb

extern "C" int cgb_op_tensor_cores(cgb_op *op, int mode, int *out) {
    if (!op) return cgb::fail(CGB_ERR_INVALID, "null handle");
    if (mode > 2) return cgb::fail(CGB_ERR_INVALID, "mode must be 0 (automatic), 1 (off) or 2 (on)");
    if (mode == 2 && !cgb::tc_supported(op))
        return cgb::fail(CGB_ERR_UNSUPPORTED, "tensor-core forward: operator shape not supported");
    if (mode >= 0) op->tc_mode = mode;
    if (out) *out = cgb::tc_forward_enabled(op) ? 1 : 0;
    return CGB_OK;
}

extern "C" int cgb_op_device_status(cgb_op *op) {
    if (!op) return cgb::fail(CGB_ERR_INVALID, "null handle");
    int dev = 0;
    CGB_CUDA(cudaGetDevice(&dev));
    CGB_CUDA(cudaSetDevice(op->device));
    cudaError_t e = cudaDeviceSynchronize();
    int h = 0;
    if (e == cudaSuccess && op->tc_err) {
        e = cudaMemcpy(&h, op->tc_err, sizeof(int), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && h) e = cudaMemset(op->tc_err, 0, sizeof(int));
    }
    cudaSetDevice(dev);
    CGB_CUDA(e);
    if (h) return cgb::fail(CGB_ERR_CUDA, "a tensor-core kernel gave up waiting (code " + std::to_string(h) + ")");
    return CGB_OK;
}
