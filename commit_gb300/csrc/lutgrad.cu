// Gradient of a loss with respect to the response-function LUTs, and LUT updates.
//
// y[v,s] depends linearly on the LUT entries: y[v,s] = sum over items of the voxel of
// c * LUT[row(item), s] with c = l*x*eval (IC), x (EC, ISO).  For an upstream gradient
// g = dLoss/dy the LUT gradient is therefore
//   G_IC[i,o,s]  = sum over IC segments j with orientation o of c_{j,i} * g[v_j, s]
//   G_EC[i,o,s]  = sum over EC elements e with orientation o of x_{EC,i,e} * g[v_e, s]
//   G_ISO[i,s]   = sum over ISO elements j of x_{ISO,i,j} * g[v_j, s].
// The items are visited in an orientation-sorted order (built once, on first use), split
// into chunks of at most kChunk items that never straddle an orientation; a warp reduces
// one chunk (lanes over samples, FP64) into a partial row, and a second pass adds the
// partial rows of each orientation in chunk order -- deterministic, no atomics.
#include <cub/cub.cuh>

#include <vector>

#include "cgb_internal.cuh"

namespace cgb {
namespace {

constexpr int kChunk = 1024;

struct GradStream {
    // items of one compartment in orientation order
    uint32_t *perm = nullptr;     // item index (voxel-ordered position for IC, element for EC)
    uint32_t *chunk_beg = nullptr, *chunk_row = nullptr;  // per chunk: first position, LUT row o
    uint32_t *row_chunk = nullptr;                        // [nrow+1] chunks of row o
    int nchunks = 0, nrows = 0;
    int64_t nitems = 0;
    ~GradStream() {
        void *p[] = {perm, chunk_beg, chunk_row, row_chunk};
        for (void *q : p)
            if (q) cudaFree(q);
    }
};

__global__ void k_iota32(uint32_t *a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (uint32_t)i;
}

__global__ void k_u16_to_u32(const uint16_t *a, uint32_t *b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

int grid_n(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 4096) g = 4096;
    if (g < 1) g = 1;
    return (int)g;
}

// Orientation-sorted order of `n` items with orientations o[] (device), chunked.
int build_stream(const uint16_t *o, int64_t n, int nrows, GradStream &S) {
    S.nitems = n;
    S.nrows = nrows;
    std::vector<uint32_t> h_off(nrows + 1, 0);
    if (n > 0) {
        uint32_t *keys = nullptr, *keys_out = nullptr, *vals = nullptr;
        void *tmp = nullptr;
        size_t bytes = 0;
        CGB_CUDA(cudaMalloc((void **)&keys, n * sizeof(uint32_t)));
        CGB_CUDA(cudaMalloc((void **)&keys_out, n * sizeof(uint32_t)));
        CGB_CUDA(cudaMalloc((void **)&vals, n * sizeof(uint32_t)));
        CGB_CUDA(cudaMalloc((void **)&S.perm, n * sizeof(uint32_t)));
        k_u16_to_u32<<<grid_n(n), 256>>>(o, keys, n);
        k_iota32<<<grid_n(n), 256>>>(vals, n);
        CGB_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys, keys_out, vals, S.perm, (int)n, 0, 16));
        CGB_CUDA(cudaMalloc(&tmp, bytes));
        CGB_CUDA(cub::DeviceRadixSort::SortPairs(tmp, bytes, keys, keys_out, vals, S.perm, (int)n, 0, 16));
        std::vector<uint32_t> h_keys(n);
        CGB_CUDA(cudaMemcpy(h_keys.data(), keys_out, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        cudaFree(keys);
        cudaFree(keys_out);
        cudaFree(vals);
        cudaFree(tmp);
        for (int64_t i = 0; i < n; ++i) h_off[h_keys[i] + 1]++;
        for (int r = 0; r < nrows; ++r) h_off[r + 1] += h_off[r];
    }
    std::vector<uint32_t> cb, cr, rc(nrows + 1, 0);
    for (int r = 0; r < nrows; ++r) {
        rc[r] = (uint32_t)cb.size();
        for (uint32_t p = h_off[r]; p < h_off[r + 1]; p += kChunk) {
            cb.push_back(p);
            cr.push_back((uint32_t)r);
        }
    }
    rc[nrows] = (uint32_t)cb.size();
    cb.push_back((uint32_t)n);  // sentinel: end of the last chunk
    S.nchunks = (int)cr.size();
    CGB_CUDA(cudaMalloc((void **)&S.chunk_beg, cb.size() * sizeof(uint32_t)));
    CGB_CUDA(cudaMalloc((void **)&S.chunk_row, (cr.size() ? cr.size() : 1) * sizeof(uint32_t)));
    CGB_CUDA(cudaMalloc((void **)&S.row_chunk, rc.size() * sizeof(uint32_t)));
    CGB_CUDA(cudaMemcpy(S.chunk_beg, cb.data(), cb.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    if (!cr.empty()) CGB_CUDA(cudaMemcpy(S.chunk_row, cr.data(), cr.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CGB_CUDA(cudaMemcpy(S.row_chunk, rc.data(), rc.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    return CGB_OK;
}

// voxel of each voxel-ordered IC position / EC element (from the CSR offsets)
__global__ void k_item_voxel(const uint32_t *ptr, int nV, uint32_t *vox) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x)
        for (uint32_t j = ptr[v]; j < ptr[v + 1]; ++j) vox[j] = (uint32_t)v;
}

// one warp per chunk: partial[chunk, s] = sum over the chunk's items of c * g[v, s]
// kind 0: IC (c = l * x[i*nF + f] * eval), kind 1: EC (c = x[ec_base + i*nE + col])
__global__ void k_grad_chunks(const OpDev P, int kind, int rf, const uint32_t *__restrict__ perm,
                              const uint32_t *__restrict__ chunk_beg, int nchunks, const uint32_t *__restrict__ vox,
                              const double *__restrict__ x, const double *__restrict__ g, double *__restrict__ partial) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int nS = P.nS;
    for (int c = warp; c < nchunks; c += nw) {
        const uint32_t b = chunk_beg[c], e = chunk_beg[c + 1];
        for (int s0 = 0; s0 < nS; s0 += 32 * 8) {
            double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (uint32_t p = b; p < e; ++p) {
                const uint32_t it = perm[p];
                double coef;
                uint32_t v;
                if (kind == 0) {
                    const size_t col = (size_t)rf * P.nF + P.seg_f[it];
                    coef = (double)P.seg_l[it] * (x[col] * (double)P.eval[col]);
                    v = vox[it];
                } else {
                    coef = x[P.ec_base + (size_t)rf * P.nE + P.ec_col[it]];
                    v = vox[it];
                }
                if (coef == 0.0) continue;
                const double *gr = g + (size_t)v * nS;
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int s = s0 + lane + 32 * k;
                    if (s < nS) acc[k] = fma(coef, gr[s], acc[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int s = s0 + lane + 32 * k;
                if (s < nS) partial[(size_t)c * nS + s] = acc[k];
            }
        }
    }
}

// out[row, s] = sum of the row's chunk partials in chunk order
__global__ void k_grad_rows(const double *__restrict__ partial, const uint32_t *__restrict__ row_chunk, int nrows,
                            int nS, double *__restrict__ out) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)nrows * nS;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(q / nS), s = (int)(q - (int64_t)r * nS);
        double t = 0.0;
        for (uint32_t c = row_chunk[r]; c < row_chunk[r + 1]; ++c) t += partial[(size_t)c * nS + s];
        out[q] = t;
    }
}

// ISO: one warp per voxel block partial over voxels, then a fixed-order sum
__global__ void k_grad_iso(const OpDev P, int rf, const double *__restrict__ x, const double *__restrict__ g,
                           double *__restrict__ partial) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int nS = P.nS;
    for (int s0 = 0; s0 < nS; s0 += 32) {
        const int s = s0 + lane;
        double acc = 0.0;
        for (int v = warp; v < P.nV; v += nw)
            for (uint32_t j = P.iso_ptr[v]; j < P.iso_ptr[v + 1]; ++j) {
                const double c = x[P.iso_base + (size_t)rf * P.nISOv + P.iso_col[j]];
                if (s < nS) acc = fma(c, g[(size_t)v * nS + s], acc);
            }
        if (s < nS) partial[(size_t)warp * nS + s] = acc;
    }
}

__global__ void k_sum_rows(const double *__restrict__ partial, int nparts, int nS, double *__restrict__ out) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nS; s += gridDim.x * blockDim.x) {
        double t = 0.0;
        for (int w = 0; w < nparts; ++w) t += partial[(size_t)w * nS + s];
        out[s] = t;
    }
}

}  // namespace

struct LutGradState {
    GradStream ic, ec;
    uint32_t *ic_vox = nullptr, *ec_vox = nullptr;
    double *partial = nullptr;
    size_t partial_len = 0;
    ~LutGradState() {
        if (ic_vox) cudaFree(ic_vox);
        if (ec_vox) cudaFree(ec_vox);
        if (partial) cudaFree(partial);
    }
};

static int ensure_grad_state(cgb_op *op) {
    if (op->gstate) return CGB_OK;
    LutGradState *G = new LutGradState();
    op->gstate = G;
    if (op->nIC > 0 && op->n > 0) {
        CGB_TRY(build_stream(op->seg_o, op->n, op->ndirs, G->ic));
        CGB_CUDA(cudaMalloc((void **)&G->ic_vox, op->n * sizeof(uint32_t)));
        k_item_voxel<<<grid_n(op->nV), 256>>>(op->vox_ptr, op->nV, G->ic_vox);
    }
    if (op->nEC > 0 && op->nE > 0) {
        // EC entries are stored voxel-ordered; perm positions refer to that order
        CGB_TRY(build_stream(op->ec_o, op->nE, op->ndirs, G->ec));
        CGB_CUDA(cudaMalloc((void **)&G->ec_vox, (size_t)op->nE * sizeof(uint32_t)));
        k_item_voxel<<<grid_n(op->nV), 256>>>(op->ec_ptr, op->nV, G->ec_vox);
    }
    const int nwarps_iso = op->nsm * 32;
    size_t need = (size_t)std::max(std::max(G->ic.nchunks, G->ec.nchunks), nwarps_iso) * op->nS;
    CGB_CUDA(cudaMalloc((void **)&G->partial, (need ? need : 1) * sizeof(double)));
    G->partial_len = need;
    CGB_CUDA(cudaDeviceSynchronize());
    return CGB_OK;
}

void free_grad_state(cgb_op *op) {
    if (op->gstate) {
        delete (LutGradState *)op->gstate;
        op->gstate = nullptr;
    }
}

}  // namespace cgb

using namespace cgb;

extern "C" {

int cgb_op_lut_grad(cgb_op *op, const double *x, const double *g, double *g_ic, double *g_ec, double *g_iso,
                    void *stream) {
    if (!op || !x || !g) return fail(CGB_ERR_INVALID, "null argument");
    if (op->nolut) return fail(CGB_ERR_UNSUPPORTED, "the LUT-free operator has no LUT");
    CGB_TRY(ensure_grad_state(op));
    LutGradState *G = (LutGradState *)op->gstate;
    cudaStream_t st = (cudaStream_t)stream;
    const OpDev P = op->dev();
    const int nS = op->nS;
    const size_t rowlen = (size_t)op->ndirs * nS;
    if (g_ic && op->nIC > 0) {
        for (int i = 0; i < op->nIC; ++i) {
            double *out = g_ic + (size_t)i * rowlen;
            if (G->ic.nchunks == 0) {
                CGB_CUDA(cudaMemsetAsync(out, 0, rowlen * sizeof(double), st));
                continue;
            }
            k_grad_chunks<<<op->nsm * 8, 256, 0, st>>>(P, 0, i, G->ic.perm, G->ic.chunk_beg, G->ic.nchunks,
                                                       G->ic_vox, x, g, G->partial);
            k_grad_rows<<<grid_n((int64_t)op->ndirs * nS), 256, 0, st>>>(G->partial, G->ic.row_chunk, op->ndirs, nS,
                                                                        out);
            CGB_CUDA(cudaGetLastError());
        }
    }
    if (g_ec && op->nEC > 0) {
        for (int i = 0; i < op->nEC; ++i) {
            double *out = g_ec + (size_t)i * rowlen;
            if (G->ec.nchunks == 0) {
                CGB_CUDA(cudaMemsetAsync(out, 0, rowlen * sizeof(double), st));
                continue;
            }
            k_grad_chunks<<<op->nsm * 8, 256, 0, st>>>(P, 1, i, G->ec.perm, G->ec.chunk_beg, G->ec.nchunks,
                                                       G->ec_vox, x, g, G->partial);
            k_grad_rows<<<grid_n((int64_t)op->ndirs * nS), 256, 0, st>>>(G->partial, G->ec.row_chunk, op->ndirs, nS,
                                                                        out);
            CGB_CUDA(cudaGetLastError());
        }
    }
    if (g_iso && op->nISO > 0) {
        const int blocks = op->nsm * 4;  // 32 warps per SM-block set -> nsm*32 partial rows
        for (int i = 0; i < op->nISO; ++i) {
            k_grad_iso<<<blocks, 256, 0, st>>>(P, i, x, g, G->partial);
            k_sum_rows<<<grid_n(nS), 256, 0, st>>>(G->partial, blocks * 8, nS, g_iso + (size_t)i * nS);
            CGB_CUDA(cudaGetLastError());
        }
    }
    return CGB_OK;
}

}  // extern "C"
