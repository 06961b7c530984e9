// Evaluation.load_dictionary's re-layout on the device (commit/core.pyx:493-580).
//
// The dictionary_*.dict files hold trk2dictionary's arrays in the order its threads wrote
// them, with voxels as linear grid indices x + X*(y + Y*z) and IC lengths in mm.  The
// reference sorts IC, EC and ISO by voxel (numpy's stable argsort, core.pyx:508-514,
// 541-545, 557-562), divides each IC length by its streamline's norm when kernels are
// normalised (core.pyx:516-525, FP32 division), and maps each voxel id to the index of that
// voxel among the mask voxels in the same linear order (a look-up table built from the
// mask, core.pyx:571-580; ids outside the mask map to 0 as the reference's zero-filled
// table does).  Here the raw arrays are already on the device: CUB's stable radix sort by
// voxel gives the same order, the look-up table is an exclusive scan of the mask, and the
// results can go straight to cgb_op_create, which accepts device pointers.
#include <cub/cub.cuh>

#include <vector>

#include "cgb_internal.cuh"

namespace cgb {
namespace {

__global__ void k_mask_u32(const uint8_t *__restrict__ m, int64_t n, uint32_t *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = m[i] ? 1u : 0u;
}

__global__ void k_iota32(uint32_t *__restrict__ a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (uint32_t)i;
}

// voxel ids that are not grid voxels are reported (bit 0) and mapped like ids outside the mask
__global__ void k_check_ids(const uint32_t *__restrict__ v, int64_t n, int64_t ngrid, unsigned int *__restrict__ bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if ((int64_t)v[i] >= ngrid) atomicOr(bad, 1u);
}

__global__ void k_gather_ic(const uint32_t *__restrict__ perm, int64_t n, const uint32_t *__restrict__ sv,
                            const uint32_t *__restrict__ f0, const uint16_t *__restrict__ o0,
                            const float *__restrict__ l0, const float *__restrict__ norm, int nF, int normalize,
                            const uint32_t *__restrict__ lut, int64_t ngrid, uint32_t *__restrict__ f,
                            uint32_t *__restrict__ v, uint16_t *__restrict__ o, float *__restrict__ l,
                            unsigned int *__restrict__ bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = perm[i];
        const uint32_t fi = f0[p];
        float li = l0[p];
        if (normalize) {
            if (fi < (uint32_t)nF) li = __fdiv_rn(li, norm[fi]);
            else atomicOr(bad, 2u);
        }
        f[i] = fi;
        if (o) o[i] = o0[p];
        l[i] = li;
        const uint32_t id = sv[i];
        v[i] = (int64_t)id < ngrid ? lut[id] : 0u;
    }
}

__global__ void k_gather_u16(const uint32_t *__restrict__ perm, int64_t n, const uint16_t *__restrict__ src,
                             uint16_t *__restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}

__global__ void k_reindex(const uint32_t *__restrict__ sv, int64_t n, const uint32_t *__restrict__ lut,
                          int64_t ngrid, uint32_t *__restrict__ v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t id = sv[i];
        v[i] = (int64_t)id < ngrid ? lut[id] : 0u;
    }
}

int grid_of(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 4096) g = 4096;
    return g < 1 ? 1 : (int)g;
}

// device scratch released on every exit path
struct Scratch {
    std::vector<void *> p;
    ~Scratch() {
        for (void *q : p) cudaFree(q);
    }
    template <class T>
    int get(T **out, size_t n) {
        *out = nullptr;
        const cudaError_t e = cudaMalloc((void **)out, (n ? n : 1) * sizeof(T));
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        p.push_back(*out);
        return CGB_OK;
    }
};

// stable sort of the voxel ids `v` (n entries) into sv, with the permutation in perm
int sort_by_voxel(const uint32_t *v, int64_t n, int64_t ngrid, uint32_t *sv, uint32_t *perm, Scratch &S,
                  cudaStream_t st) {
    if (n == 0) return CGB_OK;
    uint32_t *iota;
    CGB_TRY(S.get(&iota, n));
    k_iota32<<<grid_of(n), 256, 0, st>>>(iota, n);
    CGB_CUDA(cudaGetLastError());
    // ids beyond the grid (reported separately) still sort: all 32 key bits
    size_t tb = 0;
    CGB_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, v, sv, iota, perm, n, 0, 32, st));
    void *t;
    CGB_TRY(S.get((uint8_t **)&t, tb));
    CGB_CUDA(cub::DeviceRadixSort::SortPairs(t, tb, v, sv, iota, perm, n, 0, 32, st));
    return CGB_OK;
}

}  // namespace
}  // namespace cgb

using namespace cgb;

extern "C" int cgb_dict_relayout(const uint8_t *mask, int64_t ngrid, int64_t n, int nF, uint32_t *ICf, uint32_t *ICv,
                                 uint16_t *ICo, float *ICl, const float *trk_norm, int normalize, int64_t nE,
                                 uint32_t *ECv, uint16_t *ECo, int64_t nISOv, uint32_t *ISOv, int64_t *nV_out,
                                 void *stream) {
    if (!mask || ngrid <= 0 || !nV_out) return fail(CGB_ERR_INVALID, "mask, grid size and nV_out are required");
    if (n < 0 || nE < 0 || nISOv < 0 || nF < 0) return fail(CGB_ERR_INVALID, "negative size");
    if (ngrid >= ((int64_t)1 << 32) || n >= ((int64_t)1 << 32)) return fail(CGB_ERR_UNSUPPORTED, "more than 2^32 entries");
    if ((n > 0 && (!ICf || !ICv || !ICl)) || (n > 0 && normalize && !trk_norm) || (nE > 0 && !ECv) ||
        (nISOv > 0 && !ISOv))
        return fail(CGB_ERR_INVALID, "null dictionary array");
    NvtxRange nv("cgb_dict_relayout");
    cudaStream_t st = (cudaStream_t)stream;
    Scratch S;
    // look-up table: index of each grid voxel among the mask voxels (exclusive scan)
    uint32_t *m32, *lut;
    unsigned int *bad;
    CGB_TRY(S.get(&m32, ngrid));
    CGB_TRY(S.get(&lut, ngrid + 1));
    CGB_TRY(S.get(&bad, 1));
    CGB_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned int), st));
    k_mask_u32<<<grid_of(ngrid), 256, 0, st>>>(mask, ngrid, m32);
    CGB_CUDA(cudaGetLastError());
    size_t tb = 0;
    CGB_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, m32, lut, ngrid, st));
    void *t;
    CGB_TRY(S.get((uint8_t **)&t, tb));
    CGB_CUDA(cub::DeviceScan::ExclusiveSum(t, tb, m32, lut, ngrid, st));
    uint32_t last_lut = 0, last_m = 0;
    CGB_CUDA(cudaMemcpyAsync(&last_lut, lut + ngrid - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaMemcpyAsync(&last_m, m32 + ngrid - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    // IC: stable sort by voxel id, gather (and normalise), re-index
    if (n > 0) {
        k_check_ids<<<grid_of(n), 256, 0, st>>>(ICv, n, ngrid, bad);
        uint32_t *sv, *perm, *f0;
        uint16_t *o0 = nullptr;
        float *l0;
        CGB_TRY(S.get(&sv, n));
        CGB_TRY(S.get(&perm, n));
        CGB_TRY(S.get(&f0, n));
        CGB_TRY(S.get(&l0, n));
        CGB_CUDA(cudaMemcpyAsync(f0, ICf, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        CGB_CUDA(cudaMemcpyAsync(l0, ICl, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
        if (ICo) {
            CGB_TRY(S.get(&o0, n));
            CGB_CUDA(cudaMemcpyAsync(o0, ICo, n * sizeof(uint16_t), cudaMemcpyDeviceToDevice, st));
        }
        CGB_TRY(sort_by_voxel(ICv, n, ngrid, sv, perm, S, st));
        k_gather_ic<<<grid_of(n), 256, 0, st>>>(perm, n, sv, f0, o0, l0, trk_norm, nF, normalize, lut, ngrid, ICf,
                                                 ICv, ICo, ICl, bad);
        CGB_CUDA(cudaGetLastError());
    }
    if (nE > 0) {
        k_check_ids<<<grid_of(nE), 256, 0, st>>>(ECv, nE, ngrid, bad);
        uint32_t *sv, *perm;
        CGB_TRY(S.get(&sv, nE));
        CGB_TRY(S.get(&perm, nE));
        CGB_TRY(sort_by_voxel(ECv, nE, ngrid, sv, perm, S, st));
        if (ECo) {
            uint16_t *o0;
            CGB_TRY(S.get(&o0, nE));
            CGB_CUDA(cudaMemcpyAsync(o0, ECo, nE * sizeof(uint16_t), cudaMemcpyDeviceToDevice, st));
            k_gather_u16<<<grid_of(nE), 256, 0, st>>>(perm, nE, o0, ECo);
        }
        k_reindex<<<grid_of(nE), 256, 0, st>>>(sv, nE, lut, ngrid, ECv);
        CGB_CUDA(cudaGetLastError());
    }
    if (nISOv > 0) {
        k_check_ids<<<grid_of(nISOv), 256, 0, st>>>(ISOv, nISOv, ngrid, bad);
        uint32_t *sv, *perm;
        CGB_TRY(S.get(&sv, nISOv));
        CGB_TRY(S.get(&perm, nISOv));
        CGB_TRY(sort_by_voxel(ISOv, nISOv, ngrid, sv, perm, S, st));
        k_reindex<<<grid_of(nISOv), 256, 0, st>>>(sv, nISOv, lut, ngrid, ISOv);
        CGB_CUDA(cudaGetLastError());
    }
    unsigned int hbad = 0;
    CGB_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (hbad & 1u) return fail(CGB_ERR_INVALID, "dictionary voxel id outside the grid");
    if (hbad & 2u) return fail(CGB_ERR_INVALID, "IC streamline index >= number of streamlines");
    *nV_out = (int64_t)last_lut + (int64_t)last_m;
    return CGB_OK;
}
