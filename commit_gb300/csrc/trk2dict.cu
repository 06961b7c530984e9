// Streamline voxelisation on the device: the IC part of trk2dictionary
// (commit/trk2dictionary/trk2dictionary_c.cpp:446-870) producing the dictionary_IC_* and
// dictionary_TRK_* arrays.
//
// The reference walks each streamline on one CPU thread and merges its pieces in a
// std::map keyed by (orientation, z, y, x).  Here:
//   1. k_room          an estimate of each streamline's pieces (voxel faces crossed per
//                      step plus spares) gives it room in one piece buffer;
//   2. k_walk          one thread per streamline (longest first) runs the forward model
//                      and writes its keyed pieces (voxel, orientation, weighted length)
//                      into that room, reporting the count; a streamline that outgrew its
//                      room sends the whole call down the exact path (count walk, then
//                      emit walk at exact offsets);
//   3. a segmented stable sort by key per streamline (CUB) puts equal keys together in
//      generation order, so
//   4. k_merge sums each key's pieces in that order in FP32, exactly as the map's
//      `float += double` does, and writes the merged segments in key order;
//   5. a second segmented stable sort by voxel gives the per-voxel sums whose squares make
//      the streamline norm (k_norm), in the map's voxel order.
// The geometry is FP64 with the reference's operation order; this file is compiled with
// -fmad=false so no multiply-add is fused, and x*x replaces pow(x, 2).  The results are
// therefore bit-identical to the reference's except where atan2 (and sin / cos for blur
// replicas) of the two math libraries differ in the last place and that changes a
// rounded angle.  Streamline lengths and per-key sums stay FP32 as in the reference.
#include <cub/cub.cuh>

#include "cgb_internal.cuh"

namespace cgb {
namespace {

struct T2DCfg {
    int dimx, dimy, dimz;
    float px, py, pz, shx, shy, shz;
    float min_seg_len, min_fiber_len, max_fiber_len;
    int do_intersect, n_rep;
    const double *rho, *angle, *w;
};

struct D3 {
    double x, y, z;
};

// Vector<T>::norm() / Normalize() (Vector.h:44-58): the length is rounded to float
__device__ __forceinline__ float vlen(D3 a) { return (float)sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ D3 vunit(D3 a) {
    const float l = (float)sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    if (l == 0.f) return a;
    const double d = (double)l;
    return D3{a.x / d, a.y / d, a.z / d};
}

__device__ __forceinline__ uint64_t seg_key(unsigned o, unsigned z, unsigned y, unsigned x) {
    return ((uint64_t)o << 48) | ((uint64_t)z << 32) | ((uint64_t)y << 16) | (uint64_t)x;
}

// output of the walk for one streamline
struct Sink {
    uint64_t *key;       // null: count only
    double *len;
    int64_t n, cap;      // pieces produced; room at key / len
    float flen, flentot;
};

// (int)round(atan2(y, x) in degrees) as the reference evaluates it in FP64.  The FP64
// atan2 is the most expensive step of a piece on this part (FP64 is 1/58 of the FP32 rate),
// so it is evaluated in FP32 first (accurate to a few 1e-5 degree here) and again in FP64
// only when the FP32 value lies within 1e-3 degree of a rounding boundary, or an input is
// below FP32's normal range; the result is the FP64 one in every case.
__device__ __forceinline__ int round_deg(double y, double x) {
    const double ay = fabs(y), ax = fabs(x);
    const bool small = (ay != 0.0 && ay < 1e-30) || (ax != 0.0 && ax < 1e-30);
    if (!small) {
        const float v = atan2f((float)y, (float)x) * 57.2957795130823208768f;
        const float fr = v - floorf(v);
        if (fabsf(fr - 0.5f) > 1e-3f) return (int)floorf(v + 0.5f);
    }
    return (int)round(atan2(y, x) / 3.14159265358979323846 * 180.0);
}

__device__ void add_piece(const T2DCfg &c, D3 P1, D3 P2, int k, double w, const int16_t *__restrict__ hash,
                          const uint8_t *__restrict__ mask, Sink &S) {
    D3 d;
    d.y = P2.y - P1.y;
    if (d.y >= 0) {
        d.x = P2.x - P1.x;
        d.z = P2.z - P1.z;
    } else {
        d.x = P1.x - P2.x;
        d.y = P1.y - P2.y;
        d.z = P1.z - P2.z;
    }
    const double len = (double)vlen(d);
    if (w * len <= (double)c.min_seg_len) return;
    d = vunit(d);
    const int vx = (int)floor(0.5 * (P1.x + P2.x) / (double)c.px);
    const int vy = (int)floor(0.5 * (P1.y + P2.y) / (double)c.py);
    const int vz = (int)floor(0.5 * (P1.z + P2.z) / (double)c.pz);
    if (vx >= c.dimx || vx < 0 || vy >= c.dimy || vy < 0 || vz >= c.dimz || vz < 0) return;
    if (mask && mask[vz + (int64_t)c.dimz * (vy + (int64_t)c.dimy * vx)] == 0) return;
    const int oy = round_deg(d.y, d.x);
    const int ox = round_deg(sqrt(d.x * d.x + d.y * d.y), d.z);
    // the reference indexes hash[ox*181 + oy] unchecked; an index outside the table (which
    // it would read out of bounds) is clamped to the table
    int hi = ox * 181 + oy;
    hi = hi < 0 ? 0 : (hi > 181 * 181 - 1 ? 181 * 181 - 1 : hi);
    if (S.key && S.n < S.cap) {
        S.key[S.n] = seg_key((uint16_t)hash[hi], (unsigned)vz, (unsigned)vy, (unsigned)vx);
        S.len[S.n] = w * len;
    }
    S.n++;
    S.flentot = (float)((double)S.flentot + w * len);
    if (k == 0) S.flen = (float)((double)S.flen + len);
}

__device__ bool box_hit(D3 o, D3 d, D3 lo, D3 hi, double &t) {
    const double ix = 1.0 / d.x, iy = 1.0 / d.y, iz = 1.0 / d.z;
    double t0, t1, ty0, ty1, tz0, tz1;
    if (ix >= 0) { t0 = (lo.x - o.x) * ix; t1 = (hi.x - o.x) * ix; }
    else { t0 = (hi.x - o.x) * ix; t1 = (lo.x - o.x) * ix; }
    if (iy >= 0) { ty0 = (lo.y - o.y) * iy; ty1 = (hi.y - o.y) * iy; }
    else { ty0 = (hi.y - o.y) * iy; ty1 = (lo.y - o.y) * iy; }
    if (t0 > ty1 || ty0 > t1) return false;
    if (ty0 > t0) t0 = ty0;
    if (ty1 < t1) t1 = ty1;
    if (iz >= 0) { tz0 = (lo.z - o.z) * iz; tz1 = (hi.z - o.z) * iz; }
    else { tz0 = (hi.z - o.z) * iz; tz1 = (lo.z - o.z) * iz; }
    if (t0 > tz1 || tz0 > t1) return false;
    if (tz0 > t0) t0 = tz0;
    if (tz1 < t1) t1 = tz1;
    t = t0 <= 0 ? t1 : t0;
    return true;
}

constexpr int kMaxRep = 256;  // blur replicas handled per streamline (positions kept in local memory)

// one streamline per thread (fiberForwardModel, trk2dictionary_c.cpp:584-758)
__global__ void k_walk(const T2DCfg c, const float *__restrict__ pts, const int64_t *__restrict__ off, int64_t nfib,
                       const uint8_t *__restrict__ blur_apply, const int16_t *__restrict__ hash,
                       const uint8_t *__restrict__ mask, const int64_t *__restrict__ poff, uint64_t *__restrict__ keys,
                       double *__restrict__ lens, int64_t *__restrict__ cnt, float *__restrict__ flen,
                       float *__restrict__ flentot, const uint32_t *__restrict__ order) {
    // streamlines in order of decreasing point count, so a warp's walks have similar lengths
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (tid >= nfib) return;
    const int64_t f = order ? (int64_t)order[tid] : tid;
    Sink S;
    S.key = keys ? keys + poff[f] : nullptr;
    S.len = keys ? lens + poff[f] : nullptr;
    S.cap = keys ? poff[f + 1] - poff[f] : 0;
    S.n = 0;
    S.flen = 0.f;
    S.flentot = 0.f;
    const int64_t b = off[f];
    const int N = (int)(off[f + 1] - b);
    const float *p = pts + 3 * b;
    const bool blur = blur_apply && blur_apply[f];
    if (N > 2) {
        auto PT = [&](int i, int a) -> double {
            const float s = a == 0 ? c.shx : (a == 1 ? c.shy : c.shz);
            return (double)(p[3 * i + a] + s);
        };
        D3 P[kMaxRep];
        const D3 S1{PT(0, 0), PT(0, 1), PT(0, 2)};
        D3 dir2 = vunit(D3{PT(1, 0) - S1.x, PT(1, 1) - S1.y, PT(1, 2) - S1.z});
        D3 n = vunit(D3{dir2.y - dir2.z, dir2.z - dir2.x, dir2.x - dir2.y});
        for (int k = 0; k < c.n_rep; ++k) {
            if (!blur && k > 0) continue;
            const double R = c.rho[k], alpha = c.angle[k];
            double w = sin(alpha / 2.0);
            const D3 q{dir2.x * w, dir2.y * w, dir2.z * w};
            w = cos(alpha / 2.0);
            const D3 qn{2.0 * (q.y * n.z - q.z * n.y), 2.0 * (q.z * n.x - q.x * n.z), 2.0 * (q.x * n.y - q.y * n.x)};
            const D3 qqn{q.y * qn.z - q.z * qn.y, q.z * qn.x - q.x * qn.z, q.x * qn.y - q.y * qn.x};
            const D3 nr = vunit(D3{n.x + w * qn.x + qqn.x, n.y + w * qn.y + qqn.y, n.z + w * qn.z + qqn.z});
            P[k] = D3{S1.x + R * nr.x, S1.y + R * nr.y, S1.z + R * nr.z};
        }
        for (int i = 1; i < N; ++i) {
            const D3 S2{PT(i, 0), PT(i, 1), PT(i, 2)};
            const D3 dir1 = vunit(D3{S2.x - PT(i - 1, 0), S2.y - PT(i - 1, 1), S2.z - PT(i - 1, 2)});
            if (i == N - 1) dir2 = dir1;
            else dir2 = vunit(D3{PT(i + 1, 0) - S2.x, PT(i + 1, 1) - S2.y, PT(i + 1, 2) - S2.z});
            n = D3{0.5 * (dir1.x + dir2.x), 0.5 * (dir1.y + dir2.y), 0.5 * (dir1.z + dir2.z)};
            const double dot = dir1.x * n.x + dir1.y * n.y + dir1.z * n.z;
            n.x /= dot;
            n.y /= dot;
            n.z /= dot;
            for (int k = 0; k < c.n_rep; ++k) {
                if (!blur && k > 0) continue;
                if (c.w[k] < 1e-3) continue;
                const D3 Po = P[k];
                double len = (S2.x - Po.x) * n.x + (S2.y - Po.y) * n.y + (S2.z - Po.z) * n.z;
                if (!(len > 0)) continue;
                P[k].x += dir1.x * len;
                P[k].y += dir1.y * len;
                P[k].z += dir1.z * len;
                if (!c.do_intersect) {
                    add_piece(c, Po, P[k], k, c.w[k], hash, mask, S);
                    continue;
                }
                D3 a = Po;
                const D3 bb = P[k];
                // each pass either stops or moves a onto the next voxel face along dir1; the
                // bound only guards against a degenerate step that makes no progress
                for (int guard = 0; guard < 1 << 20; ++guard) {
                    const double ex = bb.x - a.x, ey = bb.y - a.y, ez = bb.z - a.z;
                    len = sqrt(ex * ex + ey * ey + ez * ez);
                    if (len <= (double)c.min_seg_len) break;
                    if (floor(a.x / (double)c.px) == floor(bb.x / (double)c.px) &&
                        floor(a.y / (double)c.py) == floor(bb.y / (double)c.py) &&
                        floor(a.z / (double)c.pz) == floor(bb.z / (double)c.pz)) {
                        add_piece(c, a, bb, k, c.w[k], hash, mask, S);
                        break;
                    }
                    D3 lo, hi;
                    lo.x = floor((a.x + 1e-6 * dir1.x) / (double)c.px) * (double)c.px;
                    lo.y = floor((a.y + 1e-6 * dir1.y) / (double)c.py) * (double)c.py;
                    lo.z = floor((a.z + 1e-6 * dir1.z) / (double)c.pz) * (double)c.pz;
                    hi = D3{lo.x + (double)c.px, lo.y + (double)c.py, lo.z + (double)c.pz};
                    double t;
                    if (box_hit(a, dir1, lo, hi, t) && t > 0 && t < len) {
                        const D3 pi{a.x + t * dir1.x, a.y + t * dir1.y, a.z + t * dir1.z};
                        add_piece(c, a, pi, k, c.w[k], hash, mask, S);
                        a = pi;
                    } else {
                        add_piece(c, a, bb, k, c.w[k], hash, mask, S);
                        break;
                    }
                }
            }
        }
    }
    if (cnt) {
        cnt[f] = S.n;
        flen[f] = S.flen;
        flentot[f] = S.flentot;
    }
}

// Room for the pieces of streamline f in the one-walk path: per step at most one piece per
// voxel face crossed plus the piece that ends the step, estimated from the raw points with
// three spare pieces per step, for every replica in use.  The walk writes min(count, room)
// pieces and reports the count, so a streamline whose projected steps outgrow the estimate
// is detected and the exact two-walk path is taken instead.
__global__ void k_room(const T2DCfg c, const float *__restrict__ pts, const int64_t *__restrict__ off, int64_t nfib,
                       const uint8_t *__restrict__ blur_apply, int64_t *__restrict__ room) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nfib) return;
    const int64_t b = off[f];
    const int N = (int)(off[f + 1] - b);
    if (N <= 2) {
        room[f] = 0;
        return;
    }
    const float *p = pts + 3 * b;
    float r = 0.f;
    for (int i = 1; i < N; ++i) {
        const float dx = fabsf(p[3 * i] - p[3 * i - 3]), dy = fabsf(p[3 * i + 1] - p[3 * i - 2]),
                    dz = fabsf(p[3 * i + 2] - p[3 * i - 1]);
        r += c.do_intersect ? dx / c.px + dy / c.py + dz / c.pz + 4.f : 1.f;
    }
    const int reps = (blur_apply && blur_apply[f]) ? c.n_rep : 1;
    room[f] = (int64_t)ceilf(r) * reps + 16;
}

// end of each streamline's pieces (begin + count) and whether any count exceeded its room
__global__ void k_ends(const int64_t *__restrict__ poff, const int64_t *__restrict__ cnt, int64_t nfib,
                       int64_t *__restrict__ pend, int *__restrict__ overflow) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nfib) return;
    const int64_t room = poff[f + 1] - poff[f];
    pend[f] = poff[f] + (cnt[f] < room ? cnt[f] : room);
    if (cnt[f] > room) *overflow = 1;
}

__global__ void k_npts(const int64_t *__restrict__ off, int64_t nfib, uint32_t *__restrict__ npts,
                       uint32_t *__restrict__ ids) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nfib) return;
    const int64_t n = off[f + 1] - off[f];
    npts[f] = (uint32_t)(n > 0xffffffffll ? 0xffffffffll : n);
    ids[f] = (uint32_t)f;
}

// merged segments of streamline f: runs of equal keys summed in FP32 in generation order.
// Pass 0 counts them (0 for a streamline that is not kept); pass 1 writes them.
__global__ void k_merge(int pass, int64_t nfib, const T2DCfg c, const int64_t *__restrict__ poff,
                        const int64_t *__restrict__ pend,
                        const uint64_t *__restrict__ keys, const double *__restrict__ lens,
                        const float *__restrict__ flen, const int64_t *__restrict__ soff,
                        const int64_t *__restrict__ kid, int64_t *__restrict__ mcnt, uint8_t *__restrict__ kept,
                        int64_t *__restrict__ kept64,
                        uint32_t *__restrict__ ic_f, uint32_t *__restrict__ ic_v, uint16_t *__restrict__ ic_o,
                        float *__restrict__ ic_len, uint64_t *__restrict__ vkey, float *__restrict__ vval) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nfib) return;
    const int64_t b = poff[f], e = pend[f];
    const bool keep = e > b && flen[f] > c.min_fiber_len && flen[f] < c.max_fiber_len;
    if (pass == 0) {
        kept[f] = keep ? 1 : 0;
        kept64[f] = keep ? 1 : 0;
        int64_t m = 0;
        if (keep)
            for (int64_t i = b; i < e; ++i)
                if (i == b || keys[i] != keys[i - 1]) ++m;
        mcnt[f] = m;
        return;
    }
    if (!keep) return;
    int64_t o = soff[f];
    const uint32_t fid = (uint32_t)kid[f];
    for (int64_t i = b; i < e;) {
        const uint64_t k = keys[i];
        float s = 0.f;
        int64_t j = i;
        for (; j < e && keys[j] == k; ++j) s = (float)((double)s + lens[j]);
        const unsigned x = (unsigned)(k & 0xffff), y = (unsigned)((k >> 16) & 0xffff), z = (unsigned)((k >> 32) & 0xffff);
        ic_f[o] = fid;
        ic_v[o] = x + (uint32_t)c.dimx * (y + (uint32_t)c.dimy * z);
        ic_o[o] = (uint16_t)(k >> 48);
        ic_len[o] = s;
        vkey[o] = k & 0xffffffffffffull;
        vval[o] = s;
        ++o;
        i = j;
    }
}

// fibre norm: per-voxel FP32 sums (orientations in key order), then the FP32 sum of their
// squares in voxel order and its square root (trk2dictionary_c.cpp:519-535)
__global__ void k_norm(int64_t nfib, const uint8_t *__restrict__ kept, const int64_t *__restrict__ soff,
                       const int64_t *__restrict__ kid, const uint64_t *__restrict__ vkey, const float *__restrict__ vval,
                       const float *__restrict__ flen, const float *__restrict__ flentot, float *__restrict__ norm,
                       float *__restrict__ tlen, float *__restrict__ tlentot) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nfib || !kept[f]) return;
    const int64_t b = soff[f], e = soff[f + 1];
    float acc = 0.f;
    for (int64_t i = b; i < e;) {
        float s = 0.f;
        int64_t j = i;
        for (; j < e && vkey[j] == vkey[i]; ++j) s = s + vval[j];
        acc = (float)((double)acc + (double)s * (double)s);
        i = j;
    }
    const int64_t k = kid[f];
    norm[k] = (float)sqrt((double)acc);
    tlen[k] = flen[f];
    tlentot[k] = flentot[f];
}

// track-density image (trk2dictionary_c.cpp:527): sum of segment lengths per voxel, as an
// (x, y, z) C-order array like the reference's; FP64 atomics, so the summation order (and
// the last bits) vary between runs, as they vary with the reference's thread count
__global__ void k_tdi(int64_t n, int dimx, int dimy, int dimz, const uint32_t *__restrict__ ic_v,
                      const float *__restrict__ ic_len, double *__restrict__ tdi) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = ic_v[i];
        const uint32_t x = v % (uint32_t)dimx, y = (v / (uint32_t)dimx) % (uint32_t)dimy, z = v / ((uint32_t)dimx * dimy);
        atomicAdd(tdi + ((int64_t)x * dimy + y) * dimz + z, (double)ic_len[i]);
    }
}

// EC entries from the peaks image (ECSegments, trk2dictionary_c.cpp:289-398): thread per
// voxel v = x + X*(y + Y*z) in increasing order (the reference's z, y, x loop), skipped
// where no segment passed (TDI == 0); each peak of norm >= vf_thr * the voxel's largest
// becomes one entry, its direction mapped through the affine and flips, folded to y >= 0
// and looked up in the hash table.  Pass 0 counts, pass 1 writes at off[v].
struct ECCfg {
    int dimx, dimy, dimz, np;
    float vf_thr;
    int flip[3];
    double aff[9];
};

__global__ void k_ec(int pass, const ECCfg c, const double *__restrict__ tdi, const float *__restrict__ peaks,
                     const int16_t *__restrict__ hash, int64_t *__restrict__ cnt, const int64_t *__restrict__ off,
                     uint32_t *__restrict__ ec_v, uint16_t *__restrict__ ec_o) {
    const int64_t nvox = (int64_t)c.dimx * c.dimy * c.dimz;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(v % c.dimx), iy = (int)((v / c.dimx) % c.dimy), iz = (int)(v / ((int64_t)c.dimx * c.dimy));
        const int64_t cell = iz + (int64_t)c.dimz * (iy + (int64_t)c.dimy * ix);
        int64_t m = 0;
        if (tdi[cell] != 0) {
            const float *pk = peaks + 3 * (int64_t)c.np * cell;
            float pmax = -1.f;
            for (int id = 0; id < c.np; ++id) {
                const float nrm = vlen(D3{pk[3 * id], pk[3 * id + 1], pk[3 * id + 2]});
                if (nrm > pmax) pmax = nrm;
            }
            if (pmax > 0) {
                int64_t o = pass ? off[v] : 0;
                for (int id = 0; id < c.np; ++id) {
                    const float *p = pk + 3 * id;
                    const float nrm = vlen(D3{p[0], p[1], p[2]});
                    if (nrm == 0 || nrm < c.vf_thr * pmax) continue;
                    D3 d;
                    d.x = (double)p[0] * c.aff[0] + (double)p[1] * c.aff[1] + (double)p[2] * c.aff[2];
                    d.y = (double)p[0] * c.aff[3] + (double)p[1] * c.aff[4] + (double)p[2] * c.aff[5];
                    d.z = (double)p[0] * c.aff[6] + (double)p[1] * c.aff[7] + (double)p[2] * c.aff[8];
                    d.x *= c.flip[0];
                    d.y *= c.flip[1];
                    d.z *= c.flip[2];
                    if (d.y < 0) {
                        d.x = -d.x;
                        d.y = -d.y;
                        d.z = -d.z;
                    }
                    const int ox = round_deg(sqrt(d.x * d.x + d.y * d.y), d.z);
                    const int oy = round_deg(d.y, d.x);
                    int hi = ox * 181 + oy;
                    hi = hi < 0 ? 0 : (hi > 181 * 181 - 1 ? 181 * 181 - 1 : hi);
                    if (pass) {
                        ec_v[o] = (uint32_t)v;
                        ec_o[o] = (uint16_t)hash[hi];
                        ++o;
                    }
                    ++m;
                }
            }
        }
        if (!pass) cnt[v] = m;
    }
}

// ISO voxels (ISOcompartments, trk2dictionary_c.cpp:400-440): v in increasing order where
// the ISO mask and the mask (when given) are set and some segment passed (TDI != 0)
__global__ void k_iso(int pass, int dimx, int dimy, int dimz, const double *__restrict__ tdi,
                      const uint8_t *__restrict__ mask, const uint8_t *__restrict__ iso_mask, int64_t *__restrict__ cnt,
                      const int64_t *__restrict__ off, uint32_t *__restrict__ iso_v) {
    const int64_t nvox = (int64_t)dimx * dimy * dimz;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(v % dimx), iy = (int)((v / dimx) % dimy), iz = (int)(v / ((int64_t)dimx * dimy));
        const int64_t cell = iz + (int64_t)dimz * (iy + (int64_t)dimy * ix);
        const bool in = (!iso_mask || iso_mask[cell]) && (!mask || mask[cell]) && tdi[cell] != 0;
        if (!pass) cnt[v] = in ? 1 : 0;
        else if (in) iso_v[off[v]] = (uint32_t)v;
    }
}

template <class T>
int dmalloc(T **p, size_t n, cudaStream_t st) {
    CGB_CUDA(cudaMallocAsync((void **)p, (n ? n : 1) * sizeof(T), st));
    return CGB_OK;
}

int exclusive_scan(const int64_t *in, int64_t *out, int64_t n, cudaStream_t st) {
    size_t bytes = 0;
    CGB_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, st));
    void *t = nullptr;
    CGB_TRY(dmalloc((char **)&t, bytes, st));
    const cudaError_t e = cub::DeviceScan::ExclusiveSum(t, bytes, in, out, n, st);
    cudaFreeAsync(t, st);
    CGB_CUDA(e);
    return CGB_OK;
}

template <class V>
int seg_sort(const uint64_t *kin, uint64_t *kout, const V *vin, V *vout, int64_t n, int64_t nseg, const int64_t *segoff,
             cudaStream_t st, const int64_t *segend = nullptr) {
    if (n == 0) return CGB_OK;
    if (!segend) segend = segoff + 1;
    size_t bytes = 0;
    CGB_CUDA(cub::DeviceSegmentedSort::StableSortPairs(nullptr, bytes, kin, kout, vin, vout, n, nseg, segoff,
                                                       segend, st));
    void *t = nullptr;
    CGB_TRY(dmalloc((char **)&t, bytes, st));
    const cudaError_t e = cub::DeviceSegmentedSort::StableSortPairs(t, bytes, kin, kout, vin, vout, n, nseg, segoff,
                                                                    segend, st);
    cudaFreeAsync(t, st);
    CGB_CUDA(e);
    return CGB_OK;
}

int read_i64(const int64_t *d, int64_t *h, cudaStream_t st) {
    CGB_CUDA(cudaMemcpyAsync(h, d, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    return CGB_OK;
}

}  // namespace
}  // namespace cgb

using namespace cgb;

extern "C" {

int cgb_trk2dict_free(cgb_t2d_result *r) {
    if (!r) return CGB_OK;
    void *ps[] = {r->ic_f,       r->ic_v,     r->ic_o, r->ic_len, r->trk_norm, r->trk_len,
                  r->trk_lentot, r->trk_kept, r->ec_v, r->ec_o,   r->iso_v,    r->tdi};
    for (void *p : ps)
        if (p) cudaFree(p);
    memset(r, 0, sizeof(*r));
    return CGB_OK;
}

int cgb_trk2dict(const cgb_t2d_params *prm, const float *pts, const int64_t *offsets, int64_t nfib,
                 const uint8_t *blur_apply, const int16_t *hash, const uint8_t *mask, const float *peaks,
                 const uint8_t *iso_mask, cgb_t2d_result *out, void *stream) {
    if (!prm || !out || !hash || (nfib > 0 && (!pts || !offsets))) return fail(CGB_ERR_INVALID, "null argument");
    if (nfib < 0) return fail(CGB_ERR_INVALID, "negative streamline count");
    NvtxRange nv("cgb_trk2dict");
    if (prm->dim[0] <= 0 || prm->dim[1] <= 0 || prm->dim[2] <= 0 || prm->dim[0] > 65535 || prm->dim[1] > 65535 ||
        prm->dim[2] > 65535)
        return fail(CGB_ERR_INVALID, "grid dimensions must be in 1..65535");
    if (prm->n_replicas < 1 || prm->n_replicas > kMaxRep || !prm->blur_rho || !prm->blur_angle || !prm->blur_weights)
        return fail(CGB_ERR_INVALID, "1..256 blur replicas with rho / angle / weights (device arrays)");
    memset(out, 0, sizeof(*out));
    cudaStream_t st = (cudaStream_t)stream;
    T2DCfg c;
    c.dimx = prm->dim[0];
    c.dimy = prm->dim[1];
    c.dimz = prm->dim[2];
    c.px = prm->pixdim[0];
    c.py = prm->pixdim[1];
    c.pz = prm->pixdim[2];
    c.shx = prm->fiber_shift[0] * prm->pixdim[0];
    c.shy = prm->fiber_shift[1] * prm->pixdim[1];
    c.shz = prm->fiber_shift[2] * prm->pixdim[2];
    c.min_seg_len = prm->min_seg_len;
    c.min_fiber_len = prm->min_fiber_len;
    c.max_fiber_len = prm->max_fiber_len;
    c.do_intersect = prm->do_intersect;
    c.n_rep = prm->n_replicas;
    c.rho = prm->blur_rho;
    c.angle = prm->blur_angle;
    c.w = prm->blur_weights;
    const int64_t nvox = (int64_t)c.dimx * c.dimy * c.dimz;
    const int64_t nf1 = nfib > 0 ? nfib : 1;
    int64_t *cnt = nullptr, *poff = nullptr, *mcnt = nullptr, *soff = nullptr, *kid = nullptr, *kept64 = nullptr;
    float *flen = nullptr, *flentot = nullptr;
    uint64_t *keys = nullptr, *keys2 = nullptr, *vkey = nullptr, *vkey2 = nullptr;
    double *lens = nullptr, *lens2 = nullptr;
    float *vval = nullptr, *vval2 = nullptr;
    int64_t *vcnt = nullptr, *voff = nullptr;
    uint32_t *npts = nullptr, *order = nullptr;  // [2*nfib]: counts / ids, sorted keys / sorted ids
    int64_t *pend = nullptr;                      // end of each streamline's pieces
    int *oflow = nullptr;
    int rc = CGB_OK;
    auto body = [&]() -> int {
        CGB_TRY(dmalloc(&cnt, nf1 + 1, st));
        CGB_TRY(dmalloc(&poff, nf1 + 1, st));
        CGB_TRY(dmalloc(&flen, nf1, st));
        CGB_TRY(dmalloc(&flentot, nf1, st));
        CGB_CUDA(cudaMemsetAsync(cnt, 0, (nf1 + 1) * sizeof(int64_t), st));
        const int tb = 128;
        const int gb = (int)((nfib + tb - 1) / tb);
        if (nfib > 0 && nfib < ((int64_t)1 << 31)) {
            CGB_TRY(dmalloc(&npts, 2 * nf1, st));
            CGB_TRY(dmalloc(&order, 2 * nf1, st));
            k_npts<<<gb, tb, 0, st>>>(offsets, nfib, npts, npts + nf1);
            CGB_CUDA(cudaGetLastError());
            size_t bytes = 0;
            CGB_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, bytes, npts, order + nf1, npts + nf1, order,
                                                                (int)nfib, 0, 32, st));
            void *t = nullptr;
            CGB_TRY(dmalloc((char **)&t, bytes, st));
            const cudaError_t e = cub::DeviceRadixSort::SortPairsDescending(t, bytes, npts, order + nf1, npts + nf1,
                                                                             order, (int)nfib, 0, 32, st);
            cudaFreeAsync(t, st);
            CGB_CUDA(e);
        }
        // one walk into estimated room per streamline; the exact two-walk path (count, then
        // emit) only if some streamline outgrew its room
        CGB_TRY(dmalloc(&pend, nf1, st));
        CGB_TRY(dmalloc(&oflow, 1, st));
        CGB_CUDA(cudaMemsetAsync(oflow, 0, sizeof(int), st));
        int64_t npieces = 0;
        int over = 1;
        if (nfib > 0) {
            k_room<<<gb, tb, 0, st>>>(c, pts, offsets, nfib, blur_apply, cnt);
            CGB_CUDA(cudaGetLastError());
            CGB_TRY(exclusive_scan(cnt, poff, nfib + 1, st));
            CGB_TRY(read_i64(poff + nfib, &npieces, st));
            const int64_t kMaxRoom = (int64_t)1 << 31;  // items of one segmented sort
            if (npieces < kMaxRoom) {
                CGB_TRY(dmalloc(&keys, npieces, st));
                CGB_TRY(dmalloc(&lens, npieces, st));
                k_walk<<<gb, tb, 0, st>>>(c, pts, offsets, nfib, blur_apply, hash, mask, poff, keys, lens, cnt, flen,
                                          flentot, order);
                CGB_CUDA(cudaGetLastError());
                k_ends<<<gb, tb, 0, st>>>(poff, cnt, nfib, pend, oflow);
                CGB_CUDA(cudaGetLastError());
                CGB_CUDA(cudaMemcpyAsync(&over, oflow, sizeof(int), cudaMemcpyDeviceToHost, st));
                CGB_CUDA(cudaStreamSynchronize(st));
            }
        } else {
            over = 0;
            CGB_CUDA(cudaMemsetAsync(poff, 0, sizeof(int64_t), st));
        }
        if (over) {
            if (keys) cudaFreeAsync(keys, st);
            if (lens) cudaFreeAsync(lens, st);
            keys = nullptr;
            lens = nullptr;
            k_walk<<<gb, tb, 0, st>>>(c, pts, offsets, nfib, blur_apply, hash, mask, nullptr, nullptr, nullptr, cnt,
                                      flen, flentot, order);
            CGB_CUDA(cudaGetLastError());
            CGB_TRY(exclusive_scan(cnt, poff, nfib + 1, st));
            CGB_TRY(read_i64(poff + nfib, &npieces, st));
            CGB_TRY(dmalloc(&keys, npieces, st));
            CGB_TRY(dmalloc(&lens, npieces, st));
            k_walk<<<gb, tb, 0, st>>>(c, pts, offsets, nfib, blur_apply, hash, mask, poff, keys, lens, nullptr, nullptr,
                                      nullptr, order);
            CGB_CUDA(cudaGetLastError());
            CGB_CUDA(cudaMemcpyAsync(pend, poff + 1, nfib * sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
        }
        CGB_TRY(dmalloc(&keys2, npieces, st));
        CGB_TRY(dmalloc(&lens2, npieces, st));
        CGB_TRY(seg_sort(keys, keys2, lens, lens2, npieces, nfib, poff, st, pend));
        // merge: counts, kept flags, offsets, kept ids
        CGB_TRY(dmalloc(&mcnt, nf1 + 1, st));
        CGB_TRY(dmalloc(&soff, nf1 + 1, st));
        CGB_TRY(dmalloc(&kid, nf1 + 1, st));
        CGB_TRY(dmalloc(&kept64, nf1 + 1, st));
        CGB_TRY(dmalloc(&out->trk_kept, nf1, st));
        CGB_CUDA(cudaMemsetAsync(mcnt, 0, (nf1 + 1) * sizeof(int64_t), st));
        CGB_CUDA(cudaMemsetAsync(kept64, 0, (nf1 + 1) * sizeof(int64_t), st));
        if (nfib > 0) {
            k_merge<<<gb, tb, 0, st>>>(0, nfib, c, poff, pend, keys2, lens2, flen, nullptr, nullptr, mcnt, out->trk_kept,
                                       kept64, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
            CGB_CUDA(cudaGetLastError());
        }
        CGB_TRY(exclusive_scan(mcnt, soff, nfib + 1, st));
        CGB_TRY(exclusive_scan(kept64, kid, nfib + 1, st));
        int64_t nseg = 0, nkept = 0;
        CGB_TRY(read_i64(soff + nfib, &nseg, st));
        CGB_TRY(read_i64(kid + nfib, &nkept, st));
        out->n_fibers = nfib;
        out->n_segments = nseg;
        out->n_kept = nkept;
        CGB_TRY(dmalloc(&out->ic_f, nseg, st));
        CGB_TRY(dmalloc(&out->ic_v, nseg, st));
        CGB_TRY(dmalloc(&out->ic_o, nseg, st));
        CGB_TRY(dmalloc(&out->ic_len, nseg, st));
        CGB_TRY(dmalloc(&out->trk_norm, nkept, st));
        CGB_TRY(dmalloc(&out->trk_len, nkept, st));
        CGB_TRY(dmalloc(&out->trk_lentot, nkept, st));
        CGB_TRY(dmalloc(&out->tdi, nvox, st));
        CGB_TRY(dmalloc(&vkey, nseg, st));
        CGB_TRY(dmalloc(&vkey2, nseg, st));
        CGB_TRY(dmalloc(&vval, nseg, st));
        CGB_TRY(dmalloc(&vval2, nseg, st));
        if (nfib > 0) {
            k_merge<<<gb, tb, 0, st>>>(1, nfib, c, poff, pend, keys2, lens2, flen, soff, kid, nullptr, nullptr, nullptr,
                                       out->ic_f,
                                       out->ic_v, out->ic_o, out->ic_len, vkey, vval);
            CGB_CUDA(cudaGetLastError());
        }
        CGB_TRY(seg_sort(vkey, vkey2, vval, vval2, nseg, nfib, soff, st));
        if (nfib > 0) {
            k_norm<<<gb, tb, 0, st>>>(nfib, out->trk_kept, soff, kid, vkey2, vval2, flen, flentot, out->trk_norm,
                                      out->trk_len, out->trk_lentot);
            CGB_CUDA(cudaGetLastError());
        }
        CGB_CUDA(cudaMemsetAsync(out->tdi, 0, nvox * sizeof(double), st));
        if (nseg > 0) {
            int g = (int)((nseg + 255) / 256);
            if (g > 4096) g = 4096;
            k_tdi<<<g, 256, 0, st>>>(nseg, c.dimx, c.dimy, c.dimz, out->ic_v, out->ic_len, out->tdi);
            CGB_CUDA(cudaGetLastError());
        }
        // EC and ISO compartments over the voxels (x fastest)
        CGB_TRY(dmalloc(&vcnt, nvox + 1, st));
        CGB_TRY(dmalloc(&voff, nvox + 1, st));
        int gv = (int)((nvox + 255) / 256);
        if (gv > 8192) gv = 8192;
        CGB_CUDA(cudaMemsetAsync(vcnt, 0, (nvox + 1) * sizeof(int64_t), st));
        if (peaks && prm->n_peaks > 0) {
            ECCfg e;
            e.dimx = c.dimx;
            e.dimy = c.dimy;
            e.dimz = c.dimz;
            e.np = prm->n_peaks;
            e.vf_thr = prm->vf_thr;
            for (int i = 0; i < 3; ++i) e.flip[i] = prm->flip[i];
            for (int i = 0; i < 9; ++i) e.aff[i] = prm->peaks_affine[i];
            k_ec<<<gv, 256, 0, st>>>(0, e, out->tdi, peaks, hash, vcnt, nullptr, nullptr, nullptr);
            CGB_CUDA(cudaGetLastError());
            CGB_TRY(exclusive_scan(vcnt, voff, nvox + 1, st));
            CGB_TRY(read_i64(voff + nvox, &out->n_ec, st));
            CGB_TRY(dmalloc(&out->ec_v, out->n_ec, st));
            CGB_TRY(dmalloc(&out->ec_o, out->n_ec, st));
            k_ec<<<gv, 256, 0, st>>>(1, e, out->tdi, peaks, hash, nullptr, voff, out->ec_v, out->ec_o);
            CGB_CUDA(cudaGetLastError());
        } else {
            CGB_TRY(dmalloc(&out->ec_v, 0, st));
            CGB_TRY(dmalloc(&out->ec_o, 0, st));
        }
        k_iso<<<gv, 256, 0, st>>>(0, c.dimx, c.dimy, c.dimz, out->tdi, mask, iso_mask, vcnt, nullptr, nullptr);
        CGB_CUDA(cudaGetLastError());
        CGB_TRY(exclusive_scan(vcnt, voff, nvox + 1, st));
        CGB_TRY(read_i64(voff + nvox, &out->n_iso, st));
        CGB_TRY(dmalloc(&out->iso_v, out->n_iso, st));
        k_iso<<<gv, 256, 0, st>>>(1, c.dimx, c.dimy, c.dimz, out->tdi, mask, iso_mask, nullptr, voff, out->iso_v);
        CGB_CUDA(cudaGetLastError());
        return CGB_OK;
    };
    rc = body();
    void *tmp[] = {cnt,  poff, mcnt, soff, kid,  kept64, flen, flentot, keys, keys2,
                   vkey, vkey2, lens, lens2, vval, vval2, vcnt, voff, npts, order, pend, oflow};
    for (void *q : tmp)
        if (q) cudaFreeAsync(q, st);
    if (rc == CGB_OK) {
        const cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_fail(e, "cgb_trk2dict");
    }
    if (rc != CGB_OK) {
        cudaStreamSynchronize(st);
        cgb_trk2dict_free(out);
    }
    return rc;
}

}  // extern "C"
