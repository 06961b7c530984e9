/*
 * Test infrastructure: CPU restatement of trk2dictionary's streamline voxelisation, the
 * oracle that the GPU voxeliser is checked against.  Nothing in the product links it.
 *
 * Follows commit/trk2dictionary/trk2dictionary_c.cpp:
 *   fiberForwardModel      584-758  (replicas on circles around the first point, plane
 *                                    intersections per point, optional splitting of each
 *                                    step at voxel faces)
 *   segmentForwardModel    761-809  (direction folded to y >= 0, length rounded to float,
 *                                    voxel of the centroid, mask test, orientation from the
 *                                    181x181 hash table, float accumulation per key)
 *   rayBoxIntersection     814-870
 *   ICSegments             446-560  (keep test on the streamline length, output in key
 *                                    order (o, z, y, x), fibre norm from per-voxel sums)
 * and Vector.h:44-58 (norm() and Normalize() round the length to float).
 *
 * Compiled with -ffp-contract=off so no multiply-add is fused (the reference's x86 build
 * fuses none either).  Parity with the GPU is bit-exact for everything that uses only
 * +, -, *, /, sqrt, floor and round; atan2 (and sin / cos when blur replicas are used) come
 * from two different math libraries.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int dimx, dimy, dimz;
    float px, py, pz;            /* voxel size (mm) */
    float shx, shy, shz;         /* fibre shift (mm) */
    float min_seg_len, min_fiber_len, max_fiber_len;
    int do_intersect;
    int n_rep;                   /* blur replicas (1 = none) */
    const double *rho, *angle, *w;
} t2d_cfg;

typedef struct { double x, y, z; } v3;

typedef struct {
    uint16_t x, y, z, o;
    double len;                  /* w * len of this piece */
    int64_t seq;                 /* generation order */
} piece;

typedef struct {
    /* per kept streamline */
    float *trk_norm, *trk_len, *trk_lentot;
    /* per input streamline */
    uint8_t *kept;
    /* per segment */
    uint32_t *ic_f, *ic_v;
    uint16_t *ic_o;
    float *ic_len;
    int64_t n_seg, n_kept, cap_seg;
} t2d_out;

static float vnorm(v3 a) { return (float)sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

static v3 vnormalize(v3 a) {
    const float l = (float)sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    if (l == 0) return a;
    a.x = a.x / l;
    a.y = a.y / l;
    a.z = a.z / l;
    return a;
}

typedef struct {
    piece *p;
    int64_t n, cap;
    float flen, flentot;
} fibre_acc;

static void push(fibre_acc *A, piece q) {
    if (A->n == A->cap) {
        A->cap = A->cap ? 2 * A->cap : 256;
        A->p = (piece *)realloc(A->p, (size_t)A->cap * sizeof(piece));
    }
    q.seq = A->n;
    A->p[A->n++] = q;
}

static void add_segment(const t2d_cfg *c, v3 P1, v3 P2, int k, double w, const int16_t *hash, const uint8_t *mask,
                        fibre_acc *A) {
    v3 d;
    d.y = P2.y - P1.y;
    if (d.y >= 0) {
        d.x = P2.x - P1.x;
        d.z = P2.z - P1.z;
    } else {
        d.x = P1.x - P2.x;
        d.y = P1.y - P2.y;
        d.z = P1.z - P2.z;
    }
    const double len = vnorm(d);
    if (w * len <= c->min_seg_len) return;
    d = vnormalize(d);
    const int vx = (int)floor(0.5 * (P1.x + P2.x) / c->px);
    const int vy = (int)floor(0.5 * (P1.y + P2.y) / c->py);
    const int vz = (int)floor(0.5 * (P1.z + P2.z) / c->pz);
    if (vx >= c->dimx || vx < 0 || vy >= c->dimy || vy < 0 || vz >= c->dimz || vz < 0) return;
    if (mask && mask[vz + c->dimz * (vy + c->dimy * vx)] == 0) return;
    const double lon = atan2(d.y, d.x);
    const double colat = atan2(sqrt(d.x * d.x + d.y * d.y), d.z);
    const int ox = (int)round(colat / M_PI * 180.0);
    const int oy = (int)round(lon / M_PI * 180.0);
    /* the reference indexes hash[ox*181 + oy] unchecked; out-of-table indices (which it
     * would read out of bounds) are clamped to the table */
    int hi = ox * 181 + oy;
    if (hi < 0) hi = 0;
    if (hi > 181 * 181 - 1) hi = 181 * 181 - 1;
    piece q;
    q.x = (uint16_t)vx;
    q.y = (uint16_t)vy;
    q.z = (uint16_t)vz;
    q.o = (uint16_t)hash[hi];
    q.len = w * len;
    push(A, q);
    A->flentot += w * len;
    if (k == 0) A->flen += len;
}

static int box_hit(v3 o, v3 d, v3 lo, v3 hi, double *t) {
    double ix = 1.0 / d.x, iy = 1.0 / d.y, iz = 1.0 / d.z;
    double t0, t1, ty0, ty1, tz0, tz1;
    if (ix >= 0) { t0 = (lo.x - o.x) * ix; t1 = (hi.x - o.x) * ix; }
    else { t0 = (hi.x - o.x) * ix; t1 = (lo.x - o.x) * ix; }
    if (iy >= 0) { ty0 = (lo.y - o.y) * iy; ty1 = (hi.y - o.y) * iy; }
    else { ty0 = (hi.y - o.y) * iy; ty1 = (lo.y - o.y) * iy; }
    if (t0 > ty1 || ty0 > t1) return 0;
    if (ty0 > t0) t0 = ty0;
    if (ty1 < t1) t1 = ty1;
    if (iz >= 0) { tz0 = (lo.z - o.z) * iz; tz1 = (hi.z - o.z) * iz; }
    else { tz0 = (hi.z - o.z) * iz; tz1 = (lo.z - o.z) * iz; }
    if (t0 > tz1 || tz0 > t1) return 0;
    if (tz0 > t0) t0 = tz0;
    if (tz1 < t1) t1 = tz1;
    *t = t0 <= 0 ? t1 : t0;
    return 1;
}

/* one streamline: pts[3*i + {0,1,2}] for i < N (mm); blur: replicas in use */
static void fibre_model(const t2d_cfg *c, const float *pts, int N, int blur, const int16_t *hash, const uint8_t *mask,
                        fibre_acc *A, v3 *P) {
    A->n = 0;
    A->flen = 0.f;
    A->flentot = 0.f;
    if (N <= 2) return;
#define PT(i, a) ((double)(pts[3 * (i) + (a)] + (a == 0 ? c->shx : (a == 1 ? c->shy : c->shz))))
    v3 S1 = {PT(0, 0), PT(0, 1), PT(0, 2)};
    v3 dir2 = {PT(1, 0) - S1.x, PT(1, 1) - S1.y, PT(1, 2) - S1.z};
    dir2 = vnormalize(dir2);
    v3 n = {dir2.y - dir2.z, dir2.z - dir2.x, dir2.x - dir2.y};
    n = vnormalize(n);
    for (int k = 0; k < c->n_rep; ++k) {
        if (!blur && k > 0) continue;
        const double R = c->rho[k], alpha = c->angle[k];
        double w = sin(alpha / 2.0);
        const v3 q = {dir2.x * w, dir2.y * w, dir2.z * w};
        w = cos(alpha / 2.0);
        const v3 qn = {2.0 * (q.y * n.z - q.z * n.y), 2.0 * (q.z * n.x - q.x * n.z), 2.0 * (q.x * n.y - q.y * n.x)};
        const v3 qqn = {q.y * qn.z - q.z * qn.y, q.z * qn.x - q.x * qn.z, q.x * qn.y - q.y * qn.x};
        v3 nr = {n.x + w * qn.x + qqn.x, n.y + w * qn.y + qqn.y, n.z + w * qn.z + qqn.z};
        nr = vnormalize(nr);
        P[k].x = S1.x + R * nr.x;
        P[k].y = S1.y + R * nr.y;
        P[k].z = S1.z + R * nr.z;
    }
    for (int i = 1; i < N; ++i) {
        const v3 S2 = {PT(i, 0), PT(i, 1), PT(i, 2)};
        v3 dir1 = {S2.x - PT(i - 1, 0), S2.y - PT(i - 1, 1), S2.z - PT(i - 1, 2)};
        dir1 = vnormalize(dir1);
        if (i == N - 1) {
            dir2 = dir1;
        } else {
            dir2.x = PT(i + 1, 0) - S2.x;
            dir2.y = PT(i + 1, 1) - S2.y;
            dir2.z = PT(i + 1, 2) - S2.z;
            dir2 = vnormalize(dir2);
        }
        n.x = 0.5 * (dir1.x + dir2.x);
        n.y = 0.5 * (dir1.y + dir2.y);
        n.z = 0.5 * (dir1.z + dir2.z);
        const double dot = dir1.x * n.x + dir1.y * n.y + dir1.z * n.z;
        n.x /= dot;
        n.y /= dot;
        n.z /= dot;
        for (int k = 0; k < c->n_rep; ++k) {
            if (!blur && k > 0) continue;
            if (c->w[k] < 1e-3) continue;
            const v3 Po = P[k];
            double len = (S2.x - Po.x) * n.x + (S2.y - Po.y) * n.y + (S2.z - Po.z) * n.z;
            if (!(len > 0)) continue;
            P[k].x += dir1.x * len;
            P[k].y += dir1.y * len;
            P[k].z += dir1.z * len;
            if (!c->do_intersect) {
                add_segment(c, Po, P[k], k, c->w[k], hash, mask, A);
                continue;
            }
            v3 a = Po, b = P[k];
            for (;;) {
                len = sqrt(pow(b.x - a.x, 2) + pow(b.y - a.y, 2) + pow(b.z - a.z, 2));
                if (len <= c->min_seg_len) break;
                if (floor(a.x / c->px) == floor(b.x / c->px) && floor(a.y / c->py) == floor(b.y / c->py) &&
                    floor(a.z / c->pz) == floor(b.z / c->pz)) {
                    add_segment(c, a, b, k, c->w[k], hash, mask, A);
                    break;
                }
                v3 lo, hi;
                lo.x = floor((a.x + 1e-6 * dir1.x) / c->px) * c->px;
                lo.y = floor((a.y + 1e-6 * dir1.y) / c->py) * c->py;
                lo.z = floor((a.z + 1e-6 * dir1.z) / c->pz) * c->pz;
                hi.x = lo.x + c->px;
                hi.y = lo.y + c->py;
                hi.z = lo.z + c->pz;
                double t;
                if (box_hit(a, dir1, lo, hi, &t) && t > 0 && t < len) {
                    const v3 pi = {a.x + t * dir1.x, a.y + t * dir1.y, a.z + t * dir1.z};
                    add_segment(c, a, pi, k, c->w[k], hash, mask, A);
                    a = pi;
                } else {
                    add_segment(c, a, b, k, c->w[k], hash, mask, A);
                    break;
                }
            }
        }
    }
#undef PT
}

static int cmp_key(const void *pa, const void *pb) {
    const piece *a = (const piece *)pa, *b = (const piece *)pb;
    if (a->o != b->o) return a->o < b->o ? -1 : 1;
    if (a->z != b->z) return a->z < b->z ? -1 : 1;
    if (a->y != b->y) return a->y < b->y ? -1 : 1;
    if (a->x != b->x) return a->x < b->x ? -1 : 1;
    return a->seq < b->seq ? -1 : (a->seq > b->seq);
}

typedef struct { uint16_t x, y, z; float s; int64_t seq; } vsum;

static int cmp_vox(const void *pa, const void *pb) {
    const vsum *a = (const vsum *)pa, *b = (const vsum *)pb;
    if (a->z != b->z) return a->z < b->z ? -1 : 1;
    if (a->y != b->y) return a->y < b->y ? -1 : 1;
    if (a->x != b->x) return a->x < b->x ? -1 : 1;
    return a->seq < b->seq ? -1 : (a->seq > b->seq);
}

static void out_push(t2d_out *o, uint32_t f, uint32_t v, uint16_t or_, float l) {
    if (o->n_seg == o->cap_seg) {
        o->cap_seg = o->cap_seg ? 2 * o->cap_seg : 4096;
        o->ic_f = (uint32_t *)realloc(o->ic_f, (size_t)o->cap_seg * 4);
        o->ic_v = (uint32_t *)realloc(o->ic_v, (size_t)o->cap_seg * 4);
        o->ic_o = (uint16_t *)realloc(o->ic_o, (size_t)o->cap_seg * 2);
        o->ic_len = (float *)realloc(o->ic_len, (size_t)o->cap_seg * 4);
    }
    o->ic_f[o->n_seg] = f;
    o->ic_v[o->n_seg] = v;
    o->ic_o[o->n_seg] = or_;
    o->ic_len[o->n_seg] = l;
    o->n_seg++;
}

/* All streamlines: fibre f has points pts[3*off[f] .. 3*off[f+1]); blur_apply[f] (or NULL
 * for none) selects the replicas for fibre f.  Results in *out (free with t2d_free). */
int t2d_run(const t2d_cfg *c, const float *pts, const int64_t *off, int64_t nfib, const uint8_t *blur_apply,
            const int16_t *hash, const uint8_t *mask, t2d_out *out) {
    memset(out, 0, sizeof(*out));
    out->kept = (uint8_t *)calloc((size_t)(nfib > 0 ? nfib : 1), 1);
    out->trk_norm = (float *)malloc((size_t)(nfib > 0 ? nfib : 1) * 4);
    out->trk_len = (float *)malloc((size_t)(nfib > 0 ? nfib : 1) * 4);
    out->trk_lentot = (float *)malloc((size_t)(nfib > 0 ? nfib : 1) * 4);
    fibre_acc A = {0};
    v3 *P = (v3 *)calloc((size_t)(c->n_rep > 0 ? c->n_rep : 1), sizeof(v3));
    vsum *vs = NULL;
    int64_t vs_cap = 0;
    uint32_t kept_id = 0;
    for (int64_t f = 0; f < nfib; ++f) {
        const int N = (int)(off[f + 1] - off[f]);
        fibre_model(c, pts + 3 * off[f], N, blur_apply ? blur_apply[f] : 0, hash, mask, &A, P);
        if (A.n == 0 || !(A.flen > c->min_fiber_len && A.flen < c->max_fiber_len)) continue;
        qsort(A.p, (size_t)A.n, sizeof(piece), cmp_key);
        /* merged segments in key order, float sums in generation order */
        int64_t nm = 0;
        if (vs_cap < A.n) {
            vs_cap = A.n;
            vs = (vsum *)realloc(vs, (size_t)vs_cap * sizeof(vsum));
        }
        for (int64_t i = 0; i < A.n;) {
            int64_t j = i;
            float s = 0.f;
            while (j < A.n && A.p[j].o == A.p[i].o && A.p[j].z == A.p[i].z && A.p[j].y == A.p[i].y &&
                   A.p[j].x == A.p[i].x) {
                s += A.p[j].len;
                ++j;
            }
            const piece *q = &A.p[i];
            out_push(out, kept_id, (uint32_t)q->x + (uint32_t)c->dimx * ((uint32_t)q->y + (uint32_t)c->dimy * q->z), q->o,
                     s);
            vs[nm].x = q->x;
            vs[nm].y = q->y;
            vs[nm].z = q->z;
            vs[nm].s = s;
            vs[nm].seq = nm;
            ++nm;
            i = j;
        }
        /* fibre norm: per-voxel float sums (over orientations, in key order), then the sum of
         * their squares in voxel order (z, y, x) */
        qsort(vs, (size_t)nm, sizeof(vsum), cmp_vox);
        float norm = 0.f;
        for (int64_t i = 0; i < nm;) {
            int64_t j = i;
            float s = 0.f;
            while (j < nm && vs[j].x == vs[i].x && vs[j].y == vs[i].y && vs[j].z == vs[i].z) {
                s += vs[j].s;
                ++j;
            }
            norm += pow(s, 2);
            i = j;
        }
        norm = sqrt(norm);
        out->trk_norm[out->n_kept] = norm;
        out->trk_len[out->n_kept] = A.flen;
        out->trk_lentot[out->n_kept] = A.flentot;
        out->n_kept++;
        out->kept[f] = 1;
        kept_id++;
    }
    free(A.p);
    free(P);
    free(vs);
    return 0;
}

void t2d_free(t2d_out *o) {
    free(o->trk_norm);
    free(o->trk_len);
    free(o->trk_lentot);
    free(o->kept);
    free(o->ic_f);
    free(o->ic_v);
    free(o->ic_o);
    free(o->ic_len);
    memset(o, 0, sizeof(*o));
}
