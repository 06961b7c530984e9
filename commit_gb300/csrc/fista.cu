// FISTA solver (commit/solvers.py:244-391) and proximal maps (commit/proximals.pyx:13-186)
// on the device.
//
// One solver iteration is: the smooth + proximal step fused into one elementwise pass
// (x = prox(xhat - step*grad, step), per-compartment maps of init_regularisation,
// solvers.py:16-206), the group-lasso prox as level-scheduled warp-per-group passes, one
// statistics pass giving <x-xhat,grad>, |x-xhat|^2, |x-prev_x|^2, |x|^2 and the l1 parts
// of Omega, the objective pass |sqrt(W)(A x - y)|^2 (voxel kernel with a norm epilogue,
// no y-sized write), and after the stopping tests the momentum pass and the fused
// gradient pass (A xhat - y formed per voxel in registers and fed straight into the
// adjoint).  All reductions are two-level (per block, then one block per quantity) in a
// fixed order, so a run is bitwise reproducible.  The host only reads back a handful of
// FP64 scalars once per objective evaluation to take the backtracking and stopping
// decisions exactly as the reference does.
#include <math.h>

#include <string.h>

#include <chrono>
#include <functional>
#include <vector>

#include "cgb_internal.cuh"
#include "operator_pair.cuh"

namespace cgb {
namespace {

constexpr int kStatSlots = 10;

struct RegDev {
    int64_t sIC, nIC, sEC, nEC, sISO, nISO;
    int reg_ic, reg_ec, reg_iso, nn_ic, nn_ec, nn_iso;
    double lam_ic, lam_ec, lam_iso;  // already multiplied by the prox scaling
    const double *w;
    int weighted_ic, weighted_iso;
};

struct L1Term {
    int64_t a, b;      // range [a, b)
    const double *w;   // weights or null
};

struct L1Terms {
    L1Term t[4];
    int n;
};

template <int NV>
__device__ __forceinline__ void block_sum_store_n(double (&v)[NV], double *dst) {
    __shared__ double red[NV][kBlock / 32];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
#pragma unroll
        for (int o = 16; o; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) red[j][threadIdx.x >> 5] = v[j];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            double t = threadIdx.x < kBlock / 32 ? red[j][threadIdx.x] : 0.0;
#pragma unroll
            for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) dst[j] = t;
        }
    }
}

__device__ __forceinline__ double soft(double v, double lam) {
    // proximals.pyx:25-39
    if (v > lam) return v - lam;
    if (v < -lam) return v + lam;
    return 0.0;
}

// x_out = prox(x_in - a*grad, s) for the elementwise parts of the regulariser
__global__ void k_prox_elem(double *__restrict__ xo, const double *__restrict__ xi, const double *__restrict__ grad,
                            double a, RegDev R, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = grad ? __dsub_rn(xi[i], __dmul_rn(a, grad[i])) : xi[i];
        if (i >= R.sISO && i < R.sISO + R.nISO) {
            if (R.reg_iso == CGB_REG_LASSO) v = soft(v, R.weighted_iso ? R.w[i] * R.lam_iso : R.lam_iso);
            if (R.nn_iso && v <= 0.0) v = 0.0;
        } else if (i >= R.sEC && i < R.sEC + R.nEC) {
            if (R.reg_ec == CGB_REG_LASSO) v = soft(v, R.lam_ec);
            if (R.nn_ec && v <= 0.0) v = 0.0;
        } else if (i >= R.sIC && i < R.sIC + R.nIC) {
            if (R.reg_ic == CGB_REG_LASSO || R.reg_ic == CGB_REG_SPARSE_GROUP_LASSO)
                v = soft(v, R.weighted_ic ? R.w[i] * R.lam_ic : R.lam_ic);
            if (R.nn_ic && (R.reg_ic == CGB_REG_NONE || R.reg_ic == CGB_REG_LASSO) && v <= 0.0) v = 0.0;
        }
        xo[i] = v;
    }
}

__global__ void k_nonneg(double *__restrict__ x, int64_t a, int64_t b) {
    for (int64_t i = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < b; i += (int64_t)gridDim.x * blockDim.x)
        if (x[i] <= 0.0) x[i] = 0.0;
}

__global__ void k_soft(double *__restrict__ x, const double *__restrict__ w, double lam, int64_t a, int64_t b) {
    for (int64_t i = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < b; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = soft(x[i], w ? w[i] * lam : lam);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// proximals.pyx:103-134 for the pairwise-disjoint groups [g0, g1): warp per group
__global__ void k_group_prox(double *__restrict__ x, int64_t nx, const int32_t *__restrict__ gidx,
                             const int64_t *__restrict__ gptr, const double *__restrict__ gw, int64_t g0, int64_t g1,
                             double lam, const double *__restrict__ plam) {
    if (plam) lam = *plam;  // graph mode: lam follows the device step
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t g = g0 + warp; g < g1; g += nw) {
        const int64_t beg = gptr[g], end = gptr[g + 1];
        double s = 0.0;
        for (int64_t k = beg + lane; k < end; k += 32) {
            const int64_t i = gidx[k];
            const double v = (i >= 0 && i < nx) ? x[i] : 0.0;
            s = fma(v, v, s);
        }
        s = warp_sum(s);
        const double gn = sqrt(s);
        const double wl = gw[g] * lam;
        if (gn <= wl) {
            for (int64_t k = beg + lane; k < end; k += 32) {
                const int64_t i = gidx[k];
                if (i >= 0 && i < nx) x[i] = 0.0;
            }
        } else {
            const double f = (gn - wl) / gn;
            for (int64_t k = beg + lane; k < end; k += 32) {
                const int64_t i = gidx[k];
                if (i >= 0 && i < nx) x[i] *= f;
            }
        }
    }
}

// per-group w_g*|x_g| (proximals.pyx:80-99), reduced per block into partials slot 0
__global__ void k_group_norms(const double *__restrict__ x, int64_t nx, const int32_t *__restrict__ gidx,
                              const int64_t *__restrict__ gptr, const double *__restrict__ gw, int64_t G,
                              double *__restrict__ partials) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double acc = 0.0;
    for (int64_t g = warp; g < G; g += nw) {
        double s = 0.0;
        for (int64_t k = gptr[g] + lane; k < gptr[g + 1]; k += 32) {
            const int64_t i = gidx[k];
            const double v = (i >= 0 && i < nx) ? x[i] : 0.0;
            s = fma(v, v, s);
        }
        s = warp_sum(s);
        if (lane == 0) acc += gw[g] * sqrt(s);
    }
    double v[1] = {acc};
    block_sum_store_n<1>(v, partials + (size_t)blockIdx.x * kRedSlots);
}

// FISTA statistics: slots 0 <x-xh,g>, 1 |x-xh|^2, 2 |x-p|^2, 3 |x|^2, 4.. l1 terms
__global__ void k_stats(const double *__restrict__ x, const double *__restrict__ xh, const double *__restrict__ g,
                        const double *__restrict__ p, int64_t n, L1Terms T, const double *__restrict__ xref,
                        double *__restrict__ partials) {
    double v[kStatSlots] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double xi = x[i];
        if (xh) {
            const double d = xi - xh[i];
            v[0] = fma(d, g[i], v[0]);
            v[1] = fma(d, d, v[1]);
        }
        if (p) {
            const double e = xi - p[i];
            v[2] = fma(e, e, v[2]);
        }
        v[3] = fma(xi, xi, v[3]);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < T.n && i >= T.t[k].a && i < T.t[k].b) v[4 + k] += fabs(T.t[k].w ? T.t[k].w[i] * xi : xi);
        if (xref) {
            const double r = xref[i];
            const double d = xi - r;
            v[8] = fma(d, d, v[8]);
            v[9] = fma(r, r, v[9]);
        }
    }
    block_sum_store_n<kStatSlots>(v, partials + (size_t)blockIdx.x * kRedSlots);
}

__global__ void k_dot(const double *__restrict__ a, const double *__restrict__ b, int64_t n,
                      double *__restrict__ partials) {
    double v[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[0] = fma(a[i], b[i], v[0]);
    block_sum_store_n<1>(v, partials + (size_t)blockIdx.x * kRedSlots);
}

__global__ void k_scale_range(double *__restrict__ x, int64_t a, int64_t b, double f) {
    for (int64_t i = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < b; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = f == 0.0 ? 0.0 : x[i] * f;
}

// out[j] = sum over blocks of partials[b*kRedSlots + j], j = blockIdx.x, fixed order
__global__ void k_finalize(const double *__restrict__ partials, int nblocks, double *__restrict__ out) {
    double v[1] = {0.0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v[0] += partials[(size_t)b * kRedSlots + blockIdx.x];
    double tmp[1];
    block_sum_store_n<1>(v, tmp);
    if (threadIdx.x == 0) out[blockIdx.x] = tmp[0];
}

// xhat = x + c*(x - prev); prev = x
__global__ void k_momentum(double *__restrict__ xh, const double *__restrict__ x, double *__restrict__ p, double c,
                           int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double xi = x[i];
        xh[i] = __dadd_rn(xi, __dmul_rn(c, __dsub_rn(xi, p[i])));
        p[i] = xi;
    }
}

int elem_grid(const cgb_op *op, int64_t n) {
    int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = (int64_t)op->nsm * 4;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

int finalize(const double *partials, int nblocks, int nslots, double *out, cudaStream_t st) {
    k_finalize<<<nslots, kBlock, 0, st>>>(partials, nblocks, out);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

// ------------------------------------------------------------------ graph-captured FISTA
// The whole iteration loop as one CUDA graph: a WHILE node runs the iterations, a nested
// WHILE node the backtracking steps, an IF node the momentum + gradient of a continuing
// iteration.  The decisions the host takes in Solver::run are taken by one-thread
// controller kernels on device scalars (same expressions, no fused multiply-adds, so the
// same bits), which set the conditional handles.  The host launches the graph once and
// reads the final scalars.
struct GState {
    double step, told, prev_obj, qfval, curr_obj, reg_x, res_norm, abs_obj, rel_obj, abs_x, rel_x, c;
    double tol_fun, tol_x;
    double l1coef[4];
    double group_coef;
    int nterms, group_in_omega;
    int it, crit, backtracks, max_iter;
    int bt_iter, max_bt;  // backtracks of the current iteration and their cap
    int reuse;            // A x_hat of the gradient pass comes from the stored rows
    int anchored;         // this iteration's qfval was evaluated again directly
    int anchor_req;       // the next backtracking evaluation starts with that evaluation
    int anchors;          // such evaluations over the solve
};

__device__ __forceinline__ double g_omega(const GState &S, const double *h) {
    double om = 0.0;
    for (int k = 0; k < S.nterms; ++k) om = __dadd_rn(om, __dmul_rn(S.l1coef[k], h[5 + k]));
    if (S.group_in_omega) om = __dadd_rn(om, __dmul_rn(S.group_coef, h[11]));
    return om;
}

// qfval of the iteration (solvers.py:309-313): the residual of the gradient pass
__global__ void k_ctl_begin(GState *S, const double *h) {
    const double r = __dsqrt_rn(h[12]);
    S->qfval = S->it == 1 ? S->prev_obj : __dmul_rn(__dmul_rn(0.5, r), r);
    S->bt_iter = 0;
    S->anchored = 0;
}

// whether this backtracking evaluation starts with a direct evaluation of f(x_hat)
__global__ void k_ctl_anchor_decide(const GState *S, cudaGraphConditionalHandle anchor) {
    cudaGraphSetConditional(anchor, S->anchor_req);
}

// qfval from a direct evaluation of x_hat (slot 0 of h), replacing the stored-row one
__global__ void k_ctl_anchor(GState *S, const double *h) {
    const double r = __dsqrt_rn(h[0]);
    S->qfval = __dmul_rn(__dmul_rn(0.5, r), r);
    S->anchors += 1;
}

// objective and quadratic model of the evaluated x (solvers.py:315-333); on failure of the
// sufficient-decrease test shrink the step and ask for another evaluation.  A qfval taken
// from the stored rows is rounded differently from the evaluation of x, so near convergence
// the test can fail at the rounding level for every step; its first failure in an iteration
// asks instead for f(x_hat) evaluated directly, as the reference computes it, and the same
// step is judged again (anchor_req)
__global__ void k_ctl_judge(GState *S, const double *h, cudaGraphConditionalHandle bt) {
    const double reg = g_omega(*S, h);
    const double d2 = __dsqrt_rn(h[2]);
    const double q = __dadd_rn(__dadd_rn(__dadd_rn(S->qfval, h[1]), __dmul_rn(__ddiv_rn(0.5, S->step), __dmul_rn(d2, d2))),
                               reg);
    const double rn = __dsqrt_rn(h[0]);
    const double cur = __dadd_rn(__dmul_rn(__dmul_rn(0.5, rn), rn), reg);
    S->reg_x = reg;
    S->res_norm = rn;
    S->curr_obj = cur;
    int an = 0, more = 0;
    if (cur > q && S->reuse && S->it > 1 && !S->anchored) {
        S->anchored = 1;
        an = 1;
        more = 1;
    } else if (cur > q && S->bt_iter >= S->max_bt) {
        S->crit = -1;  // cap reached: leave the backtracking loop, k_ctl_stop ends the solve
    } else if (cur > q) {
        S->step = __dmul_rn(0.9, S->step);
        S->backtracks += 1;
        S->bt_iter += 1;
        more = 1;
    }
    S->anchor_req = an;
    cudaGraphSetConditional(bt, more);
}

// stopping tests (solvers.py:335-357) and the FISTA coefficients (solvers.py:359-368)
__global__ void k_ctl_stop(GState *S, const double *h, cudaGraphConditionalHandle hmain,
                           cudaGraphConditionalHandle hcont) {
    if (S->crit == -1) {
        cudaGraphSetConditional(hmain, 0);
        cudaGraphSetConditional(hcont, 0);
        return;
    }
    const double eps = 2.220446049250313e-16;
    const double a = fabs(__dsub_rn(S->curr_obj, S->prev_obj));
    S->abs_obj = a;
    S->rel_obj = __ddiv_rn(a, S->curr_obj);
    S->abs_x = __dsqrt_rn(h[3]);
    S->rel_x = __ddiv_rn(S->abs_x, __dadd_rn(__dsqrt_rn(h[4]), eps));
    int crit = -1;
    if (S->abs_obj < eps) crit = 0;
    else if (S->rel_obj < S->tol_fun) crit = 1;
    else if (S->abs_x < eps) crit = 2;
    else if (S->rel_x < S->tol_x) crit = 3;
    else if (S->it >= S->max_iter) crit = 4;
    if (crit >= 0) {
        S->crit = crit;
        cudaGraphSetConditional(hmain, 0);
        cudaGraphSetConditional(hcont, 0);
        return;
    }
    const double t = __dmul_rn(0.5, __dadd_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(__dmul_rn(4.0, S->told), S->told)))));
    S->c = __ddiv_rn(__dsub_rn(S->told, 1.0), t);
    S->told = t;
    S->prev_obj = S->curr_obj;
    S->it += 1;
    cudaGraphSetConditional(hcont, 1);
}

__global__ void k_prox_elem_dev(double *__restrict__ xo, const double *__restrict__ xi, const double *__restrict__ grad,
                                const GState *__restrict__ S, RegDev R, int64_t n) {
    const double s = S->step;
    R.lam_ic = __dmul_rn(s, R.lam_ic);
    R.lam_ec = __dmul_rn(s, R.lam_ec);
    R.lam_iso = __dmul_rn(s, R.lam_iso);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = __dsub_rn(xi[i], __dmul_rn(s, grad[i]));
        if (i >= R.sISO && i < R.sISO + R.nISO) {
            if (R.reg_iso == CGB_REG_LASSO) v = soft(v, R.weighted_iso ? R.w[i] * R.lam_iso : R.lam_iso);
            if (R.nn_iso && v <= 0.0) v = 0.0;
        } else if (i >= R.sEC && i < R.sEC + R.nEC) {
            if (R.reg_ec == CGB_REG_LASSO) v = soft(v, R.lam_ec);
            if (R.nn_ec && v <= 0.0) v = 0.0;
        } else if (i >= R.sIC && i < R.sIC + R.nIC) {
            if (R.reg_ic == CGB_REG_LASSO || R.reg_ic == CGB_REG_SPARSE_GROUP_LASSO)
                v = soft(v, R.weighted_ic ? R.w[i] * R.lam_ic : R.lam_ic);
            if (R.nn_ic && (R.reg_ic == CGB_REG_NONE || R.reg_ic == CGB_REG_LASSO) && v <= 0.0) v = 0.0;
        }
        xo[i] = v;
    }
}

__global__ void k_momentum_dev(double *__restrict__ xh, const double *__restrict__ x, double *__restrict__ p,
                               const GState *__restrict__ S, int64_t n) {
    const double c = S->c;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double xi = x[i];
        xh[i] = __dadd_rn(xi, __dmul_rn(c, __dsub_rn(xi, p[i])));
        p[i] = xi;
    }
}

// One elementwise pass of an evaluation of x (regularisers without groups): optionally the
// deferred momentum of the iteration (xhat = x + c*(x - prev), prev = x, exactly as
// k_momentum), then x = prox(xhat - a*grad) (k_prox_elem / k_prox_elem_dev) and the
// statistics of k_stats, with the fixed-order final sums of k_finalize done by the last
// block to finish (out[0..9]; out[10], the group penalty, is 0).  Same expressions and the
// same summation order as the separate kernels, so the iterates are bitwise the same.
template <bool DEV>
__global__ void k_prox_stats(double *__restrict__ x, double *__restrict__ xh, const double *__restrict__ g,
                             double *__restrict__ p, double a, RegDev R, int64_t n, int mom, double c,
                             const GState *__restrict__ S, L1Terms T, const double *__restrict__ xref,
                             double *__restrict__ partials, unsigned int *__restrict__ counter,
                             double *__restrict__ out) {
    if (DEV) {
        const double s = S->step;
        a = s;
        R.lam_ic = __dmul_rn(s, R.lam_ic);
        R.lam_ec = __dmul_rn(s, R.lam_ec);
        R.lam_iso = __dmul_rn(s, R.lam_iso);
    }
    double v[kStatSlots] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double xhi, pi;
        if (mom) {
            const double xo = x[i];
            xhi = __dadd_rn(xo, __dmul_rn(c, __dsub_rn(xo, p[i])));
            xh[i] = xhi;
            p[i] = xo;
            pi = xo;
        } else {
            xhi = xh[i];
            pi = p[i];
        }
        const double gi = g[i];
        double w = __dsub_rn(xhi, __dmul_rn(a, gi));
        if (i >= R.sISO && i < R.sISO + R.nISO) {
            if (R.reg_iso == CGB_REG_LASSO) w = soft(w, R.weighted_iso ? R.w[i] * R.lam_iso : R.lam_iso);
            if (R.nn_iso && w <= 0.0) w = 0.0;
        } else if (i >= R.sEC && i < R.sEC + R.nEC) {
            if (R.reg_ec == CGB_REG_LASSO) w = soft(w, R.lam_ec);
            if (R.nn_ec && w <= 0.0) w = 0.0;
        } else if (i >= R.sIC && i < R.sIC + R.nIC) {
            if (R.reg_ic == CGB_REG_LASSO || R.reg_ic == CGB_REG_SPARSE_GROUP_LASSO)
                w = soft(w, R.weighted_ic ? R.w[i] * R.lam_ic : R.lam_ic);
            if (R.nn_ic && (R.reg_ic == CGB_REG_NONE || R.reg_ic == CGB_REG_LASSO) && w <= 0.0) w = 0.0;
        }
        x[i] = w;
        const double d = w - xhi;
        v[0] = fma(d, gi, v[0]);
        v[1] = fma(d, d, v[1]);
        const double e = w - pi;
        v[2] = fma(e, e, v[2]);
        v[3] = fma(w, w, v[3]);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < T.n && i >= T.t[k].a && i < T.t[k].b) v[4 + k] += fabs(T.t[k].w ? T.t[k].w[i] * w : w);
        if (xref) {
            const double r = xref[i];
            const double dd = w - r;
            v[8] = fma(dd, dd, v[8]);
            v[9] = fma(r, r, v[9]);
        }
    }
    block_sum_store_n<kStatSlots>(v, partials + (size_t)blockIdx.x * kRedSlots);
    // the last block to finish forms the final sums, in k_finalize's order
    __shared__ unsigned int is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    for (int j = 0; j < kStatSlots; ++j) {
        double t[1] = {0.0};
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) t[0] += __ldcg(partials + (size_t)b * kRedSlots + j);
        double tot[1];
        block_sum_store_n<1>(t, tot);
        if (threadIdx.x == 0) out[j] = tot[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[kStatSlots] = 0.0;
        *counter = 0u;
    }
}

// graph mode with momentum reuse: A x_hat = (1+c) A x - c A x_prev from the stored rows,
// with c the device-side momentum coefficient and the rounding of the gradient kernels'
// own combination (ax_combine), so the graph's iterates are those of the host loop
__global__ void k_ax_combine_dev(double *__restrict__ out, const double *__restrict__ a, const double *__restrict__ b,
                                 const GState *__restrict__ S, int64_t n) {
    const double c = S->c;
    const double ca = __dadd_rn(1.0, c), cb = -c;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = detail::ax_combine(ca, a[i], cb, b[i]);
}

__global__ void k_ax_combine32_dev(float *__restrict__ out, const float *__restrict__ a, const float *__restrict__ b,
                                   const GState *__restrict__ S, int64_t n) {
    const double c = S->c;
    const float ca = (float)__dadd_rn(1.0, c), cb = (float)(-c);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = detail::ax_combine(ca, a[i], cb, b[i]);
}

// lam = lam_base * step for the group prox of the graph (the host path passes it directly)
__global__ void k_scale_lam(const GState *__restrict__ S, double lam_base, double *__restrict__ out) {
    *out = __dmul_rn(S->step, lam_base);
}

}  // namespace

// ------------------------------------------------------------------ solver workspace
struct FistaWS {
    int64_t ncols = 0, nrows = 0;
    double *xhat = nullptr, *prev = nullptr, *grad = nullptr, *ax[3] = {nullptr, nullptr, nullptr};
    double *pstats = nullptr, *pgrp = nullptr, *pres = nullptr;
    unsigned int *counter = nullptr;  // arrival counter of the fused elementwise pass (k_prox_stats)
    // reduced-precision path: FP32 copies of y and sqrt(W), FP32 A*x buffers
    float *y32 = nullptr, *sqw32 = nullptr, *ax32[3] = {nullptr, nullptr, nullptr};
    cudaStream_t st = nullptr;  // allocations are stream-ordered on the solver's stream
    ~FistaWS() {
        void *ps[] = {xhat, prev, grad, ax[0], ax[1], ax[2], pstats, pgrp, pres, y32, sqw32, ax32[0], ax32[1], ax32[2],
                      counter};
        for (void *p : ps)
            if (p) cudaFreeAsync(p, st);
    }
};

namespace {

// stream-ordered allocation: no device-wide synchronisation, so solvers on other streams
// (e.g. one regularisation path per tractogram) keep running
template <class T>
int ws_alloc(T **p, size_t n, cudaStream_t st) {
    CGB_CUDA(cudaMallocAsync((void **)p, (n ? n : 1) * sizeof(T), st));
    return CGB_OK;
}

struct Solver {
    cgb_op *op;
    const double *y, *sqw;
    const cgb_reg *reg;
    const cgb_fista_params *prm;
    cudaStream_t st;
    FistaWS ws;
    L1Terms terms;
    double l1coef[4];
    int has_group_prox = 0, group_in_omega = 0;
    int fused_elem = 0;  // regulariser without groups: one fused elementwise pass per evaluation
    double group_omega_coef = 0.0;
    int calls = 0;

    bool mixed = false;
    bool batch_member = false;  // one problem of a batch: row buffers belong to the batch
    double *dsc = nullptr;      // this problem's 16 device scalars
    const GState *gdev = nullptr;  // graph mode: the device-side state (step) kernels read
    double *glam = nullptr;        // graph mode: device copy of the group-prox lambda

    int init() {
        const int64_t nc = op->ncols, nr = op->nrows;
        const int rb = partial_blocks(op);
        mixed = prm->arith == CGB_ARITH_BF16 || prm->arith == CGB_ARITH_FP16 || prm->arith == CGB_ARITH_F32;
        if (!dsc) dsc = op->dscal;
        ws.st = st;
        CGB_TRY(ws_alloc(&ws.xhat, nc, st));
        CGB_TRY(ws_alloc(&ws.prev, nc, st));
        CGB_TRY(ws_alloc(&ws.grad, nc, st));
        if (batch_member) {
        } else if (mixed) {
            CGB_TRY(ensure_reduced(op, prm->arith));
            CGB_TRY(ws_alloc(&ws.y32, nr, st));
            CGB_TRY(convert_f64_to_f32(y, ws.y32, nr, st));
            if (sqw) {
                CGB_TRY(ws_alloc(&ws.sqw32, nr, st));
                CGB_TRY(convert_f64_to_f32(sqw, ws.sqw32, nr, st));
            }
            if (prm->momentum_reuse) {
                CGB_TRY(ws_alloc(&ws.ax32[0], nr, st));
                CGB_TRY(ws_alloc(&ws.ax32[1], nr, st));
                if (prm->graph) CGB_TRY(ws_alloc(&ws.ax32[2], nr, st));
            }
        } else if (prm->momentum_reuse) {
            CGB_TRY(ws_alloc(&ws.ax[0], nr, st));
            CGB_TRY(ws_alloc(&ws.ax[1], nr, st));
            if (prm->graph) CGB_TRY(ws_alloc(&ws.ax[2], nr, st));
        }
        CGB_TRY(ws_alloc(&ws.pstats, (size_t)rb * kRedSlots, st));
        CGB_TRY(ws_alloc(&ws.pgrp, (size_t)rb * kRedSlots, st));
        CGB_TRY(ws_alloc(&ws.pres, (size_t)rb * kRedSlots, st));
        // l1 parts of Omega with the reference's slicing (solvers.py:68, 150, 183)
        terms.n = 0;
        auto clamp = [&](int64_t v) { return v < 0 ? 0 : (v > nc ? nc : v); };
        auto add = [&](int64_t a, int64_t b, const double *w, double c) {
            a = clamp(a);
            b = clamp(b);
            if (b <= a || c == 0.0) return;
            terms.t[terms.n] = L1Term{a, b, w};
            l1coef[terms.n] = c;
            terms.n++;
        };
        const cgb_reg &R = *reg;
        if (R.reg_ic == CGB_REG_LASSO) {
            // x[startIC:sizeIC]
            add(R.start_ic, R.size_ic, R.weighted_ic ? R.coeff_weights : nullptr, R.lambda_ic);
        } else if (R.reg_ic == CGB_REG_SPARSE_GROUP_LASSO) {
            // whole x (proximals.pyx:150, 177-178); weighted with all_coeff_weights
            if (R.lambda_ic != 0.0 || R.lambda_ic_group != 0.0)
                add(0, nc, R.weighted_ic ? R.coeff_weights : nullptr, R.lambda_ic);
        }
        if (R.reg_ec == CGB_REG_LASSO) add(R.start_ec, R.start_ec + R.size_ec, nullptr, R.lambda_ec);
        if (R.reg_iso == CGB_REG_LASSO) {
            if (R.weighted_iso) add(R.start_iso, R.size_iso, R.coeff_weights, R.lambda_iso);  // [startISO:sizeISO]
            else add(R.start_iso, R.start_iso + R.size_iso, nullptr, R.lambda_iso);
        }
        if (R.reg_ic == CGB_REG_GROUP_LASSO || R.reg_ic == CGB_REG_SPARSE_GROUP_LASSO) {
            const double lg = R.reg_ic == CGB_REG_GROUP_LASSO ? R.lambda_ic : R.lambda_ic_group;
            has_group_prox = R.ngroups > 0;
            if (R.reg_ic == CGB_REG_GROUP_LASSO) {
                group_in_omega = lg != 0.0;
                group_omega_coef = lg;
            } else {
                group_in_omega = (R.lambda_ic != 0.0 || lg != 0.0);
                group_omega_coef = lg;
            }
            if (R.ngroups > 0 && (!R.group_idx || !R.group_ptr || !R.group_w))
                return fail(CGB_ERR_INVALID, "group arrays are NULL");
        }
        if ((R.weighted_ic || R.weighted_iso) && !R.coeff_weights)
            return fail(CGB_ERR_INVALID, "weighted regulariser without coeff_weights");
        const bool grp = R.reg_ic == CGB_REG_GROUP_LASSO || R.reg_ic == CGB_REG_SPARSE_GROUP_LASSO;
        fused_elem = nc > 0 && !has_group_prox && !group_in_omega && !grp;
        if (fused_elem) {
            CGB_TRY(ws_alloc(&ws.counter, 1, st));
            CGB_CUDA(cudaMemsetAsync(ws.counter, 0, sizeof(unsigned int), st));
        }
        return CGB_OK;
    }

    // x = prox(xhat - a*grad) and its statistics in one pass (fused_elem); mom: apply the
    // iteration's deferred momentum with coefficient c first
    int prox_stats(double *x, double a, int mom, double c) {
        const int64_t nc = op->ncols;
        const int gb = elem_grid(op, nc);
        if (gdev)
            k_prox_stats<true><<<gb, kBlock, 0, st>>>(x, ws.xhat, ws.grad, ws.prev, 0.0, regdev(1.0), nc, 0, 0.0, gdev,
                                                      terms, prm->x_ref, ws.pstats, ws.counter, dsc + 1);
        else
            k_prox_stats<false><<<gb, kBlock, 0, st>>>(x, ws.xhat, ws.grad, ws.prev, a, regdev(a), nc, mom, c, nullptr,
                                                       terms, prm->x_ref, ws.pstats, ws.counter, dsc + 1);
        CGB_CUDA(cudaGetLastError());
        return CGB_OK;
    }

    RegDev regdev(double s) const {
        const cgb_reg &R = *reg;
        RegDev d;
        d.sIC = R.start_ic; d.nIC = R.size_ic; d.sEC = R.start_ec; d.nEC = R.size_ec;
        d.sISO = R.start_iso; d.nISO = R.size_iso;
        d.reg_ic = R.reg_ic; d.reg_ec = R.reg_ec; d.reg_iso = R.reg_iso;
        d.nn_ic = R.nn_ic; d.nn_ec = R.nn_ec; d.nn_iso = R.nn_iso;
        d.lam_ic = s * R.lambda_ic;
        d.lam_ec = s * R.lambda_ec;
        d.lam_iso = s * R.lambda_iso;
        d.w = R.coeff_weights;
        d.weighted_ic = R.weighted_ic; d.weighted_iso = R.weighted_iso;
        return d;
    }

    // x_out = prox(x_in - a*grad, s) (grad may be null), in place allowed
    int prox(double *xo, const double *xi, const double *grad, double a, double s) {
        const int64_t nc = op->ncols;
        if (nc == 0) return CGB_OK;
        if (gdev) {
            // graph mode: step (= a = s) read on the device
            k_prox_elem_dev<<<elem_grid(op, nc), kBlock, 0, st>>>(xo, xi, grad, gdev, regdev(1.0), nc);
        } else {
            k_prox_elem<<<elem_grid(op, nc), kBlock, 0, st>>>(xo, xi, grad, a, regdev(s), nc);
        }
        CGB_CUDA(cudaGetLastError());
        const cgb_reg &R = *reg;
        if (has_group_prox) {
            const double lam_base = R.reg_ic == CGB_REG_GROUP_LASSO ? R.lambda_ic : R.lambda_ic_group;
            const double lam = gdev ? lam_base : s * lam_base;
            if (gdev && lam_base != 0.0) {
                k_scale_lam<<<1, 1, 0, st>>>(gdev, lam_base, glam);
                CGB_CUDA(cudaGetLastError());
            }
            if (lam != 0.0) {
                for (int64_t k = 0; k < R.nlevels; ++k) {
                    const int64_t g0 = R.level_ptr[k], g1 = R.level_ptr[k + 1];
                    if (g1 <= g0) continue;
                    int64_t blocks = ((g1 - g0) * 32 + kBlock - 1) / kBlock;
                    if (blocks > op->nsm * 8) blocks = op->nsm * 8;
                    k_group_prox<<<(int)blocks, kBlock, 0, st>>>(xo, op->ncols, R.group_idx, R.group_ptr, R.group_w, g0, g1,
                                                                lam, gdev ? glam : nullptr);
                    CGB_CUDA(cudaGetLastError());
                }
            }
        }
        if (R.nn_ic && (R.reg_ic == CGB_REG_GROUP_LASSO || R.reg_ic == CGB_REG_SPARSE_GROUP_LASSO) && R.size_ic > 0) {
            k_nonneg<<<elem_grid(op, R.size_ic), kBlock, 0, st>>>(xo, R.start_ic, R.start_ic + R.size_ic);
            CGB_CUDA(cudaGetLastError());
        }
        return CGB_OK;
    }

    // statistics of x (and omega pieces) into dscal[1..8], group omega into dscal[9]
    int stats(const double *x, const double *xh, const double *g, const double *p) {
        const int64_t nc = op->ncols;
        const int gb = elem_grid(op, nc);
        k_stats<<<gb, kBlock, 0, st>>>(x, xh, g, p, nc, terms, xh ? prm->x_ref : nullptr, ws.pstats);
        CGB_CUDA(cudaGetLastError());
        CGB_TRY(finalize(ws.pstats, gb, kStatSlots, dsc + 1, st));
        if (group_in_omega) {
            int64_t blocks = (reg->ngroups * 32 + kBlock - 1) / kBlock;
            if (blocks > op->nsm * 4) blocks = op->nsm * 4;
            if (blocks < 1) blocks = 1;
            k_group_norms<<<(int)blocks, kBlock, 0, st>>>(x, op->ncols, reg->group_idx, reg->group_ptr, reg->group_w,
                                                         reg->ngroups, ws.pgrp);
            CGB_CUDA(cudaGetLastError());
            CGB_TRY(finalize(ws.pgrp, (int)blocks, 1, dsc + 11, st));
        } else {
            CGB_CUDA(cudaMemsetAsync(dsc + 11, 0, sizeof(double), st));
        }
        return CGB_OK;
    }

    double omega_from(const double *h) const {
        double om = 0.0;
        for (int k = 0; k < terms.n; ++k) om += l1coef[k] * h[5 + k];
        if (group_in_omega) om += group_omega_coef * h[11];
        return om;
    }

    // |sqw*(A x - y)|^2 -> dscal[0]; with slot >= 0, A x -> A*x buffer `slot`
    int objective(const double *x, int slot) {
        int g = 0;
        if (mixed) {
            CGB_TRY(launch_resnorm_mix(op, x, ws.y32, ws.sqw32, op->partials, slot >= 0 ? ws.ax32[slot] : nullptr,
                                       nullptr, st, prm->arith, &g));
        } else {
            CGB_TRY(launch_resnorm_grid(op, x, y, sqw, op->partials, slot >= 0 ? ws.ax[slot] : nullptr, st,
                                        prm->arith, &g));
        }
        calls++;
        if (g > 0) {
            CGB_TRY(finalize(op->partials, g, 1, op->dscal + 0, st));
        } else {
            CGB_CUDA(cudaMemsetAsync(op->dscal, 0, sizeof(double), st));
        }
        return CGB_OK;
    }

    // grad = A'(W (A x - y)) (or, with sa >= 0, A x = ca*ax[sa] + cb*ax[sb]), |r|^2 -> dscal[10]
    int gradient(const double *x, double *grad, int sa, int sb, double ca, double cb) {
        int g = 0;
        if (mixed) {
            CGB_TRY(launch_gradient_mix(op, x, ws.y32, ws.sqw32, grad, ws.pres, sa >= 0 ? ws.ax32[sa] : nullptr,
                                        sb >= 0 ? ws.ax32[sb] : nullptr, (float)ca, (float)cb, st, prm->arith, &g));
        } else {
            CGB_TRY(launch_gradient_grid(op, x, y, sqw, grad, ws.pres, sa >= 0 ? ws.ax[sa] : nullptr,
                                         sb >= 0 ? ws.ax[sb] : nullptr, ca, cb, st, prm->arith, &g));
        }
        calls += sa >= 0 ? 1 : 2;
        if (g > 0) {
            CGB_TRY(finalize(ws.pres, g, 1, op->dscal + 12, st));
        } else {
            CGB_CUDA(cudaMemsetAsync(op->dscal + 12, 0, sizeof(double), st));
        }
        return CGB_OK;
    }

    int fetch(double *h) {
        CGB_CUDA(cudaMemcpyAsync(h, op->dscal, 16 * sizeof(double), cudaMemcpyDeviceToHost, st));
        CGB_CUDA(cudaStreamSynchronize(st));
        return CGB_OK;
    }

    int run(double *x, cgb_fista_result *res) {
        const int max_bt = prm->max_backtracks > 0 ? prm->max_backtracks : (prm->max_backtracks < 0 ? 0 : 1000);
        const int64_t nc = op->ncols;
        const double eps = 2.220446049250313e-16;
        double *h = op->h_scal;
        const double beta = 0.9;
        int backtracks = 0;
        const auto t_start = std::chrono::steady_clock::now();
        // initialisation (solvers.py:260-286)
        CGB_CUDA(cudaMemcpyAsync(ws.xhat, x, nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
        CGB_TRY(gradient(ws.xhat, ws.grad, -1, -1, 0.0, 0.0));
        CGB_TRY(prox(ws.xhat, ws.xhat, nullptr, 0.0, 1.0));
        CGB_TRY(stats(ws.xhat, nullptr, nullptr, nullptr));
        CGB_TRY(fetch(h));
        double res_norm = sqrt(h[12]);
        double reg_term = omega_from(h);
        double prev_obj = 0.5 * res_norm * res_norm + reg_term;
        double told = 1.0;
        CGB_CUDA(cudaMemcpyAsync(ws.prev, ws.xhat, nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
        double qfval = prev_obj;
        // step size from one Rayleigh quotient of grad (solvers.py:282-286)
        {
            int g = 0;
            k_dot<<<elem_grid(op, nc), kBlock, 0, st>>>(ws.grad, ws.grad, nc, ws.pstats);
            CGB_CUDA(cudaGetLastError());
            CGB_TRY(finalize(ws.pstats, elem_grid(op, nc), 1, op->dscal + 13, st));
            if (mixed) {
                CGB_TRY(launch_resnorm_mix(op, ws.grad, nullptr, ws.sqw32, op->partials, nullptr, nullptr, st,
                                           prm->arith, &g));
            } else {
                CGB_TRY(launch_resnorm_grid(op, ws.grad, nullptr, sqw, op->partials, nullptr, st, prm->arith, &g));
            }
            calls++;
            if (g > 0) {
                CGB_TRY(finalize(op->partials, g, 1, op->dscal + 14, st));
            } else {
                CGB_CUDA(cudaMemsetAsync(op->dscal + 14, 0, sizeof(double), st));
            }
            CGB_TRY(fetch(h));
        }
        const double Ln = sqrt(h[14]) / sqrt(h[13]);
        const double L = Ln * Ln;
        double step = 1.9 / L;
        if (prm->verbose == 4) {
            printf("\n      |  1/2||Ax-y||^2      Omega      |  Cost function    Abs error      Rel error    |"
                   "      Abs x          Rel x    \n");
            printf("------|--------------------------------|-----------------------------------------------|"
                   "------------------------------\n");
        }
        int it = 1;
        int cur = 0;          // ax buffer written by objective(x)
        int have_prev_ax = 0; // ax[1-cur] holds A*prev_x
        double curr_obj = 0, reg_term_x = 0, abs_obj = 0, rel_obj = 0, abs_x = 0, rel_x = 0;
        int crit = 4;
        int anchors = 0;      // direct evaluations of f(x_hat) (see k_ctl_judge)
        bool q_rows = false;  // this iteration's qfval comes from the stored rows
        int pend_mom = 0;     // momentum deferred into the next evaluation's fused pass
        double pend_c = 0.0;
        while (true) {
            NvtxRange nvi("fista iteration");
            auto eval_x = [&](double s) -> int {
                if (fused_elem) {
                    CGB_TRY(prox_stats(x, s, pend_mom, pend_c));
                    pend_mom = 0;
                } else {
                    CGB_TRY(prox(x, ws.xhat, ws.grad, s, s));
                    CGB_TRY(stats(x, ws.xhat, ws.grad, ws.prev));
                }
                CGB_TRY(objective(x, prm->momentum_reuse ? cur : -1));
                return fetch(h);
            };
            CGB_TRY(eval_x(step));
            qfval = 0.5 * sqrt(h[12]) * sqrt(h[12]);
            if (it == 1) qfval = prev_obj;
            reg_term_x = omega_from(h);
            double q = qfval + h[1] + 0.5 / step * (sqrt(h[2]) * sqrt(h[2])) + reg_term_x;
            res_norm = sqrt(h[0]);
            curr_obj = 0.5 * res_norm * res_norm + reg_term_x;
            int bt_iter = 0;
            bool anchored = false;
            while (curr_obj > q) {
                if (q_rows && !anchored) {
                    // qfval from the stored rows: judge this step again against f(x_hat)
                    // evaluated directly, as the reference computes it (see k_ctl_judge)
                    anchored = true;
                    anchors++;
                    CGB_TRY(objective(ws.xhat, -1));
                    CGB_TRY(fetch(h));
                    qfval = 0.5 * sqrt(h[0]) * sqrt(h[0]);
                    CGB_TRY(eval_x(step));
                    reg_term_x = omega_from(h);
                    q = qfval + h[1] + 0.5 / step * (sqrt(h[2]) * sqrt(h[2])) + reg_term_x;
                    res_norm = sqrt(h[0]);
                    curr_obj = 0.5 * res_norm * res_norm + reg_term_x;
                    continue;
                }
                if (bt_iter >= max_bt)
                    return fail(CGB_ERR_BACKTRACK, "FISTA: backtracking of iteration " + std::to_string(it) +
                                                       " reached its cap of " + std::to_string(max_bt) + " step reductions");
                ++bt_iter;
                step = beta * step;
                backtracks++;
                CGB_TRY(eval_x(step));
                reg_term_x = omega_from(h);
                q = qfval + h[1] + 0.5 / step * (sqrt(h[2]) * sqrt(h[2])) + reg_term_x;
                res_norm = sqrt(h[0]);
                curr_obj = 0.5 * res_norm * res_norm + reg_term_x;
            }
            if (prm->trace && prm->x_ref && it <= prm->trace_len) {
                const int w = prm->trace_cost ? 3 : 2;
                double *t = prm->trace + (size_t)w * (it - 1);
                t[0] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
                t[1] = sqrt(h[9]) / sqrt(h[10]);
                if (w == 3) t[2] = curr_obj;
            }
            abs_obj = fabs(curr_obj - prev_obj);
            rel_obj = abs_obj / curr_obj;
            abs_x = sqrt(h[3]);
            rel_x = abs_x / (sqrt(h[4]) + eps);
            if (prm->verbose == 4)
                printf("%4d  |  %13.7e  %13.7e  |  %13.7e  %13.7e  %13.7e  |  %13.7e  %13.7e\n", it,
                       0.5 * res_norm * res_norm, reg_term_x, curr_obj, abs_obj, rel_obj, abs_x, rel_x);
            if (abs_obj < eps) { crit = 0; break; }
            if (rel_obj < prm->tol_fun) { crit = 1; break; }
            if (abs_x < eps) { crit = 2; break; }
            if (rel_x < prm->tol_x) { crit = 3; break; }
            if (it >= prm->max_iter) { crit = 4; break; }
            // FISTA update (solvers.py:359-368); with restart, a rise of the objective resets
            // the momentum
            if (prm->restart && curr_obj > prev_obj) told = 1.0;
            const double t = 0.5 * (1.0 + sqrt(1.0 + 4.0 * told * told));
            const double c = (told - 1.0) / t;
            if (prm->momentum_reuse && (c == 0.0 || have_prev_ax)) {
                // A*xhat = (1+c) A*x - c A*prev_x: the gradient does not read xhat, so with a
                // fused elementwise pass the momentum itself waits for the next evaluation
                if (fused_elem) {
                    pend_mom = 1;
                    pend_c = c;
                } else {
                    k_momentum<<<elem_grid(op, nc), kBlock, 0, st>>>(ws.xhat, x, ws.prev, c, nc);
                    CGB_CUDA(cudaGetLastError());
                }
                CGB_TRY(gradient(ws.xhat, ws.grad, cur, have_prev_ax ? 1 - cur : cur, 1.0 + c, -c));
                q_rows = true;
            } else {
                k_momentum<<<elem_grid(op, nc), kBlock, 0, st>>>(ws.xhat, x, ws.prev, c, nc);
                CGB_CUDA(cudaGetLastError());
                CGB_TRY(gradient(ws.xhat, ws.grad, -1, -1, 0.0, 0.0));
                q_rows = false;
            }
            if (prm->momentum_reuse) {
                cur = 1 - cur;
                have_prev_ax = 1;
            }
            it += 1;
            prev_obj = curr_obj;
            told = t;
        }
        if (prm->verbose == 4) {
            static const char *names[] = {"Absolute tolerance on the objective", "Relative tolerance on the objective",
                                          "Absolute tolerance on the unknowns", "Relative tolerance on the unknowns",
                                          "Maximum number of iterations"};
            printf("< Stopping criterion: %s >\n", names[crit]);
        }
        res->residual = 0.5 * res_norm * res_norm;
        res->regterm = reg_term_x;
        res->cost_function = curr_obj;
        res->abs_cost = abs_obj;
        res->rel_cost = rel_obj;
        res->abs_x = abs_x;
        res->rel_x = rel_x;
        res->iterations = it;
        res->stopping_criterion = crit;
        res->backtracks = backtracks;
        res->operator_calls = calls;
        res->anchors = anchors;
        CGB_CUDA(cudaStreamSynchronize(st));
        return CGB_OK;
    }

    // --------------------------------------------------------------- graph mode
    // One evaluation of x = prox(xhat - step*grad) with its statistics and objective.
    int eval_dev(double *x, int slot) {
        if (fused_elem) {
            CGB_TRY(prox_stats(x, 0.0, 0, 0.0));
        } else {
            CGB_TRY(prox(x, ws.xhat, ws.grad, 0.0, 0.0));
            CGB_TRY(stats(x, ws.xhat, ws.grad, ws.prev));
        }
        return objective(x, slot);
    }

    // add a conditional node at the current point of the capture on `cap`, capture its body
    // on `body_st` with f(), and continue the capture after the node
    template <class F>
    int conditional(cudaStream_t cap, cudaStream_t body_st, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                    F &&f) {
        cudaStreamCaptureStatus status;
        cudaGraph_t cg;
        const cudaGraphNode_t *deps = nullptr;
        size_t ndeps = 0;
        CGB_CUDA(cudaStreamGetCaptureInfo(cap, &status, nullptr, &cg, &deps, nullptr, &ndeps));
        cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
        np.conditional.handle = h;
        np.conditional.type = type;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        CGB_CUDA(cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &np));
        cudaGraph_t body = np.conditional.phGraph_out[0];
        const cudaStream_t outer = st;
        st = body_st;
        CGB_CUDA(cudaStreamBeginCaptureToGraph(body_st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        int rc = f();
        cudaGraph_t done = nullptr;
        const cudaError_t e = cudaStreamEndCapture(body_st, &done);
        st = outer;
        CGB_TRY(rc);
        CGB_CUDA(e);
        CGB_CUDA(cudaStreamUpdateCaptureDependencies(cap, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        return CGB_OK;
    }

    // FISTA with the iteration loop as one graph launch (no trace).  With momentum reuse the
    // body holds two iterations, so the two stored A x rows alternate with fixed pointers.
    int run_graph(double *x, cgb_fista_result *res) {
        const int64_t nc = op->ncols;
        const bool reuse = prm->momentum_reuse != 0;
        double *h = op->h_scal;
        // initialisation on the host path (solvers.py:260-286), as in run()
        CGB_CUDA(cudaMemcpyAsync(ws.xhat, x, nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
        CGB_TRY(gradient(ws.xhat, ws.grad, -1, -1, 0.0, 0.0));
        CGB_TRY(prox(ws.xhat, ws.xhat, nullptr, 0.0, 1.0));
        CGB_TRY(stats(ws.xhat, nullptr, nullptr, nullptr));
        CGB_TRY(fetch(h));
        double res_norm = sqrt(h[12]);
        const double prev_obj = 0.5 * res_norm * res_norm + omega_from(h);
        CGB_CUDA(cudaMemcpyAsync(ws.prev, ws.xhat, nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
        {
            int g = 0;
            k_dot<<<elem_grid(op, nc), kBlock, 0, st>>>(ws.grad, ws.grad, nc, ws.pstats);
            CGB_CUDA(cudaGetLastError());
            CGB_TRY(finalize(ws.pstats, elem_grid(op, nc), 1, op->dscal + 13, st));
            if (mixed) {
                CGB_TRY(launch_resnorm_mix(op, ws.grad, nullptr, ws.sqw32, op->partials, nullptr, nullptr, st,
                                           prm->arith, &g));
            } else {
                CGB_TRY(launch_resnorm_grid(op, ws.grad, nullptr, sqw, op->partials, nullptr, st, prm->arith, &g));
            }
            calls++;
            if (g > 0) {
                CGB_TRY(finalize(op->partials, g, 1, op->dscal + 14, st));
            } else {
                CGB_CUDA(cudaMemsetAsync(op->dscal + 14, 0, sizeof(double), st));
            }
            CGB_TRY(fetch(h));
        }
        const double Ln = sqrt(h[14]) / sqrt(h[13]);
        GState G;
        memset(&G, 0, sizeof(G));
        G.step = 1.9 / (Ln * Ln);
        G.told = 1.0;
        G.prev_obj = prev_obj;
        G.tol_fun = prm->tol_fun;
        G.tol_x = prm->tol_x;
        G.nterms = terms.n;
        for (int k = 0; k < terms.n; ++k) G.l1coef[k] = l1coef[k];
        G.group_in_omega = group_in_omega;
        G.group_coef = group_omega_coef;
        G.it = 1;
        G.crit = 4;
        G.max_iter = prm->max_iter;
        G.max_bt = prm->max_backtracks > 0 ? prm->max_backtracks : (prm->max_backtracks < 0 ? 0 : 1000);
        G.reuse = reuse;
        GState *gs = nullptr;
        CGB_TRY(ws_alloc(&gs, 1, st));
        CGB_TRY(ws_alloc(&glam, 1, st));
        CGB_CUDA(cudaMemcpyAsync(gs, &G, sizeof(G), cudaMemcpyHostToDevice, st));
        CGB_CUDA(cudaStreamSynchronize(st));
        gdev = gs;
        if (reuse) {
            // the first iteration combines A x with a zero "previous" row (c = 0 there)
            if (mixed) CGB_CUDA(cudaMemsetAsync(ws.ax32[1], 0, op->nrows * sizeof(float), st));
            else CGB_CUDA(cudaMemsetAsync(ws.ax[1], 0, op->nrows * sizeof(double), st));
        }
        // graph: WHILE(main) { ITER(0) } without reuse, WHILE(main) { ITER(0, IF(cont) { ITER(1) }) }
        // with it, where ITER(s) = begin; eval; judge; WHILE(bt) { eval; judge }; stop;
        // IF(cont) { momentum; gradient; ... } and eval writes A x to stored row s
        cudaStream_t s0 = nullptr, s1 = nullptr, s2 = nullptr, s3 = nullptr, s4 = nullptr;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        const cudaStream_t user = st;
        double *d = op->dscal;
        auto build = [&]() -> int {
            CGB_CUDA(cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking));
            CGB_CUDA(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking));
            CGB_CUDA(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
            CGB_CUDA(cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking));
            CGB_CUDA(cudaStreamCreateWithFlags(&s4, cudaStreamNonBlocking));
            CGB_CUDA(cudaGraphCreate(&graph, 0));
            // every handle belongs to exactly one conditional node: the anchors' IF nodes
            // exist only with momentum reuse, and so do their handles
            cudaGraphConditionalHandle hmain, hbt, hcont, hbt2 = 0, hcont2 = 0, hq = 0, hq2 = 0;
            if (reuse) {
                CGB_CUDA(cudaGraphConditionalHandleCreate(&hq, graph, 0, cudaGraphCondAssignDefault));
                CGB_CUDA(cudaGraphConditionalHandleCreate(&hq2, graph, 0, cudaGraphCondAssignDefault));
            }
            CGB_CUDA(cudaGraphConditionalHandleCreate(&hmain, graph, 1, cudaGraphCondAssignDefault));
            CGB_CUDA(cudaGraphConditionalHandleCreate(&hbt, graph, 0, cudaGraphCondAssignDefault));
            CGB_CUDA(cudaGraphConditionalHandleCreate(&hcont, graph, 0, cudaGraphCondAssignDefault));
            if (reuse) {
                CGB_CUDA(cudaGraphConditionalHandleCreate(&hbt2, graph, 0, cudaGraphCondAssignDefault));
                CGB_CUDA(cudaGraphConditionalHandleCreate(&hcont2, graph, 0, cudaGraphCondAssignDefault));
            }
            const int64_t nr = op->nrows;
            // one iteration captured on `cap`: evaluation into stored row `slot` (-1: none),
            // backtracking (WHILE(bt) { IF(anchor) { f(x_hat) directly }; eval; judge }),
            // stopping test, and for a continuing iteration the momentum, the gradient at
            // x_hat and then `more`.  The anchor's IF node and the kernel that sets its handle
            // sit in the backtracking body; its body is captured on `sif`, which is free until
            // the backtracking node is complete.
            std::function<int(cudaStream_t, cudaStream_t, cudaStream_t, cudaGraphConditionalHandle,
                              cudaGraphConditionalHandle, cudaGraphConditionalHandle, int, std::function<int()>)>
                iteration = [&](cudaStream_t cap, cudaStream_t sbt, cudaStream_t sif, cudaGraphConditionalHandle hb,
                                cudaGraphConditionalHandle hc, cudaGraphConditionalHandle ha, int slot,
                                std::function<int()> more) -> int {
                k_ctl_begin<<<1, 1, 0, cap>>>(gs, d);
                CGB_CUDA(cudaGetLastError());
                CGB_TRY(eval_dev(x, slot));
                k_ctl_judge<<<1, 1, 0, cap>>>(gs, d, hb);
                CGB_CUDA(cudaGetLastError());
                CGB_TRY(conditional(cap, sbt, hb, cudaGraphCondTypeWhile, [&]() -> int {
                    if (reuse) {
                        k_ctl_anchor_decide<<<1, 1, 0, st>>>(gs, ha);
                        CGB_CUDA(cudaGetLastError());
                        CGB_TRY(conditional(st, sif, ha, cudaGraphCondTypeIf, [&]() -> int {
                            CGB_TRY(objective(ws.xhat, -1));
                            k_ctl_anchor<<<1, 1, 0, st>>>(gs, d);
                            CGB_CUDA(cudaGetLastError());
                            return CGB_OK;
                        }));
                    }
                    CGB_TRY(eval_dev(x, slot));
                    k_ctl_judge<<<1, 1, 0, st>>>(gs, d, hb);
                    CGB_CUDA(cudaGetLastError());
                    return CGB_OK;
                }));
                k_ctl_stop<<<1, 1, 0, cap>>>(gs, d, hmain, hc);
                CGB_CUDA(cudaGetLastError());
                return conditional(cap, sif, hc, cudaGraphCondTypeIf, [&]() -> int {
                    k_momentum_dev<<<elem_grid(op, nc), kBlock, 0, st>>>(ws.xhat, x, ws.prev, gs, nc);
                    CGB_CUDA(cudaGetLastError());
                    if (slot < 0) {
                        CGB_TRY(gradient(ws.xhat, ws.grad, -1, -1, 0.0, 0.0));
                    } else {
                        if (mixed)
                            k_ax_combine32_dev<<<elem_grid(op, nr), kBlock, 0, st>>>(ws.ax32[2], ws.ax32[slot],
                                                                                     ws.ax32[1 - slot], gs, nr);
                        else
                            k_ax_combine_dev<<<elem_grid(op, nr), kBlock, 0, st>>>(ws.ax[2], ws.ax[slot],
                                                                                   ws.ax[1 - slot], gs, nr);
                        CGB_CUDA(cudaGetLastError());
                        CGB_TRY(gradient(ws.xhat, ws.grad, 2, 2, 1.0, 0.0));
                    }
                    return more();
                });
            };
            cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
            np.conditional.handle = hmain;
            np.conditional.type = cudaGraphCondTypeWhile;
            np.conditional.size = 1;
            cudaGraphNode_t wnode;
            CGB_CUDA(cudaGraphAddNode(&wnode, graph, nullptr, nullptr, 0, &np));
            cudaGraph_t body = np.conditional.phGraph_out[0];
            st = s0;
            CGB_CUDA(cudaStreamBeginCaptureToGraph(s0, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            int rc = [&]() -> int {
                if (!reuse) return iteration(s0, s1, s2, hbt, hcont, hq, -1, [] { return CGB_OK; });
                return iteration(s0, s1, s2, hbt, hcont, hq, 0, [&]() -> int {
                    return iteration(s2, s3, s4, hbt2, hcont2, hq2, 1, [] { return CGB_OK; });
                });
            }();
            cudaGraph_t done = nullptr;
            const cudaError_t e = cudaStreamEndCapture(s0, &done);
            st = user;
            CGB_TRY(rc);
            CGB_CUDA(e);
            CGB_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            return CGB_OK;
        };
        const int calls_init = calls;  // the captures below count their calls once more
        int rc = build();
        st = user;
        if (rc == CGB_OK) {
            const cudaError_t e = cudaGraphLaunch(exec, st);
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaGraphLaunch");
        }
        if (rc == CGB_OK) {
            cudaMemcpyAsync(&G, gs, sizeof(G), cudaMemcpyDeviceToHost, st);
            const cudaError_t e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) rc = cuda_fail(e, "graph FISTA");
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (cudaStream_t q : {s0, s1, s2, s3, s4})
            if (q) cudaStreamDestroy(q);
        gdev = nullptr;
        cudaFreeAsync(gs, st);
        cudaFreeAsync(glam, st);
        glam = nullptr;
        CGB_TRY(rc);
        if (G.crit == -1)
            return fail(CGB_ERR_BACKTRACK, "FISTA (graph): backtracking of iteration " + std::to_string(G.it) +
                                               " reached its cap of " + std::to_string(G.max_bt) + " step reductions");
        res->residual = 0.5 * G.res_norm * G.res_norm;
        res->regterm = G.reg_x;
        res->cost_function = G.curr_obj;
        res->abs_cost = G.abs_obj;
        res->rel_cost = G.rel_obj;
        res->abs_x = G.abs_x;
        res->rel_x = G.rel_x;
        res->iterations = G.it;
        res->stopping_criterion = G.crit;
        res->backtracks = G.backtracks;
        res->anchors = G.anchors;
        // init: 2 (gradient) + 1 (Rayleigh quotient); per evaluation 1 (an anchored iteration
        // evaluates x once more and x_hat once); per gradient 2, or 1 when A x_hat comes from
        // the stored rows
        res->operator_calls =
            calls_init + (G.it + G.backtracks + 2 * G.anchors) + (reuse ? 1 : 2) * (G.it - 1);
        return CGB_OK;
    }
};

// out[off[j]] = sum over blocks of partials[b*kRedSlots + j] for the j with off[j] >= 0
struct SlotMap {
    int off[kMaxRhs];
};
__global__ void k_finalize_scatter(const double *__restrict__ partials, int nblocks, SlotMap M, double *__restrict__ out) {
    double v[1] = {0.0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v[0] += partials[(size_t)b * kRedSlots + blockIdx.x];
    double tmp[1];
    block_sum_store_n<1>(v, tmp);
    if (threadIdx.x == 0 && M.off[blockIdx.x] >= 0) out[M.off[blockIdx.x]] = tmp[0];
}

// A regularisation path (or any set of problems sharing A, y and sqrt(W)) solved together:
// every problem follows commit/solvers.py:244-391 exactly as Solver does (its own step,
// momentum, backtracking and stopping tests), but the operator passes of all problems that
// need one at the same point run as multi-right-hand-side passes (BF16 LUT, FP32 rows,
// R = 2 or 4 vectors per pass), which load each segment's LUT row once for R vectors.
// A problem that has stopped leaves the passes; x of each problem is its own device array.
struct BatchSolver {
    cgb_op *op;
    const double *y, *sqw;
    const cgb_reg *regs;
    int P;
    const cgb_fista_params *prm;
    cudaStream_t st;
    std::vector<Solver> S;
    float *y32 = nullptr, *sqw32 = nullptr;
    float *scr[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<float *> ax32;  // 2 per problem with momentum reuse
    double *bscal = nullptr, *partials = nullptr;
    std::vector<double> hbv;  // host copy of the scalars (pageable: freeing it needs no device sync)
    double *hb = nullptr;
    int R = 4;
    int calls = 0;

    ~BatchSolver() {
        if (y32) cudaFreeAsync(y32, st);
        if (sqw32) cudaFreeAsync(sqw32, st);
        for (float *p : scr)
            if (p) cudaFreeAsync(p, st);
        for (float *p : ax32)
            if (p) cudaFreeAsync(p, st);
        if (bscal) cudaFreeAsync(bscal, st);
        if (partials) cudaFreeAsync(partials, st);
    }

    int init() {
        const int64_t nr = op->nrows;
        CGB_TRY(ensure_reduced(op, CGB_ARITH_BF16));
        CGB_TRY(ws_alloc(&bscal, (size_t)P * 16, st));
        CGB_CUDA(cudaMemsetAsync(bscal, 0, (size_t)P * 16 * sizeof(double), st));
        hbv.assign((size_t)P * 16, 0.0);
        hb = hbv.data();
        CGB_TRY(ws_alloc(&partials, (size_t)partial_blocks(op) * kRedSlots, st));
        CGB_TRY(ws_alloc(&y32, nr, st));
        CGB_TRY(convert_f64_to_f32(y, y32, nr, st));
        if (sqw) {
            CGB_TRY(ws_alloc(&sqw32, nr, st));
            CGB_TRY(convert_f64_to_f32(sqw, sqw32, nr, st));
        }
        const size_t nscr = (size_t)(op->n > 0 ? op->n : 1) * (op->nIC > 0 ? op->nIC : 1);
        for (int r = 0; r < 4; ++r) CGB_TRY(ws_alloc(&scr[r], nscr, st));
        if (prm->momentum_reuse && (prm->momentum_reuse != 2 || op->batch_reuse != 1)) {
            ax32.assign((size_t)2 * P, nullptr);
            for (auto &p : ax32) CGB_TRY(ws_alloc(&p, nr, st));
        }
        S.resize(P);
        for (int p = 0; p < P; ++p) {
            Solver &s = S[p];
            s.op = op;
            s.y = y;
            s.sqw = sqw;
            s.reg = regs + p;
            s.prm = prm;
            s.st = st;
            s.batch_member = true;
            s.dsc = bscal + (size_t)16 * p;
            CGB_TRY(s.init());
        }
        R = op->batch_rhs == 2 ? 2 : 4;
        return CGB_OK;
    }

    // chunks of the problem list J: full chunks of R, a remainder of 3 as R = 4 with one idle
    // slot, of 2 as R = 2, of 1 through the single-vector kernels
    template <class F>
    int chunks(const std::vector<int> &J, F &&f) {
        size_t i = 0;
        while (i < J.size()) {
            const size_t left = J.size() - i;
            int take, rr;
            if (left >= (size_t)R) take = rr = R;
            else if (left == 3) take = 3, rr = 4;
            else if (left == 2) take = rr = 2;
            else take = rr = 1;
            CGB_TRY(f(&J[i], take, rr));
            i += take;
        }
        return CGB_OK;
    }

    // |sqw*(A x_p - yobs)|^2 -> slot of each problem in J (yobs null: |sqw*A x_p|^2);
    // with ax, A x_p is also kept in ax32[2p + slot_ax[p]]
    int forward(const std::vector<int> &J, double *const *xs, const float *yobs, int slot, const int *slot_ax) {
        return chunks(J, [&](const int *pp, int take, int rr) -> int {
            int g = 0;
            SlotMap M;
            for (int r = 0; r < kMaxRhs; ++r) M.off[r] = -1;
            if (rr == 1) {
                const int p = pp[0];
                float *ax = slot_ax ? ax32[2 * p + slot_ax[p]] : nullptr;
                CGB_TRY(launch_resnorm_mix(op, xs[p], yobs, sqw32, partials, ax, nullptr, st, CGB_ARITH_BF16, &g));
                M.off[0] = 16 * p + slot;
            } else {
                RhsPtrs V;
                memset(&V, 0, sizeof(V));
                for (int r = 0; r < rr; ++r) {
                    const int p = pp[r < take ? r : 0];
                    V.x[r] = xs[p];
                    V.active[r] = r < take;
                    if (r < take) {
                        if (slot_ax) V.ax[r] = ax32[2 * p + slot_ax[p]];
                        M.off[r] = 16 * p + slot;
                    }
                }
                CGB_TRY(launch_forward_R(op, rr, V, yobs, sqw32, partials, st, &g));
            }
            calls += take;
            if (g > 0) {
                k_finalize_scatter<<<rr, kBlock, 0, st>>>(partials, g, M, bscal);
                CGB_CUDA(cudaGetLastError());
            } else {
                for (int r = 0; r < take; ++r) CGB_CUDA(cudaMemsetAsync(bscal + M.off[r], 0, sizeof(double), st));
            }
            return CGB_OK;
        });
    }

    // grad_p = A'(W(A xhat_p - y)), |r_p|^2 -> slot 12; with reuse, A xhat_p = ca*ax[sa] + cb*ax[sb]
    int gradient(const std::vector<int> &J, bool reuse, const int *sa, const int *sb, const double *ca,
                 const double *cb) {
        return chunks(J, [&](const int *pp, int take, int rr) -> int {
            int g = 0;
            SlotMap M;
            for (int r = 0; r < kMaxRhs; ++r) M.off[r] = -1;
            if (op->nV == 0) {
                for (int r = 0; r < take; ++r) {
                    const int p = pp[r];
                    if (op->ncols > 0) CGB_CUDA(cudaMemsetAsync(S[p].ws.grad, 0, op->ncols * sizeof(double), st));
                    CGB_CUDA(cudaMemsetAsync(bscal + 16 * p + 12, 0, sizeof(double), st));
                }
                return CGB_OK;
            }
            if (rr == 1) {
                const int p = pp[0];
                CGB_TRY(launch_gradient_mix(op, S[p].ws.xhat, y32, sqw32, S[p].ws.grad, partials,
                                            reuse ? ax32[2 * p + sa[p]] : nullptr, reuse ? ax32[2 * p + sb[p]] : nullptr,
                                            reuse ? (float)ca[p] : 0.f, reuse ? (float)cb[p] : 0.f, st, CGB_ARITH_BF16,
                                            &g));
                M.off[0] = 16 * p + 12;
            } else {
                RhsPtrs V;
                memset(&V, 0, sizeof(V));
                for (int r = 0; r < rr; ++r) {
                    const int p = pp[r < take ? r : 0];
                    V.x[r] = S[p].ws.xhat;
                    V.active[r] = r < take;
                    V.scr[r] = scr[r];
                    V.xout[r] = S[p].ws.grad;
                    if (reuse) {
                        V.axa[r] = ax32[2 * p + sa[p]];
                        V.axb[r] = ax32[2 * p + sb[p]];
                        V.ca[r] = (float)ca[p];
                        V.cb[r] = (float)cb[p];
                    }
                    if (r < take) M.off[r] = 16 * p + 12;
                }
                if (op->nslab > 1) {
                    // slab by slab, the fibre passes right after each voxel pass (terms in L2),
                    // each vector's running fibre sums in its own accumulator
                    CGB_TRY(ensure_fib_acc(op, take));
                    int g0 = 0;
                    CGB_TRY(slab_schedule(
                        op, st,
                        [&](int sl, cudaStream_t q) {
                            VoxelRange vr(op, op->slab_v[sl], op->slab_v[sl + 1]);
                            int gs = 0;
                            const int rc = launch_adjoint_R(op, rr, V, reuse ? 2 : 1, y32, sqw32,
                                                            partials + (size_t)sl * g0 * kRedSlots, q, &gs);
                            if (sl == 0) g0 = gs;
                            return rc;
                        },
                        [&](int sl, cudaStream_t q) {
                            for (int r = 0; r < take; ++r)
                                CGB_TRY(fibre_sum32_slab(op, scr[r], S[pp[r]].ws.grad, sl, q, r));
                            return CGB_OK;
                        }));
                    g = g0 * op->nslab;
                } else {
                    CGB_TRY(launch_adjoint_R(op, rr, V, reuse ? 2 : 1, y32, sqw32, partials, st, &g));
                    for (int r = 0; r < take; ++r) CGB_TRY(fibre_sum32_from(op, scr[r], S[pp[r]].ws.grad, st));
                }
            }
            calls += take * (reuse ? 1 : 2);
            if (g > 0) {
                k_finalize_scatter<<<rr, kBlock, 0, st>>>(partials, g, M, bscal);
                CGB_CUDA(cudaGetLastError());
            }
            return CGB_OK;
        });
    }

    int fetch() {
        CGB_CUDA(cudaMemcpyAsync(hb, bscal, (size_t)P * 16 * sizeof(double), cudaMemcpyDeviceToHost, st));
        CGB_CUDA(cudaStreamSynchronize(st));
        return CGB_OK;
    }

    // Autotuner, run on first use and kept on the handle: the vectors per pass (R = 2 or 4)
    // and, when params->momentum_reuse is 2 (automatic), whether the gradient takes
    // A x_hat from the stored A x rows (saves a forward product, costs three FP32 row-sized
    // transfers per problem) or recomputes it in the fused pass.  Each candidate is timed
    // on one iteration's operator passes of up to 4 problems (one warm-up round first).
    bool reuse = false;
    int tune() {
        const bool want_r = op->batch_rhs == 0 && P >= 4;
        const bool want_shape = op->batch_lpv == 0;
        const bool want_reuse = prm->momentum_reuse == 2 && op->batch_reuse == 0;
        if (op->nV == 0 || (!want_r && !want_shape && !want_reuse)) {
            if (op->batch_lpv == 0) op->batch_lpv = 1;
            return CGB_OK;
        }
        std::vector<int> J;
        for (int p = 0; p < P && p < 4; ++p) J.push_back(p);
        std::vector<double *> xh(P);
        for (int p = 0; p < P; ++p) xh[p] = S[p].ws.xhat;
        std::vector<int> zero(P, 0);
        std::vector<double> one(P, 1.0), nil(P, 0.0);
        cudaEvent_t e[2];
        for (auto &ev : e) CGB_CUDA(cudaEventCreate(&ev));
        auto timed = [&](auto &&f, float *ms) -> int {
            CGB_CUDA(cudaEventRecord(e[0], st));
            CGB_TRY(f());
            CGB_CUDA(cudaEventRecord(e[1], st));
            CGB_CUDA(cudaEventSynchronize(e[1]));
            CGB_CUDA(cudaEventElapsedTime(ms, e[0], e[1]));
            return CGB_OK;
        };
        // candidates: vectors per pass x voxel shape (default, or a warp per voxel when that
        // is a different shape); each timed on one iteration's passes, with and without reuse
        const int widths[2] = {4, 2};
        const int nw = want_r ? 2 : 1;
        const bool wide_differs = detail::wide_pair_shape(op->nS).lpv != detail::pick_pair_shape(op->nS).lpv;
        const int ns = want_shape && wide_differs ? 2 : 1;
        float cost[2][2][2] = {};  // [shape][width][reuse]
        for (int rep = 0; rep < 2; ++rep) {
            for (int h = 0; h < ns; ++h) {
                op->batch_lpv = want_shape ? h + 1 : op->batch_lpv;
                for (int k = 0; k < nw; ++k) {
                    R = want_r ? widths[k] : (op->batch_rhs == 2 ? 2 : 4);
                    float t0 = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f;
                    CGB_TRY(timed([&] { return forward(J, xh.data(), y32, 0, nullptr); }, &t0));
                    CGB_TRY(timed([&] { return gradient(J, false, nullptr, nullptr, nullptr, nullptr); }, &t1));
                    if (!ax32.empty()) {
                        CGB_TRY(timed([&] { return forward(J, xh.data(), y32, 0, zero.data()); }, &t2));
                        CGB_TRY(timed(
                            [&] { return gradient(J, true, zero.data(), zero.data(), one.data(), nil.data()); }, &t3));
                    }
                    if (rep == 1) {
                        cost[h][k][0] = t0 + t1;
                        cost[h][k][1] = t2 + t3;
                    }
                }
            }
        }
        for (auto &ev : e) cudaEventDestroy(ev);
        // reuse: -1 to be chosen, else fixed (by the caller or an earlier tuning)
        const int ru = want_reuse ? -1 : (prm->momentum_reuse == 2 ? op->batch_reuse == 2 : prm->momentum_reuse != 0);
        float best = 1e30f;
        int bh = 0, bk = 0, bu = 0;
        for (int h = 0; h < ns; ++h)
            for (int k = 0; k < nw; ++k)
                for (int u = 0; u < 2; ++u) {
                    if (ru >= 0 && u != ru) continue;
                    if (u == 1 && ax32.empty()) continue;
                    if (cost[h][k][u] < best) {
                        best = cost[h][k][u];
                        bh = h;
                        bk = k;
                        bu = u;
                    }
                }
        if (want_shape) op->batch_lpv = bh + 1;
        if (want_r) op->batch_rhs = widths[bk];
        if (want_reuse) op->batch_reuse = bu ? 2 : 1;
        R = op->batch_rhs == 2 ? 2 : 4;
        return CGB_OK;
    }

    int run(double *const *xs, cgb_fista_result *res) {
        const int64_t nc = op->ncols;
        const double eps = 2.220446049250313e-16;
        const double beta = 0.9;
        std::vector<int> all(P);
        for (int p = 0; p < P; ++p) all[p] = p;
        for (int p = 0; p < P; ++p)
            CGB_CUDA(cudaMemcpyAsync(S[p].ws.xhat, xs[p], nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
        CGB_TRY(tune());
        reuse = prm->momentum_reuse == 2 ? op->batch_reuse == 2 : prm->momentum_reuse != 0;
        // initialisation (solvers.py:260-286), all problems at once
        CGB_TRY(gradient(all, false, nullptr, nullptr, nullptr, nullptr));
        std::vector<double *> gp(P);
        for (int p = 0; p < P; ++p) {
            Solver &s = S[p];
            CGB_TRY(s.prox(s.ws.xhat, s.ws.xhat, nullptr, 0.0, 1.0));
            CGB_TRY(s.stats(s.ws.xhat, nullptr, nullptr, nullptr));
            k_dot<<<elem_grid(op, nc), kBlock, 0, st>>>(s.ws.grad, s.ws.grad, nc, s.ws.pstats);
            CGB_CUDA(cudaGetLastError());
            CGB_TRY(finalize(s.ws.pstats, elem_grid(op, nc), 1, s.dsc + 13, st));
            gp[p] = s.ws.grad;
        }
        CGB_TRY(forward(all, gp.data(), nullptr, 14, nullptr));
        CGB_TRY(fetch());
        std::vector<double> step(P), told(P, 1.0), prev_obj(P), qfval(P), res_norm(P), reg_x(P), curr(P, 0.0),
            abs_obj(P, 0.0), rel_obj(P, 0.0), abs_x(P, 0.0), rel_x(P, 0.0), cc(P, 0.0), ca(P), cb(P);
        std::vector<int> crit(P, 4), iters(P, 1), bts(P, 0), cur(P, 0), sa(P), sb(P), bt_it(P, 0);
        std::vector<char> anchored(P, 0);
        std::vector<int> anchors(P, 0);
        const int max_bt = prm->max_backtracks > 0 ? prm->max_backtracks : (prm->max_backtracks < 0 ? 0 : 1000);
        for (int p = 0; p < P; ++p) {
            const double *h = hb + 16 * p;
            res_norm[p] = sqrt(h[12]);
            prev_obj[p] = 0.5 * res_norm[p] * res_norm[p] + S[p].omega_from(h);
            qfval[p] = prev_obj[p];
            const double Ln = sqrt(h[14]) / sqrt(h[13]);
            step[p] = 1.9 / (Ln * Ln);
            CGB_CUDA(cudaMemcpyAsync(S[p].ws.prev, S[p].ws.xhat, nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
        const bool reuse_on = reuse;
        int have_prev_ax = 0;
        std::vector<int> J = all;
        int it = 1;
        while (!J.empty()) {
            auto eval = [&](const std::vector<int> &K) -> int {
                for (int p : K) {
                    Solver &s = S[p];
                    CGB_TRY(s.prox(xs[p], s.ws.xhat, s.ws.grad, step[p], step[p]));
                    CGB_TRY(s.stats(xs[p], s.ws.xhat, s.ws.grad, s.ws.prev));
                }
                CGB_TRY(forward(K, xs, y32, 0, reuse_on ? cur.data() : nullptr));
                return fetch();
            };
            auto judge = [&](int p, double &q) {
                const double *h = hb + 16 * p;
                reg_x[p] = S[p].omega_from(h);
                q = qfval[p] + h[1] + 0.5 / step[p] * (sqrt(h[2]) * sqrt(h[2])) + reg_x[p];
                res_norm[p] = sqrt(h[0]);
                curr[p] = 0.5 * res_norm[p] * res_norm[p] + reg_x[p];
            };
            CGB_TRY(eval(J));
            std::vector<int> B;
            for (int p : J) {
                const double *h = hb + 16 * p;
                qfval[p] = it == 1 ? prev_obj[p] : 0.5 * sqrt(h[12]) * sqrt(h[12]);
                anchored[p] = 0;
                bt_it[p] = 0;
                double q;
                judge(p, q);
                if (curr[p] > q) B.push_back(p);
            }
            while (!B.empty()) {
                // a qfval from the stored rows is evaluated again directly on the first
                // failure of the test and the same step judged again (as in Solver::run)
                std::vector<int> An;
                for (int p : B) {
                    if (reuse_on && it > 1 && !anchored[p]) {
                        anchored[p] = 1;
                        anchors[p]++;
                        An.push_back(p);
                    } else {
                        if (bt_it[p] >= max_bt)
                            return fail(CGB_ERR_BACKTRACK, "batched FISTA: backtracking of problem " +
                                                                    std::to_string(p) + ", iteration " +
                                                                    std::to_string(it) + " reached its cap of " +
                                                                    std::to_string(max_bt) + " step reductions");
                        bt_it[p]++;
                        step[p] *= beta;
                        bts[p]++;
                    }
                }
                if (!An.empty()) {
                    std::vector<double *> xh(P, nullptr);
                    for (int p : An) xh[p] = S[p].ws.xhat;
                    CGB_TRY(forward(An, xh.data(), y32, 0, nullptr));
                    CGB_TRY(fetch());
                    for (int p : An) {
                        const double r = sqrt(hb[16 * p]);
                        qfval[p] = 0.5 * r * r;
                    }
                }
                CGB_TRY(eval(B));
                std::vector<int> B2;
                for (int p : B) {
                    double q;
                    judge(p, q);
                    if (curr[p] > q) B2.push_back(p);
                }
                B.swap(B2);
            }
            std::vector<int> next;
            for (int p : J) {
                const double *h = hb + 16 * p;
                abs_obj[p] = fabs(curr[p] - prev_obj[p]);
                rel_obj[p] = abs_obj[p] / curr[p];
                abs_x[p] = sqrt(h[3]);
                rel_x[p] = abs_x[p] / (sqrt(h[4]) + eps);
                iters[p] = it;
                int c = -1;
                if (abs_obj[p] < eps) c = 0;
                else if (rel_obj[p] < prm->tol_fun) c = 1;
                else if (abs_x[p] < eps) c = 2;
                else if (rel_x[p] < prm->tol_x) c = 3;
                else if (it >= prm->max_iter) c = 4;
                if (c >= 0) crit[p] = c;
                else next.push_back(p);
            }
            if (next.empty()) break;
            // FISTA update (solvers.py:359-368) for the problems that go on
            for (int p : next) {
                const double t = 0.5 * (1.0 + sqrt(1.0 + 4.0 * told[p] * told[p]));
                cc[p] = (told[p] - 1.0) / t;
                told[p] = t;
                Solver &s = S[p];
                k_momentum<<<elem_grid(op, nc), kBlock, 0, st>>>(s.ws.xhat, xs[p], s.ws.prev, cc[p], nc);
                CGB_CUDA(cudaGetLastError());
                sa[p] = cur[p];
                sb[p] = have_prev_ax ? 1 - cur[p] : cur[p];
                ca[p] = 1.0 + cc[p];
                cb[p] = -cc[p];
                prev_obj[p] = curr[p];
            }
            // every problem starts with c = 0, so the reuse condition is the same for all
            CGB_TRY(gradient(next, reuse_on, sa.data(), sb.data(), ca.data(), cb.data()));
            if (reuse_on) {
                for (int p : next) cur[p] = 1 - cur[p];
                have_prev_ax = 1;
            }
            J.swap(next);
            it += 1;
        }
        for (int p = 0; p < P; ++p) {
            cgb_fista_result &r = res[p];
            r.residual = 0.5 * res_norm[p] * res_norm[p];
            r.regterm = reg_x[p];
            r.cost_function = curr[p];
            r.abs_cost = abs_obj[p];
            r.rel_cost = rel_obj[p];
            r.abs_x = abs_x[p];
            r.rel_x = rel_x[p];
            r.iterations = iters[p];
            r.stopping_criterion = crit[p];
            r.backtracks = bts[p];
            r.operator_calls = 0;
            r.anchors = anchors[p];
        }
        if (P > 0) res[0].operator_calls = calls;
        CGB_CUDA(cudaStreamSynchronize(st));
        return CGB_OK;
    }
};

}  // namespace
}  // namespace cgb

using namespace cgb;

struct DevGuard {
    int prev = -1;
    explicit DevGuard(int d) {
        cudaGetDevice(&prev);
        if (prev != d) cudaSetDevice(d);
    }
    ~DevGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

extern "C" {

int cgb_fista_run(cgb_op *op, const double *y, const double *sqrt_w, const cgb_reg *reg,
                  const cgb_fista_params *params, double *x, cgb_fista_result *result, void *stream) {
    if (!op || !y || !reg || !params || !x || !result) return fail(CGB_ERR_INVALID, "null argument");
    if (params->arith < CGB_ARITH_F64 || params->arith > CGB_ARITH_F32)
        return fail(CGB_ERR_INVALID, "unknown FISTA arith");
    if (reg->reg_ec > CGB_REG_LASSO || reg->reg_iso > CGB_REG_LASSO)
        return fail(CGB_ERR_INVALID, "EC/ISO regularisers must be none or lasso");
    if ((reg->reg_ic == CGB_REG_GROUP_LASSO || reg->reg_ic == CGB_REG_SPARSE_GROUP_LASSO) && reg->ngroups > 0 &&
        (!reg->level_ptr || reg->nlevels < 1))
        return fail(CGB_ERR_INVALID, "group regulariser needs a level schedule");
    if (params->graph && ((params->trace && params->x_ref) || params->verbose == 4 || params->restart))
        return fail(CGB_ERR_UNSUPPORTED, "graph mode runs without restart, trace or verbose output");
    NvtxRange nv("cgb_fista_run");
    DevGuard g(op->device);
    Solver S;
    S.op = op;
    S.y = y;
    S.sqw = sqrt_w;
    S.reg = reg;
    S.prm = params;
    S.st = (cudaStream_t)stream;
    CGB_TRY(S.init());
    return params->graph ? S.run_graph(x, result) : S.run(x, result);
}

int cgb_fista_batch_run(cgb_op *op, const double *y, const double *sqrt_w, const cgb_reg *regs, int nprob,
                        const cgb_fista_params *params, double *const *x, cgb_fista_result *results, void *stream) {
    if (!op || !y || !regs || !params || !x || !results) return fail(CGB_ERR_INVALID, "null argument");
    if (nprob < 1) return fail(CGB_ERR_INVALID, "nprob must be >= 1");
    if (params->arith != CGB_ARITH_BF16) return fail(CGB_ERR_UNSUPPORTED, "batched FISTA runs in BF16-LUT arithmetic");
    NvtxRange nv("cgb_fista_batch_run");
    for (int p = 0; p < nprob; ++p) {
        const cgb_reg *reg = regs + p;
        if (!x[p]) return fail(CGB_ERR_INVALID, "null x");
        if (reg->reg_ec > CGB_REG_LASSO || reg->reg_iso > CGB_REG_LASSO)
            return fail(CGB_ERR_INVALID, "EC/ISO regularisers must be none or lasso");
        if ((reg->reg_ic == CGB_REG_GROUP_LASSO || reg->reg_ic == CGB_REG_SPARSE_GROUP_LASSO) && reg->ngroups > 0 &&
            (!reg->level_ptr || reg->nlevels < 1))
            return fail(CGB_ERR_INVALID, "group regulariser needs a level schedule");
    }
    DevGuard g(op->device);
    BatchSolver B;
    B.op = op;
    B.y = y;
    B.sqw = sqrt_w;
    B.regs = regs;
    B.P = nprob;
    B.prm = params;
    B.st = (cudaStream_t)stream;
    CGB_TRY(B.init());
    return B.run(x, results);
}

int cgb_op_batch_width(cgb_op *op, int set, int *width) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (set >= 0) {
        if (set != 0 && set != 2 && set != 4) return fail(CGB_ERR_INVALID, "width must be 0, 2 or 4");
        op->batch_rhs = set;
    }
    if (width) *width = op->batch_rhs;
    return CGB_OK;
}

int cgb_op_batch_shape(cgb_op *op, int set, int *shape) {
    if (!op) return fail(CGB_ERR_INVALID, "null handle");
    if (set >= 0) {
        if (set > 2) return fail(CGB_ERR_INVALID, "shape must be 0 (tune), 1 (default) or 2 (a warp per voxel)");
        op->batch_lpv = set;
    }
    if (shape) *shape = op->batch_lpv;
    return CGB_OK;
}

int cgb_op_apply_batch(cgb_op *op, int adjoint, int nvec, const void *const *in, void *const *out, void *stream) {
    if (!op || !in || !out) return fail(CGB_ERR_INVALID, "null argument");
    if (nvec < 1) return fail(CGB_ERR_INVALID, "nvec must be >= 1");
    for (int r = 0; r < nvec; ++r)
        if (!in[r] || !out[r]) return fail(CGB_ERR_INVALID, "null vector");
    DevGuard g(op->device);
    cudaStream_t st = (cudaStream_t)stream;
    CGB_TRY(ensure_reduced(op, CGB_ARITH_BF16));
    if (op->nV == 0) {
        for (int r = 0; r < nvec; ++r) {
            if (adjoint && op->ncols > 0) CGB_CUDA(cudaMemsetAsync(out[r], 0, op->ncols * sizeof(double), st));
            if (!adjoint && op->nrows > 0) CGB_CUDA(cudaMemsetAsync(out[r], 0, op->nrows * sizeof(float), st));
        }
        return CGB_OK;
    }
    const int W = op->batch_rhs == 2 ? 2 : 4;
    std::vector<float *> scr;
    if (adjoint) {
        const size_t nscr = (size_t)(op->n > 0 ? op->n : 1) * (op->nIC > 0 ? op->nIC : 1);
        for (int r = 0; r < W; ++r) {
            float *p = nullptr;
            const cudaError_t e = cudaMallocAsync((void **)&p, nscr * sizeof(float), st);
            if (e != cudaSuccess) {
                for (float *q : scr) cudaFreeAsync(q, st);
                return cuda_fail(e, "cudaMallocAsync");
            }
            scr.push_back(p);
        }
    }
    int rc = CGB_OK;
    for (int i = 0; i < nvec && rc == CGB_OK;) {
        const int left = nvec - i;
        const int take = left >= W ? W : (left == 3 ? 3 : (left >= 2 ? 2 : 1));
        const int rr = take == 3 ? 4 : (take == 1 ? 2 : take);
        RhsPtrs V;
        memset(&V, 0, sizeof(V));
        for (int r = 0; r < rr; ++r) {
            const int k = i + (r < take ? r : 0);
            V.active[r] = r < take;
            if (adjoint) {
                V.yin[r] = (const float *)in[k];
                V.xout[r] = (double *)out[k];
                V.scr[r] = scr[r];
            } else {
                V.x[r] = (const double *)in[k];
                V.y[r] = (float *)out[k];
            }
        }
        if (adjoint) {
            rc = launch_adjoint_R(op, rr, V, 0, nullptr, nullptr, nullptr, st, nullptr);
            for (int r = 0; r < take && rc == CGB_OK; ++r) rc = fibre_sum32_from(op, scr[r], (double *)out[i + r], st);
        } else {
            rc = launch_forward_R(op, rr, V, nullptr, nullptr, nullptr, st, nullptr);
        }
        i += take;
    }
    for (float *q : scr) cudaFreeAsync(q, st);
    return rc;
}

// ------------------------------------------------------------------ standalone proximal maps
static int grid_n(int64_t n) {
    int64_t g = (n + kBlock - 1) / kBlock;
    if (g > 4096) g = 4096;
    if (g < 1) g = 1;
    return (int)g;
}

int cgb_prox_non_negativity(double *x, int64_t start, int64_t size, void *stream) {
    if (size <= 0) return CGB_OK;
    if (!x || start < 0) return fail(CGB_ERR_INVALID, "bad argument");
    k_nonneg<<<grid_n(size), kBlock, 0, (cudaStream_t)stream>>>(x, start, start + size);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

int cgb_prox_soft_thresholding(double *x, double lam, int64_t start, int64_t size, void *stream) {
    if (size <= 0) return CGB_OK;
    if (!x || start < 0) return fail(CGB_ERR_INVALID, "bad argument");
    k_soft<<<grid_n(size), kBlock, 0, (cudaStream_t)stream>>>(x, nullptr, lam, start, start + size);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

int cgb_prox_w_soft_thresholding(double *x, const double *w, double lam, int64_t start, int64_t size,
                                 void *stream) {
    if (size <= 0) return CGB_OK;
    if (!x || !w || start < 0) return fail(CGB_ERR_INVALID, "bad argument");
    k_soft<<<grid_n(size), kBlock, 0, (cudaStream_t)stream>>>(x, w, lam, start, start + size);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

static int sum_sq_range(const double *x, int64_t start, int64_t size, double *out, cudaStream_t st) {
    const int g = grid_n(size) > 1024 ? 1024 : grid_n(size);
    double *part = nullptr, *dres = nullptr;
    CGB_CUDA(cudaMallocAsync((void **)&part, (size_t)g * kRedSlots * sizeof(double), st));
    CGB_CUDA(cudaMallocAsync((void **)&dres, sizeof(double), st));
    k_dot<<<g, kBlock, 0, st>>>(x + start, x + start, size, part);
    k_finalize<<<1, kBlock, 0, st>>>(part, g, dres);
    cudaError_t e = cudaMemcpyAsync(out, dres, sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFreeAsync(part, st);
    cudaFreeAsync(dres, st);
    CGB_CUDA(e);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

int cgb_prox_projection_onto_l2_ball(double *x, double lam, int64_t start, int64_t size, void *stream) {
    // proximals.pyx:59-77
    if (size <= 0) return CGB_OK;
    if (!x || start < 0) return fail(CGB_ERR_INVALID, "bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    double s2 = 0.0;
    CGB_TRY(sum_sq_range(x, start, size, &s2, st));
    const double xn = sqrt(s2);
    const double f = xn > lam ? 1.0 - lam / xn : 0.0;
    k_scale_range<<<grid_n(size), kBlock, 0, st>>>(x, start, start + size, f);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

int cgb_prox_group_lasso(double *x, int64_t nx, const int32_t *group_idx, const int64_t *group_ptr, const double *group_w,
                         int64_t ngroups, const int64_t *level_ptr, int64_t nlevels, double lam, void *stream) {
    if (lam == 0.0 || ngroups <= 0) return CGB_OK;
    if (!x || !group_idx || !group_ptr || !group_w || !level_ptr) return fail(CGB_ERR_INVALID, "bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    for (int64_t k = 0; k < nlevels; ++k) {
        const int64_t g0 = level_ptr[k], g1 = level_ptr[k + 1];
        if (g1 <= g0) continue;
        int64_t blocks = ((g1 - g0) * 32 + kBlock - 1) / kBlock;
        if (blocks > 4096) blocks = 4096;
        k_group_prox<<<(int)blocks, kBlock, 0, st>>>(x, nx, group_idx, group_ptr, group_w, g0, g1, lam, nullptr);
        CGB_CUDA(cudaGetLastError());
    }
    return CGB_OK;
}

static int group_omega(const double *x, int64_t nx, const int32_t *gidx, const int64_t *gptr, const double *gw, int64_t G,
                       double *out, cudaStream_t st) {
    int64_t blocks = (G * 32 + kBlock - 1) / kBlock;
    if (blocks > 1024) blocks = 1024;
    if (blocks < 1) blocks = 1;
    double *part = nullptr, *dres = nullptr;
    CGB_CUDA(cudaMallocAsync((void **)&part, (size_t)blocks * kRedSlots * sizeof(double), st));
    CGB_CUDA(cudaMallocAsync((void **)&dres, sizeof(double), st));
    k_group_norms<<<(int)blocks, kBlock, 0, st>>>(x, nx, gidx, gptr, gw, G, part);
    k_finalize<<<1, kBlock, 0, st>>>(part, (int)blocks, dres);
    cudaError_t e = cudaMemcpyAsync(out, dres, sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFreeAsync(part, st);
    cudaFreeAsync(dres, st);
    CGB_CUDA(e);
    CGB_CUDA(cudaGetLastError());
    return CGB_OK;
}

int cgb_omega_group_lasso(const double *x, int64_t nx, const int32_t *group_idx, const int64_t *group_ptr,
                          const double *group_w, int64_t ngroups, double lam, double *out, void *stream) {
    if (!out) return fail(CGB_ERR_INVALID, "out is NULL");
    *out = 0.0;
    if (lam == 0.0 || ngroups <= 0) return CGB_OK;
    double s = 0.0;
    CGB_TRY(group_omega(x, nx, group_idx, group_ptr, group_w, ngroups, &s, (cudaStream_t)stream));
    *out = lam * s;
    return CGB_OK;
}

static int l1_sum(const double *x, const double *w, int64_t a, int64_t b, double *out, cudaStream_t st) {
    *out = 0.0;
    if (b <= a) return CGB_OK;
    const int g = grid_n(b - a) > 1024 ? 1024 : grid_n(b - a);
    double *part = nullptr, *dres = nullptr;
    CGB_CUDA(cudaMallocAsync((void **)&part, (size_t)g * kRedSlots * sizeof(double), st));
    CGB_CUDA(cudaMallocAsync((void **)&dres, kStatSlots * sizeof(double), st));
    L1Terms T;
    T.n = 1;
    T.t[0] = L1Term{a, b, w};
    k_stats<<<g, kBlock, 0, st>>>(x, nullptr, nullptr, nullptr, b, T, nullptr, part);
    k_finalize<<<kStatSlots, kBlock, 0, st>>>(part, g, dres);
    double h[8];
    cudaError_t e = cudaMemcpyAsync(h, dres, 8 * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFreeAsync(part, st);
    cudaFreeAsync(dres, st);
    CGB_CUDA(e);
    CGB_CUDA(cudaGetLastError());
    *out = h[4];
    return CGB_OK;
}

int cgb_omega_l1(const double *x, const double *w, int64_t start, int64_t size, double lam, double *out,
                 void *stream) {
    if (!out || !x) return fail(CGB_ERR_INVALID, "null argument");
    double s = 0.0;
    CGB_TRY(l1_sum(x, w, start, start + size, &s, (cudaStream_t)stream));
    *out = lam * s;
    return CGB_OK;
}

int cgb_omega_sparse_group_lasso(const double *x, int64_t nx, const double *w, const int32_t *group_idx,
                                 const int64_t *group_ptr, const double *group_w, int64_t ngroups, double lam1,
                                 double lam2, double *out, void *stream) {
    if (!out || !x) return fail(CGB_ERR_INVALID, "null argument");
    *out = 0.0;
    if (lam1 == 0.0 && lam2 == 0.0) return CGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    double o1 = 0.0, o2 = 0.0;
    CGB_TRY(l1_sum(x, w, 0, nx, &o1, st));
    if (ngroups > 0) CGB_TRY(group_omega(x, nx, group_idx, group_ptr, group_w, ngroups, &o2, st));
    *out = lam1 * o1 + lam2 * o2;
    return CGB_OK;
}

}  // extern "C"
