/*
 * ORACLE -- test infrastructure only.  A plain-C restatement of COMMIT's CPU operator
 * (A*x and A'*y over the IC, EC and ISO compartments, with and without LUT), used by the
 * tests as the checker and by the benchmark as the timed CPU baseline ("port").  Nothing
 * in the commit_gb300 package calls it.
 *
 * Semantics follow the generated C of the reference:
 *   A  (IC)  setup_operator.py:50-109   y[v,:] += l * sum_i x[i*nF+f]*eval[i*nF+f] * LUT_IC[i,o,:]
 *   A  (EC)  setup_operator.py:111-165  y[v,:] += sum_i x[nIC*nF + i*nE + e] * LUT_EC[i,o,:]
 *   A  (ISO) setup_operator.py:167-218  y[v,:] += sum_i x[nIC*nF + nEC*nE + i*nISO + j] * LUT_ISO[i,:]
 *   A' (IC)  setup_operator.py:370-442  x[i*nF+f] += l * <LUT_IC[i,o,:], y[v,:]> * eval[i*nF+f]
 *   A' (EC)  setup_operator.py:444-504  x[nIC*nF + i*nE + e] += <LUT_EC[i,o,:], y[v,:]>
 *   A' (ISO) setup_operator.py:506-563  x[... + i*nISO + j] += <LUT_ISO[i,:], y[v,:]>
 *   nolut    setup_operator.py:713-915  (nS == 1, no LUT, one ISO response)
 * Outputs are accumulated into, so callers pass zeroed buffers (operator.pyx:133).
 * A coefficient set that is all zero skips its segment (setup_operator.py:66,88).
 *
 * Work is split over threads the way the reference splits it: A by contiguous voxel
 * ranges balanced on IC segment counts (commit/core.pyx:626-667); A' IC by fibre
 * ownership with every thread scanning all segments (core.pyx:673-693,
 * setup_operator.py:412-435); A' EC/ISO by equal contiguous ranges (core.pyx:695-722).
 * The input arrays must be sorted by voxel (load_dictionary, core.pyx:508-562) for more
 * than one thread; otherwise a single thread is used.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MAX_THREADS 256

typedef struct {
    const double *x; double *y;
    int nS, nF, nE, nV, nISOv;
    int64_t n;
    const uint32_t *ICf, *ICeval, *ICv, *ECv, *ISOv;
    const uint16_t *ICo, *ECo;
    const float *ICl, *lutIC, *lutEC, *lutISO;
    int ndirs, nIC, nEC, nISO;
    /* partitions */
    int64_t ic0, ic1, ec0, ec1, iso0, iso1;
    uint32_t f0, f1;
} job_t;

static int64_t lower_bound_u32(const uint32_t *a, int64_t n, uint32_t key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) { int64_t mid = (lo + hi) / 2; if (a[mid] < key) lo = mid + 1; else hi = mid; }
    return lo;
}

static int is_sorted_u32(const uint32_t *a, int64_t n) {
    for (int64_t i = 1; i < n; i++) if (a[i] < a[i - 1]) return 0;
    return 1;
}

static void run_threads(void *(*fn)(void *), job_t *jobs, int T) {
    pthread_t th[ORACLE_MAX_THREADS];
    for (int t = 1; t < T; t++) pthread_create(&th[t], NULL, fn, &jobs[t]);
    fn(&jobs[0]);
    for (int t = 1; t < T; t++) pthread_join(th[t], NULL);
}

/* ----------------------------------------------------------------------------- A*x */
static void *a_block(void *arg) {
    const job_t *J = (const job_t *)arg;
    const int nS = J->nS;
    double xs[32];
    /* IC */
    for (int64_t s = J->ic0; s < J->ic1; s++) {
        const uint32_t f = J->ICf[s];
        int any = 0;
        for (int i = 0; i < J->nIC; i++) {
            xs[i] = J->x[(int64_t)i * J->nF + f] * (double)J->ICeval[(int64_t)i * J->nF + f];
            any |= (xs[i] != 0);
        }
        if (!any) continue;
        const double w = (double)J->ICl[s];
        double *Y = J->y + (int64_t)nS * J->ICv[s];
        const int64_t off = (int64_t)nS * J->ICo[s];
        for (int k = 0; k < nS; k++) {
            double acc = 0.0;
            for (int i = 0; i < J->nIC; i++)
                acc += xs[i] * (double)J->lutIC[(int64_t)i * J->ndirs * nS + off + k];
            Y[k] += w * acc;
        }
    }
    /* EC */
    const double *xEC = J->x + (int64_t)J->nIC * J->nF;
    for (int64_t e = J->ec0; e < J->ec1; e++) {
        int any = 0;
        for (int i = 0; i < J->nEC; i++) { xs[i] = xEC[(int64_t)i * J->nE + e]; any |= (xs[i] != 0); }
        if (!any) continue;
        double *Y = J->y + (int64_t)nS * J->ECv[e];
        const int64_t off = (int64_t)nS * J->ECo[e];
        for (int k = 0; k < nS; k++) {
            double acc = 0.0;
            for (int i = 0; i < J->nEC; i++)
                acc += xs[i] * (double)J->lutEC[(int64_t)i * J->ndirs * nS + off + k];
            Y[k] += acc;
        }
    }
    /* ISO */
    const double *xISO = xEC + (int64_t)J->nEC * J->nE;
    for (int64_t j = J->iso0; j < J->iso1; j++) {
        int any = 0;
        for (int i = 0; i < J->nISO; i++) { xs[i] = xISO[(int64_t)i * J->nISOv + j]; any |= (xs[i] != 0); }
        if (!any) continue;
        double *Y = J->y + (int64_t)nS * J->ISOv[j];
        for (int k = 0; k < nS; k++) {
            double acc = 0.0;
            for (int i = 0; i < J->nISO; i++) acc += xs[i] * (double)J->lutISO[(int64_t)i * nS + k];
            Y[k] += acc;
        }
    }
    return NULL;
}

/* voxel-aligned split of [0,n) IC segments into T ranges with about n/T segments each */
static int split_A(job_t *base, job_t *jobs, int T) {
    const int64_t n = base->n;
    uint32_t vb[ORACLE_MAX_THREADS + 1];
    vb[0] = 0;
    for (int t = 1; t < T; t++) {
        int64_t s = n * t / T;
        uint32_t v = (n > 0 && s < n) ? base->ICv[s] : (uint32_t)base->nV;
        vb[t] = v > vb[t - 1] ? v : vb[t - 1];
    }
    vb[T] = 0xffffffffu;
    for (int t = 0; t < T; t++) {
        jobs[t] = *base;
        jobs[t].ic0 = t ? lower_bound_u32(base->ICv, n, vb[t]) : 0;
        jobs[t].ic1 = (t < T - 1) ? lower_bound_u32(base->ICv, n, vb[t + 1]) : n;
        jobs[t].ec0 = t ? lower_bound_u32(base->ECv, base->nE, vb[t]) : 0;
        jobs[t].ec1 = (t < T - 1) ? lower_bound_u32(base->ECv, base->nE, vb[t + 1]) : base->nE;
        jobs[t].iso0 = t ? lower_bound_u32(base->ISOv, base->nISOv, vb[t]) : 0;
        jobs[t].iso1 = (t < T - 1) ? lower_bound_u32(base->ISOv, base->nISOv, vb[t + 1]) : base->nISOv;
    }
    return T;
}

int oracle_A(const double *x, double *y, int nS, int ndirs, int nF, int64_t n, int nE, int nV, int nISOv,
             const uint32_t *ICf, const uint32_t *ICeval, const uint32_t *ICv, const uint16_t *ICo, const float *ICl,
             const uint32_t *ECv, const uint16_t *ECo, const uint32_t *ISOv,
             const float *lutIC, const float *lutEC, const float *lutISO,
             int nIC, int nEC, int nISO, int nThreads) {
    if (nIC > 32 || nEC > 32 || nISO > 32) return -1;
    job_t base = {x, y, nS, nF, nE, nV, nISOv, n, ICf, ICeval, ICv, ECv, ISOv, ICo, ECo, ICl, lutIC, lutEC, lutISO,
                  ndirs, nIC, nEC, nISO, 0, n, 0, nE, 0, nISOv, 0, 0};
    if (nIC == 0) { base.ic1 = 0; }
    if (nEC == 0) { base.ec1 = 0; }
    if (nISO == 0) { base.iso1 = 0; }
    int T = nThreads < 1 ? 1 : (nThreads > ORACLE_MAX_THREADS ? ORACLE_MAX_THREADS : nThreads);
    if (!is_sorted_u32(ICv, n) || !is_sorted_u32(ECv, nE) || !is_sorted_u32(ISOv, nISOv)) T = 1;
    job_t jobs[ORACLE_MAX_THREADS];
    if (T == 1) { a_block(&base); return 0; }
    split_A(&base, jobs, T);
    for (int t = 0; t < T; t++) {
        if (nIC == 0) { jobs[t].ic0 = jobs[t].ic1 = 0; }
        if (nEC == 0) { jobs[t].ec0 = jobs[t].ec1 = 0; }
        if (nISO == 0) { jobs[t].iso0 = jobs[t].iso1 = 0; }
    }
    run_threads(a_block, jobs, T);
    return 0;
}

/* ---------------------------------------------------------------------------- A'*y */
static void *at_block(void *arg) {
    const job_t *J = (const job_t *)arg;
    const int nS = J->nS;
    /* IC: scan every segment, keep those whose fibre this thread owns */
    if (J->nIC > 0) {
        for (int64_t s = 0; s < J->n; s++) {
            const uint32_t f = J->ICf[s];
            if (f < J->f0 || f >= J->f1) continue;
            const double *Y = J->y + (int64_t)nS * J->ICv[s];
            const int64_t off = (int64_t)nS * J->ICo[s];
            const double w = (double)J->ICl[s];
            for (int i = 0; i < J->nIC; i++) {
                const float *L = J->lutIC + (int64_t)i * J->ndirs * nS + off;
                double d = 0.0;
                for (int k = 0; k < nS; k++) d += (double)L[k] * Y[k];
                double *xo = (double *)J->x + (int64_t)i * J->nF + f;
                *xo += w * d * (double)J->ICeval[(int64_t)i * J->nF + f];
            }
        }
    }
    double *xEC = (double *)J->x + (int64_t)J->nIC * J->nF;
    for (int64_t e = J->ec0; e < J->ec1; e++) {
        const double *Y = J->y + (int64_t)nS * J->ECv[e];
        const int64_t off = (int64_t)nS * J->ECo[e];
        for (int i = 0; i < J->nEC; i++) {
            const float *L = J->lutEC + (int64_t)i * J->ndirs * nS + off;
            double d = 0.0;
            for (int k = 0; k < nS; k++) d += (double)L[k] * Y[k];
            xEC[(int64_t)i * J->nE + e] += d;
        }
    }
    double *xISO = xEC + (int64_t)J->nEC * J->nE;
    for (int64_t j = J->iso0; j < J->iso1; j++) {
        const double *Y = J->y + (int64_t)nS * J->ISOv[j];
        for (int i = 0; i < J->nISO; i++) {
            const float *L = J->lutISO + (int64_t)i * nS;
            double d = 0.0;
            for (int k = 0; k < nS; k++) d += (double)L[k] * Y[k];
            xISO[(int64_t)i * J->nISOv + j] += d;
        }
    }
    return NULL;
}

/* x (output, accumulated into) is passed through job.x with the const cast above */
int oracle_At(const double *y, double *x, int nS, int ndirs, int nF, int64_t n, int nE, int nV, int nISOv,
              const uint32_t *ICf, const uint32_t *ICeval, const uint32_t *ICv, const uint16_t *ICo, const float *ICl,
              const uint32_t *ECv, const uint16_t *ECo, const uint32_t *ISOv,
              const float *lutIC, const float *lutEC, const float *lutISO,
              int nIC, int nEC, int nISO, int nThreads) {
    if (nIC > 32 || nEC > 32 || nISO > 32) return -1;
    int T = nThreads < 1 ? 1 : (nThreads > ORACLE_MAX_THREADS ? ORACLE_MAX_THREADS : nThreads);
    job_t base = {x, (double *)y, nS, nF, nE, nV, nISOv, n, ICf, ICeval, ICv, ECv, ISOv, ICo, ECo, ICl, lutIC, lutEC,
                  lutISO, ndirs, nIC, nEC, nISO, 0, n, 0, nE, 0, nISOv, 0, (uint32_t)nF};
    job_t jobs[ORACLE_MAX_THREADS];
    /* fibre ownership balanced on segment counts */
    int64_t *cnt = (int64_t *)calloc((size_t)nF + 1, sizeof(int64_t));
    if (!cnt) return -2;
    for (int64_t s = 0; s < n; s++) cnt[ICf[s]]++;
    uint32_t fb[ORACLE_MAX_THREADS + 1];
    fb[0] = 0;
    int t = 1;
    int64_t acc = 0;
    for (uint32_t f = 0; f < (uint32_t)nF && t < T; f++) {
        acc += cnt[f];
        if (acc >= n * t / T) fb[t++] = f + 1;
    }
    while (t <= T) fb[t++] = (uint32_t)nF;
    free(cnt);
    for (t = 0; t < T; t++) {
        jobs[t] = base;
        jobs[t].f0 = fb[t];
        jobs[t].f1 = fb[t + 1];
        jobs[t].ec0 = (int64_t)nE * t / T;
        jobs[t].ec1 = (int64_t)nE * (t + 1) / T;
        jobs[t].iso0 = (int64_t)nISOv * t / T;
        jobs[t].iso1 = (int64_t)nISOv * (t + 1) / T;
        if (nEC == 0) jobs[t].ec0 = jobs[t].ec1 = 0;
        if (nISO == 0) jobs[t].iso0 = jobs[t].iso1 = 0;
    }
    run_threads(at_block, jobs, T);
    return 0;
}

/* ------------------------------------------------------------------------ nolut */
static void *a_nolut_block(void *arg) {
    const job_t *J = (const job_t *)arg;
    for (int64_t s = J->ic0; s < J->ic1; s++) {
        const uint32_t f = J->ICf[s];
        const double x0 = J->x[f] * (double)J->ICeval[f];
        if (x0 != 0) J->y[J->ICv[s]] += (double)J->ICl[s] * x0;
    }
    if (J->nISO > 0)
        for (int64_t j = J->iso0; j < J->iso1; j++) {
            const double x0 = J->x[(int64_t)J->nF + j];
            if (x0 != 0) J->y[J->ISOv[j]] += x0;
        }
    return NULL;
}

int oracle_A_nolut(const double *x, double *y, int nF, int64_t n, int nV, int nISOv,
                   const uint32_t *ICf, const uint32_t *ICeval, const uint32_t *ICv, const float *ICl,
                   const uint32_t *ISOv, int nISO, int nThreads) {
    int T = nThreads < 1 ? 1 : (nThreads > ORACLE_MAX_THREADS ? ORACLE_MAX_THREADS : nThreads);
    if (!is_sorted_u32(ICv, n) || !is_sorted_u32(ISOv, nISOv)) T = 1;
    job_t base;
    memset(&base, 0, sizeof(base));
    base.x = x; base.y = y; base.nS = 1; base.nF = nF; base.n = n; base.nV = nV; base.nISOv = nISOv;
    base.ICf = ICf; base.ICeval = ICeval; base.ICv = ICv; base.ICl = ICl; base.ISOv = ISOv; base.nISO = nISO;
    base.ECv = ISOv; base.nE = 0;
    base.ic0 = 0; base.ic1 = n; base.iso0 = 0; base.iso1 = nISOv;
    if (T == 1) { a_nolut_block(&base); return 0; }
    job_t jobs[ORACLE_MAX_THREADS];
    split_A(&base, jobs, T);
    run_threads(a_nolut_block, jobs, T);
    return 0;
}

static void *at_nolut_block(void *arg) {
    const job_t *J = (const job_t *)arg;
    double *x = (double *)J->x;
    for (int64_t s = 0; s < J->n; s++) {
        const uint32_t f = J->ICf[s];
        if (f < J->f0 || f >= J->f1) continue;
        x[f] += (double)J->ICl[s] * J->y[J->ICv[s]] * (double)J->ICeval[f];
    }
    if (J->nISO > 0)
        for (int64_t j = J->iso0; j < J->iso1; j++) x[(int64_t)J->nF + j] += J->y[J->ISOv[j]];
    return NULL;
}

int oracle_At_nolut(const double *y, double *x, int nF, int64_t n, int nV, int nISOv,
                    const uint32_t *ICf, const uint32_t *ICeval, const uint32_t *ICv, const float *ICl,
                    const uint32_t *ISOv, int nISO, int nThreads) {
    int T = nThreads < 1 ? 1 : (nThreads > ORACLE_MAX_THREADS ? ORACLE_MAX_THREADS : nThreads);
    job_t base;
    memset(&base, 0, sizeof(base));
    base.x = x; base.y = (double *)y; base.nF = nF; base.n = n; base.nV = nV; base.nISOv = nISOv;
    base.ICf = ICf; base.ICeval = ICeval; base.ICv = ICv; base.ICl = ICl; base.ISOv = ISOv; base.nISO = nISO;
    job_t jobs[ORACLE_MAX_THREADS];
    for (int t = 0; t < T; t++) {
        jobs[t] = base;
        jobs[t].f0 = (uint32_t)((int64_t)nF * t / T);
        jobs[t].f1 = (uint32_t)((int64_t)nF * (t + 1) / T);
        jobs[t].iso0 = (int64_t)nISOv * t / T;
        jobs[t].iso1 = (int64_t)nISOv * (t + 1) / T;
    }
    run_threads(at_nolut_block, jobs, T);
    return 0;
}
