"""ORACLE -- test infrastructure only.

CPU restatement of COMMIT's hot path, used as the checker by ``tests/``, by
``__graft_entry__.smoke()`` and as the CPU baseline leg of ``bench.py``.  The product
package (``commit_gb300``) never imports this module.

Contents
--------
* ``PortOperator``: the C restatement in ``oracle/commit_oracle.c`` behind the
  ``LinearOperator`` surface of commit/operator/operator.pyx:10-184 (``dot``, ``T``,
  ``shape``, ``nROWS``, ``nCOLS``, ``adjoint``).
* ``RefOperator``: the reference's own generated C operator (setup_operator.py) compiled
  into ``oracle/_ref`` by ``oracle/build_ref.py``, driven with the reference's THREADS
  partitions (restated in ``set_threads``).
* ``set_threads``: restatement of Evaluation.set_threads, commit/core.pyx:586-724.
* ``init_regularisation``, ``solve``, ``fista``, ``evaluate_model``: numpy restatement of
  commit/solvers.py:16-391.
* proximal maps and penalties: numpy restatement of commit/proximals.pyx:13-186.
"""
from __future__ import annotations

import ctypes
import os
import sys
from math import sqrt

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, '_build')
REF_DIR = os.path.join(HERE, '_ref')
PORT_LIB = os.path.join(BUILD_DIR, 'libcommit_oracle.so')
REF_LIB = os.path.join(REF_DIR, 'libcommit_ref_operator.so')

eps = np.finfo(float).eps

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags='C')
_u16p = np.ctypeslib.ndpointer(dtype=np.uint16, flags='C')
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags='C')
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags='C')
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags='C')


def build_port(force: bool = False) -> str:
    """Compile oracle/commit_oracle.c with gcc (no fast-math) into oracle/_build."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, 'commit_oracle.c')
    if force or not os.path.exists(PORT_LIB) or os.path.getmtime(PORT_LIB) < os.path.getmtime(src):
        cmd = f'gcc -O3 -fPIC -shared -o {PORT_LIB}.tmp {src} -lpthread && mv {PORT_LIB}.tmp {PORT_LIB}'
        if os.system(cmd) != 0:
            raise RuntimeError('failed to build the oracle: ' + cmd)
    return PORT_LIB


_port = None


def port_lib():
    global _port
    if _port is None:
        build_port()
        L = ctypes.CDLL(PORT_LIB)
        i32, i64 = ctypes.c_int, ctypes.c_int64
        args = [_f64p, _f64p, i32, i32, i32, i64, i32, i32, i32,
                _u32p, _u32p, _u32p, _u16p, _f32p, _u32p, _u16p, _u32p, _f32p, _f32p, _f32p, i32, i32, i32, i32]
        for name in ('oracle_A', 'oracle_At'):
            getattr(L, name).argtypes = args
            getattr(L, name).restype = ctypes.c_int
        nl = [_f64p, _f64p, i32, i64, i32, i32, _u32p, _u32p, _u32p, _f32p, _u32p, i32, i32]
        for name in ('oracle_A_nolut', 'oracle_At_nolut'):
            getattr(L, name).argtypes = nl
            getattr(L, name).restype = ctypes.c_int
        _port = L
    return _port


def _arr(a, dt):
    a = np.asarray(a, dtype=dt)
    if a.size == 0:
        return np.zeros(1, dtype=dt)
    return np.ascontiguousarray(a)


class _OperatorBase:
    """The LinearOperator surface of commit/operator/operator.pyx:10-111."""

    def __init__(self, DICTIONARY, KERNELS, THREADS=None, nolut=False, nthreads=None):
        self.DICTIONARY, self.KERNELS, self.THREADS = DICTIONARY, KERNELS, THREADS
        IC, EC, ISO = DICTIONARY['IC'], DICTIONARY['EC'], DICTIONARY['ISO']
        self.ICn, self.ICnSTR, self.ICnVOX = int(IC['n']), int(IC['nSTR']), int(IC['nVOX'])
        self.ECn, self.ISOn = int(EC['n']), int(ISO['n'])
        self.ICnRF, self.ECnRF, self.ISOnRF = KERNELS['wmr'].shape[0], KERNELS['wmh'].shape[0], KERNELS['iso'].shape[0]
        if KERNELS['wmr'].size > 0:
            self.nSAMPLES = KERNELS['wmr'].shape[2]
        elif KERNELS['wmh'].size > 0:
            self.nSAMPLES = KERNELS['wmh'].shape[2]
        else:
            self.nSAMPLES = KERNELS['wmr'].shape[1]
        self.ndirs = KERNELS['wmr'].shape[1]
        self.nolut = bool(nolut)
        self.adjoint = 0
        self.nROWS = self.ICnVOX * self.nSAMPLES
        self.nCOLS = self.ICnSTR * self.ICnRF + self.ECn * self.ECnRF + self.ISOn * self.ISOnRF
        self.nthreads = int(nthreads or (THREADS or {}).get('n', 1) or 1)
        self.ICf = _arr(IC['str'], np.uint32); self.ICv = _arr(IC['vox'], np.uint32)
        self.ICo = _arr(IC['dir'], np.uint16); self.ICl = _arr(IC['len'], np.float32)
        self.ICeval = _arr(IC.get('eval', np.ones(self.ICnSTR * self.ICnRF, np.uint32)), np.uint32)
        self.ECv = _arr(EC['vox'], np.uint32); self.ECo = _arr(EC['dir'], np.uint16)
        self.ISOv = _arr(ISO['vox'], np.uint32)
        self.LUT_IC = _arr(KERNELS['wmr'], np.float32).ravel()
        self.LUT_EC = _arr(KERNELS['wmh'], np.float32).ravel()
        self.LUT_ISO = _arr(KERNELS['iso'], np.float32).ravel()

    def _copy(self):
        C = object.__new__(type(self))
        C.__dict__.update(self.__dict__)
        return C

    @property
    def T(self):
        C = self._copy()
        C.adjoint = 1 - self.adjoint
        return C

    @property
    def shape(self):
        return (self.nROWS, self.nCOLS) if not self.adjoint else (self.nCOLS, self.nROWS)

    def dot(self, v_in):
        v_in = np.ascontiguousarray(v_in, dtype=np.float64)
        if v_in.size != self.shape[1]:
            raise RuntimeError("A.dot(): dimensions do not match")
        v_out = np.zeros(self.shape[0], dtype=np.float64)
        self._apply(v_in, v_out)
        return v_out


class PortOperator(_OperatorBase):
    """The C restatement in commit_oracle.c."""

    def _apply(self, vin, vout):
        L = port_lib()
        vin1 = vin if vin.size else np.zeros(1)
        vout1 = vout if vout.size else np.zeros(1)
        if self.nolut:
            fn = L.oracle_At_nolut if self.adjoint else L.oracle_A_nolut
            rc = fn(vin1, vout1, self.ICnSTR, self.ICn, self.ICnVOX, self.ISOn, self.ICf, self.ICeval, self.ICv,
                    self.ICl, self.ISOv, self.ISOnRF, self.nthreads)
        else:
            fn = L.oracle_At if self.adjoint else L.oracle_A
            rc = fn(vin1, vout1, self.nSAMPLES, self.ndirs, self.ICnSTR, self.ICn, self.ECn, self.ICnVOX, self.ISOn,
                    self.ICf, self.ICeval, self.ICv, self.ICo, self.ICl, self.ECv, self.ECo, self.ISOv,
                    self.LUT_IC, self.LUT_EC, self.LUT_ISO, self.ICnRF, self.ECnRF, self.ISOnRF, self.nthreads)
        if rc != 0:
            raise RuntimeError(f'oracle operator failed ({rc})')


# ------------------------------------------------------------------ reference (oracle/_ref)
_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError('oracle/_ref is not built (run oracle/build_ref.py)')
        L = ctypes.CDLL(REF_LIB)
        u32 = ctypes.c_uint32
        i32 = ctypes.c_int
        # commit/operator/operator.pyx:189-227 declarations
        L.COMMIT_A.argtypes = [_f64p, _f64p, i32, i32, i32, i32, i32, _u32p, _u32p, _u32p, _u16p, _f32p, _u32p, _u16p,
                               _u32p, _f32p, _f32p, _f32p, _u32p, _u32p, _u32p, u32, u32, u32, u32]
        L.COMMIT_At.argtypes = [_f64p, _f64p, i32, i32, i32, i32, i32, i32, _u32p, _u32p, _u32p, _u16p, _f32p, _u32p,
                                _u16p, _u32p, _f32p, _f32p, _f32p, _u8p, _u32p, _u32p, u32, u32, u32, u32]
        L.COMMIT_A_nolut.argtypes = [_f64p, _f64p, i32, _u32p, _u32p, _u32p, _f32p, _u32p, _u32p, _u32p, u32, u32]
        L.COMMIT_At_nolut.argtypes = [_f64p, _f64p, i32, i32, _u32p, _u32p, _u32p, _f32p, _u32p, _u8p, _u32p, u32, u32]
        for f in (L.COMMIT_A, L.COMMIT_At, L.COMMIT_A_nolut, L.COMMIT_At_nolut):
            f.restype = None
        _ref = L
    return _ref


class RefOperator(_OperatorBase):
    """The reference's compiled operator, called the way operator.pyx:136-182 calls it."""

    def __init__(self, DICTIONARY, KERNELS, THREADS, nolut=False):
        super().__init__(DICTIONARY, KERNELS, THREADS, nolut)
        T = THREADS
        self.nThreads = int(T['n'])
        z32 = np.zeros(self.nThreads + 1, np.uint32)
        self.ICthreads = _arr(T['IC'] if T['IC'] is not None else z32, np.uint32)
        self.ECthreads = _arr(T['EC'] if T['EC'] is not None else z32, np.uint32)
        self.ISOthreads = _arr(T['ISO'] if T['ISO'] is not None else z32, np.uint32)
        self.ICthreadsT = _arr(T['ICt'] if T['ICt'] is not None else np.zeros(1, np.uint8), np.uint8)
        self.ECthreadsT = _arr(T['ECt'] if T['ECt'] is not None else z32, np.uint32)
        self.ISOthreadsT = _arr(T['ISOt'] if T['ISOt'] is not None else z32, np.uint32)

    def _apply(self, vin, vout):
        L = ref_lib()
        if not self.adjoint:
            if self.nolut:
                L.COMMIT_A_nolut(vin, vout, self.ICnSTR, self.ICf, self.ICeval, self.ICv, self.ICl, self.ISOv,
                                 self.ICthreads, self.ISOthreads, self.ISOnRF, self.nThreads)
            else:
                L.COMMIT_A(vin, vout, self.nSAMPLES, self.ndirs, self.ICnSTR, self.ECn, self.ISOn,
                           self.ICf, self.ICeval, self.ICv, self.ICo, self.ICl, self.ECv, self.ECo, self.ISOv,
                           self.LUT_IC, self.LUT_EC, self.LUT_ISO, self.ICthreads, self.ECthreads, self.ISOthreads,
                           self.ICnRF, self.ECnRF, self.ISOnRF, self.nThreads)
        else:
            if self.nolut:
                L.COMMIT_At_nolut(vin, vout, self.ICnSTR, self.ICn, self.ICf, self.ICeval, self.ICv, self.ICl,
                                  self.ISOv, self.ICthreadsT, self.ISOthreadsT, self.ISOnRF, self.nThreads)
            else:
                L.COMMIT_At(vin, vout, self.nSAMPLES, self.ndirs, self.ICnSTR, self.ICn, self.ECn, self.ISOn,
                            self.ICf, self.ICeval, self.ICv, self.ICo, self.ICl, self.ECv, self.ECo, self.ISOv,
                            self.LUT_IC, self.LUT_EC, self.LUT_ISO, self.ICthreadsT, self.ECthreadsT,
                            self.ISOthreadsT, self.ICnRF, self.ECnRF, self.ISOnRF, self.nThreads)


def set_threads(DICTIONARY: dict, n: int) -> dict:
    """Restatement of Evaluation.set_threads (commit/core.pyx:586-724)."""
    if n < 1 or n > 255:
        raise ValueError('Number of threads must be between 1 and 255')
    IC, EC, ISO = DICTIONARY['IC'], DICTIONARY['EC'], DICTIONARY['ISO']
    T = {'n': n}
    # A*x (core.pyx:626-667)
    if IC['n'] > 0:
        T['IC'] = np.zeros(n + 1, dtype=np.uint32)
        if n > 1:
            N = np.floor(IC['n'] / n)
            t = 1
            tot = 0
            C = np.bincount(IC['vox'])
            for c in C:
                tot += c
                if tot >= N and t <= n:
                    T['IC'][t] = T['IC'][t - 1] + tot
                    t += 1
                    tot = 0
        T['IC'][n] = IC['n']
        if np.count_nonzero(np.diff(T['IC'].astype(np.int32)) <= 0):
            raise RuntimeError('Too many threads for the IC compartments to evaluate; try decreasing the number')
    else:
        T['IC'] = None
    if EC['n'] > 0:
        T['EC'] = np.zeros(n + 1, dtype=np.uint32)
        for i in range(n):
            T['EC'][i] = np.searchsorted(EC['vox'], IC['vox'][T['IC'][i]])
        T['EC'][n] = EC['n']
        if np.count_nonzero(np.diff(T['EC'].astype(np.int32)) <= 0):
            raise RuntimeError('Too many threads for the EC compartments to evaluate; try decreasing the number')
    else:
        T['EC'] = None
    if ISO['n'] > 0:
        T['ISO'] = np.zeros(n + 1, dtype=np.uint32)
        for i in range(n):
            T['ISO'][i] = np.searchsorted(ISO['vox'], IC['vox'][T['IC'][i]])
        T['ISO'][n] = ISO['n']
    else:
        T['ISO'] = None
    # A'*y (core.pyx:673-722)
    if IC['n'] > 0:
        T['ICt'] = np.full(IC['n'], n - 1, dtype=np.uint8)
        if n > 1:
            idx = np.argsort(IC['str'], kind='mergesort')
            C = np.bincount(IC['str'])
            t = tot = i1 = i2 = 0
            N = np.floor(IC['n'] / n)
            for c in C:
                i2 += c
                tot += c
                if tot >= N:
                    T['ICt'][i1:i2] = t
                    t += 1
                    if t == n - 1:
                        break
                    i1 = i2
                    tot = c
            T['ICt'][idx] = T['ICt'].copy()
    else:
        T['ICt'] = None
    for key, comp in (('ECt', EC), ('ISOt', ISO)):
        if comp['n'] > 0:
            T[key] = np.zeros(n + 1, dtype=np.uint32)
            N = np.floor(comp['n'] / n)
            for i in range(1, n):
                T[key][i] = T[key][i - 1] + N
            T[key][n] = comp['n']
            if np.count_nonzero(np.diff(T[key].astype(np.int32)) <= 0):
                raise RuntimeError(f'Too many threads for the {key[:-1]} compartments to evaluate')
        else:
            T[key] = None
    return T


# ------------------------------------------------------------------ proximals.pyx restatement
def non_negativity(x, compartment_start, compartment_size):
    """proximals.pyx:13-22 (in place; x <= 0 -> 0)."""
    s = slice(compartment_start, compartment_start + compartment_size)
    v = x[s]
    v[v <= 0.0] = 0.0
    return x


def soft_thresholding(x, lam, compartment_start, compartment_size):
    """proximals.pyx:25-39."""
    s = slice(compartment_start, compartment_start + compartment_size)
    v = x[s]
    x[s] = np.where(v > lam, v - lam, np.where(v < -lam, v + lam, 0.0))
    return x


def w_soft_thresholding(x, w, lam, compartment_start, compartment_size):
    """proximals.pyx:42-56."""
    s = slice(compartment_start, compartment_start + compartment_size)
    v = x[s]
    wl = w[s] * lam
    x[s] = np.where(v > wl, v - wl, np.where(v < -wl, v + wl, 0.0))
    return x


def omega_group_lasso(x, group_idx, group_size, group_weight, lam):
    """proximals.pyx:80-99."""
    omega = 0.0
    if lam != 0:
        j = 0
        for k in range(group_size.size):
            N = int(group_size[k])
            g = x[group_idx[j:j + N]]
            omega += group_weight[k] * sqrt(float(np.dot(g, g)))
            j += N
    return lam * omega


def prox_group_lasso(x, group_idx, group_size, group_weight, lam):
    """proximals.pyx:103-134: groups processed in order, in place."""
    if lam != 0:
        j = 0
        for k in range(group_size.size):
            N = int(group_size[k])
            idx = group_idx[j:j + N]
            g = x[idx]
            gNorm = sqrt(float(np.dot(g, g)))
            wl = group_weight[k] * lam
            if gNorm <= wl:
                x[idx] = 0.0
            else:
                x[idx] = g * ((gNorm - wl) / gNorm)
            j += N
    return x


def omega_sparse_group_lasso(x, group_idx, group_size, group_weight, lam1, lam2):
    """proximals.pyx:138-159 (the l1 term covers the whole x)."""
    omega1 = omega2 = 0.0
    if lam1 != 0 or lam2 != 0:
        omega1 = float(np.sum(np.abs(x)))
        omega2 = omega_group_lasso(x, group_idx, group_size, group_weight, 1.0)
    return lam1 * omega1 + lam2 * omega2


def omega_w_sparse_group_lasso(x, w, group_idx, group_size, group_weight, lam1, lam2):
    """proximals.pyx:162-186 (the weighted l1 term covers the whole x)."""
    omega1 = omega2 = 0.0
    if lam1 != 0 or lam2 != 0:
        omega1 = float(np.sum(np.abs(w[:x.shape[0]] * x)))
        omega2 = omega_group_lasso(x, group_idx, group_size, group_weight, 1.0)
    return lam1 * omega1 + lam2 * omega2


# ------------------------------------------------------------------ solvers.py restatement
def _flatten_groups(group_idx_kept):
    N = int(np.sum([g.size for g in group_idx_kept]))
    gidx = np.zeros(N, dtype=np.int32)
    gsize = np.zeros(len(group_idx_kept), dtype=np.int32)
    pos = 0
    for i, g in enumerate(group_idx_kept):
        gsize[i] = g.size
        gidx[pos:pos + g.size] = g[:]
        pos += g.size
    return gidx, gsize


def init_regularisation(rp: dict) -> dict:
    """Restatement of commit/solvers.py:16-206 (omega/prox closures per compartment)."""
    lst = [None, 'lasso', 'group_lasso', 'sparse_group_lasso']
    if rp['regIC'] not in lst or rp['regEC'] not in lst or rp['regISO'] not in lst:
        raise ValueError('Regularisation not in the list')
    sIC, nIC = rp.get('startIC'), rp.get('sizeIC')
    sEC, nEC = rp.get('startEC'), rp.get('sizeEC')
    sISO, nISO = rp.get('startISO'), rp.get('sizeISO')
    acw = np.ones(nIC + nEC + nISO, dtype=np.float64)
    dIC = rp.get('dictIC_params')
    dISO = rp.get('dictISO_params')
    if dIC is not None and 'coeff_weights_kept' in dIC:
        acw[sIC:sIC + nIC] = dIC['coeff_weights_kept']
    if dISO is not None and 'coeff_weights' in dISO:
        acw[sISO:sISO + nISO] = dISO['coeff_weights']

    nn = lambda v, a, b: non_negativity(v, a, b)
    reg = rp['regIC']
    if reg is None:
        omegaIC = lambda x: 0.0
        proxIC = (lambda x, _: nn(x, sIC, nIC)) if rp.get('nnIC') == True else (lambda x, _: x)  # noqa: E712
    elif reg == 'lasso':
        lam = rp['lambdaIC']
        if dIC is not None and 'coeff_weights_kept' in dIC:
            omegaIC = lambda x: lam * np.linalg.norm(acw[sIC:nIC] * x[sIC:nIC], 1)  # solvers.py:68 slicing
            if rp.get('nnIC'):
                proxIC = lambda x, s: nn(w_soft_thresholding(x, acw, s * lam, sIC, nIC), sIC, nIC)
            else:
                proxIC = lambda x, s: w_soft_thresholding(x, acw, s * lam, sIC, nIC)
        else:
            omegaIC = lambda x: lam * np.linalg.norm(x[sIC:nIC], 1)
            if rp.get('nnIC'):
                proxIC = lambda x, s: nn(soft_thresholding(x, s * lam, sIC, nIC), sIC, nIC)
            else:
                proxIC = lambda x, s: soft_thresholding(x, s * lam, sIC, nIC)
    elif reg == 'group_lasso':
        lam = rp['lambdaIC']
        gidx, gsize = _flatten_groups(dIC['group_idx_kept'])
        gw = dIC['group_weights']
        omegaIC = lambda x: omega_group_lasso(x, gidx, gsize, gw, lam)
        if rp.get('nnIC'):
            proxIC = lambda x, s: nn(prox_group_lasso(x, gidx, gsize, gw, s * lam), sIC, nIC)
        else:
            proxIC = lambda x, s: prox_group_lasso(x, gidx, gsize, gw, s * lam)
    else:  # sparse_group_lasso
        lam1, lam2 = rp['lambdaIC'][0], rp['lambdaIC'][1]
        gidx, gsize = _flatten_groups(dIC['group_idx_kept'])
        gw = dIC['group_weights']
        if 'coeff_weights_kept' in dIC:
            omegaIC = lambda x: omega_w_sparse_group_lasso(x, acw, gidx, gsize, gw, lam1, lam2)
            inner = lambda x, s: prox_group_lasso(w_soft_thresholding(x, acw, s * lam1, sIC, nIC), gidx, gsize, gw, s * lam2)
        else:
            omegaIC = lambda x: omega_sparse_group_lasso(x, gidx, gsize, gw, lam1, lam2)
            inner = lambda x, s: prox_group_lasso(soft_thresholding(x, s * lam1, sIC, nIC), gidx, gsize, gw, s * lam2)
        if rp.get('nnIC'):
            proxIC = lambda x, s: nn(inner(x, s), sIC, nIC)
        else:
            proxIC = inner

    reg = rp['regEC']
    if reg is None:
        omegaEC = lambda x: 0.0
        proxEC = (lambda x, _: nn(x, sEC, nEC)) if rp.get('nnEC') == True else (lambda x, _: x)  # noqa: E712
    elif reg == 'lasso':
        lamE = rp.get('lambdaEC')
        omegaEC = lambda x: lamE * np.linalg.norm(x[sEC:sEC + nEC], 1)
        if rp.get('nnEC'):
            proxEC = lambda x, s: nn(soft_thresholding(x, s * lamE, sEC, nEC), sEC, nEC)
        else:
            proxEC = lambda x, s: soft_thresholding(x, s * lamE, sEC, nEC)
    else:
        raise ValueError('EC regulariser not supported by the reference')

    reg = rp['regISO']
    if reg is None:
        omegaISO = lambda x: 0.0
        proxISO = (lambda x, _: nn(x, sISO, nISO)) if rp.get('nnISO') == True else (lambda x, _: x)  # noqa: E712
    elif reg == 'lasso':
        lamI = rp.get('lambdaISO')
        if dISO is not None and 'coeff_weights' in dISO:
            omegaISO = lambda x: lamI * np.linalg.norm(acw[sISO:nISO] * x[sISO:nISO], 1)  # solvers.py:183 slicing
            if rp.get('nnISO'):
                proxISO = lambda x, s: nn(w_soft_thresholding(x, acw, s * lamI, sISO, nISO), sISO, nISO)
            else:
                proxISO = lambda x, s: w_soft_thresholding(x, acw, s * lamI, sISO, nISO)
        else:
            omegaISO = lambda x: lamI * np.linalg.norm(x[sISO:sISO + nISO], 1)
            if rp.get('nnISO'):
                proxISO = lambda x, s: nn(soft_thresholding(x, s * lamI, sISO, nISO), sISO, nISO)
            else:
                proxISO = lambda x, s: soft_thresholding(x, s * lamI, sISO, nISO)
    else:
        raise ValueError('ISO regulariser not supported by the reference')

    rp['omega'] = lambda x: omegaIC(x) + omegaEC(x) + omegaISO(x)
    rp['prox'] = lambda x, s: proxIC(proxEC(proxISO(x, s), s), s)
    return rp


def evaluate_model(y, A, x, regularisation=None):
    """solvers.py:209-215."""
    omega = (lambda x: 0.0) if regularisation is None else init_regularisation(regularisation)['omega']
    return 0.5 * np.linalg.norm(A.dot(x) - y) ** 2 + omega(x)


def solve(y, A, At, tol_fun=1e-4, tol_x=1e-6, max_iter=1000, verbose=True, x0=None, regularisation=None,
          confidence_array=None):
    """solvers.py:218-241."""
    if regularisation is None:
        omega = lambda x: 0.0
        prox = lambda x, _: x
    else:
        omega, prox = regularisation['omega'], regularisation['prox']
    if x0 is None:
        x0 = np.zeros(A.shape[1])
    if confidence_array is not None:
        confidence_array = np.sqrt(confidence_array)
    return fista(y, A, At, omega, prox, confidence_array, tol_fun, tol_x, max_iter, verbose, x0)


def fista(y, A, At, omega, prox, sqrt_W=None, tol_fun=1e-4, tol_x=1e-6, max_iter=1000, verbose=False, x0=None):
    """Restatement of commit/solvers.py:244-391 (FISTA with backtracking)."""
    if x0 is None:
        x0 = np.zeros(A.shape[1])
    xhat = x0.copy()
    if sqrt_W is not None:
        res = sqrt_W * (A.dot(xhat) - y)
        grad = np.asarray(At.dot(sqrt_W * res))
    else:
        res = A.dot(xhat) - y
        grad = np.asarray(At.dot(res))
    prox(xhat, 1.0)
    reg_term = omega(xhat)
    prev_obj = 0.5 * np.linalg.norm(res) ** 2 + reg_term
    told = 1
    beta = 0.9
    prev_x = xhat.copy()
    qfval = prev_obj
    if sqrt_W is not None:
        L = (np.linalg.norm(sqrt_W * A.dot(grad)) / np.linalg.norm(grad)) ** 2
    else:
        L = (np.linalg.norm(A.dot(grad)) / np.linalg.norm(grad)) ** 2
    step_size = 1.9 / L
    it = 1
    while True:
        x = xhat - step_size * grad
        prox(x, step_size)
        reg_term_x = omega(x)
        tmp = x - xhat
        q = qfval + np.real(np.dot(tmp, grad)) + 0.5 / step_size * np.linalg.norm(tmp) ** 2 + reg_term_x
        res = sqrt_W * (A.dot(x) - y) if sqrt_W is not None else A.dot(x) - y
        res_norm = np.linalg.norm(res)
        curr_obj = 0.5 * res_norm ** 2 + reg_term_x
        while curr_obj > q:
            step_size = beta * step_size
            x = xhat - step_size * grad
            prox(x, step_size)
            reg_term_x = omega(x)
            tmp = x - xhat
            q = qfval + np.real(np.dot(tmp, grad)) + 0.5 / step_size * np.linalg.norm(tmp) ** 2 + reg_term_x
            res = sqrt_W * (A.dot(x) - y) if sqrt_W is not None else A.dot(x) - y
            res_norm = np.linalg.norm(res)
            curr_obj = 0.5 * res_norm ** 2 + reg_term_x
        abs_obj = abs(curr_obj - prev_obj)
        rel_obj = abs_obj / curr_obj
        abs_x = np.linalg.norm(x - prev_x)
        rel_x = abs_x / (np.linalg.norm(x) + eps)
        if abs_obj < eps:
            criterion = "Absolute tolerance on the objective"
            break
        elif rel_obj < tol_fun:
            criterion = "Relative tolerance on the objective"
            break
        elif abs_x < eps:
            criterion = "Absolute tolerance on the unknowns"
            break
        elif rel_x < tol_x:
            criterion = "Relative tolerance on the unknowns"
            break
        elif it >= max_iter:
            criterion = "Maximum number of iterations"
            break
        t = 0.5 * (1 + sqrt(1 + 4 * told ** 2))
        xhat = x + (told - 1) / t * (x - prev_x)
        if sqrt_W is not None:
            res = sqrt_W * (A.dot(xhat) - y)
            grad = np.asarray(At.dot(sqrt_W * res))
        else:
            res = A.dot(xhat) - y
            grad = np.asarray(At.dot(res))
        it += 1
        prev_obj = curr_obj
        prev_x = x.copy()
        told = t
        qfval = 0.5 * np.linalg.norm(res) ** 2
    return x, {'residual': 0.5 * res_norm ** 2, 'regterm': reg_term_x, 'cost_function': curr_obj,
               'abs_cost': abs_obj, 'rel_cost': rel_obj, 'abs_x': abs_x, 'rel_x': rel_x,
               'iterations': it, 'stopping_criterion': criterion}


def reg_params(D: dict, K: dict, regularisers=(None, None, None), is_nonnegative=(True, True, True)) -> dict:
    """The compartment layout part of Evaluation.set_regularisation (commit/core.pyx:1030-1046)."""
    rp = {}
    rp['startIC'] = 0
    rp['sizeIC'] = int(D['IC']['nSTR'] * K['wmr'].shape[0])
    rp['startEC'] = rp['sizeIC']
    rp['sizeEC'] = int(D['EC']['n'] * K['wmh'].shape[0])
    rp['startISO'] = rp['sizeIC'] + rp['sizeEC']
    rp['sizeISO'] = int(D['ISO']['n'] * K['iso'].shape[0])
    rp['regIC'], rp['regEC'], rp['regISO'] = regularisers
    rp['nnIC'], rp['nnEC'], rp['nnISO'] = is_nonnegative
    rp['dictIC_params'] = rp['dictEC_params'] = rp['dictISO_params'] = None
    return rp


def voxel_maps(D: dict, K: dict, x, y_est, y_mea=None, conf=None, norm_fib=None) -> dict:
    """Maps of Evaluation.save_results (commit/core.pyx:1662-1750), numpy restatement.
    y_est = A x.  Error maps compare FP32-rounded signals (core.pyx:1664-1665) with FP64
    sums; bincount lengths are the number of mask voxels."""
    nV = int(D['IC']['nVOX'])
    nSTR = int(D['IC']['nSTR'])
    nE = int(D['EC']['n'])
    nIC, nEC, nISO = K['wmr'].shape[0], K['wmh'].shape[0], K['iso'].shape[0]
    x = np.asarray(x, dtype=np.float64)
    out = {}
    if nIC > 0:                                                  # core.pyx:1717-1725
        off = nSTR * nIC
        w = np.ones(off) if norm_fib is None else np.asarray(norm_fib, dtype=np.float64)
        tmp = (x[:off].reshape((-1, nSTR)) * w.reshape((-1, nSTR))).sum(axis=0)
        out['compartment_IC'] = np.bincount(D['IC']['vox'], minlength=nV,
                                            weights=tmp[D['IC']['str']] * D['IC']['len'])
    else:
        out['compartment_IC'] = np.zeros(nV)
    if nEC > 0 and nE > 0:                                       # core.pyx:1731-1736
        off = nSTR * nIC
        tmp = x[off:off + nE * nEC].reshape((-1, nE)).sum(axis=0)
        out['compartment_EC'] = np.bincount(D['EC']['vox'], weights=tmp, minlength=nV)
    else:
        out['compartment_EC'] = np.zeros(nV)
    nI = int(D['ISO']['n'])
    if nISO > 0 and nI > 0:                                      # core.pyx:1742-1748
        off = nSTR * nIC + nE * nEC
        tmp = x[off:off + nI * nISO].reshape((-1, nI)).sum(axis=0)
        out['compartment_ISO'] = np.bincount(D['ISO']['vox'], weights=tmp, minlength=nV)
    else:
        out['compartment_ISO'] = np.zeros(nV)
    if y_mea is not None:                                        # core.pyx:1662-1680
        ym = np.asarray(y_mea).astype(np.float32).reshape((nV, -1))
        ye = np.asarray(y_est).astype(np.float32).reshape((nV, -1))
        d2 = ((ym - ye).astype(np.float64)) ** 2
        y2 = ym.astype(np.float64) ** 2
        out['fit_RMSE'] = np.sqrt(d2.mean(axis=1))
        tmp = y2.sum(axis=1)
        idx = np.where(tmp < 1e-12)
        tmp[idx] = 1
        tmp = np.sqrt(d2.sum(axis=1) / tmp)
        tmp[idx] = 0
        out['fit_NRMSE'] = tmp
        if conf is not None:                                     # core.pyx:1682-1705
            c = np.asarray(conf).astype(np.float32).astype(np.float64).reshape((nV, -1))
            for name, den in (('fit_RMSE_adjusted', c.sum(axis=1)), ('fit_NRMSE_adjusted', (c * y2).sum(axis=1))):
                idx = np.where(den < 1e-12)
                den[idx] = 1
                t = np.sqrt((c * d2).sum(axis=1) / den)
                t[idx] = 0
                out[name] = t
    return out
