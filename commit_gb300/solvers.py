"""GB300 drop-in for commit/solvers.py (init_regularisation, evaluate_model, solve, fista).

``init_regularisation`` accepts the dict ``Evaluation.set_regularisation`` builds
(commit/core.pyx:1030-1046 and solvers.py:16-206) and returns it with ``omega`` and
``prox`` entries, as the reference does; here they are device-backed callables that also
carry the regulariser description, which ``solve``/``fista`` hand to the CUDA solver
(``cgb_fista_run``).  FISTA itself runs on the GPU with the reference's step-size rule,
backtracking, stopping criteria and returned ``opt_details`` (solvers.py:244-391).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check, lib
from .operator import LinearOperator

eps = np.finfo(float).eps
list_regularizers = [None, 'lasso', 'group_lasso', 'sparse_group_lasso']


def _dev(a, dtype, device):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).to(device)


def level_schedule(groups):
    """Order groups into levels of pairwise-disjoint groups that reproduce the sequential
    prox_group_lasso loop (proximals.pyx:103-134): a group's level is one more than the
    highest level of any earlier group it overlaps, so overlapping groups keep their
    relative order and disjoint ones run together.  Returns (order, level_ptr)."""
    ng = len(groups)
    if ng == 0:
        return np.zeros(0, np.int64), np.zeros(1, np.int64)
    top = max((int(g.max()) for g in groups if g.size), default=-1) + 1
    touch = np.full(max(top, 1), -1, dtype=np.int64)
    level = np.zeros(ng, dtype=np.int64)
    for k, g in enumerate(groups):
        lv = int(touch[g].max()) + 1 if g.size else 0
        level[k] = lv
        if g.size:
            touch[g] = lv
    order = np.argsort(level, kind='stable')
    counts = np.bincount(level, minlength=int(level.max()) + 1)
    return order, np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)


class RegSpec:
    """Device description of a regularisation dict (the omega/prox pair of the reference)."""

    def __init__(self, rp: dict):
        self.rp = rp
        self.sIC, self.nIC = int(rp.get('startIC') or 0), int(rp.get('sizeIC') or 0)
        self.sEC, self.nEC = int(rp.get('startEC') or 0), int(rp.get('sizeEC') or 0)
        self.sISO, self.nISO = int(rp.get('startISO') or 0), int(rp.get('sizeISO') or 0)
        self.ncols = self.nIC + self.nEC + self.nISO
        self.reg_ic, self.reg_ec, self.reg_iso = rp.get('regIC'), rp.get('regEC'), rp.get('regISO')
        # nn flags: `== True` when no regulariser is set, truthiness otherwise (solvers.py:54-206)
        self.nn_ic = bool(rp.get('nnIC') == True) if self.reg_ic is None else bool(rp.get('nnIC'))  # noqa: E712
        self.nn_ec = bool(rp.get('nnEC') == True) if self.reg_ec is None else bool(rp.get('nnEC'))  # noqa: E712
        self.nn_iso = bool(rp.get('nnISO') == True) if self.reg_iso is None else bool(rp.get('nnISO'))  # noqa: E712
        dIC = rp.get('dictIC_params')
        dISO = rp.get('dictISO_params')
        acw = np.ones(self.ncols, dtype=np.float64)
        self.weighted_ic = False
        self.weighted_iso = False
        if dIC is not None and 'coeff_weights_kept' in dIC:
            acw[self.sIC:self.sIC + self.nIC] = dIC['coeff_weights_kept']
            self.weighted_ic = self.reg_ic in ('lasso', 'sparse_group_lasso')
        if dISO is not None and 'coeff_weights' in dISO:
            acw[self.sISO:self.sISO + self.nISO] = dISO['coeff_weights']
            self.weighted_iso = self.reg_iso == 'lasso'
        self.acw = acw
        self.lam_ic = self.lam_ic_group = self.lam_ec = self.lam_iso = 0.0
        if self.reg_ic == 'lasso':
            self.lam_ic = float(rp['lambdaIC'])
        elif self.reg_ic == 'group_lasso':
            self.lam_ic = float(rp['lambdaIC'])
        elif self.reg_ic == 'sparse_group_lasso':
            self.lam_ic, self.lam_ic_group = float(rp['lambdaIC'][0]), float(rp['lambdaIC'][1])
        if self.reg_ec == 'lasso':
            self.lam_ec = float(rp.get('lambdaEC'))
        if self.reg_iso == 'lasso':
            self.lam_iso = float(rp.get('lambdaISO'))
        self.groups = None
        if self.reg_ic in ('group_lasso', 'sparse_group_lasso'):
            if not len(dIC['group_idx_kept']) == len(dIC['group_weights']):
                raise ValueError('Number of groups and weights do not match')
            groups = [np.asarray(g, dtype=np.int64).ravel() for g in dIC['group_idx_kept']]
            order, level_ptr = level_schedule(groups)
            gw = np.asarray(dIC['group_weights'], dtype=np.float64)
            og = [groups[k] for k in order]
            sizes = np.array([g.size for g in og], dtype=np.int64)
            self.group_idx = np.concatenate(og).astype(np.int32) if og else np.zeros(0, np.int32)
            self.group_ptr = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
            self.group_w = gw[order]
            self.level_ptr = level_ptr
            self.groups = groups
        self._dev = {}

    def device_arrays(self, device):
        key = str(device)
        if key not in self._dev:
            d = {'acw': _dev(self.acw, torch.float64, device)}
            if self.groups is not None:
                d['gidx'] = _dev(self.group_idx, torch.int32, device)
                d['gptr'] = _dev(self.group_ptr, torch.int64, device)
                d['gw'] = _dev(self.group_w, torch.float64, device)
            self._dev[key] = d
        return self._dev[key]

    def cstruct(self, device) -> tuple:
        d = self.device_arrays(device)
        r = _lib.CgbReg()
        r.start_ic, r.size_ic, r.start_ec, r.size_ec = self.sIC, self.nIC, self.sEC, self.nEC
        r.start_iso, r.size_iso = self.sISO, self.nISO
        r.reg_ic, r.reg_ec, r.reg_iso = _lib.REG[self.reg_ic], _lib.REG[self.reg_ec], _lib.REG[self.reg_iso]
        r.nn_ic, r.nn_ec, r.nn_iso = int(self.nn_ic), int(self.nn_ec), int(self.nn_iso)
        r.lambda_ic, r.lambda_ic_group = self.lam_ic, self.lam_ic_group
        r.lambda_ec, r.lambda_iso = self.lam_ec, self.lam_iso
        r.coeff_weights = d['acw'].data_ptr()
        r.weighted_ic, r.weighted_iso = int(self.weighted_ic), int(self.weighted_iso)
        keep = [d]
        if self.groups is not None:
            r.group_idx, r.group_ptr, r.group_w = d['gidx'].data_ptr(), d['gptr'].data_ptr(), d['gw'].data_ptr()
            r.ngroups = len(self.groups)
            lp = np.ascontiguousarray(self.level_ptr, dtype=np.int64)
            keep.append(lp)
            r.level_ptr = lp.ctypes.data
            r.nlevels = lp.size - 1
        return r, keep


def _no_reg_spec(ncols: int) -> RegSpec:
    return RegSpec({'startIC': 0, 'sizeIC': ncols, 'startEC': ncols, 'sizeEC': 0, 'startISO': ncols, 'sizeISO': 0,
                    'regIC': None, 'regEC': None, 'regISO': None, 'nnIC': False, 'nnEC': False, 'nnISO': False})


class _Omega:
    """omega(x) of init_regularisation, evaluated on the device."""

    def __init__(self, spec: RegSpec):
        self.spec = spec

    def __call__(self, x) -> float:
        from . import proximals as P
        s = self.spec
        xt, _ = P._as_device(x)
        total = 0.0
        acw = s.device_arrays(xt.device)['acw']
        if s.reg_ic == 'lasso':
            total += P._l1(xt, acw if s.weighted_ic else None, s.sIC, s.nIC - s.sIC) * s.lam_ic
        elif s.reg_ic == 'group_lasso':
            total += P._omega_groups(xt, s, s.lam_ic)
        elif s.reg_ic == 'sparse_group_lasso':
            if s.lam_ic != 0 or s.lam_ic_group != 0:
                total += s.lam_ic * P._l1(xt, acw if s.weighted_ic else None, 0, xt.numel())
                total += P._omega_groups(xt, s, s.lam_ic_group, force=True)
        if s.reg_ec == 'lasso':
            total += s.lam_ec * P._l1(xt, None, s.sEC, s.nEC)
        if s.reg_iso == 'lasso':
            if s.weighted_iso:
                total += s.lam_iso * P._l1(xt, acw, s.sISO, min(s.nISO, xt.numel()) - s.sISO)
            else:
                total += s.lam_iso * P._l1(xt, None, s.sISO, s.nISO)
        return float(total)


class _Prox:
    """prox(x, scaling) of init_regularisation: in place on a numpy array or CUDA tensor."""

    def __init__(self, spec: RegSpec):
        self.spec = spec

    def __call__(self, x, scaling):
        from . import proximals as P
        return P._apply_spec(x, self.spec, float(scaling))


def init_regularisation(regularisation_params: dict) -> dict:
    """commit/solvers.py:16-206: adds 'omega' and 'prox' to the regularisation dict."""
    rp = regularisation_params
    if rp['regIC'] not in list_regularizers or rp['regEC'] not in list_regularizers or \
            rp['regISO'] not in list_regularizers:
        raise ValueError('Regularisation not in the list')
    if rp['regEC'] not in (None, 'lasso') or rp['regISO'] not in (None, 'lasso'):
        raise ValueError('EC and ISO compartments support only None or "lasso"')
    spec = RegSpec(rp)
    rp['omega'] = _Omega(spec)
    rp['prox'] = _Prox(spec)
    rp['_spec'] = spec
    return rp


def evaluate_model(y, A, x, regularisation=None):
    """solvers.py:209-215."""
    omega = (lambda x: 0.0) if regularisation is None else init_regularisation(regularisation)['omega']
    r = A.dot(x)
    if isinstance(r, torch.Tensor):
        return 0.5 * float(torch.linalg.norm(r - torch.as_tensor(y, device=r.device))) ** 2 + omega(x)
    return 0.5 * np.linalg.norm(r - y) ** 2 + omega(x)


def solve(y, A, At, tol_fun=1e-4, tol_x=1e-6, max_iter=1000, verbose=True, x0=None, regularisation=None,
          confidence_array=None, arith=None, momentum_reuse=True, x_ref=None, graph=False, max_backtracks=0,
          restart=False):
    """solvers.py:218-241: regularised least squares by FISTA, on the GPU.

    graph=True runs the iteration loop as one CUDA graph launch whose backtracking and
    stopping decisions are taken on the device (conditional graph nodes), with or without
    momentum reuse; it takes no x_ref / verbose output and no restart.  max_backtracks caps the step
    reductions of one iteration (0: 1000, negative: none); reaching the cap raises CgbError (the
    reference's backtracking loop has no cap, solvers.py:322-333).  restart=True resets the
    momentum after an iteration whose objective rose (function-value restart; not in the
    reference, whose FISTA never restarts: solvers.py:359-368)."""
    if regularisation is None:
        spec = _no_reg_spec(A.shape[1])
    else:
        spec = regularisation.get('_spec') if isinstance(regularisation, dict) else None
        if spec is None:
            spec = init_regularisation(regularisation)['_spec']
    sqrt_W = None
    if confidence_array is not None:
        sqrt_W = np.sqrt(np.asarray(confidence_array)) if not isinstance(confidence_array, torch.Tensor) \
            else torch.sqrt(confidence_array)
    return _fista(y, A, spec, sqrt_W, tol_fun, tol_x, max_iter, verbose, x0, arith, momentum_reuse, x_ref, graph,
                  max_backtracks, restart)


def fista(y, A, At, omega, prox, sqrt_W=None, tol_fun=1e-4, tol_x=1e-6, max_iter=1000, verbose=False, x0=None,
          arith=None, momentum_reuse=True):
    """solvers.py:244-391.  omega/prox must come from init_regularisation (or be the
    no-regulariser pair of ``solve``)."""
    spec = getattr(prox, 'spec', None)
    if spec is None:
        spec = _no_reg_spec(A.shape[1])
        if not (callable(prox) and _is_identity(prox, A.shape[1])):
            raise TypeError('commit_gb300 fista needs omega/prox from commit_gb300.solvers.init_regularisation')
    return _fista(y, A, spec, sqrt_W, tol_fun, tol_x, max_iter, verbose, x0, arith, momentum_reuse)


def _is_identity(prox, n) -> bool:
    probe = np.linspace(-1.0, 1.0, 7)
    try:
        out = prox(probe.copy(), 1.0)
    except Exception:
        return False
    return out is not None and np.array_equal(np.asarray(out), probe)


def _fista(y, A, spec: RegSpec, sqrt_W, tol_fun, tol_x, max_iter, verbose, x0, arith, momentum_reuse, x_ref=None,
           graph=False, max_backtracks=0, restart=False):
    """With x_ref given, details['trace'] holds, per accepted iteration, the seconds since
    the solve started, |x_k - x_ref| / |x_ref| and the cost function."""
    if not isinstance(A, LinearOperator):
        raise TypeError('A must be a commit_gb300.operator.LinearOperator')
    if A.adjoint:
        raise ValueError('A must be the forward operator')
    dev = torch.device('cuda', A.device)
    host = not isinstance(y, torch.Tensor)
    yd = torch.as_tensor(np.ascontiguousarray(y, dtype=np.float64) if host else y, dtype=torch.float64).to(dev)
    yd = yd.contiguous()
    if yd.numel() != A.nROWS:
        raise RuntimeError("A.dot(): dimensions do not match")
    if x0 is None:
        xd = torch.zeros(A.nCOLS, dtype=torch.float64, device=dev)
    else:
        xd = torch.as_tensor(np.asarray(x0, dtype=np.float64) if not isinstance(x0, torch.Tensor) else x0,
                             dtype=torch.float64).to(dev).clone()
    sw = None
    if sqrt_W is not None:
        sw = torch.as_tensor(np.asarray(sqrt_W, dtype=np.float64) if not isinstance(sqrt_W, torch.Tensor) else sqrt_W,
                             dtype=torch.float64).to(dev).contiguous()
    if spec.ncols != A.nCOLS:
        raise ValueError('regularisation sizes do not match the operator')
    reg, keep = spec.cstruct(dev)
    prm = _lib.CgbFistaParams(float(tol_fun), float(tol_x), int(max_iter), int(verbose) if verbose is not True else 1,
                              _lib.ARITH[arith or A.arith], int(bool(momentum_reuse)))
    prm.graph = int(bool(graph))
    prm.max_backtracks = int(max_backtracks)
    prm.restart = int(bool(restart))
    if graph and (x_ref is not None or verbose == 4):
        raise ValueError('graph mode takes no x_ref and no verbose output')
    trace = None
    if x_ref is not None:
        xr = torch.as_tensor(np.asarray(x_ref, dtype=np.float64) if not isinstance(x_ref, torch.Tensor) else x_ref,
                             dtype=torch.float64).to(dev).contiguous()
        trace = np.full((int(max_iter), 3), np.nan)
        prm.x_ref = xr.data_ptr()
        prm.trace = trace.ctypes.data
        prm.trace_len = int(max_iter)
        prm.trace_cost = 1
    res = _lib.CgbFistaResult()
    st = torch.cuda.current_stream(dev).cuda_stream
    check(lib().cgb_fista_run(A.handle, ctypes.c_void_p(yd.data_ptr()),
                              ctypes.c_void_p(sw.data_ptr()) if sw is not None else None, ctypes.byref(reg),
                              ctypes.byref(prm), ctypes.c_void_p(xd.data_ptr()), ctypes.byref(res),
                              ctypes.c_void_p(st)))
    del keep
    details = {'residual': res.residual, 'regterm': res.regterm, 'cost_function': res.cost_function,
               'abs_cost': res.abs_cost, 'rel_cost': res.rel_cost, 'abs_x': res.abs_x, 'rel_x': res.rel_x,
               'iterations': int(res.iterations), 'stopping_criterion': _lib.CRITERIA[res.stopping_criterion]}
    if trace is not None:
        details['trace'] = trace[:int(res.iterations)]
    details['backtracks'] = int(res.backtracks)
    details['operator_calls'] = int(res.operator_calls)
    details['anchors'] = int(res.anchors)
    x = xd.cpu().numpy() if host else xd
    return x, details


def solve_mixed(y, A, tol_fun=1e-4, tol_x=1e-6, max_iter=1000, verbose=0, x0=None, regularisation=None,
                confidence_array=None, arith='fp16', refine_arith=None, refine_max_iter=None,
                refine_tol_fun=None, refine_tol_x=None, x_ref=None, restart=False):
    """Reduced-precision FISTA followed by an FP64 refinement solve.

    Phase 1 runs FISTA with the operator in ``arith`` ('bf16', 'fp16' or 'f32': LUT in
    that format, FP16 lengths, FP32 accumulation; FISTA vectors, the Lipschitz estimate
    and every objective / stopping reduction in FP64).  The default is FP16, with a tenth of
    BF16's error (solution within 4e-4 instead of 4e-3 of the FP64 one on the demo case);
    BF16 is the faster choice on dense dictionaries, where it runs on the tensor cores (141
    against 65 operator pairs/s for FP16 at 1M streamlines).  Phase 2 restarts the plain FP64
    solver (float-float by default) from the phase-1 solution, which removes the bias of
    the reduced-precision operator.  Returns (x, details) with details['mixed'] and
    details['refine'] holding each phase's opt_details.  restart applies the function-value
    momentum restart of ``solve`` in both phases.
    """
    import time
    t0 = time.perf_counter()
    x1, d1 = solve(y, A, A.T, tol_fun=tol_fun, tol_x=tol_x, max_iter=max_iter, verbose=verbose, x0=x0,
                   regularisation=regularisation, confidence_array=confidence_array, arith=arith, x_ref=x_ref,
                   restart=restart)
    t1 = time.perf_counter() - t0
    x2, d2 = solve(y, A, A.T, tol_fun=refine_tol_fun if refine_tol_fun is not None else tol_fun,
                   tol_x=refine_tol_x if refine_tol_x is not None else tol_x,
                   max_iter=refine_max_iter if refine_max_iter is not None else max_iter, verbose=verbose, x0=x1,
                   regularisation=regularisation, confidence_array=confidence_array, arith=refine_arith, x_ref=x_ref,
                   restart=restart)
    det = dict(d2)
    if x_ref is not None:
        tr2 = d2['trace'].copy()
        tr2[:, 0] += t1
        det['trace'] = np.concatenate([d1['trace'], tr2])
    det['mixed'] = d1
    det['refine'] = d2
    det['iterations'] = d1['iterations'] + d2['iterations']
    return x2, det


def solve_batch(y, A, regularisations, tol_fun=1e-4, tol_x=1e-6, max_iter=1000, x0=None, confidence_array=None,
                momentum_reuse='auto'):
    """Several problems on one operator and one y, e.g. a regularisation path over lambda.

    ``regularisations`` is a list of regularisation dicts (as for ``solve``; None for no
    regulariser).  Every problem runs the FISTA of commit/solvers.py:244-391 with its own
    step size, backtracking and stopping test; the operator runs in BF16-LUT arithmetic and
    the products of all problems at the same stage share multi-right-hand-side passes
    (``cgb_fista_batch_run``).  Returns a list of (x, opt_details), x on the device of A when
    y is a CUDA tensor, numpy otherwise.  Polish a solution with ``solve(..., x0=x)`` in FP64
    where the BF16 operator's bias matters (as ``solve_mixed`` does for one problem).
    ``momentum_reuse``: True, False, or 'auto' (chosen by timing on the first batched solve
    on this operator, together with the vectors per pass)."""
    if not isinstance(A, LinearOperator):
        raise TypeError('A must be a commit_gb300.operator.LinearOperator')
    if A.adjoint:
        raise ValueError('A must be the forward operator')
    P = len(regularisations)
    if P == 0:
        return []
    dev = torch.device('cuda', A.device)
    host = not isinstance(y, torch.Tensor)
    yd = torch.as_tensor(np.ascontiguousarray(y, dtype=np.float64) if host else y, dtype=torch.float64).to(dev)
    yd = yd.contiguous()
    if yd.numel() != A.nROWS:
        raise RuntimeError("A.dot(): dimensions do not match")
    sw = None
    if confidence_array is not None:
        c = confidence_array
        sw = torch.sqrt(torch.as_tensor(np.asarray(c, dtype=np.float64) if not isinstance(c, torch.Tensor) else c,
                                        dtype=torch.float64).to(dev)).contiguous()
    specs = []
    for rp in regularisations:
        if rp is None:
            specs.append(_no_reg_spec(A.shape[1]))
        else:
            sp = rp.get('_spec') if isinstance(rp, dict) else None
            specs.append(sp if sp is not None else init_regularisation(rp)['_spec'])
    for sp in specs:
        if sp.ncols != A.nCOLS:
            raise ValueError('regularisation sizes do not match the operator')
    regs = (_lib.CgbReg * P)()
    keep = []
    for p, sp in enumerate(specs):
        r, k = sp.cstruct(dev)
        regs[p] = r
        keep.append(k)
    xs = []
    for p in range(P):
        x0p = x0[p] if isinstance(x0, (list, tuple)) else x0
        if x0p is None:
            xs.append(torch.zeros(A.nCOLS, dtype=torch.float64, device=dev))
        else:
            xs.append(torch.as_tensor(np.asarray(x0p, dtype=np.float64) if not isinstance(x0p, torch.Tensor) else x0p,
                                      dtype=torch.float64).to(dev).clone().contiguous())
    ptrs = (ctypes.c_void_p * P)(*[x.data_ptr() for x in xs])
    mr = 2 if momentum_reuse == 'auto' else int(bool(momentum_reuse))
    prm = _lib.CgbFistaParams(float(tol_fun), float(tol_x), int(max_iter), 0, _lib.ARITH['bf16'], mr)
    res = (_lib.CgbFistaResult * P)()
    st = torch.cuda.current_stream(dev).cuda_stream
    check(lib().cgb_fista_batch_run(A.handle, ctypes.c_void_p(yd.data_ptr()),
                                    ctypes.c_void_p(sw.data_ptr()) if sw is not None else None, regs, P,
                                    ctypes.byref(prm), ptrs, res, ctypes.c_void_p(st)))
    del keep
    out = []
    for p in range(P):
        r = res[p]
        det = {'residual': r.residual, 'regterm': r.regterm, 'cost_function': r.cost_function,
               'abs_cost': r.abs_cost, 'rel_cost': r.rel_cost, 'abs_x': r.abs_x, 'rel_x': r.rel_x,
               'iterations': int(r.iterations), 'stopping_criterion': _lib.CRITERIA[r.stopping_criterion],
               'backtracks': int(r.backtracks), 'anchors': int(r.anchors)}
        if p == 0:
            det['batch_operator_calls'] = int(r.operator_calls)
        out.append((xs[p].cpu().numpy() if host else xs[p], det))
    return out


def solve_batches(jobs, n_streams: int = 4, **kw):
    """Regularisation paths on several operators (e.g. tractograms of uneven size) at once.

    jobs: list of (y, A, regularisations).  Each job runs ``solve_batch`` on a CUDA stream
    from a host thread (the library releases the GIL and allocates stream-ordered), up to
    n_streams at a time, so the device overlaps one job's host decisions and small passes
    with another job's work.  Jobs are taken largest first (segments x problems) from one
    queue by whichever stream is free, so the last jobs to finish are the small ones.
    Returns one list of (x, details) per job, in order."""
    import queue
    import threading
    if not jobs:
        return []
    n_streams = max(1, min(int(n_streams), len(jobs)))
    devs = [torch.device('cuda', A.device) for _, A, _ in jobs]
    streams = [torch.cuda.Stream(device=devs[0]) for _ in range(n_streams)]
    for s in streams:
        s.wait_stream(torch.cuda.current_stream(devs[0]))
    order = sorted(range(len(jobs)), key=lambda k: -(jobs[k][1].ICn * jobs[k][1].ICnRF * max(1, len(jobs[k][2]))))
    todo = queue.Queue()
    for k in order:
        todo.put(k)
    res, errors = {}, []

    def worker(w):
        s = streams[w]
        while True:
            try:
                k = todo.get_nowait()
            except queue.Empty:
                return
            try:
                y, A, regs = jobs[k]
                with torch.cuda.device(devs[k]), torch.cuda.stream(s):
                    res[k] = solve_batch(y, A, regs, **kw)
                s.synchronize()
            except BaseException as e:  # noqa: BLE001 - re-raised on the calling thread
                errors.append(e)
                return

    if n_streams == 1:
        worker(0)
    else:
        threads = [threading.Thread(target=worker, args=(w,)) for w in range(n_streams)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    if errors:
        raise errors[0]
    return [res[k] for k in range(len(jobs))]
