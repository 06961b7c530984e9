"""GB300 drop-in for commit/proximals.pyx:13-186.

Same names and arguments as the reference.  Each map works in place and returns the
array: on a CUDA float64 tensor it runs on the tensor's device and torch's current
stream; on a numpy array the data is copied to the GPU, transformed there, and written
back into the array.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import check, lib


def _stream(t: torch.Tensor):
    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _as_device(x):
    """(device tensor, numpy array to write back or None)."""
    if isinstance(x, torch.Tensor):
        if not x.is_cuda or x.dtype != torch.float64 or not x.is_contiguous():
            raise TypeError('expected a contiguous CUDA float64 tensor')
        return x, None
    arr = np.asarray(x)
    if arr.dtype != np.float64:
        raise TypeError('expected a float64 array')
    return torch.from_numpy(np.ascontiguousarray(arr)).to('cuda'), arr


def _finish(t, host):
    if host is None:
        return t
    host[...] = t.cpu().numpy()
    return np.asarray(host)


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _range(n, start, size):
    a = max(0, int(start))
    b = min(n, int(start) + int(size))
    return a, max(0, b - a)


def non_negativity(x, compartment_start, compartment_size):
    """proximals.pyx:13-22."""
    t, h = _as_device(x)
    a, n = _range(t.numel(), compartment_start, compartment_size)
    check(lib().cgb_prox_non_negativity(_vp(t), a, n, _stream(t)))
    return _finish(t, h)


def soft_thresholding(x, lam, compartment_start, compartment_size):
    """proximals.pyx:25-39."""
    t, h = _as_device(x)
    a, n = _range(t.numel(), compartment_start, compartment_size)
    check(lib().cgb_prox_soft_thresholding(_vp(t), float(lam), a, n, _stream(t)))
    return _finish(t, h)


def w_soft_thresholding(x, w, lam, compartment_start, compartment_size):
    """proximals.pyx:42-56."""
    t, h = _as_device(x)
    wt = w if isinstance(w, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(w, dtype=np.float64)).to(t.device)
    a, n = _range(t.numel(), compartment_start, compartment_size)
    check(lib().cgb_prox_w_soft_thresholding(_vp(t), _vp(wt), float(lam), a, n, _stream(t)))
    return _finish(t, h)


def projection_onto_l2_ball(x, lam, compartment_start, compartment_size):
    """proximals.pyx:59-77."""
    t, h = _as_device(x)
    a, n = _range(t.numel(), compartment_start, compartment_size)
    check(lib().cgb_prox_projection_onto_l2_ball(_vp(t), float(lam), a, n, _stream(t)))
    return _finish(t, h)


def _groups_from_flat(group_idx, group_size):
    gi = np.asarray(group_idx, dtype=np.int64)
    gs = np.asarray(group_size, dtype=np.int64)
    return np.split(gi, np.cumsum(gs)[:-1]) if gs.size else []


class _GroupArrays:
    def __init__(self, groups, weights, device):
        from .solvers import level_schedule
        order, level_ptr = level_schedule(groups)
        og = [groups[k] for k in order]
        sizes = np.array([g.size for g in og], dtype=np.int64)
        self.gidx = torch.as_tensor(np.concatenate(og).astype(np.int32) if og else np.zeros(1, np.int32)).to(device)
        self.gptr = torch.as_tensor(np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)).to(device)
        self.gw = torch.as_tensor(np.asarray(weights, dtype=np.float64)[order] if len(groups) else np.zeros(1)).to(device)
        self.level_ptr = np.ascontiguousarray(level_ptr, dtype=np.int64)
        self.n = len(groups)


def omega_group_lasso(x, group_idx, group_size, group_weight, lam):
    """proximals.pyx:80-99."""
    t, _ = _as_device(x)
    G = _GroupArrays(_groups_from_flat(group_idx, group_size), group_weight, t.device)
    out = ctypes.c_double()
    check(lib().cgb_omega_group_lasso(_vp(t), t.numel(), _vp(G.gidx), _vp(G.gptr), _vp(G.gw), G.n, float(lam),
                                      ctypes.byref(out), _stream(t)))
    return out.value


def prox_group_lasso(x, group_idx, group_size, group_weight, lam):
    """proximals.pyx:103-134 (groups in order; overlapping groups via a level schedule)."""
    t, h = _as_device(x)
    G = _GroupArrays(_groups_from_flat(group_idx, group_size), group_weight, t.device)
    check(lib().cgb_prox_group_lasso(_vp(t), t.numel(), _vp(G.gidx), _vp(G.gptr), _vp(G.gw), G.n,
                                     G.level_ptr.ctypes.data_as(ctypes.c_void_p), G.level_ptr.size - 1, float(lam),
                                     _stream(t)))
    return _finish(t, h)


def omega_sparse_group_lasso(x, group_idx, group_size, group_weight, lam1, lam2):
    """proximals.pyx:138-159 (l1 part over the whole vector)."""
    t, _ = _as_device(x)
    G = _GroupArrays(_groups_from_flat(group_idx, group_size), group_weight, t.device)
    out = ctypes.c_double()
    check(lib().cgb_omega_sparse_group_lasso(_vp(t), t.numel(), None, _vp(G.gidx), _vp(G.gptr), _vp(G.gw), G.n,
                                             float(lam1), float(lam2), ctypes.byref(out), _stream(t)))
    return out.value


def omega_w_sparse_group_lasso(x, w, group_idx, group_size, group_weight, lam1, lam2):
    """proximals.pyx:162-186 (weighted l1 part over the whole vector)."""
    t, _ = _as_device(x)
    wt = w if isinstance(w, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(w, dtype=np.float64)).to(t.device)
    G = _GroupArrays(_groups_from_flat(group_idx, group_size), group_weight, t.device)
    out = ctypes.c_double()
    check(lib().cgb_omega_sparse_group_lasso(_vp(t), t.numel(), _vp(wt), _vp(G.gidx), _vp(G.gptr), _vp(G.gw), G.n,
                                             float(lam1), float(lam2), ctypes.byref(out), _stream(t)))
    return out.value


# ------------------------------------------------------------------ helpers for solvers.py
def _l1(t, w, start, size) -> float:
    if size <= 0:
        return 0.0
    out = ctypes.c_double()
    check(lib().cgb_omega_l1(_vp(t), _vp(w) if w is not None else None, int(start), int(size), 1.0,
                             ctypes.byref(out), _stream(t)))
    return out.value


def _omega_groups(t, spec, lam, force=False) -> float:
    if lam == 0 and not force:
        return 0.0
    d = spec.device_arrays(t.device)
    out = ctypes.c_double()
    check(lib().cgb_omega_group_lasso(_vp(t), t.numel(), _vp(d['gidx']), _vp(d['gptr']), _vp(d['gw']), len(spec.groups), 1.0,
                                      ctypes.byref(out), _stream(t)))
    return lam * out.value


def _apply_spec(x, spec, s):
    """prox of an init_regularisation spec: proxIC(proxEC(proxISO(x, s), s), s)."""
    t, h = _as_device(x)
    st = _stream(t)
    d = spec.device_arrays(t.device)
    L = lib()
    # ISO
    if spec.reg_iso == 'lasso':
        if spec.weighted_iso:
            check(L.cgb_prox_w_soft_thresholding(_vp(t), _vp(d['acw']), s * spec.lam_iso, spec.sISO, spec.nISO, st))
        else:
            check(L.cgb_prox_soft_thresholding(_vp(t), s * spec.lam_iso, spec.sISO, spec.nISO, st))
    if spec.nn_iso:
        check(L.cgb_prox_non_negativity(_vp(t), spec.sISO, spec.nISO, st))
    # EC
    if spec.reg_ec == 'lasso':
        check(L.cgb_prox_soft_thresholding(_vp(t), s * spec.lam_ec, spec.sEC, spec.nEC, st))
    if spec.nn_ec:
        check(L.cgb_prox_non_negativity(_vp(t), spec.sEC, spec.nEC, st))
    # IC
    if spec.reg_ic in ('lasso', 'sparse_group_lasso'):
        if spec.weighted_ic:
            check(L.cgb_prox_w_soft_thresholding(_vp(t), _vp(d['acw']), s * spec.lam_ic, spec.sIC, spec.nIC, st))
        else:
            check(L.cgb_prox_soft_thresholding(_vp(t), s * spec.lam_ic, spec.sIC, spec.nIC, st))
    if spec.reg_ic in ('group_lasso', 'sparse_group_lasso'):
        lam = s * (spec.lam_ic if spec.reg_ic == 'group_lasso' else spec.lam_ic_group)
        lp = spec.level_ptr
        check(L.cgb_prox_group_lasso(_vp(t), t.numel(), _vp(d['gidx']), _vp(d['gptr']), _vp(d['gw']), len(spec.groups),
                                     lp.ctypes.data_as(ctypes.c_void_p), lp.size - 1, lam, st))
    if spec.nn_ic:
        check(L.cgb_prox_non_negativity(_vp(t), spec.sIC, spec.nIC, st))
    return _finish(t, h)
