"""The allocation-free A'*y entry point, cgb_op_adjoint_noalloc, through the C ABI.

It exists for callers that cannot let the library call cudaMalloc -- an application
that owns all GPU memory through its own pool, or one that cannot accept cudaMalloc's
device-wide synchronisation on its stream.  Such a caller hands over only its own device
buffers; the entry point's working memory is a fixed static device array.  This test
plays that caller: it places the reference-layout arrays in device buffers itself, calls
the entry point twice in a row (the second call must not see the first call's leftovers
in the shared static array), and compares with the existing A' (LinearOperator.T.dot).
"""
import ctypes

import numpy as np
import pytest
import torch

import golden_io as G

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _dev(a, dtype):
    a = np.ascontiguousarray(a)
    if a.size == 0:
        a = np.zeros(1, dtype=a.dtype)
    return torch.from_numpy(a.astype(dtype, copy=False)).cuda()


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _call(L, c, y, stream=None):
    D, K = c['D'], c['K']
    IC, EC, ISO = D['IC'], D['EC'], D['ISO']
    nIC, nEC, nISO = K['wmr'].shape[0], K['wmh'].shape[0], K['iso'].shape[0]
    nS, ndirs = K['wmr'].shape[2], K['wmr'].shape[1]
    nF, n = IC['nSTR'], IC['n']
    # fibre index: segment indices grouped by fibre (stable), and each fibre's range
    perm = np.argsort(IC['str'], kind='stable').astype(np.uint32)
    ptr = np.concatenate([[0], np.cumsum(np.bincount(IC['str'], minlength=nF))]).astype(np.uint32)
    bufs = dict(ICf=_dev(IC['str'], np.uint32), ICeval=_dev(IC['eval'], np.uint32), ICv=_dev(IC['vox'], np.uint32),
                ICo=_dev(IC['dir'].astype(np.int16), np.int16), ICl=_dev(IC['len'], np.float32),
                ECv=_dev(EC['vox'], np.uint32), ECo=_dev(EC['dir'].astype(np.int16), np.int16),
                ISOv=_dev(ISO['vox'], np.uint32), lutIC=_dev(K['wmr'], np.float32),
                lutEC=_dev(K['wmh'], np.float32), lutISO=_dev(K['iso'], np.float32),
                fib_ptr=_dev(ptr, np.uint32), fib_perm=_dev(perm, np.uint32))
    ncols = nF * nIC + EC['n'] * nEC + ISO['n'] * nISO
    yd = torch.from_numpy(np.ascontiguousarray(y)).cuda()
    xd = torch.full((ncols,), np.nan, dtype=torch.float64, device='cuda')
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = L.cgb_op_adjoint_noalloc(nS, ndirs, nF, n, EC['n'], IC['nVOX'], ISO['n'], _vp(yd), _vp(xd),
                                  _vp(bufs['ICf']), _vp(bufs['ICeval']), _vp(bufs['ICv']), _vp(bufs['ICo']),
                                  _vp(bufs['ICl']), _vp(bufs['ECv']), _vp(bufs['ECo']), _vp(bufs['ISOv']),
                                  _vp(bufs['lutIC']), _vp(bufs['lutEC']), _vp(bufs['lutISO']), nIC, nEC, nISO,
                                  _vp(bufs['fib_ptr']), _vp(bufs['fib_perm']), ctypes.c_void_p(st))
    torch.cuda.synchronize()
    return rc, xd.cpu().numpy()


@pytest.mark.parametrize('name', ['szb', 'multi_rf', 'eval_gaps', 'scalar_map'])
def test_adjoint_noalloc_matches_adjoint_twice(name):
    from commit_gb300 import _lib
    from commit_gb300.operator import LinearOperator
    L = _lib.lib()
    c = G.load_case(name)
    A = LinearOperator(c['D'], c['K'], None, arith='ff')
    rng = np.random.default_rng(7)
    for y in (c['y_in'], rng.normal(size=A.nROWS) * 3.0):
        rc, x = _call(L, c, y)
        assert rc == 0, L.cgb_last_error().decode()
        assert G.rel(x, A.T.dot(y)) <= TOL


def test_adjoint_noalloc_rejects_sizes_beyond_its_scratch():
    from commit_gb300 import _lib
    L = _lib.lib()
    big = _lib.lib().cgb_op_adjoint_noalloc
    n = (1 << 20) + 1
    rc = big(1, 1, 1, n, 0, 1, 0, ctypes.c_void_p(8), ctypes.c_void_p(8), None, None, None, None, None, None, None,
             None, None, None, None, 1, 0, 0, None, None, None)
    assert rc == _lib.CGB_ERR_UNSUPPORTED
    assert b'exceeds its static scratch' in L.cgb_last_error()
