"""The allocation-free A'*y entry point, cgb_op_adjoint_noalloc, through the C ABI.

It exists for callers that cannot let the library call cudaMalloc -- an application
that owns all GPU memory through its own pool, or one that cannot accept cudaMalloc's
device-wide synchronisation on its stream.  Such a caller hands over only its own device
buffers; the entry point's working memory is a fixed static device array.  This test
plays that caller: it places the reference-layout arrays in device buffers itself, calls
the entry point twice in a row (the second call must not see the first call's leftovers
in the shared static array), and compares with the reference's own A' (golden vectors
made by its compiled operator) and with the existing A' (LinearOperator.T.dot).  It also
checks that a call after the first one leaves the device's free memory unchanged, and
runs the entry point on a stream of its own.
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


def _buffers(c):
    D, K = c['D'], c['K']
    IC, EC, ISO = D['IC'], D['EC'], D['ISO']
    nF = IC['nSTR']
    # fibre index: segment indices grouped by fibre (stable), and each fibre's range
    perm = np.argsort(IC['str'], kind='stable').astype(np.uint32)
    ptr = np.concatenate([[0], np.cumsum(np.bincount(IC['str'], minlength=nF))]).astype(np.uint32)
    return dict(ICf=_dev(IC['str'], np.uint32), ICeval=_dev(IC['eval'], np.uint32), ICv=_dev(IC['vox'], np.uint32),
                ICo=_dev(IC['dir'].astype(np.int16), np.int16), ICl=_dev(IC['len'], np.float32),
                ECv=_dev(EC['vox'], np.uint32), ECo=_dev(EC['dir'].astype(np.int16), np.int16),
                ISOv=_dev(ISO['vox'], np.uint32), lutIC=_dev(K['wmr'], np.float32),
                lutEC=_dev(K['wmh'], np.float32), lutISO=_dev(K['iso'], np.float32),
                fib_ptr=_dev(ptr, np.uint32), fib_perm=_dev(perm, np.uint32))


def _launch(L, c, bufs, yd, xd, st):
    D, K = c['D'], c['K']
    IC, EC, ISO = D['IC'], D['EC'], D['ISO']
    nIC, nEC, nISO = K['wmr'].shape[0], K['wmh'].shape[0], K['iso'].shape[0]
    nS, ndirs = K['wmr'].shape[2], K['wmr'].shape[1]
    return L.cgb_op_adjoint_noalloc(nS, ndirs, IC['nSTR'], IC['n'], EC['n'], IC['nVOX'], ISO['n'], _vp(yd), _vp(xd),
                                    _vp(bufs['ICf']), _vp(bufs['ICeval']), _vp(bufs['ICv']), _vp(bufs['ICo']),
                                    _vp(bufs['ICl']), _vp(bufs['ECv']), _vp(bufs['ECo']), _vp(bufs['ISOv']),
                                    _vp(bufs['lutIC']), _vp(bufs['lutEC']), _vp(bufs['lutISO']), nIC, nEC, nISO,
                                    _vp(bufs['fib_ptr']), _vp(bufs['fib_perm']), ctypes.c_void_p(st))


def _ncols(c):
    D, K = c['D'], c['K']
    return D['IC']['nSTR'] * K['wmr'].shape[0] + D['EC']['n'] * K['wmh'].shape[0] + D['ISO']['n'] * K['iso'].shape[0]


def _call(L, c, y, stream=None):
    bufs = _buffers(c)
    yd = torch.from_numpy(np.ascontiguousarray(y)).cuda()
    xd = torch.full((_ncols(c),), np.nan, dtype=torch.float64, device='cuda')
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = _launch(L, c, bufs, yd, xd, st)
    torch.cuda.synchronize()
    return rc, xd.cpu().numpy()


@pytest.mark.parametrize('name', ['szb', 'multi_rf', 'eval_gaps', 'scalar_map'])
def test_adjoint_noalloc_matches_adjoint_twice(name):
    from commit_gb300 import _lib
    from commit_gb300.operator import LinearOperator
    L = _lib.lib()
    c = G.load_case(name)
    A = LinearOperator(c['D'], c['K'], None, arith='ff')
    # the reference's own A' on the golden input, then a second call on another vector
    rc, x = _call(L, c, c['y_in'])
    assert rc == 0, L.cgb_last_error().decode()
    assert G.rel(x, c['Aty']) <= TOL
    assert G.rel(x, A.T.dot(c['y_in'])) <= TOL
    y2 = np.random.default_rng(7).normal(size=A.nROWS) * 3.0
    rc, x2 = _call(L, c, y2)
    assert rc == 0, L.cgb_last_error().decode()
    assert G.rel(x2, A.T.dot(y2)) <= TOL


def test_adjoint_noalloc_allocates_nothing_after_the_first_call():
    """Once the first call on the device has done its set-up, calls leave the device's
    free memory exactly as it was, on the default stream and on a stream of its own."""
    from commit_gb300 import _lib
    L = _lib.lib()
    c = G.load_case('multi_rf')
    bufs = _buffers(c)
    yd = torch.from_numpy(np.ascontiguousarray(c['y_in'])).cuda()
    xd = torch.empty(_ncols(c), dtype=torch.float64, device='cuda')
    side = torch.cuda.Stream()
    assert _launch(L, c, bufs, yd, xd, torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for st in (torch.cuda.current_stream().cuda_stream, side.cuda_stream):
        xd.fill_(np.nan)
        torch.cuda.synchronize()
        assert _launch(L, c, bufs, yd, xd, st) == 0, L.cgb_last_error().decode()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        assert G.rel(xd.cpu().numpy(), c['Aty']) <= TOL


def test_adjoint_noalloc_setup_call():
    """A call whose sizes are all zero does only the per-device set-up and succeeds."""
    from commit_gb300 import _lib
    L = _lib.lib()
    y = torch.zeros(1, dtype=torch.float64, device='cuda')
    rc = L.cgb_op_adjoint_noalloc(1, 1, 0, 0, 0, 0, 0, _vp(y), None, None, None, None, None, None, None, None,
                                  None, None, None, None, 0, 0, 0, None, None, None)
    assert rc == 0, L.cgb_last_error().decode()


def test_adjoint_noalloc_rejects_sizes_beyond_its_scratch():
    from commit_gb300 import _lib
    L = _lib.lib()
    big = _lib.lib().cgb_op_adjoint_noalloc
    n = (1 << 20) + 1
    rc = big(1, 1, 1, n, 0, 1, 0, ctypes.c_void_p(8), ctypes.c_void_p(8), None, None, None, None, None, None, None,
             None, None, None, None, 1, 0, 0, None, None, None)
    assert rc == _lib.CGB_ERR_UNSUPPORTED
    assert b'exceeds its static scratch' in L.cgb_last_error()
