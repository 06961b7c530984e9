"""Differentiation through the operator: loss = 1/2|A x - y|^2 + lambda |x|_1, lambda = 1e-3.

Gradients with respect to x and to the IC / EC / ISO LUT entries are checked against FP64
central finite differences (h = 1e-6) on 64 random coordinates each, evaluated with the
oracle (the reference operator restated in C, FP64 accumulation), and the adjoint used for
dLoss/dx is checked against the oracle's A' by the dot test <Ax, y> = <x, A'y>.
"""
import numpy as np
import pytest
import torch

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu

LAM = 1e-3
H = 1e-6


def _problem():
    from commit_gb300 import synth
    D, K = synth.make_dictionary(synth.scaled_spec('demo_5k', n_fibers=50000))
    D['IC']['eval'] = np.ones(D['IC']['nSTR'], np.uint32)
    P = O.PortOperator(D, K, None, nthreads=8)
    x = synth.make_x(P.nCOLS, 1) * 0.5
    y = synth.make_signal(P.dot(synth.make_x(P.nCOLS, 11)), 2)
    return D, K, P, x, y


def _loss_fp64(P, x, y):
    r = P.dot(x) - y
    return 0.5 * float(np.dot(r, r)) + LAM * float(np.abs(x).sum())


def test_gradients_against_central_differences():
    from commit_gb300.autograd import commit_apply
    from commit_gb300.operator import LinearOperator
    D, K, P, x, y = _problem()
    A = LinearOperator(D, K, None)
    xt = torch.from_numpy(x).cuda().requires_grad_(True)
    luts = [torch.from_numpy(K[k]).cuda().requires_grad_(True) for k in ('wmr', 'wmh', 'iso')]
    yt = torch.from_numpy(y).cuda()
    pred = commit_apply(A, xt, *luts)
    loss = 0.5 * ((pred - yt) ** 2).sum() + LAM * xt.abs().sum()
    loss.backward()
    gx = xt.grad.cpu().numpy()
    gl = [t.grad.double().cpu().numpy() for t in luts]
    rng = np.random.default_rng(0)
    # dLoss/dx: central differences of the FP64 oracle loss
    for k in rng.choice(x.size, size=64, replace=False):
        xp, xm = x.copy(), x.copy()
        xp[k] += H
        xm[k] -= H
        lp, lm = _loss_fp64(P, xp, y), _loss_fp64(P, xm, y)
        fd = (lp - lm) / (2 * H)
        fd_err = 8 * np.finfo(float).eps * max(lp, lm) / (2 * H)
        assert abs(gx[k] - fd) <= 4 * fd_err + 1e-7 * abs(fd), (k, gx[k], fd, fd_err)
    # dLoss/dLUT: y is linear in a LUT entry, so loss(theta +- h) follows from r and the
    # entry's column of coefficients; evaluate it in FP64 and difference centrally
    r = P.dot(x) - y
    nS = K['wmr'].shape[2]
    IC = D['IC']
    coef_ic = IC['len'].astype(np.float64) * x[IC['str']]
    ecv, eco = D['EC']['vox'], D['EC']['dir']
    base_ec = IC['nSTR']
    for which, grad in (('wmr', gl[0]), ('wmh', gl[1]), ('iso', gl[2])):
        for _ in range(64 if which != 'iso' else 16):
            s = int(rng.integers(nS))
            d = np.zeros_like(r)
            if which == 'iso':
                i = int(rng.integers(K['iso'].shape[0]))
                xi = x[base_ec + D['EC']['n'] + i * D['ISO']['n']: base_ec + D['EC']['n'] + (i + 1) * D['ISO']['n']]
                np.add.at(d, D['ISO']['vox'].astype(np.int64) * nS + s, xi)
                g_kernel = grad[i, s]
            elif which == 'wmr':
                o = int(rng.choice(IC['dir']))
                sel = IC['dir'] == o
                np.add.at(d, IC['vox'][sel].astype(np.int64) * nS + s, coef_ic[sel])
                g_kernel = grad[0, o, s]
            else:
                o = int(rng.choice(eco))
                sel = eco == o
                np.add.at(d, ecv[sel].astype(np.int64) * nS + s, x[base_ec + np.flatnonzero(sel)])
                g_kernel = grad[0, o, s]
            lp = 0.5 * float(np.dot(r + H * d, r + H * d))
            lm = 0.5 * float(np.dot(r - H * d, r - H * d))
            fd = (lp - lm) / (2 * H)
            # the difference quotient itself is accurate to about eps * loss / h
            fd_err = 8 * np.finfo(float).eps * max(lp, lm) / (2 * H)
            assert abs(g_kernel - fd) <= 4 * fd_err + 1e-7 * abs(fd), (which, g_kernel, fd, fd_err)


def test_adjoint_dot_test_against_oracle():
    from commit_gb300.operator import LinearOperator
    D, K, P, x, y = _problem()
    A = LinearOperator(D, K, None)
    rng = np.random.default_rng(1)
    u = rng.normal(size=P.nCOLS)
    w = rng.normal(size=P.nROWS)
    lhs = float(np.dot(P.dot(u), w))
    rhs = float(np.dot(u, A.T.dot(w)))
    assert abs(lhs - rhs) <= 1e-11 * max(1.0, abs(lhs))
    assert G.rel(A.T.dot(w), P.T.dot(w)) <= 1e-10


def test_set_lut_changes_the_operator():
    from commit_gb300.autograd import commit_apply
    from commit_gb300.operator import LinearOperator
    c = G.load_case('szb')
    A = LinearOperator(c['D'], c['K'], None)
    K2 = {k: v.copy() for k, v in c['K'].items()}
    K2['wmr'] *= np.float32(1.5)
    P2 = O.PortOperator(c['D'], K2, None)
    x = torch.from_numpy(c['x_in']).cuda()
    y = commit_apply(A, x, torch.from_numpy(K2['wmr']).cuda(), None, None)
    assert G.rel(y.cpu().numpy(), P2.dot(c['x_in'])) <= 1e-10
