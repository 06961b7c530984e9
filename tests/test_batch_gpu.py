"""Multi-right-hand-side operator passes and the batched FISTA driver.

The multi-vector BF16 kernels must give, vector by vector, what the single-vector BF16
kernels give (same LUT rounding, FP32 accumulation; only the summation grouping differs) and
stay within the BF16 bound of the FP64 oracle.  The batched solver runs each problem's
FISTA (commit/solvers.py:244-391) with its own step size, backtracking and stopping test:
its solutions must track sequential single-problem BF16 solves and the FP64 solution.
"""
import numpy as np
import pytest
import torch

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu


def _demo(nS_spec='demo_5k', **kw):
    from commit_gb300 import synth
    D, K = synth.make_dictionary(synth.scaled_spec(nS_spec, **kw))
    P = O.PortOperator(D, K, None, nthreads=8)
    y = synth.make_signal(P.dot(synth.make_x(P.nCOLS, 1)), 2)
    return D, K, P, y


@pytest.mark.parametrize('width', [2, 4])
@pytest.mark.parametrize('nvec', [1, 2, 3, 5, 8])
def test_dot_batch_matches_single_vector(nvec, width):
    from commit_gb300.operator import LinearOperator
    D, K, P, _ = _demo()
    A = LinearOperator(D, K, None)
    A.tensor_cores(1)  # the batched passes are CUDA-core BF16: compare with the same single-vector kernels
    A.batch_width(width)
    rng = np.random.default_rng(nvec)
    xs32 = [torch.from_numpy(rng.uniform(0, 1, P.nCOLS).astype(np.float32)).cuda() for _ in range(nvec)]
    ys = A.dot_batch([x.double() for x in xs32])
    for x32, yb in zip(xs32, ys):
        ysingle = A.dot(x32, arith='bf16')
        assert G.rel(yb.cpu().numpy(), ysingle.cpu().numpy()) <= 1e-5
        assert G.rel(yb.cpu().numpy(), P.dot(x32.double().cpu().numpy())) <= 1.5e-2
    ws32 = [torch.from_numpy(rng.normal(size=P.nROWS).astype(np.float32)).cuda() for _ in range(nvec)]
    xs = A.T.dot_batch(ws32)
    for w32, xb in zip(ws32, xs):
        xsingle = A.T.dot(w32, arith='bf16')
        assert G.rel(xb.cpu().numpy(), xsingle.double().cpu().numpy()) <= 1e-5
        assert G.rel(xb.cpu().numpy(), P.T.dot(w32.double().cpu().numpy())) <= 1.5e-2


def test_dot_batch_full_acquisition():
    """nS = 288 (18 b0 + 3 shells x 90 directions), the batched workload's acquisition."""
    from commit_gb300.operator import LinearOperator
    D, K, P, _ = _demo('demo_5k', n_b0=18, shells=[(1000.0, 90), (2000.0, 90), (3000.0, 90)], n_fibers=2000)
    A = LinearOperator(D, K, None)
    rng = np.random.default_rng(3)
    xs = [torch.from_numpy(rng.uniform(0, 1, P.nCOLS)).cuda() for _ in range(4)]
    for x, yb in zip(xs, A.dot_batch(xs)):
        assert G.rel(yb.cpu().numpy(), P.dot(x.cpu().numpy())) <= 1.5e-2
    ws = [torch.from_numpy(rng.normal(size=P.nROWS).astype(np.float32)).cuda() for _ in range(3)]
    for w, xb in zip(ws, A.T.dot_batch(ws)):
        assert G.rel(xb.cpu().numpy(), P.T.dot(w.double().cpu().numpy())) <= 1.5e-2


def _path_regs(A, D, K, y, fracs, ngroups=8):
    from commit_gb300 import evaluation, synth
    groups = synth.bundle_groups(D['IC']['nSTR'], ngroups, seed=5)
    regs = []
    for f in fracs:
        regs.append(evaluation.set_regularisation(
            A, y, D, K, regularisers=('group_lasso', None, None), lambdas=(f, None, None),
            is_nonnegative=(True, True, True),
            params=({'group_idx': groups, 'group_weights_cardinality': True, 'group_weights_adaptive': False},
                    None, None)))
    return regs


@pytest.mark.parametrize('reuse', [True, False])
def test_batched_path_tracks_sequential_solves(reuse):
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    D, K, P, y = _demo()
    A = LinearOperator(D, K, None)
    A.tensor_cores(1)  # the batched passes are CUDA-core BF16: compare with the same single-vector kernels
    fracs = [1e-4, 1e-3, 3e-3, 1e-2, 3e-2]   # 5 problems: a 4-vector pass and a single one
    regs = _path_regs(A, D, K, y, fracs)
    out = solvers.solve_batch(y, A, regs, tol_fun=1e-5, tol_x=1e-7, max_iter=150, momentum_reuse=reuse)
    assert len(out) == len(fracs)
    for (xb, db), rp in zip(out, regs):
        xs, ds = solvers.solve(y, A, A.T, tol_fun=1e-5, tol_x=1e-7, max_iter=150, verbose=0, regularisation=rp,
                               arith='bf16', momentum_reuse=reuse)
        assert abs(db['iterations'] - ds['iterations']) <= max(3, ds['iterations'] // 20), (db, ds)
        assert G.rel(xb, xs) <= 2e-3
        assert abs(db['cost_function'] - ds['cost_function']) <= 1e-4 * ds['cost_function']
        # against the FP64 solver: within the BF16 operator's accuracy
        xf, df = solvers.solve(y, A, A.T, tol_fun=1e-5, tol_x=1e-7, max_iter=150, verbose=0, regularisation=rp,
                               arith='ff')
        assert G.rel(xb, xf) <= 5e-2
        assert abs(db['cost_function'] - df['cost_function']) <= 1e-2 * df['cost_function']
    # stronger regularisation gives a lower data fit and no larger group support
    costs = [d['residual'] for _, d in out]
    assert costs[-1] >= costs[0]


def test_batch_widths_agree_and_problems_stop_independently():
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    D, K, P, y = _demo()
    A = LinearOperator(D, K, None)
    regs = _path_regs(A, D, K, y, [1e-4, 1e-2, 5e-2, 1e-1])
    res = {}
    for w in (2, 4):
        A.batch_width(w)
        res[w] = solvers.solve_batch(y, A, regs, tol_fun=1e-4, tol_x=1e-6, max_iter=300)
    for (x2, d2), (x4, d4) in zip(res[2], res[4]):
        assert abs(d2['iterations'] - d4['iterations']) <= 3
        assert G.rel(x2, x4) <= 2e-3
    its = [d['iterations'] for _, d in res[4]]
    assert len(set(its)) > 1, its          # each problem has its own stopping point
    A.batch_width(0)
    solvers.solve_batch(y, A, regs, tol_fun=1e-4, tol_x=1e-6, max_iter=5)
    assert A.batch_width() in (2, 4)        # tuned on the first batched solve


def test_batch_rejects_bad_arguments():
    import ctypes
    from commit_gb300 import _lib, solvers
    from commit_gb300.operator import LinearOperator
    c = G.load_case('szb')
    A = LinearOperator(c['D'], c['K'], None)
    assert solvers.solve_batch(c['y_obs'], A, []) == []
    with pytest.raises(RuntimeError):
        solvers.solve_batch(c['y_obs'][:-1], A, [None])
    with pytest.raises(_lib.CgbError):
        A.batch_width(3)
    y = torch.from_numpy(c['y_obs']).cuda()
    x = torch.zeros(A.nCOLS, dtype=torch.float64, device='cuda')
    reg, keep = solvers._no_reg_spec(A.nCOLS).cstruct(x.device)
    prm = _lib.CgbFistaParams(1e-4, 1e-6, 10, 0, _lib.ARITH['ff'], 1)
    res = (_lib.CgbFistaResult * 1)()
    ptrs = (ctypes.c_void_p * 1)(x.data_ptr())
    rc = _lib.lib().cgb_fista_batch_run(A.handle, ctypes.c_void_p(y.data_ptr()), None, ctypes.byref(reg), 1,
                                        ctypes.byref(prm), ptrs, res, None)
    assert rc == _lib.CGB_ERR_UNSUPPORTED


def test_concurrent_paths_match_one_at_a_time():
    """solve_batches runs each operator's path on its own stream and thread; with the
    width and momentum reuse fixed the results are bitwise those of solve_batch."""
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    jobs = []
    for seed in (21, 22, 23):
        D, K = synth.make_dictionary(synth.scaled_spec('demo_5k', seed=seed, n_fibers=3000))
        P = O.PortOperator(D, K, None, nthreads=8)
        y = synth.make_signal(P.dot(synth.make_x(P.nCOLS, 1)), 2)
        A = LinearOperator(D, K, None)
        A.batch_width(2)
        jobs.append((y, A, _path_regs(A, D, K, y, [1e-4, 1e-3, 1e-2])))
    kw = dict(tol_fun=1e-5, tol_x=1e-7, max_iter=60, momentum_reuse=True)
    seq = [solvers.solve_batch(y, A, regs, **kw) for y, A, regs in jobs]
    con = solvers.solve_batches(jobs, n_streams=3, **kw)
    for a, b in zip(seq, con):
        for (x1, d1), (x2, d2) in zip(a, b):
            assert d1['iterations'] == d2['iterations']
            assert np.array_equal(x1, x2)


def test_batched_path_with_adjoint_slabs_is_bitwise_unchanged():
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    D, K, P, y = _demo()
    A = LinearOperator(D, K, None)
    A.batch_width(2)
    regs = _path_regs(A, D, K, y, [1e-4, 1e-3, 1e-2])
    out = {}
    for s in (1, 4):
        assert A.set_slabs(s) == s
        out[s] = solvers.solve_batch(y, A, regs, tol_fun=1e-5, tol_x=1e-7, max_iter=40, momentum_reuse=False)
    for (x1, d1), (x4, d4) in zip(out[1], out[4]):
        assert d1['iterations'] == d4['iterations']
        assert np.array_equal(x1, x4)


@pytest.mark.parametrize('shape', [1, 2])
def test_batch_voxel_shapes_agree(shape):
    """Both voxel shapes of the multi-vector kernels (the single-vector kernels' lanes per
    voxel, a warp per voxel) give the same products to FP32 summation-order accuracy."""
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    D, K, P, y = _demo('demo_5k', n_b0=18, shells=[(1000.0, 90), (2000.0, 90), (3000.0, 90)], n_fibers=2000)
    A = LinearOperator(D, K, None)
    A.tensor_cores(1)  # the batched passes are CUDA-core BF16: compare with the same single-vector kernels
    A.batch_width(4)
    A.batch_shape(shape)
    rng = np.random.default_rng(8)
    xs = [torch.from_numpy(rng.uniform(0, 1, P.nCOLS)).cuda() for _ in range(4)]
    for x, yb in zip(xs, A.dot_batch(xs)):
        assert G.rel(yb.cpu().numpy(), P.dot(x.cpu().numpy())) <= 1.5e-2
    ws = [torch.from_numpy(rng.normal(size=P.nROWS).astype(np.float32)).cuda() for _ in range(4)]
    for w, xb in zip(ws, A.T.dot_batch(ws)):
        xsingle = A.T.dot(w, arith='bf16')
        assert G.rel(xb.cpu().numpy(), xsingle.double().cpu().numpy()) <= 1e-5
    regs = _path_regs(A, D, K, y, [1e-4, 1e-2])
    out = solvers.solve_batch(y, A, regs, tol_fun=1e-5, tol_x=1e-7, max_iter=60, momentum_reuse=False)
    for (xb, db), rp in zip(out, regs):
        xs1, ds1 = solvers.solve(y, A, A.T, tol_fun=1e-5, tol_x=1e-7, max_iter=60, verbose=0, regularisation=rp,
                                 arith='bf16', momentum_reuse=False)
        assert G.rel(xb, xs1) <= 2e-3
    assert A.batch_shape() == shape


def test_batch_single_and_three_problems():
    """One problem (single-vector kernels) and three (a 4-vector pass with an idle slot)
    match sequential BF16 solves."""
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    D, K, P, y = _demo()
    A = LinearOperator(D, K, None)
    A.tensor_cores(1)  # the batched passes are CUDA-core BF16: compare with the same single-vector kernels
    A.batch_width(4)
    for fr in ([1e-3], [1e-4, 1e-3, 1e-2]):
        regs = _path_regs(A, D, K, y, fr)
        out = solvers.solve_batch(y, A, regs, tol_fun=1e-5, tol_x=1e-7, max_iter=50, momentum_reuse=False)
        for (xb, db), rp in zip(out, regs):
            xs1, ds1 = solvers.solve(y, A, A.T, tol_fun=1e-5, tol_x=1e-7, max_iter=50, verbose=0, regularisation=rp,
                                     arith='bf16', momentum_reuse=False)
            assert G.rel(xb, xs1) <= 2e-3
            assert abs(db['iterations'] - ds1['iterations']) <= 3
