"""Parity of the GPU FISTA solver with the reference solvers.solve (golden fixtures).

Acceptance follows the reference's own test (tests/test_demo.py:120-141): identical
iteration count and stopping criterion, fit details within 1e-4; plus x within 1e-8
relative of the reference solution.
"""
import numpy as np
import pytest

import golden_io as G

pytestmark = pytest.mark.gpu


def _fit_cases():
    out = []
    for name in G.case_names():
        c = G.load_case(name)
        for v in c['fits']:
            out.append((name, v))
    return out


def _solve(c, f, arith, reuse):
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    A = LinearOperator(c['D'], c['K'], None, nolut=c['nolut'], arith=arith)
    reg = solvers.init_regularisation(G.fresh_reg(f['reg']))
    return solvers.solve(c['y_obs'], A, A.T, tol_fun=1e-5, tol_x=1e-7, max_iter=f['details']['iterations'],
                         verbose=0, regularisation=reg, confidence_array=f['conf'], arith=arith,
                         momentum_reuse=reuse)


@pytest.mark.parametrize('name,variant', _fit_cases())
def test_fista_matches_reference(name, variant):
    c = G.load_case(name)
    f = c['fits'][variant]
    x, det = _solve(c, f, 'ff', True)
    ref = f['details']
    assert det['iterations'] == ref['iterations']
    assert det['stopping_criterion'] == ref['stopping_criterion']
    assert G.rel(x, f['x']) <= 1e-8
    for k in ('residual', 'regterm', 'cost_function', 'abs_cost', 'rel_cost', 'abs_x', 'rel_x'):
        assert abs(det[k] - ref[k]) <= 1e-4 * max(1.0, abs(ref[k])), k


@pytest.mark.parametrize('arith,reuse', [('f64', False), ('ff', False), ('f64', True)])
@pytest.mark.parametrize('variant', ['nnls', 'lasso_ic_nn', 'group_lasso_hier', 'nnls_confidence'])
def test_fista_variants_of_arithmetic(variant, arith, reuse):
    c = G.load_case('szb')
    f = c['fits'][variant]
    x, det = _solve(c, f, arith, reuse)
    assert det['iterations'] == f['details']['iterations']
    assert G.rel(x, f['x']) <= 1e-8


def test_fista_demo_scale_against_oracle():
    """200 nnls iterations on the 5k-streamline demo workload vs the numpy/C oracle."""
    import oracle as O
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.SPECS['demo_5k'])
    P = O.PortOperator(D, K, None, nthreads=8)
    y = synth.make_signal(P.dot(synth.make_x(P.nCOLS, 1)), 2)
    rp = O.reg_params(D, K)
    xo, do = O.solve(y, P, P.T, tol_fun=1e-12, tol_x=1e-12, max_iter=200, verbose=0,
                     regularisation=O.init_regularisation(dict(rp)))
    A = LinearOperator(D, K, None)
    xg, dg = solvers.solve(y, A, A.T, tol_fun=1e-12, tol_x=1e-12, max_iter=200, verbose=0,
                           regularisation=solvers.init_regularisation(dict(rp)))
    assert dg['iterations'] == do['iterations'] == 200
    assert G.rel(xg, xo) <= 1e-8
    assert abs(dg['cost_function'] - do['cost_function']) <= 1e-8 * do['cost_function']


@pytest.mark.parametrize('arith,tol', [('bf16', 5e-2), ('fp16', 1e-2), ('f32', 1e-4)])
def test_mixed_fista_and_refinement(arith, tol):
    """Reduced-precision FISTA tracks the FP64 iterates to its operator's accuracy, and the
    FP64 refinement from its solution reaches a lower objective than FP64 FISTA alone with
    the same FP64 iteration budget."""
    import oracle as O
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.SPECS['demo_5k'])
    A = LinearOperator(D, K, None)
    P = O.PortOperator(D, K, None, nthreads=8)
    y = synth.make_signal(P.dot(synth.make_x(P.nCOLS, 1)), 2)
    rp = O.reg_params(D, K)
    reg = lambda: solvers.init_regularisation(dict(rp))  # noqa: E731
    n1, n2 = 400, 200
    x_plain, d_plain = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=n1, verbose=0, regularisation=reg())
    x_mix, d_mix = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=n1, verbose=0, regularisation=reg(),
                                 arith=arith)
    assert d_mix['iterations'] == n1
    assert G.rel(x_mix, x_plain) <= tol
    x_ref, d_ref = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=n2, verbose=0, regularisation=reg())
    xm, dm = solvers.solve_mixed(y, A, tol_fun=0.0, tol_x=0.0, max_iter=n1, verbose=0, regularisation=reg(),
                                 arith=arith, refine_max_iter=n2)
    assert dm['iterations'] == n1 + n2
    assert dm['cost_function'] <= d_ref['cost_function'] * (1 + 1e-9)


@pytest.mark.parametrize('reuse', [False, True])
@pytest.mark.parametrize('name,variant', [(n, v) for n, v in _fit_cases() if n in ('szb', 'multi_rf', 'eval_gaps')])
def test_graph_mode_matches_host_loop(name, variant, reuse):
    """The iteration loop as one CUDA graph (device-side backtracking and stopping; with
    momentum reuse, A x_hat formed on the device from the two stored rows) gives the
    host-driven loop's iterates bit for bit, and the reference's fit."""
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    c = G.load_case(name)
    f = c['fits'][variant]
    A = LinearOperator(c['D'], c['K'], None, nolut=c['nolut'])
    kw = dict(tol_fun=1e-5, tol_x=1e-7, max_iter=f['details']['iterations'], verbose=0,
              confidence_array=f['conf'], momentum_reuse=reuse)
    xh, dh = solvers.solve(c['y_obs'], A, A.T, regularisation=solvers.init_regularisation(G.fresh_reg(f['reg'])), **kw)
    xg, dg = solvers.solve(c['y_obs'], A, A.T, regularisation=solvers.init_regularisation(G.fresh_reg(f['reg'])),
                           graph=True, **kw)
    assert dg['iterations'] == dh['iterations'] == f['details']['iterations']
    assert dg['stopping_criterion'] == dh['stopping_criterion'] == f['details']['stopping_criterion']
    assert dg['backtracks'] == dh['backtracks']
    assert dg['anchors'] == dh['anchors']
    assert np.array_equal(xg, xh)
    assert G.rel(xg, f['x']) <= 1e-8
    for k in ('residual', 'regterm', 'cost_function', 'abs_cost', 'rel_cost', 'abs_x', 'rel_x'):
        assert dg[k] == dh[k], k


@pytest.mark.parametrize('reuse', [False, True])
def test_graph_mode_with_adjoint_slabs(reuse):
    """Inside the graph capture the slab schedule runs its steps in order on one stream; the
    iterates stay bit-identical to the host loop's (three-stream schedule)."""
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.scaled_spec('demo_5k', n_fibers=8000))
    A = LinearOperator(D, K, None)
    assert A.set_slabs(4) == 4
    x0 = synth.make_x(A.nCOLS, 1)
    y = synth.make_signal(A.dot(x0), 2)
    kw = dict(tol_fun=1e-6, tol_x=1e-8, max_iter=60, verbose=0, momentum_reuse=reuse)
    xh, dh = solvers.solve(y, A, A.T, **kw)
    xg, dg = solvers.solve(y, A, A.T, graph=True, **kw)
    assert dg['iterations'] == dh['iterations']
    assert np.array_equal(xg, xh)


def test_backtracking_cap_ends_the_solve():
    """A fit that backtracks, run with no step reduction allowed, stops with the
    backtracking status in both the host loop and the graph (whose backtracking WHILE node
    is bounded); with the default cap it finishes as before."""
    from commit_gb300 import _lib, solvers
    from commit_gb300.operator import LinearOperator
    found = False
    for name, variant in _fit_cases():
        c = G.load_case(name)
        f = c['fits'][variant]
        A = LinearOperator(c['D'], c['K'], None, nolut=c['nolut'])
        kw = dict(tol_fun=1e-5, tol_x=1e-7, max_iter=f['details']['iterations'], verbose=0,
                  confidence_array=f['conf'], momentum_reuse=False)
        reg = lambda: solvers.init_regularisation(G.fresh_reg(f['reg']))  # noqa: E731
        _, d = solvers.solve(c['y_obs'], A, A.T, regularisation=reg(), **kw)
        if d['backtracks'] == 0:
            continue
        found = True
        for graph in (False, True):
            with pytest.raises(_lib.CgbError, match='backtracking') as ei:
                solvers.solve(c['y_obs'], A, A.T, regularisation=reg(), graph=graph, max_backtracks=-1, **kw)
            assert ei.value.code == _lib.CGB_ERR_BACKTRACK
        _, d2 = solvers.solve(c['y_obs'], A, A.T, regularisation=reg(), graph=True, **kw)
        assert d2['iterations'] == d['iterations'] and d2['backtracks'] == d['backtracks']
        break
    assert found, 'no golden fit backtracks'


@pytest.mark.parametrize('name', ['szb', 'multi_rf'])
def test_solve_far_past_convergence(name):
    """Tolerances off, up to 4000 nnls iterations: near the minimum the sufficient-decrease
    test is decided at the rounding level.  With momentum reuse qfval comes from the stored
    rows and rounds differently from the evaluation of x; on a failed test the solver then
    evaluates f(x_hat) directly (an anchor) instead of shrinking the step without end.  The
    host loop (with and without restart) and the graph end without error, on the iteration
    cap or on the reference's absolute tests (|f_k - f_k-1| or |x_k - x_k-1| below eps),
    the graph with the host loop's iterates, backtracks and anchors bit for bit, and all
    stay at the no-reuse run's cost (to 1e-3: without restart FISTA still oscillates around
    the minimum after 4000 iterations, and x itself is not identifiable on these small fits,
    whose columns are nearly collinear)."""
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    c = G.load_case(name)
    f = c['fits']['nnls']
    A = LinearOperator(c['D'], c['K'], None, nolut=c['nolut'])
    kw = dict(tol_fun=0.0, tol_x=0.0, max_iter=4000, verbose=0)
    reg = lambda: solvers.init_regularisation(G.fresh_reg(f['reg']))  # noqa: E731
    x0, d0 = solvers.solve(c['y_obs'], A, A.T, regularisation=reg(), momentum_reuse=False, **kw)
    xh, dh = solvers.solve(c['y_obs'], A, A.T, regularisation=reg(), **kw)
    xg, dg = solvers.solve(c['y_obs'], A, A.T, regularisation=reg(), graph=True, **kw)
    xr, dr = solvers.solve(c['y_obs'], A, A.T, regularisation=reg(), restart=True, **kw)
    assert d0['anchors'] == 0
    ends = ('Maximum number of iterations', 'Absolute tolerance on the objective',
            'Absolute tolerance on the unknowns')
    for d in (d0, dh, dg, dr):
        assert d['stopping_criterion'] in ends
    for k in ('iterations', 'backtracks', 'anchors', 'cost_function'):
        assert dg[k] == dh[k], k
    assert np.array_equal(xg, xh)
    for d in (dh, dr):
        assert abs(d['cost_function'] - d0['cost_function']) <= 1e-3 * d0['cost_function']
