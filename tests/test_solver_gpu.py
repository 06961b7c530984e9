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


@pytest.mark.parametrize('arith', ['bf16', 'fp16'])
def test_mixed_fista_with_refinement_reaches_fp64_solution(arith):
    """Reduced-precision FISTA + FP64 refinement reaches the FP64 solution within 1e-4."""
    import oracle as O
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.SPECS['demo_5k'])
    A = LinearOperator(D, K, None)
    P = O.PortOperator(D, K, None, nthreads=8)
    y = synth.make_signal(P.dot(synth.make_x(P.nCOLS, 1)), 2)
    rp = O.reg_params(D, K)
    x_ref, _ = solvers.solve(y, A, A.T, tol_fun=1e-12, tol_x=1e-12, max_iter=3000, verbose=0,
                             regularisation=solvers.init_regularisation(dict(rp)))
    xm, dm = solvers.solve_mixed(y, A, tol_fun=1e-9, tol_x=1e-9, max_iter=1500, verbose=0,
                                 regularisation=solvers.init_regularisation(dict(rp)), arith=arith,
                                 refine_tol_fun=1e-12, refine_tol_x=1e-12, refine_max_iter=3000)
    assert G.rel(xm, x_ref) <= 1e-4
