"""Pin the oracle (C port + numpy solver) against the reference's own outputs.

The golden fixtures were produced by running the reference's generated C operator
(setup_operator.py) and its solvers.py / proximals.pyx (tests/golden/make_golden.py).
When oracle/_ref is built on this machine the port is also compared with it directly.
"""
import numpy as np
import pytest

import golden_io as G
import oracle as O

CASES = G.case_names()


@pytest.mark.parametrize('name', CASES)
def test_port_operator_matches_reference(name):
    c = G.load_case(name)
    for nt in (1, c['threads']):
        A = O.PortOperator(c['D'], c['K'], None, nolut=c['nolut'], nthreads=nt)
        assert A.shape == (c['Ax'].size, c['x_in'].size)
        assert G.rel(A.dot(c['x_in']), c['Ax']) < 1e-13
        assert G.rel(A.T.dot(c['y_in']), c['Aty']) < 1e-13
    if 'Ax_mt' in c:
        assert G.rel(c['Ax_mt'], c['Ax']) < 1e-13


@pytest.mark.parametrize('name', CASES)
def test_port_dimension_check(name):
    c = G.load_case(name)
    A = O.PortOperator(c['D'], c['K'], None, nolut=c['nolut'])
    with pytest.raises(RuntimeError, match='dimensions do not match'):
        A.dot(np.zeros(A.nCOLS + 1))


def _fit_cases():
    out = []
    for name in CASES:
        c = G.load_case(name)
        for v in c['fits']:
            out.append((name, v))
    return out


@pytest.mark.parametrize('name,variant', _fit_cases())
def test_oracle_solver_matches_reference(name, variant):
    c = G.load_case(name)
    f = c['fits'][variant]
    A = O.PortOperator(c['D'], c['K'], None, nolut=c['nolut'], nthreads=2)
    reg = O.init_regularisation(G.fresh_reg(f['reg']))
    x, det = O.solve(c['y_obs'], A, A.T, tol_fun=1e-5, tol_x=1e-7, max_iter=f['details']['iterations'] + 5
                     if f['details']['stopping_criterion'] != 'Maximum number of iterations'
                     else f['details']['iterations'], verbose=0, regularisation=reg, confidence_array=f['conf'])
    ref = f['details']
    assert det['iterations'] == ref['iterations']
    assert det['stopping_criterion'] == ref['stopping_criterion']
    assert G.rel(x, f['x']) < 1e-8
    for k in ('residual', 'regterm', 'cost_function', 'abs_cost', 'rel_cost', 'abs_x', 'rel_x'):
        assert abs(det[k] - ref[k]) <= 1e-4 * max(1.0, abs(ref[k])), k


@pytest.mark.skipif(not O.ref_available(), reason='oracle/_ref not built on this machine')
@pytest.mark.parametrize('nt', [1, 3, 8])
def test_port_vs_reference_library(nt):
    from commit_gb300 import synth
    D, K = synth.make_dictionary(synth.ProblemSpec(dim=(16, 16, 8), n_mask=1500, n_fibers=400, ndirs=100,
                                                   shells=[(1000.0, 20)], seed=3))
    D['IC']['eval'] = np.ones(D['IC']['nSTR'], np.uint32)
    R = O.RefOperator(D, K, O.set_threads(D, nt))
    P = O.PortOperator(D, K, None, nthreads=nt)
    rng = np.random.default_rng(5)
    x = rng.normal(size=R.nCOLS)
    y = rng.normal(size=R.nROWS)
    assert G.rel(P.dot(x), R.dot(x)) < 1e-13
    assert G.rel(P.T.dot(y), R.T.dot(y)) < 1e-13
