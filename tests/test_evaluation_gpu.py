"""The operator's callers in Evaluation: lambda_max / group weights (set_regularisation,
commit/core.pyx:861-1192) and the debias re-fit (core.pyx:1476-1508), against the same
flow run on the oracle."""
import numpy as np
import pytest

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu


def _case():
    c = G.load_case('szb')
    return c['D'], c['K'], c['y_obs']


def test_lambda_max_lasso_and_group():
    from commit_gb300 import evaluation
    from commit_gb300.operator import LinearOperator
    D, K, y = _case()
    A = LinearOperator(D, K, None)
    P = O.PortOperator(D, K, None)
    Aty = P.T.dot(y)
    nF = D['IC']['nSTR']
    reg = evaluation.set_regularisation(A, y, D, K, regularisers=('lasso', 'lasso', 'lasso'),
                                        lambdas=(0.1, 0.2, 0.3))
    assert abs(reg['lambdaIC_max'] - np.max(np.abs(Aty[:nF]))) <= 1e-12 * reg['lambdaIC_max']
    nE = D['EC']['n']
    assert abs(reg['lambdaEC_max'] - np.max(np.abs(Aty[nF:nF + nE]))) <= 1e-12 * reg['lambdaEC_max']
    assert abs(reg['lambdaISO'] - 0.3 * np.max(np.abs(Aty[nF + nE:]))) <= 1e-12 * reg['lambdaISO']
    # groups: cardinality weights, adaptive weights from an nnls solution
    rng = np.random.default_rng(0)
    groups = np.empty(6, dtype=object)
    groups[:] = [np.sort(g) for g in np.array_split(rng.permutation(nF), 6)]
    x_nnls = np.abs(rng.normal(size=A.nCOLS))
    reg = evaluation.set_regularisation(A, y, D, K, regularisers=('group_lasso', None, None),
                                        lambdas=(0.05, None, None), params=({'group_idx': groups}, None, None),
                                        x_nnls=x_nnls)
    w = np.sqrt([g.size for g in groups]) / np.array([np.linalg.norm(x_nnls[g]) + 1e-12 for g in groups])
    np.testing.assert_allclose(reg['dictIC_params']['group_weights'], w, rtol=1e-14)
    lm = max(np.linalg.norm(Aty[g]) / w[k] for k, g in enumerate(groups))
    assert abs(reg['lambdaIC'] - 0.05 * lm) <= 1e-12 * reg['lambdaIC']
    with pytest.raises(ValueError):
        evaluation.set_regularisation(A, y, D, K, regularisers=('group_lasso', None, None), lambdas=(0.1, None, None),
                                      params=({'group_idx': groups[:3]}, None, None), x_nnls=x_nnls)


def test_debias_fit_matches_oracle_flow():
    from commit_gb300 import evaluation
    from commit_gb300.operator import LinearOperator
    D, K, y = _case()
    A = LinearOperator(D, K, None)
    reg = evaluation.set_regularisation(A, y, D, K, regularisers=('lasso', None, None), lambdas=(1e-3, None, None))
    x, det, Ad = evaluation.fit(D, K, y, regularisation=reg, tol_fun=1e-6, max_iter=150, debias=True)
    # oracle: the same two solves
    P = O.PortOperator(D, K, None)
    rp = O.reg_params(D, K, regularisers=('lasso', None, None))
    rp['lambdaIC'] = reg['lambdaIC']
    x1, _ = O.solve(y, P, P.T, tol_fun=1e-6, tol_x=1e-6, max_iter=150, verbose=0,
                    regularisation=O.init_regularisation(rp))
    nF = D['IC']['nSTR']
    mask = np.ones(nF, dtype=np.uint32)
    mask[x1[:nF] < 1e-15] = 0
    assert 0 < mask.sum() < nF      # the lasso removes some streamlines and keeps others
    D2 = {'IC': dict(D['IC'], eval=mask), 'EC': D['EC'], 'ISO': D['ISO']}
    P2 = O.PortOperator(D2, K, None)
    xd = x1.copy()
    xd[:nF] *= mask
    xd[nF:] = 0
    ym = P2.dot(xd)
    ym = (ym > 0).astype(np.float64)
    x2, d2 = O.solve(y * ym, P2, P2.T, tol_fun=1e-6, tol_x=1e-6, max_iter=150, verbose=0,
                     regularisation=O.init_regularisation(O.reg_params(D, K)))
    assert det['iterations'] == d2['iterations']
    assert G.rel(x, x2) <= 1e-8
