"""Device proximal maps and penalties vs the proximals.pyx restatement (oracle)."""
import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu


def _groups(rng, n, hier):
    base = [np.sort(g).astype(np.int32) for g in np.array_split(rng.permutation(n), 5)]
    if hier:
        base = [base[0], base[1], np.union1d(base[0], base[1]).astype(np.int32)] + base[2:]
    gidx = np.concatenate(base).astype(np.int32)
    gsz = np.array([g.size for g in base], np.int32)
    return gidx, gsz, rng.uniform(0.5, 2.0, size=len(base))


@pytest.mark.parametrize('seed', [0, 1])
def test_elementwise_maps(seed):
    from commit_gb300 import proximals as P
    rng = np.random.default_rng(seed)
    x = rng.normal(size=1000)
    w = rng.uniform(0.1, 2.0, size=1000)
    for fn, args in ((P.non_negativity, (100, 500)), (P.soft_thresholding, (0.3, 50, 700)),
                     (P.w_soft_thresholding, (w, 0.3, 10, 900))):
        ref = getattr(O, fn.__name__)(x.copy(), *args)
        got = fn(x.copy(), *args)
        np.testing.assert_array_equal(got, ref)
        # on a device tensor, in place
        t = torch.from_numpy(x.copy()).cuda()
        fn(t, *[torch.from_numpy(a).cuda() if isinstance(a, np.ndarray) else a for a in args])
        np.testing.assert_array_equal(t.cpu().numpy(), ref)


def test_projection_onto_l2_ball():
    from commit_gb300 import proximals as P
    rng = np.random.default_rng(3)
    x = rng.normal(size=300)
    got = P.projection_onto_l2_ball(x.copy(), 2.0, 20, 200)
    ref = x.copy()
    xn = np.linalg.norm(ref[20:220])
    ref[20:220] = ref[20:220] * (1 - 2.0 / xn) if xn > 2.0 else 0.0
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize('hier', [False, True])
def test_group_lasso_prox_and_penalties(hier):
    from commit_gb300 import proximals as P
    rng = np.random.default_rng(4)
    x = rng.normal(size=200)
    gidx, gsz, gw = _groups(rng, 200, hier)
    np.testing.assert_allclose(P.prox_group_lasso(x.copy(), gidx, gsz, gw, 0.7),
                               O.prox_group_lasso(x.copy(), gidx, gsz, gw, 0.7), rtol=1e-12, atol=1e-14)
    assert abs(P.omega_group_lasso(x, gidx, gsz, gw, 0.7) - O.omega_group_lasso(x, gidx, gsz, gw, 0.7)) < 1e-11
    assert abs(P.omega_sparse_group_lasso(x, gidx, gsz, gw, 0.2, 0.7)
               - O.omega_sparse_group_lasso(x, gidx, gsz, gw, 0.2, 0.7)) < 1e-10
    w = rng.uniform(0.5, 1.5, size=200)
    assert abs(P.omega_w_sparse_group_lasso(x, w, gidx, gsz, gw, 0.2, 0.7)
               - O.omega_w_sparse_group_lasso(x, w, gidx, gsz, gw, 0.2, 0.7)) < 1e-10
    assert P.omega_group_lasso(x, gidx, gsz, gw, 0.0) == 0.0


def test_init_regularisation_prox_and_omega_match_oracle():
    import golden_io as G
    from commit_gb300 import solvers
    c = G.load_case('szb')
    rng = np.random.default_rng(5)
    for name, f in c['fits'].items():
        x = rng.normal(size=c['x_in'].size)
        mine = solvers.init_regularisation(G.fresh_reg(f['reg']))
        ref = O.init_regularisation(G.fresh_reg(f['reg']))
        np.testing.assert_allclose(mine['prox'](x.copy(), 0.37), ref['prox'](x.copy(), 0.37), rtol=1e-12,
                                   atol=1e-14, err_msg=name)
        assert abs(mine['omega'](x) - ref['omega'](x)) <= 1e-10 * max(1.0, abs(ref['omega'](x))), name
