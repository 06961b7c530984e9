"""Voxelwise maps of a fit (Evaluation.save_results, commit/core.pyx:1614-1750) on the device
against the oracle's numpy restatement: compartment maps to 1e-12 relative (FP64 sums in a
different order), error maps to 1e-10 (both compare the same FP32-rounded signals)."""
import numpy as np
import pytest

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name', ['szb', 'multi_rf', 'ball_stick', 'eval_gaps'])
def test_voxel_maps_match_oracle(name):
    from commit_gb300 import evaluation
    from commit_gb300.operator import LinearOperator
    c = G.load_case(name)
    D, K = c['D'], c['K']
    A = LinearOperator(D, K, None, nolut=c['nolut'])
    P = O.PortOperator(D, K, None, nolut=c['nolut'])
    rng = np.random.default_rng(7)
    x = rng.uniform(0, 1, A.nCOLS)
    y = c['y_obs']
    conf = rng.uniform(0, 1, A.nROWS)
    conf[:A.nSAMPLES] = 0.0                     # a voxel with zero confidence
    nf = rng.uniform(0.5, 2.0, A.ICnSTR * A.ICnRF)
    got = evaluation.voxel_maps(A, x, y, conf, nf)
    want = O.voxel_maps(D, K, x, P.dot(x), y, conf, nf)
    for k in ('compartment_IC', 'compartment_EC', 'compartment_ISO'):
        assert G.rel(got[k].astype(np.float64), want[k].astype(np.float32).astype(np.float64)) <= 1e-6, k
    for k in ('fit_RMSE', 'fit_NRMSE', 'fit_RMSE_adjusted', 'fit_NRMSE_adjusted'):
        assert G.rel(got[k].astype(np.float64), want[k].astype(np.float32).astype(np.float64)) <= 1e-6, k
    assert got['fit_RMSE_adjusted'][0] == 0.0


def test_voxel_maps_volumes_and_normalisation():
    from commit_gb300 import evaluation, synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.SPECS['demo_5k'])
    A = LinearOperator(D, K, None)
    x = synth.make_x(A.nCOLS, 1)
    m = evaluation.voxel_maps(A, x, normalize_maps=True, DICTIONARY=D)
    tot = m['compartment_IC'] + m['compartment_EC'] + m['compartment_ISO']
    assert np.all(np.abs(tot - 1.0) < 1e-5)
    vol = m['compartment_IC_vol']
    assert vol.shape == D['MASK'].shape
    assert np.array_equal(vol[D['MASK_ix'], D['MASK_iy'], D['MASK_iz']], m['compartment_IC'])


def test_voxel_maps_reject_bad_sizes():
    from commit_gb300 import evaluation
    from commit_gb300.operator import LinearOperator
    c = G.load_case('szb')
    A = LinearOperator(c['D'], c['K'], None)
    with pytest.raises(RuntimeError):
        evaluation.voxel_maps(A, np.zeros(A.nCOLS - 1))
    with pytest.raises(RuntimeError):
        evaluation.voxel_maps(A, np.zeros(A.nCOLS), y=np.zeros(A.nROWS + 1))
    m = evaluation.voxel_maps(A, np.zeros(A.nCOLS), y=c['y_obs'])
    assert not m['compartment_IC'].any() and m['fit_RMSE'].max() > 0
