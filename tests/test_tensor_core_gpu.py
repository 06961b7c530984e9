"""The reduced-precision BF16 operator on the tensor cores (tcgen05) against the oracle and
against the CUDA-core BF16 kernels.

Both use the same BF16 LUT values.  The tensor-core forward merges each voxel's items per
LUT row in FP32 and splits the sums into BF16 high and low parts (about 16 bits); the
tensor-core adjoint splits the input rows the same way.  So the two paths agree to ~1e-5
and both stay within the BF16 bound against the FP64 oracle.
Bars: 1.5e-2 against the oracle (the BF16 bound of the CUDA-core path), 1e-4 against the
CUDA-core kernels, bitwise equal on repeated calls.
"""
import numpy as np
import pytest
import torch

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu

BF16_TOL = 1.5e-2
TC_VS_CC = 1e-4
SHAPES = [(1, [(1000.0, 6)]), (3, [(1000.0, 30)]), (1, [(1000.0, 45), (2000.0, 45)]),
          (18, [(1000.0, 90), (2000.0, 90), (3000.0, 90)])]


def _forward_both(A, x):
    xt = torch.from_numpy(x).float().cuda()
    assert A.tensor_cores(2)
    y_tc = A.dot(xt, arith='bf16').double().cpu().numpy()
    y_tc2 = A.dot(xt, arith='bf16').double().cpu().numpy()
    A.device_status()
    A.tensor_cores(1)
    y_cc = A.dot(xt, arith='bf16').double().cpu().numpy()
    return y_tc, y_tc2, y_cc


def _adjoint_both(A, y):
    yt = torch.from_numpy(y).float().cuda()
    assert A.tensor_cores(2)
    g_tc = A.T.dot(yt, arith='bf16').cpu().numpy()
    g_tc2 = A.T.dot(yt, arith='bf16').cpu().numpy()
    A.device_status()
    A.tensor_cores(1)
    g_cc = A.T.dot(yt, arith='bf16').cpu().numpy()
    return g_tc, g_tc2, g_cc


def _small(n_b0, shells):
    from commit_gb300 import synth
    spec = synth.ProblemSpec(dim=(24, 24, 16), n_mask=5000, n_fibers=800, ndirs=200, n_b0=n_b0, shells=shells, seed=5)
    return synth.make_dictionary(spec)


@pytest.mark.parametrize('name', ['szb', 'multi_rf', 'ball_stick', 'eval_gaps', 'scalar_map'])
def test_tensor_core_forward_golden_shapes(name):
    from commit_gb300.operator import LinearOperator
    c = G.load_case(name)
    A = LinearOperator(c['D'], c['K'], None)
    y_tc, y_tc2, y_cc = _forward_both(A, c['x_in'])
    assert np.array_equal(y_tc, y_tc2)
    assert G.rel(y_tc, c['Ax']) <= BF16_TOL
    assert G.rel(y_tc, y_cc) <= TC_VS_CC


@pytest.mark.parametrize('name', ['szb', 'multi_rf', 'ball_stick', 'eval_gaps', 'scalar_map'])
def test_tensor_core_adjoint_golden_shapes(name):
    from commit_gb300.operator import LinearOperator
    c = G.load_case(name)
    A = LinearOperator(c['D'], c['K'], None)
    g_tc, g_tc2, g_cc = _adjoint_both(A, c['y_in'])
    assert np.array_equal(g_tc, g_tc2)
    assert G.rel(g_tc, c['Aty']) <= BF16_TOL
    assert G.rel(g_tc, g_cc) <= TC_VS_CC


@pytest.mark.parametrize('n_b0,shells', SHAPES)
def test_tensor_core_sample_counts(n_b0, shells):
    """nS = 7, 33, 91 and 288 (padded to 32, 64, 96, 288 samples; 1, 1, 2, 5 K-blocks of 64
    samples in the adjoint), 200 LUT directions."""
    from commit_gb300.operator import LinearOperator
    D, K = _small(n_b0, shells)
    P = O.PortOperator(D, K, None, nthreads=8)
    rng = np.random.default_rng(3)
    x = rng.uniform(0.0, 1.0, size=P.nCOLS)
    y = rng.normal(size=P.nROWS)
    A = LinearOperator(D, K, None)
    y_tc, y_tc2, y_cc = _forward_both(A, x)
    assert np.array_equal(y_tc, y_tc2)
    assert G.rel(y_tc, P.dot(x)) <= BF16_TOL
    assert G.rel(y_tc, y_cc) <= TC_VS_CC
    g_tc, g_tc2, g_cc = _adjoint_both(A, y)
    assert np.array_equal(g_tc, g_tc2)
    assert G.rel(g_tc, P.T.dot(y)) <= BF16_TOL
    assert G.rel(g_tc, g_cc) <= TC_VS_CC


def test_tensor_core_demo_scale():
    """The 5k-streamline demo (nS = 66, 500 directions, ~580k segments, many tiles per SM)."""
    from commit_gb300 import synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.SPECS['demo_5k'])
    P = O.PortOperator(D, K, None, nthreads=8)
    rng = np.random.default_rng(2)
    x = rng.uniform(-0.2, 1.0, size=P.nCOLS)
    y = rng.uniform(0.0, 1.0, size=P.nROWS)
    A = LinearOperator(D, K, None)
    y_tc, y_tc2, y_cc = _forward_both(A, x)
    assert np.array_equal(y_tc, y_tc2)
    assert G.rel(y_tc, P.dot(x)) <= BF16_TOL
    assert G.rel(y_tc, y_cc) <= TC_VS_CC
    g_tc, g_tc2, g_cc = _adjoint_both(A, y)
    assert np.array_equal(g_tc, g_tc2)
    assert G.rel(g_tc, P.T.dot(y)) <= BF16_TOL
    assert G.rel(g_tc, g_cc) <= TC_VS_CC


def test_tensor_core_fista():
    """Reduced-precision FISTA (fused residual-norm epilogue, gradient from stored A x rows)
    on the tensor cores follows the CUDA-core run: same iterations, close solutions."""
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    c = G.load_case('szb')
    rp = O.reg_params(c['D'], c['K'])
    kw = dict(tol_fun=0.0, tol_x=0.0, max_iter=40, verbose=0, arith='bf16')
    A = LinearOperator(c['D'], c['K'], None)
    A.tensor_cores(2)
    x1, d1 = solvers.solve(c['y_obs'], A, A.T, regularisation=solvers.init_regularisation(dict(rp)), **kw)
    A.device_status()
    A.tensor_cores(1)
    x2, d2 = solvers.solve(c['y_obs'], A, A.T, regularisation=solvers.init_regularisation(dict(rp)), **kw)
    assert d1['iterations'] == d2['iterations']
    assert G.rel(x1, x2) <= 1e-3
    assert abs(d1['cost_function'] - d2['cost_function']) <= 1e-4 * abs(d2['cost_function'])
