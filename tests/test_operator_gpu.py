"""Parity of the GB300 operator with the reference operator (golden fixtures) and the oracle.

Bar (FP64 path, both arithmetics): relative error <= 1e-10 (2-norm) on A*x and A'*y.
"""
import numpy as np
import pytest
import torch

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10
CASES = G.case_names()


def _op(c, arith='ff', D=None):
    from commit_gb300.operator import LinearOperator
    return LinearOperator(D or c['D'], c['K'], None, nolut=c['nolut'], arith=arith)


@pytest.mark.parametrize('arith', ['ff', 'f64'])
@pytest.mark.parametrize('name', CASES)
def test_operator_matches_reference_golden(name, arith):
    c = G.load_case(name)
    A = _op(c, arith)
    assert A.shape == (c['Ax'].size, c['x_in'].size)
    assert A.T.shape == (c['x_in'].size, c['Ax'].size)
    assert G.rel(A.dot(c['x_in']), c['Ax']) <= TOL
    assert G.rel(A.T.dot(c['y_in']), c['Aty']) <= TOL


@pytest.mark.parametrize('name', CASES)
def test_operator_device_tensors(name):
    c = G.load_case(name)
    A = _op(c)
    x = torch.from_numpy(c['x_in']).cuda()
    y = torch.from_numpy(c['y_in']).cuda()
    ax = A.dot(x)
    aty = A.T.dot(y)
    assert ax.is_cuda and aty.is_cuda
    assert G.rel(ax.cpu().numpy(), c['Ax']) <= TOL
    assert G.rel(aty.cpu().numpy(), c['Aty']) <= TOL


@pytest.mark.parametrize('name', CASES)
def test_dimension_mismatch_raises(name):
    c = G.load_case(name)
    A = _op(c)
    with pytest.raises(RuntimeError, match='dimensions do not match'):
        A.dot(np.zeros(A.nCOLS + 1))
    with pytest.raises(RuntimeError, match='dimensions do not match'):
        A.T.dot(np.zeros(A.nROWS - 1))


@pytest.mark.parametrize('name', ['szb', 'multi_rf', 'eval_gaps'])
def test_unsorted_dictionary_gives_same_operator(name):
    """The device re-layout sorts; a shuffled dictionary defines the same A."""
    c = G.load_case(name)
    D = c['D']
    rng = np.random.default_rng(0)
    p = rng.permutation(D['IC']['n'])
    IC = dict(D['IC'])
    for k in ('str', 'vox', 'dir', 'len'):
        IC[k] = np.ascontiguousarray(IC[k][p])
    D2 = {'IC': IC, 'EC': D['EC'], 'ISO': D['ISO']}
    A = _op(c, D=D2)
    assert G.rel(A.dot(c['x_in']), c['Ax']) <= TOL
    assert G.rel(A.T.dot(c['y_in']), c['Aty']) <= TOL


@pytest.mark.parametrize('name', CASES)
def test_dot_product_identity(name):
    c = G.load_case(name)
    A = _op(c)
    rng = np.random.default_rng(1)
    x = rng.normal(size=A.nCOLS)
    y = rng.normal(size=A.nROWS)
    lhs = float(np.dot(A.dot(x), y))
    rhs = float(np.dot(x, A.T.dot(y)))
    assert abs(lhs - rhs) <= 1e-11 * max(1.0, abs(lhs))


def test_invalid_dictionary_is_rejected():
    from commit_gb300._lib import CgbError
    c = G.load_case('szb')
    D = c['D']
    IC = dict(D['IC'])
    IC['vox'] = IC['vox'].copy()
    IC['vox'][3] = D['IC']['nVOX'] + 5
    with pytest.raises(CgbError, match='IC voxel index'):
        _op(c, D={'IC': IC, 'EC': D['EC'], 'ISO': D['ISO']})


def test_demo_scale_against_oracle():
    """The 5k-streamline demo workload (nS=66, ~580k segments) against the C port."""
    from commit_gb300 import synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.SPECS['demo_5k'])
    P = O.PortOperator(D, K, None, nthreads=8)
    rng = np.random.default_rng(2)
    x = rng.uniform(-0.2, 1.0, size=P.nCOLS)
    y = rng.normal(size=P.nROWS)
    ax, aty = P.dot(x), P.T.dot(y)
    for arith in ('ff', 'f64'):
        A = LinearOperator(D, K, None, arith=arith)
        assert G.rel(A.dot(x), ax) <= TOL
        assert G.rel(A.T.dot(y), aty) <= TOL


def test_repeatable_bitwise():
    c = G.load_case('szb')
    A = _op(c)
    a1 = A.T.dot(c['y_in'])
    a2 = A.T.dot(c['y_in'])
    assert np.array_equal(a1, a2)


@pytest.mark.parametrize('n_b0,shells', [(1, [(1000.0, 6)]), (3, [(1000.0, 30)]), (1, [(1000.0, 45), (2000.0, 45)]),
                                         (18, [(1000.0, 90), (2000.0, 90), (3000.0, 90)])])
def test_sample_counts_against_oracle(n_b0, shells):
    """nS = 7, 33, 91 (odd: scalar row stores) and 288 (the full-brain acquisition)."""
    from commit_gb300 import synth
    from commit_gb300.operator import LinearOperator
    spec = synth.ProblemSpec(dim=(24, 24, 16), n_mask=5000, n_fibers=800, ndirs=200, n_b0=n_b0, shells=shells,
                             seed=5)
    D, K = synth.make_dictionary(spec)
    P = O.PortOperator(D, K, None, nthreads=8)
    rng = np.random.default_rng(3)
    x = rng.uniform(-0.3, 1.0, size=P.nCOLS)
    y = rng.normal(size=P.nROWS)
    ax, aty = P.dot(x), P.T.dot(y)
    for arith in ('ff', 'f64'):
        A = LinearOperator(D, K, None, arith=arith)
        assert G.rel(A.dot(x), ax) <= TOL, arith
        assert G.rel(A.T.dot(y), aty) <= TOL, arith


@pytest.mark.parametrize('arith,tol', [('bf16', 1.5e-2), ('fp16', 4e-3), ('f32', 2e-5)])
def test_reduced_precision_operator(arith, tol):
    """LUT in BF16/FP16 (or FP32), FP16 lengths, FP32 accumulation vs the FP64 oracle."""
    from commit_gb300 import synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.SPECS['demo_5k'])
    P = O.PortOperator(D, K, None, nthreads=8)
    rng = np.random.default_rng(4)
    x = rng.uniform(0.0, 1.0, size=P.nCOLS)
    y = rng.uniform(0.0, 1.0, size=P.nROWS)
    A = LinearOperator(D, K, None)
    ax = A.dot(torch.from_numpy(x).float().cuda(), arith=arith).double().cpu().numpy()
    aty = A.T.dot(torch.from_numpy(y).float().cuda(), arith=arith).double().cpu().numpy()
    assert G.rel(ax, P.dot(x)) <= tol
    assert G.rel(aty, P.T.dot(y)) <= tol
    # the reduced operator is itself an exact adjoint pair up to FP32 rounding
    xs = rng.normal(size=P.nCOLS)
    ys = rng.normal(size=P.nROWS)
    lhs = float(np.dot(A.dot(torch.from_numpy(xs).float().cuda(), arith=arith).double().cpu().numpy(), ys))
    rhs = float(np.dot(xs, A.T.dot(torch.from_numpy(ys).float().cuda(), arith=arith).double().cpu().numpy()))
    assert abs(lhs - rhs) <= 1e-4 * (abs(lhs) + abs(rhs))


def test_occupancy_builds_give_identical_results():
    """Both register builds of each tuned kernel compute the same operations in the same
    order: forcing either gives bitwise-equal products (FP64 float-float and BF16 paths)."""
    import torch
    from commit_gb300 import synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.scaled_spec('demo_5k', n_fibers=2000, n_b0=18,
                                                   shells=[(1000.0, 90), (2000.0, 90), (3000.0, 90)]))
    A = LinearOperator(D, K, None)
    rng = np.random.default_rng(0)
    x = torch.from_numpy(rng.uniform(0, 1, A.nCOLS)).cuda()
    w = torch.from_numpy(rng.normal(size=A.nROWS)).cuda()
    w32 = w.float()
    res = {}
    for c in (1, 2):
        A.occupancy({k: c for k in A.OCC_SLOTS})
        res[c] = (A.dot(x).cpu().numpy(), A.T.dot(w).cpu().numpy(), A.T.dot(w32, arith='bf16').cpu().numpy())
    for a, b in zip(res[1], res[2]):
        assert np.array_equal(a, b)
    A.occupancy({k: 0 for k in A.OCC_SLOTS})
    A.dot(x)
    A.T.dot(w)
    st = A.occupancy()
    assert st['ff_forward'][0] in (1, 2) and st['ff_adjoint'][0] in (1, 2)
    assert st['ff_forward'][1] > 0 and st['ff_forward'][2] > 0


def test_host_pipeline_matches_device_path():
    """Host-buffer products on a problem large enough for the copy/compute pipeline
    (nROWS >= 2^22) equal the device-buffer products bit for bit."""
    import torch
    from commit_gb300 import synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.scaled_spec('demo_5k', dim=(64, 64, 32), n_mask=80000, n_fibers=20000,
                                                   n_b0=18, shells=[(1000.0, 90)]))
    A = LinearOperator(D, K, None)
    assert A.nROWS >= 1 << 22
    rng = np.random.default_rng(5)
    x = rng.uniform(0, 1, A.nCOLS)
    w = rng.normal(size=A.nROWS)
    yh = A.dot(x)
    xh = A.T.dot(w)
    yd = A.dot(torch.from_numpy(x).cuda()).cpu().numpy()
    xd = A.T.dot(torch.from_numpy(w).cuda()).cpu().numpy()
    assert np.array_equal(yh, yd)
    assert np.array_equal(xh, xd)


@pytest.mark.parametrize('nslab', [2, 5, 16])
def test_adjoint_slabs_give_identical_sums(nslab):
    """A' slab by slab (fibre pass right after each slab's voxel pass) adds each fibre's
    terms in the same order as the one-slab adjoint: bitwise-equal results, for the FP64
    products, the reduced-precision product and the FISTA gradient pass (solver)."""
    import torch
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.scaled_spec('demo_5k', n_fibers=20000))
    A = LinearOperator(D, K, None)
    rng = np.random.default_rng(2)
    w = torch.from_numpy(rng.normal(size=A.nROWS)).cuda()
    x = synth.make_x(A.nCOLS, 1)
    y = synth.make_signal(A.dot(x), 2)
    res = {}
    for s in (1, nslab):
        assert A.set_slabs(s) == s
        fit = solvers.solve(y, A, A.T, tol_fun=1e-6, tol_x=1e-8, max_iter=30, verbose=0)
        res[s] = (A.T.dot(w).cpu().numpy(), A.T.dot(w.float(), arith='bf16').cpu().numpy(), A.T.dot(w.cpu().numpy()),
                  fit[0], fit[1]['iterations'])
    for a, b in zip(res[1], res[nslab]):
        assert np.array_equal(np.asarray(a), np.asarray(b))
    assert A.set_slabs(0) >= 1


@pytest.mark.parametrize('mode', [0, 1])
def test_page_locked_host_rows_direct_and_staged(mode):
    """Page-locked host rows are read / written in place by the kernels (mode 0) or staged
    (mode 1); both equal the device-buffer products bit for bit."""
    import torch
    from commit_gb300 import synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.scaled_spec('demo_5k', dim=(64, 64, 32), n_mask=80000, n_fibers=20000,
                                                   n_b0=18, shells=[(1000.0, 90)]))
    A = LinearOperator(D, K, None)
    assert A.host_mode(mode) == mode
    rng = np.random.default_rng(6)
    xh = torch.empty(A.nCOLS, dtype=torch.float64, pin_memory=True).numpy()
    xh[:] = rng.uniform(0, 1, A.nCOLS)
    wh = torch.empty(A.nROWS, dtype=torch.float64, pin_memory=True).numpy()
    wh[:] = rng.normal(size=A.nROWS)
    yh = torch.empty(A.nROWS, dtype=torch.float64, pin_memory=True).numpy()
    gh = torch.empty(A.nCOLS, dtype=torch.float64, pin_memory=True).numpy()
    A.dot(xh, out=yh)
    A.T.dot(wh, out=gh)
    yd = A.dot(torch.from_numpy(xh.copy()).cuda()).cpu().numpy()
    gd = A.T.dot(torch.from_numpy(wh.copy()).cuda()).cpu().numpy()
    assert np.array_equal(yh, yd)
    assert np.array_equal(gh, gd)


@pytest.mark.parametrize('name', ['szb', 'multi_rf', 'eval_gaps', 'ball_stick'])
def test_scalar_float_float_kernels_match_golden(name):
    """The one-sample-per-lane float-float kernels (the other kernel family) against the
    reference's golden products."""
    from commit_gb300.operator import LinearOperator
    c = G.load_case(name)
    A = LinearOperator(c['D'], c['K'], None, nolut=c['nolut'])
    assert A.ff_kernels(0) == 0
    assert G.rel(A.dot(c['x_in']), c['Ax']) <= 1e-10
    assert G.rel(A.T.dot(c['y_in']), c['Aty']) <= 1e-10


def test_handles_release_their_device_memory():
    """Creating, using (float-float, reduced precision, slabs, batched, solver) and
    destroying handles returns the device memory: no growth over repeated cycles."""
    import gc
    import torch
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    D, K = synth.make_dictionary(synth.scaled_spec('demo_5k', n_fibers=3000))
    x = torch.from_numpy(synth.make_x(synth.n_cols(D, K), 1)).cuda()

    def cycle():
        A = LinearOperator(D, K, None)
        A.set_slabs(3)
        y = A.dot(x)
        A.T.dot(y)
        A.T.dot(y.float(), arith='bf16')
        A.dot_batch([x, x])
        solvers.solve(y, A, A.T, tol_fun=0, tol_x=0, max_iter=5, verbose=0)
        solvers.solve_batch(y, A, [None, None, None], tol_fun=0, tol_x=0, max_iter=5)
        del A
        gc.collect()
        torch.cuda.synchronize()

    cycle()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        cycle()
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < 64 << 20, (free0, free1)


@pytest.mark.parametrize('name', ['szb', 'multi_rf', 'eval_gaps', 'ball_stick', 'scalar_map'])
def test_float_float_voxel_shapes_match_golden(name):
    """Both voxel shapes of the float-float pair kernels (default lanes per voxel, a warp
    per voxel) reproduce the reference's products, and the FISTA fits."""
    from commit_gb300 import solvers
    from commit_gb300.operator import LinearOperator
    c = G.load_case(name)
    out = {}
    for shape in (1, 2):
        A = LinearOperator(c['D'], c['K'], None, nolut=c['nolut'])
        A.ff_shape(shape)
        out[shape] = (A.dot(c['x_in']), A.T.dot(c['y_in']))
        assert G.rel(out[shape][0], c['Ax']) <= 1e-10
        assert G.rel(out[shape][1], c['Aty']) <= 1e-10
        f = c['fits']['nnls']
        x, det = solvers.solve(c['y_obs'], A, A.T, tol_fun=1e-5, tol_x=1e-7, max_iter=f['details']['iterations'],
                               verbose=0, regularisation=solvers.init_regularisation(G.fresh_reg(f['reg'])),
                               confidence_array=f['conf'])
        assert det['iterations'] == f['details']['iterations']
        assert G.rel(x, f['x']) <= 1e-8
    assert G.rel(out[1][0], out[2][0]) <= 1e-13
    assert G.rel(out[1][1], out[2][1]) <= 1e-13


@pytest.mark.parametrize('scale', [1e30, 1e-30, 1e45, 1e-45, 1e200, 1e-200])
@pytest.mark.parametrize('arith', ['ff', 'f64'])
@pytest.mark.parametrize('name', ['szb', 'multi_rf'])
def test_range_guard_scaled_inputs(name, arith, scale):
    """FP64 inputs far outside FP32's exponent range (the float-float words are FP32): the
    kernels scale them by an exact power of two, so A(s x) and A'(s y) stay within the FP64
    bar of the oracle run on the same scaled inputs, on host and device vectors."""
    c = G.load_case(name)
    A = _op(c, arith)
    P = O.PortOperator(c['D'], c['K'], None)
    xs, ys = c['x_in'] * scale, c['y_in'] * scale
    ax, aty = P.dot(xs), P.T.dot(ys)
    assert np.all(np.isfinite(ax)) and np.all(np.isfinite(aty))

    def rel(a, b):  # on the unscaled magnitudes, so the norms themselves do not overflow
        return G.rel(np.asarray(a) / scale, np.asarray(b) / scale)

    assert rel(A.dot(xs), ax) <= TOL
    assert rel(A.T.dot(ys), aty) <= TOL
    assert rel(A.dot(torch.from_numpy(xs).cuda()).cpu().numpy(), ax) <= TOL
    assert rel(A.T.dot(torch.from_numpy(ys).cuda()).cpu().numpy(), aty) <= TOL


def test_range_guard_mixed_row_magnitudes():
    """Rows of y spanning 1e-40 .. 1e40 (each voxel row is scaled on its own) and x mixing
    1e40 and O(1) entries stay within the FP64 bar."""
    c = G.load_case('szb')
    A = _op(c)
    P = O.PortOperator(c['D'], c['K'], None)
    nS = c['K']['wmr'].shape[2]
    rng = np.random.default_rng(7)
    y = c['y_in'] * np.repeat(10.0 ** rng.choice([-40.0, 0.0, 40.0], size=c['y_in'].size // nS), nS)
    x = c['x_in'] * np.where(rng.uniform(size=c['x_in'].size) < 0.5, 1e40, 1.0)
    assert G.rel(A.T.dot(y), P.T.dot(y)) <= TOL
    assert G.rel(A.dot(x), P.dot(x)) <= TOL


def test_range_guard_in_fista():
    """FISTA on y * 2^140 (beyond FP32's range) follows the unscaled solve: the iterates
    scale exactly with the data (nnls, fixed iteration count)."""
    from commit_gb300 import solvers
    c = G.load_case('szb')
    A = _op(c)
    rp = O.reg_params(c['D'], c['K'])
    s = 2.0 ** 140
    kw = dict(tol_fun=0.0, tol_x=0.0, max_iter=30, verbose=0)
    x1, d1 = solvers.solve(c['y_obs'], A, A.T, regularisation=solvers.init_regularisation(dict(rp)), **kw)
    x2, d2 = solvers.solve(c['y_obs'] * s, A, A.T, regularisation=solvers.init_regularisation(dict(rp)), **kw)
    assert d1['iterations'] == d2['iterations']
    assert np.all(np.isfinite(x2))
    assert G.rel(x2 / s, x1) <= 1e-8
