"""Parity at the full-brain workload the operator benchmark runs on: 1M seeded streamlines
(~1.2e8 IC segments), 145x174x145 grid, nS = 288, SZB 1 IC / 1 EC / 2 ISO.

The reference operator (its own generated C, compiled in oracle/_ref; the C restatement
when it was not compiled) runs on a central voxel slab holding about a quarter of the
segments.  The slab's A x is the full A x's rows of the slab, and its A' y is the full A'
of y zeroed outside those rows, read at the slab's columns (synth.voxel_slab), so the GPU
operator over the whole workload is compared with the reference on every row and column
the slab touches.  Bars: FP64 path (float-float and native FP64) <= 1e-10 relative
(2-norm), reduced-precision LUTs at the bounds the demo-scale tests state.
"""
import os

import numpy as np
import pytest
import torch

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10
REDUCED_TOL = {'bf16': 1.5e-2, 'fp16': 4e-3, 'f32': 2e-5}


@pytest.fixture(scope='module')
def hcp():
    from commit_gb300 import synth
    spec = synth.SPECS['hcp_1m']
    D, K = synth.make_dictionary(spec, device='cuda')
    D['IC']['eval'] = np.ones(D['IC']['nSTR'] * K['wmr'].shape[0], np.uint32)
    S = synth.voxel_slab(D, K, 0.25)
    threads = min(os.cpu_count() or 1, 255)
    if O.ref_available():
        R = O.RefOperator(S['D'], K, O.set_threads(S['D'], threads))
    else:
        R = O.PortOperator(S['D'], K, None, nthreads=threads)
    nS = K['wmr'].shape[2]
    ncols = synth.n_cols(D, K)
    nrows = synth.n_rows(D, K)
    x = synth.make_x(ncols, spec.seed + 1)
    lo, hi = S['voxels']
    r0, r1 = lo * nS, hi * nS
    y = np.random.default_rng(spec.seed + 5).normal(size=r1 - r0)
    ax_ref = R.dot(x[S['cols']])
    aty_ref = np.zeros(ncols)
    aty_ref[S['cols']] = R.T.dot(y)
    ym = np.zeros(nrows)
    ym[r0:r1] = y
    return {'D': D, 'K': K, 'S': S, 'x': x, 'ym': ym, 'rows': (r0, r1), 'ax_ref': ax_ref, 'aty_ref': aty_ref,
            'n_segments': int(D['IC']['n'])}


def test_workload_shape(hcp):
    """The slab is a real sample of the headline workload (nS = 288, ~1.2e8 segments)."""
    assert hcp['K']['wmr'].shape[2] == 288
    assert hcp['n_segments'] > 100_000_000
    assert 0.2 <= hcp['S']['share'] <= 0.6


@pytest.mark.parametrize('arith', ['ff', 'f64'])
def test_fp64_path_matches_reference(hcp, arith):
    from commit_gb300.operator import LinearOperator
    A = LinearOperator(hcp['D'], hcp['K'], None, arith=arith)
    r0, r1 = hcp['rows']
    ax = A.dot(torch.from_numpy(hcp['x']).cuda())
    assert G.rel(ax[r0:r1].cpu().numpy(), hcp['ax_ref']) <= TOL
    aty = A.T.dot(torch.from_numpy(hcp['ym']).cuda()).cpu().numpy()
    assert G.rel(aty, hcp['aty_ref']) <= TOL
    # columns the slab does not touch receive exactly zero
    outside = np.ones(aty.size, bool)
    outside[hcp['S']['cols']] = False
    assert not np.any(aty[outside])


@pytest.mark.parametrize('arith', ['bf16', 'fp16', 'f32'])
def test_reduced_precision_matches_reference(hcp, arith):
    from commit_gb300.operator import LinearOperator
    A = LinearOperator(hcp['D'], hcp['K'], None)
    r0, r1 = hcp['rows']
    ax = A.dot(torch.from_numpy(hcp['x']).cuda().float(), arith=arith)
    assert G.rel(ax[r0:r1].double().cpu().numpy(), hcp['ax_ref']) <= REDUCED_TOL[arith]
    aty = A.T.dot(torch.from_numpy(hcp['ym']).cuda().float(), arith=arith)
    assert G.rel(aty.double().cpu().numpy(), hcp['aty_ref']) <= REDUCED_TOL[arith]


def test_tensor_cores_at_full_workload(hcp):
    """The tensor-core BF16 operator at 1M streamlines (the default there: 212 IC segments per
    voxel) against the CUDA-core BF16 kernels on the same BF16 LUT (1e-4), bitwise
    repeatable."""
    from commit_gb300.operator import LinearOperator
    A = LinearOperator(hcp['D'], hcp['K'], None)
    x = torch.from_numpy(hcp['x']).cuda().float()
    y = torch.from_numpy(hcp['ym']).cuda().float()
    assert A.tensor_cores(None)  # chosen by density
    ax1, ax2 = A.dot(x, arith='bf16'), A.dot(x, arith='bf16')
    g1, g2 = A.T.dot(y, arith='bf16'), A.T.dot(y, arith='bf16')
    A.device_status()
    A.tensor_cores(1)
    axc, gc = A.dot(x, arith='bf16'), A.T.dot(y, arith='bf16')
    assert torch.equal(ax1, ax2) and torch.equal(g1, g2)
    assert G.rel(ax1.double().cpu().numpy(), axc.double().cpu().numpy()) <= 1e-4
    assert G.rel(g1.double().cpu().numpy(), gc.double().cpu().numpy()) <= 1e-4
