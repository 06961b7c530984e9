"""Device voxeliser (cgb_trk2dict) against the reference's own trk2dictionary outputs
(golden vectors) and the oracle: IC segments, streamline norms / lengths / kept flags, EC
entries and ISO voxels bit-exact; the track-density image (FP64 atomics, order-dependent)
to 1e-12 relative."""
import glob
import os

import numpy as np
import pytest

import trk2dict as T

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(glob.glob(os.path.join(HERE, 'golden', 't2d_*.npz')))


@pytest.mark.parametrize('path', CASES, ids=[os.path.basename(p)[4:-4] for p in CASES])
def test_device_voxeliser_matches_reference(path):
    from commit_gb300 import trk2dictionary as V
    from test_t2d_oracle import load
    z, kw = load(path)
    r = V.voxelise(z['pts'], z['off'], tuple(z['dim']), tuple(z['pix']), z['hash'], **kw)
    for comp in ('IC', 'TRK', 'EC', 'ISO'):
        for k, a in r[comp].items():
            assert np.array_equal(a, z[f'out_{comp}_{k}']), (comp, k)
    ref = z['out_TDI']
    assert np.allclose(r['TDI'], ref, rtol=1e-12, atol=0) and np.array_equal(r['TDI'] != 0, ref != 0)


def test_device_voxeliser_matches_oracle_at_scale():
    """20k streamlines of up to 300 points on a 64^3 grid: IC / TRK bit-exact vs the oracle."""
    import sys
    sys.path.insert(0, os.path.join(HERE, 'golden'))
    import make_t2d_golden as M
    from commit_gb300 import trk2dictionary as V
    dim, pix = (64, 64, 64), (1.0, 1.0, 1.0)
    pts, off = M.streamlines(20000, dim, pix, seed=9)
    H = V.hash_table(M.directions(500, 4))
    a = V.voxelise(pts, off, dim, pix, H)
    b = T.voxelise(pts, off, dim, pix, H)
    for comp in ('IC', 'TRK'):
        for k in b[comp]:
            assert np.array_equal(a[comp][k], b[comp][k]), (comp, k)


def test_voxelised_dictionary_loads_into_the_operator(tmp_path):
    """voxelise -> .dict files -> load_dictionary -> LinearOperator, checked against the oracle."""
    import oracle as O
    from commit_gb300 import dictionary, synth
    from commit_gb300 import trk2dictionary as V
    from commit_gb300.operator import LinearOperator
    z, kw = load_case('intersect_mask_peaks')
    r = V.voxelise(z['pts'], z['off'], tuple(z['dim']), tuple(z['pix']), z['hash'], **kw)
    V.write(str(tmp_path), r)
    D = dictionary.load_dictionary(str(tmp_path), r['TDI'] > 0)
    dirs = np.random.default_rng(0).normal(size=(500, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    bvals, bvecs = synth.make_scheme(2, [(1000.0, 12)])
    K = synth.szb_kernels(bvals, bvecs, dirs)
    A = LinearOperator(D, K, None)
    P = O.PortOperator(D, K, None)
    x = np.random.default_rng(1).uniform(0, 1, A.nCOLS)
    y = A.dot(x)
    assert np.linalg.norm(y - P.dot(x)) <= 1e-10 * np.linalg.norm(P.dot(x))


def load_case(name):
    from test_t2d_oracle import load
    return load(os.path.join(HERE, 'golden', f't2d_{name}.npz'))


def test_voxeliser_edge_cases():
    """No streamlines; streamlines of 0, 1, 2 points (no segments, not kept); a streamline
    entirely outside the grid; identical to the oracle in every case."""
    from commit_gb300 import trk2dictionary as V
    dim, pix = (8, 8, 8), (1.0, 1.0, 1.0)
    H = V.hash_table(np.eye(3))
    r = V.voxelise(np.zeros((0, 3), np.float32), np.array([0]), dim, pix, H)
    assert r['IC']['f'].size == 0 and r['TRK']['kept'].size == 0 and not r['TDI'].any()
    pts = np.array([[1.5, 1.5, 1.5],                                   # 1 point
                    [2.2, 2.1, 2.0], [2.9, 2.5, 2.4],                   # 2 points
                    [20.0, 20.0, 20.0], [21.0, 20.5, 20.0], [22.0, 21.0, 20.0],   # outside
                    [0.5, 0.5, 0.5], [1.7, 0.9, 0.6], [2.9, 1.4, 0.8], [3.6, 2.2, 1.5]],  # inside
                   np.float32)
    off = np.array([0, 0, 1, 3, 6, 10])                                 # first streamline empty
    a = V.voxelise(pts, off, dim, pix, H)
    b = T.voxelise(pts, off, dim, pix, H)
    for comp in ('IC', 'TRK'):
        for k in b[comp]:
            assert np.array_equal(a[comp][k], b[comp][k]), (comp, k)
    assert list(a['TRK']['kept']) == [0, 0, 0, 0, 1]
    assert set(np.unique(a['IC']['f'])) == {0}
