"""Evaluation.load_dictionary's re-layout on the device (cgb_dict_relayout) against the numpy
restatement (commit/core.pyx:493-580), on dictionaries made by the reference's own
trk2dictionary (the t2d_* golden outputs, written out as dictionary_*.dict files).

Bar: identical arrays (stable sort by voxel, FP32 length normalisation, voxel re-index),
and an operator built from the device arrays gives the same products as one built from
the host arrays.
"""
import glob
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
T2D = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, 't2d_*.npz')))


def _write(z, path):
    from commit_gb300 import dictionary
    raw = {'IC': {'str': z['out_IC_f'], 'vox': z['out_IC_v'], 'dir': z['out_IC_o'], 'len': z['out_IC_len']},
           'EC': {'vox': z['out_EC_v'], 'dir': z['out_EC_o']},
           'ISO': {'vox': z['out_ISO_v']},
           'TRK': {'norm': z['out_TRK_norm'], 'kept': z['out_TRK_kept']}}
    dictionary.write_dictionary(path, raw)
    return (z['out_TDI'] > 0).astype(np.uint8)


@pytest.mark.parametrize('name', T2D)
@pytest.mark.parametrize('normalize', [True, False])
def test_device_relayout_matches_host(name, normalize, tmp_path):
    from commit_gb300 import dictionary
    z = np.load(os.path.join(GOLDEN, name + '.npz'))
    mask = _write(z, str(tmp_path))
    H = dictionary.load_dictionary(str(tmp_path), mask, normalize_kernels=normalize)
    Dd = dictionary.load_dictionary(str(tmp_path), mask, normalize_kernels=normalize, device=0)
    assert isinstance(Dd['IC']['vox'], torch.Tensor) and Dd['IC']['vox'].is_cuda
    D = dictionary.to_host(Dd)
    for comp, keys in (('IC', ('str', 'vox', 'dir', 'len')), ('EC', ('vox', 'dir')), ('ISO', ('vox',))):
        for k in keys:
            assert D[comp][k].dtype == H[comp][k].dtype, (comp, k)
            assert np.array_equal(D[comp][k], H[comp][k]), (comp, k)
    for k in ('n', 'nSTR', 'nVOX'):
        assert D['IC'][k] == H['IC'][k]
    assert D['EC']['n'] == H['EC']['n'] and D['ISO']['n'] == H['ISO']['n']


@pytest.mark.parametrize('name', T2D)
def test_operator_from_device_dictionary(name, tmp_path):
    """The device arrays go to cgb_op_create without a host round trip and define the same A."""
    from commit_gb300 import dictionary
    from commit_gb300.operator import LinearOperator
    z = np.load(os.path.join(GOLDEN, name + '.npz'))
    mask = _write(z, str(tmp_path))
    H = dictionary.load_dictionary(str(tmp_path), mask)
    Dd = dictionary.load_dictionary(str(tmp_path), mask, device=0)
    ndirs = int(max(z['out_IC_o'].max(initial=0), z['out_EC_o'].max(initial=0))) + 1
    rng = np.random.default_rng(0)
    K = {'wmr': rng.uniform(0.1, 1.0, (1, ndirs, 12)).astype(np.float32),
         'wmh': rng.uniform(0.1, 1.0, (1, ndirs, 12)).astype(np.float32),
         'iso': rng.uniform(0.1, 1.0, (2, 12)).astype(np.float32)}
    for D in (H, Dd):
        D['IC']['eval'] = np.ones(H['IC']['nSTR'], np.uint32)
    Ah = LinearOperator(H, K, None)
    Ad = LinearOperator(Dd, K, None)
    for A in (Ah, Ad):  # one voxel shape for both (the timed choice may differ, and so would the sum order)
        A.ff_shape(1)
    x = rng.uniform(0.0, 1.0, Ah.nCOLS)
    y = rng.normal(size=Ah.nROWS)
    assert np.array_equal(Ah.dot(x), Ad.dot(x))
    assert np.array_equal(Ah.T.dot(y), Ad.T.dot(y))


def test_voxel_outside_the_grid_is_rejected(tmp_path):
    from commit_gb300 import dictionary
    from commit_gb300._lib import CgbError
    z = dict(np.load(os.path.join(GOLDEN, T2D[0] + '.npz')))
    v = z['out_IC_v'].copy()
    v[0] = np.uint32(z['out_TDI'].size + 7)
    z['out_IC_v'] = v
    mask = _write(z, str(tmp_path))
    with pytest.raises(CgbError, match='outside the grid'):
        dictionary.load_dictionary(str(tmp_path), mask, device=0)
