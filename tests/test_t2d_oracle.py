"""The voxelisation oracle (oracle/trk2dict_oracle.c + the EC / ISO restatement in
oracle/trk2dict.py) against golden vectors made by the reference's own trk2dictionary
(tests/golden/make_t2d_golden.py): bit-exact."""
import glob
import os

import numpy as np
import pytest

import trk2dict as T

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(glob.glob(os.path.join(HERE, 'golden', 't2d_*.npz')))


def load(path):
    z = np.load(path)
    kw = {}
    for k in ('mask', 'blur_apply', 'iso_mask', 'peaks'):
        if k in z:
            kw[k] = z[k]
    if 'blur' in z:
        kw['blur'] = tuple(z['blur'])
    for k in z.files:
        if k.startswith('arg_'):
            v = z[k]
            kw[k[4:]] = tuple(v.tolist()) if v.ndim == 1 else (v if v.ndim == 2 else v.item())
    return z, kw


@pytest.mark.parametrize('path', CASES, ids=[os.path.basename(p)[4:-4] for p in CASES])
def test_oracle_matches_reference_voxelisation(path):
    z, kw = load(path)
    ic_kw = {k: v for k, v in kw.items() if k not in ('peaks', 'iso_mask', 'vf_thr', 'peaks_affine')}
    r = T.voxelise(z['pts'], z['off'], tuple(z['dim']), tuple(z['pix']), z['hash'], **ic_kw)
    for comp in ('IC', 'TRK'):
        for k, a in r[comp].items():
            assert np.array_equal(a, z[f'out_{comp}_{k}']), (comp, k)
    # track density from the merged segments, in the reference's summation order
    tdi = np.zeros(tuple(z['dim']), dtype=np.float64).ravel(order='F')
    np.add.at(tdi, r['IC']['v'].astype(np.int64), r['IC']['len'].astype(np.float64))
    tdi = tdi.reshape(tuple(z['dim']), order='F')
    assert np.array_equal(tdi, z['out_TDI'])
    if 'peaks' in kw:
        v, o = T.ec_entries(tdi, kw['peaks'], z['hash'], kw.get('vf_thr', 0.1), (1, 1, 1), kw.get('peaks_affine'))
        assert np.array_equal(v, z['out_EC_v']) and np.array_equal(o, z['out_EC_o'])
    else:
        assert z['out_EC_v'].size == 0
    iso = T.iso_voxels(tdi, kw.get('mask'), kw.get('iso_mask'))
    assert np.array_equal(iso, z['out_ISO_v'])


@pytest.mark.skipif(not T.ref_available(), reason='reference voxeliser not built (needs the reference tree)')
def test_oracle_matches_reference_on_fresh_streamlines(tmp_path):
    import sys
    sys.path.insert(0, os.path.join(HERE, 'golden'))
    import make_t2d_golden as M
    dim, pix = (24, 20, 12), (1.0, 1.5, 2.5)
    pts, off = M.streamlines(400, dim, pix, seed=77)
    th = np.deg2rad(np.arange(181.0))[:, None]
    ph = np.deg2rad(np.arange(181.0))[None, :]
    v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th) + 0 * ph], -1).reshape(-1, 3)
    H = np.abs(v @ M.directions(300, 5).T).argmax(1).astype(np.int16)
    for kw in (dict(), dict(do_intersect=False, min_fiber_len=3.0)):
        a = T.voxelise(pts, off, dim, pix, H, **kw)
        b = T.reference_voxelise(str(tmp_path / 'ref'), pts, off, dim, pix, H, **kw)
        for comp in ('IC', 'TRK'):
            for k in a[comp]:
                assert np.array_equal(a[comp][k], b[comp][k]), (comp, k)
