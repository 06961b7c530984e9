"""Golden vectors for the streamline voxeliser, produced by the reference itself.

Runs the reference's trk2dictionary (commit/trk2dictionary/trk2dictionary_c.cpp, compiled
into oracle/_ref by oracle/build_ref.py) on seeded synthetic streamlines written as a .trk
file, and stores inputs and outputs in tests/golden/t2d_<case>.npz.  Run in a container
that has the reference tree:  python tests/golden/make_t2d_golden.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, 'oracle'))
import trk2dict as T  # noqa: E402


def streamlines(n, dim, pix, seed):
    """Random smooth curves of 1-120 points (steps of 0.7 mm), some leaving the grid."""
    rng = np.random.default_rng(seed)
    ext = np.array(dim) * np.array(pix)
    pts, off = [], [0]
    for _ in range(n):
        N = int(rng.integers(1, 120))
        p = rng.uniform(0.1, 0.9, 3) * ext
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        P = []
        for _ in range(N):
            P.append(p.copy())
            d = d + 0.3 * rng.normal(size=3)
            d /= np.linalg.norm(d)
            p = p + 0.7 * d
        pts.append(np.array(P, np.float32))
        off.append(off[-1] + N)
    return np.concatenate(pts), np.array(off, dtype=np.int64)


def directions(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[d[:, 1] < 0] *= -1
    return d


def case(name, seed, **kw):
    dim, pix = (20, 18, 16), (1.25, 1.25, 2.0)
    pts, off = streamlines(300, dim, pix, seed)
    rng = np.random.default_rng(seed + 100)
    dirs = directions(500, seed + 200)
    th = np.deg2rad(np.arange(181.0))[:, None]
    ph = np.deg2rad(np.arange(181.0))[None, :]
    v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th) + 0 * ph], -1).reshape(-1, 3)
    H = np.abs(v @ dirs.T).argmax(1).astype(np.int16)
    args = dict(kw)
    if args.pop('with_mask', False):
        args['mask'] = (rng.uniform(size=dim) > 0.1).astype(np.float32)
    if args.pop('with_peaks', False):
        pk = rng.normal(size=dim + (3, 3)).astype(np.float32)
        pk[rng.uniform(size=dim + (3,)) < 0.3] = 0
        args['peaks'] = pk
    if args.pop('with_iso_mask', False):
        args['iso_mask'] = (rng.uniform(size=dim) > 0.2).astype(np.float32)
    with tempfile.TemporaryDirectory() as tmp:
        r = T.reference_voxelise(tmp, pts, off, dim, pix, H, **args)
    save = {'pts': pts, 'off': off, 'dim': np.array(dim), 'pix': np.array(pix, np.float32), 'hash': H}
    for k in ('mask', 'peaks', 'iso_mask', 'blur_apply'):
        if k in args:
            save[k] = np.asarray(args[k])
    if 'blur' in args:
        save['blur'] = np.stack([np.asarray(a, np.float64) for a in args['blur']])
    for k in ('fiber_shift', 'min_fiber_len', 'max_fiber_len', 'do_intersect', 'vf_thr', 'peaks_affine'):
        if k in args:
            save['arg_' + k] = np.asarray(args[k])
    for comp in ('IC', 'TRK', 'EC', 'ISO'):
        for k, a in r[comp].items():
            save[f'out_{comp}_{k}'] = a
    save['out_TDI'] = r['TDI']
    np.savez_compressed(os.path.join(HERE, f't2d_{name}.npz'), **save)
    print(name, 'segments', r['IC']['f'].size, 'kept', int(r['TRK']['kept'].sum()), 'EC', r['EC']['v'].size,
          'ISO', r['ISO']['v'].size)


if __name__ == '__main__':
    if not T.ref_available():
        sys.exit('oracle/_ref/libt2d_ref.so missing: run oracle/build_ref.py with the reference tree present')
    case('intersect_mask_peaks', 1, with_mask=True, with_peaks=True, vf_thr=0.2)
    case('plain_blur_limits', 2, do_intersect=False, min_fiber_len=5.0, max_fiber_len=40.0,
         blur=(np.array([0.0, 0.5, 0.5, 1.0]), np.array([0.0, 0.3, 2.0, 4.0]), np.array([1.0, 0.6, 0.4, 0.0005])),
         blur_apply=(np.arange(300) % 3 != 0).astype(np.uint8))
    case('shift_isomask_affine', 3, fiber_shift=(0.5, -0.25, 0.5), with_iso_mask=True, with_peaks=True,
         peaks_affine=np.array([[0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, -1.0]]))
