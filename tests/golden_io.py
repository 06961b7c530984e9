"""Load the golden fixtures written by tests/golden/make_golden.py."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def case_names():
    """Operator / solver cases (the voxeliser's t2d_*.npz fixtures have their own loader)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, '*.npz'))
                  if not os.path.basename(p).startswith('t2d_'))


def load_case(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False)
    manifest = json.loads(bytes(z['manifest']).decode())
    n, nSTR, nVOX, nE, nISO = [int(v) for v in z['D.counts']]
    D = {'IC': {'str': z['D.IC.str'], 'vox': z['D.IC.vox'], 'dir': z['D.IC.dir'], 'len': z['D.IC.len'],
                'eval': z['D.IC.eval'], 'n': n, 'nSTR': nSTR, 'nVOX': nVOX},
         'EC': {'vox': z['D.EC.vox'], 'dir': z['D.EC.dir'], 'n': nE},
         'ISO': {'vox': z['D.ISO.vox'], 'n': nISO}}
    K = {'wmr': z['K.wmr'], 'wmh': z['K.wmh'], 'iso': z['K.iso']}
    out = {'name': name, 'D': D, 'K': K, 'nolut': manifest['nolut'], 'threads': manifest['threads'],
           'x_in': z['x_in'], 'y_in': z['y_in'], 'y_obs': z['y_obs'], 'Ax': z['ref.Ax'], 'Aty': z['ref.Aty'],
           'fits': {}}
    if 'ref.Ax_mt' in z:
        out['Ax_mt'] = z['ref.Ax_mt']
        out['Aty_mt'] = z['ref.Aty_mt']
    for vname, info in manifest['fits'].items():
        pre = f'fit.{vname}.'
        rp = dict(info['meta'])
        for key in ('lambdaIC',):
            if isinstance(rp.get(key), list):
                rp[key] = tuple(rp[key])
        for k in z.files:
            if not k.startswith(pre + 'reg.'):
                continue
            rest = k[len(pre + 'reg.'):]
            parts = rest.split('.')
            dname, field = parts[0], parts[1]
            rp.setdefault(dname, {})
            if rp[dname] is None:
                rp[dname] = {}
            if field == 'group_idx_kept':
                if parts[2] == 'idx':
                    idx = z[k]
                    sizes = z[pre + f'reg.{dname}.group_idx_kept.size']
                    groups = np.split(idx, np.cumsum(sizes)[:-1])
                    arr = np.empty(len(groups), dtype=object)
                    arr[:] = groups
                    rp[dname]['group_idx_kept'] = arr
            else:
                rp[dname][field] = z[k]
        for dname in ('dictIC_params', 'dictEC_params', 'dictISO_params'):
            rp.setdefault(dname, None)
        conf = z[pre + 'conf'] if pre + 'conf' in z else None
        out['fits'][vname] = {'x': z[pre + 'x'], 'details': info['details'], 'reg': rp, 'conf': conf}
    return out


def fresh_reg(rp: dict) -> dict:
    """A copy of a regularisation input, safe to hand to init_regularisation."""
    out = {}
    for k, v in rp.items():
        out[k] = dict(v) if isinstance(v, dict) else v
    return out


def rel(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
