"""Generate the golden fixtures in tests/golden/ from the reference implementation itself.

Runs only where the reference tree and Cython are present: builds oracle/_ref (the
reference's generated C operator, plus its Cython proximals) with oracle/build_ref.py,
imports the reference ``commit/solvers.py`` against that build, and records, on small
seeded synthetic problems:

* A*x and A'*y of the reference operator (commit/operator/operator.pyx:114-184) for
  random x and y, with 1 and several CPU threads (partitions from core.pyx:586-724);
* ``solvers.solve`` outputs (x and fit details, solvers.py:218-391) for the regularisers
  of ``init_regularisation`` (solvers.py:16-206), with lambdas set the way
  ``Evaluation.set_regularisation`` sets them (core.pyx:961-976, 1146-1192).

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))

import build_ref  # noqa: E402
import oracle as O  # noqa: E402
from commit_gb300 import synth  # noqa: E402


def _small(**kw):
    base = dict(dim=(10, 10, 6), n_mask=420, n_fibers=90, ndirs=60, n_b0=2, shells=[(1000.0, 14)], seed=7)
    base.update(kw)
    return synth.ProblemSpec(**base)


def golden_cases():
    """Small seeded problems covering the operator's shapes and edge cases."""
    cases = []
    D, K = synth.make_dictionary(_small())
    cases.append(dict(name='szb', D=D, K=K, nolut=False, seed=7, threads=4, fista=True, max_iter=300))

    D, K = synth.make_dictionary(_small(seed=11, n_ic=3, d_perps=(0.51e-3, 0.3e-3), d_isos=(1.7e-3, 3.0e-3, 0.8e-3)))
    cases.append(dict(name='multi_rf', D=D, K=K, nolut=False, seed=11, threads=3, fista=True, max_iter=150))

    # ball-and-stick: EC peaks in the dictionary but no EC response (tests/test_demo.py:52-83)
    D, K = synth.make_dictionary(_small(seed=13))
    K['wmh'] = np.zeros((0,) + K['wmh'].shape[1:], dtype=np.float32)
    cases.append(dict(name='ball_stick', D=D, K=K, nolut=False, seed=13, threads=2, fista=True, max_iter=150))

    # per-column eval mask with zeros (the debias operator, core.pyx:1481-1486) and
    # voxels with EC/ISO but no IC segments (use_all_voxels_in_mask=True)
    D, K = synth.make_dictionary(_small(seed=17))
    r = np.random.default_rng(17)
    D['IC']['eval'] = (r.uniform(size=D['IC']['nSTR'] * K['wmr'].shape[0]) > 0.3).astype(np.uint32)
    nV = D['IC']['nVOX']
    newv = lambda v: (v + v // 3).astype(np.uint32)
    nV2 = int(newv(np.array([nV - 1]))[0]) + 2
    D['IC']['vox'] = newv(D['IC']['vox'])
    D['IC']['nVOX'] = nV2
    ecn = r.integers(0, 4, size=nV2)
    D['EC'] = {'vox': np.repeat(np.arange(nV2, dtype=np.uint32), ecn),
               'dir': r.integers(0, 60, size=int(ecn.sum())).astype(np.uint16), 'n': int(ecn.sum())}
    D['ISO'] = {'vox': np.arange(nV2, dtype=np.uint32), 'n': nV2}
    cases.append(dict(name='eval_gaps', D=D, K=K, nolut=False, seed=17, threads=3, fista=True, max_iter=150))

    # ScalarMap-like: one sample, one direction, unit IC LUT and a negative ISO LUT
    # (commit/models.pyx:75-80); the same dictionary through the nolut kernels
    D, K = synth.make_dictionary(_small(seed=19, ndirs=1, d_perps=()))
    K = {'wmr': np.ones((1, 1, 1), np.float32), 'wmh': np.ones((0, 1, 1), np.float32),
         'iso': -np.ones((1, 1), np.float32)}
    cases.append(dict(name='scalar_map', D=D, K=K, nolut=False, seed=19, threads=2, fista=True, max_iter=100))
    K2 = {'wmr': np.ones((1, 1, 1), np.float32), 'wmh': np.ones((0, 1, 1), np.float32),
          'iso': np.ones((1, 1), np.float32)}
    cases.append(dict(name='nolut', D=D, K=K2, nolut=True, seed=19, threads=2, fista=True, max_iter=100))
    for c in cases:
        c['D']['IC'].setdefault('eval', np.ones(c['D']['IC']['nSTR'] * c['K']['wmr'].shape[0], dtype=np.uint32))
    return cases


DICT_KEYS = [('IC', 'str'), ('IC', 'vox'), ('IC', 'dir'), ('IC', 'len'), ('IC', 'eval'), ('EC', 'vox'), ('EC', 'dir'),
             ('ISO', 'vox')]


def load_reference_solvers():
    build_ref.main(['--python'])
    sys.path.insert(0, build_ref.PY_DIR)
    import commit.proximals  # noqa: F401  (the compiled reference proximals.pyx)
    path = os.path.join(build_ref.reference_root(), 'commit', 'solvers.py')
    spec = importlib.util.spec_from_file_location('commit.solvers', path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules['commit.solvers'] = mod
    spec.loader.exec_module(mod)
    return mod


def lambda_max_lasso(At, y, start, size, w):
    Aty = np.asarray(At.dot(y))
    return float(np.max(np.abs(Aty[start:start + size]) / w))


def lambda_max_group(At, y, w_group, groups):
    Aty = np.asarray(At.dot(y))
    return float(max(np.sqrt(np.sum(Aty[g] ** 2)) / w_group[k] for k, g in enumerate(groups)))


def regularisation_variants(D, K, A, y, rng):
    """(name, regularisation dict input, confidence) triples covering init_regularisation."""
    base = O.reg_params(D, K)
    nF = base['sizeIC']
    out = []
    out.append(('nnls', dict(base), None))
    out.append(('unconstrained', dict(base, nnIC=False, nnEC=False, nnISO=False), None))
    lm = lambda_max_lasso(A.T, y, 0, nF, np.ones(nF))
    out.append(('lasso_ic_nn', dict(base, regIC='lasso', lambdaIC=0.05 * lm), None))
    out.append(('lasso_ic_free', dict(base, regIC='lasso', lambdaIC=0.02 * lm, nnIC=False), None))
    w = rng.uniform(0.5, 2.0, size=nF)
    lmw = lambda_max_lasso(A.T, y, 0, nF, w)
    out.append(('lasso_ic_weighted', dict(base, regIC='lasso', lambdaIC=0.05 * lmw,
                                          dictIC_params={'coeff_weights_kept': w}), None))
    # non-overlapping groups: a random partition of the streamlines into 8 bundles
    perm = rng.permutation(nF)
    groups = [np.sort(g).astype(np.int32) for g in np.array_split(perm, 8)]
    gw = np.sqrt(np.array([g.size for g in groups], dtype=np.float64))
    lg = lambda_max_group(A.T, y, gw, groups)
    gobj = np.empty(len(groups), dtype=object)
    gobj[:] = groups
    out.append(('group_lasso', dict(base, regIC='group_lasso', lambdaIC=0.1 * lg,
                                    dictIC_params={'group_idx_kept': gobj, 'group_weights': gw}), None))
    # hierarchical (overlapping) groups: two children then their union, in that order
    h = [groups[0], groups[1], np.sort(np.concatenate([groups[0], groups[1]])).astype(np.int32)] + groups[2:]
    hobj = np.empty(len(h), dtype=object)
    hobj[:] = h
    hw = np.sqrt(np.array([g.size for g in h], dtype=np.float64))
    out.append(('group_lasso_hier', dict(base, regIC='group_lasso', lambdaIC=0.1 * lg, nnIC=False,
                                         dictIC_params={'group_idx_kept': hobj, 'group_weights': hw}), None))
    out.append(('sparse_group_lasso', dict(base, regIC='sparse_group_lasso', lambdaIC=(0.02 * lm, 0.05 * lg),
                                           dictIC_params={'group_idx_kept': gobj, 'group_weights': gw}), None))
    out.append(('sparse_group_lasso_w', dict(base, regIC='sparse_group_lasso', lambdaIC=(0.02 * lmw, 0.05 * lg),
                                             dictIC_params={'group_idx_kept': gobj, 'group_weights': gw,
                                                            'coeff_weights_kept': w}), None))
    if base['sizeEC'] > 0:
        le = lambda_max_lasso(A.T, y, base['startEC'], base['sizeEC'], np.ones(base['sizeEC']))
        out.append(('lasso_ec', dict(base, regEC='lasso', lambdaEC=0.05 * le), None))
    if base['sizeISO'] > 0:
        li = lambda_max_lasso(A.T, y, base['startISO'], base['sizeISO'], np.ones(base['sizeISO']))
        out.append(('lasso_iso', dict(base, regISO='lasso', lambdaISO=0.05 * li, nnISO=False), None))
        wi = rng.uniform(0.5, 2.0, size=base['sizeISO'])
        out.append(('lasso_iso_weighted', dict(base, regISO='lasso', lambdaISO=0.05 * li,
                                               dictISO_params={'coeff_weights': wi}), None))
    conf = rng.uniform(0.2, 1.0, size=A.nROWS).astype(np.float32)
    out.append(('nnls_confidence', dict(base), conf))
    return out


def pack_reg(rp: dict) -> dict:
    """Arrays of a regularisation input as flat npz entries (groups as idx + sizes)."""
    arrs = {}
    meta = {}
    for k, v in rp.items():
        if k in ('dictIC_params', 'dictEC_params', 'dictISO_params'):
            if v is None:
                continue
            for kk, vv in v.items():
                if kk in ('group_idx_kept',):
                    arrs[f'{k}.{kk}.idx'] = np.concatenate(list(vv)).astype(np.int32)
                    arrs[f'{k}.{kk}.size'] = np.array([g.size for g in vv], dtype=np.int32)
                else:
                    arrs[f'{k}.{kk}'] = np.asarray(vv)
        else:
            meta[k] = list(v) if isinstance(v, tuple) else v
    return arrs, meta


def main():
    ref_solvers = load_reference_solvers()
    for case in golden_cases():
        name, D, K, nolut = case['name'], case['D'], case['K'], case['nolut']
        rng = np.random.default_rng(case['seed'] + 100)
        T1 = O.set_threads(D, 1)
        A = O.RefOperator(D, K, T1, nolut=nolut)
        x_in = rng.uniform(-0.5, 1.0, size=A.nCOLS)
        y_in = rng.normal(size=A.nROWS)
        rec = {}
        rec['Ax'] = A.dot(x_in)
        rec['Aty'] = A.T.dot(y_in)
        nt = case['threads']
        if nt > 1:
            Tn = O.set_threads(D, nt)
            An = O.RefOperator(D, K, Tn, nolut=nolut)
            rec['Ax_mt'] = An.dot(x_in)
            rec['Aty_mt'] = An.T.dot(y_in)
        # observed signal for the fits
        y_obs = synth.make_signal(A.dot(synth.make_x(A.nCOLS, case['seed'] + 1)), case['seed'] + 2)
        fits = {}
        if case['fista']:
            for vname, rp, conf in regularisation_variants(D, K, A, y_obs, rng):
                rp_in = {k: (dict(v) if isinstance(v, dict) else v) for k, v in rp.items()}
                reg = ref_solvers.init_regularisation(dict(rp_in))
                xs, det = ref_solvers.solve(y_obs, A, A.T, tol_fun=1e-5, tol_x=1e-7, max_iter=case['max_iter'],
                                            verbose=0, regularisation=reg, confidence_array=conf)
                arrs, meta = pack_reg(rp_in)
                fits[vname] = {'x': xs, 'details': det, 'arrs': arrs, 'meta': meta, 'conf': conf}
        out = {'x_in': x_in, 'y_in': y_in, 'y_obs': y_obs}
        for a, b in DICT_KEYS:
            out[f'D.{a}.{b}'] = np.asarray(D[a][b])
        for k in ('wmr', 'wmh', 'iso'):
            out[f'K.{k}'] = K[k]
        out['D.counts'] = np.array([D['IC']['n'], D['IC']['nSTR'], D['IC']['nVOX'], D['EC']['n'], D['ISO']['n']],
                                   dtype=np.int64)
        for k, v in rec.items():
            out['ref.' + k] = v
        manifest = {'name': name, 'nolut': nolut, 'threads': nt, 'fits': {}}
        for vname, f in fits.items():
            out[f'fit.{vname}.x'] = f['x']
            if f['conf'] is not None:
                out[f'fit.{vname}.conf'] = f['conf']
            for k, v in f['arrs'].items():
                out[f'fit.{vname}.reg.{k}'] = v
            det = {k: (float(v) if not isinstance(v, str) and k != 'iterations' else v) for k, v in f['details'].items()}
            det['iterations'] = int(f['details']['iterations'])
            manifest['fits'][vname] = {'details': det, 'meta': f['meta']}
        out['manifest'] = np.frombuffer(json.dumps(manifest).encode(), dtype=np.uint8)
        path = os.path.join(HERE, f'{name}.npz')
        np.savez_compressed(path, **out)
        print(f'{name}: {os.path.getsize(path) / 1024:.0f} KB, {len(fits)} fits,',
              ', '.join(f"{k}:{v['details']['iterations']}" for k, v in manifest['fits'].items()))


if __name__ == '__main__':
    main()
