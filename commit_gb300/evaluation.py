"""The operator's callers in COMMIT's Evaluation, on the GB300 path.

``set_regularisation`` restates Evaluation.set_regularisation (commit/core.pyx:861-1192):
compartment ranges, parameter checks, group re-indexing to kept streamlines, group
weights (cardinality, adaptive, extra), and lambda = fraction * lambda_max with
lambda_max from one A'y (Kim et al. for lasso, Yuan & Lin for groups, core.pyx:961-976).
``fit`` restates Evaluation.fit's solver and debias logic (core.pyx:1353-1519) without the
NIfTI I/O: solve, then optionally mask IC columns with x < 1e-15, rebuild the operator
with that eval mask, binarise A*x_debias into a mask of y, and solve again without a
regulariser.  Arrays (DICTIONARY, KERNELS, y, confidence) are passed in directly.
"""
from __future__ import annotations

import numpy as np
import torch

from . import solvers
from .operator import LinearOperator


def _Aty(A: LinearOperator, y):
    r = A.T.dot(y)
    return r.cpu().numpy() if isinstance(r, torch.Tensor) else np.asarray(r)


def lambda_max_lasso(A, y, start, size, w_coeff):
    """core.pyx:961-966."""
    Aty = _Aty(A, y)
    return float(np.max(np.abs(Aty[start:start + size]) / w_coeff))


def lambda_max_group(A, y, w_group, idx_group):
    """core.pyx:968-976."""
    Aty = _Aty(A, y)
    return float(max(np.sqrt(np.sum(Aty[np.asarray(g)] ** 2)) / w_group[k] for k, g in enumerate(idx_group)))


def set_regularisation(A: LinearOperator, y, DICTIONARY, KERNELS, regularisers=(None, None, None),
                       lambdas=(None, None, None), is_nonnegative=(True, True, True), params=(None, None, None),
                       x_nnls=None):
    """Regularisation dict as Evaluation.set_regularisation builds it, passed through
    commit_gb300.solvers.init_regularisation."""
    nIC_rf, nEC_rf, nISO_rf = KERNELS['wmr'].shape[0], KERNELS['wmh'].shape[0], KERNELS['iso'].shape[0]
    nSTR = DICTIONARY['IC']['nSTR']
    kept = DICTIONARY.get('TRK', {}).get('kept')
    if kept is None:
        kept = np.ones(nSTR, dtype=np.uint8)
    reg = {'startIC': 0, 'sizeIC': int(nSTR * nIC_rf)}
    reg['startEC'] = reg['sizeIC']
    reg['sizeEC'] = int(DICTIONARY['EC']['n'] * nEC_rf)
    reg['startISO'] = reg['sizeIC'] + reg['sizeEC']
    reg['sizeISO'] = int(DICTIONARY['ISO']['n'] * nISO_rf)
    reg['regIC'], reg['regEC'], reg['regISO'] = regularisers
    reg['nnIC'], reg['nnEC'], reg['nnISO'] = is_nonnegative
    dIC, dEC, dISO = [dict(p) if p is not None else None for p in params]
    allowed = ['group_idx', 'group_weights_cardinality', 'group_weights_adaptive', 'group_weights_extra',
               'coeff_weights', 'group_weights', 'group_idx_kept', 'coeff_weights_kept']
    if dIC is not None:
        for k in dIC:
            if k not in allowed:
                raise ValueError(f'Unexpected key "{k}" in the IC parameters')

    # ---- IC (core.pyx:1050-1206)
    rIC = reg['regIC']
    if rIC in ('lasso', 'group_lasso'):
        if lambdas[0] is None:
            raise ValueError('Missing regularisation parameter for the IC compartment')
        if lambdas[0] < 0:
            raise ValueError('Regularisation parameter for the IC compartment must be greater than 0')
        reg['lambdaIC_perc'] = lambdas[0]
    elif rIC == 'sparse_group_lasso':
        if len(lambdas[0]) != 2:
            raise ValueError('Regularisation parameters for the IC compartment ara not exactly two')
        if lambdas[0][0] < 0 or lambdas[0][1] < 0:
            raise ValueError('Regularisation parameters for the IC compartment must be greater than 0')
        reg['lambdaIC_perc'] = lambdas[0]
    elif rIC is not None:
        raise ValueError('Regularisation not in the list')
    if rIC in ('group_lasso', 'sparse_group_lasso') and (dIC is None or dIC.get('group_idx') is None):
        raise ValueError('Group structure for the IC compartment not provided')
    if rIC in ('lasso', 'sparse_group_lasso') and dIC is not None and 'coeff_weights' in dIC:
        cw = np.asarray(dIC['coeff_weights'], dtype=np.float64)
        if np.any(cw < 0):
            raise ValueError('All coefficients weights must be non-negative')
        if cw.size != kept.size:
            raise ValueError('"coeff_weights" must have the same size as the number of elements in the IC compartment')
        dIC['coeff_weights_kept'] = cw[kept == 1]
    if rIC in ('group_lasso', 'sparse_group_lasso'):
        dIC.setdefault('group_weights_cardinality', True)
        dIC.setdefault('group_weights_adaptive', True)
        for key in ('group_weights_cardinality', 'group_weights_adaptive'):
            v = dIC[key]
            if isinstance(v, str):
                if v.lower() not in ('true', 'false'):
                    raise ValueError(f'"{key}" must be a boolean or a string')
                dIC[key] = v.lower() == 'true'
            elif not isinstance(v, bool):
                raise ValueError(f'"{key}" must be a boolean or a string')
        groups = [np.asarray(g, dtype=np.int64) for g in dIC['group_idx']]
        all_in = np.sort(np.unique(np.concatenate(groups)))
        if all_in.size != kept.size or np.any(all_in != np.arange(kept.size)):
            raise ValueError('Group indices must contain all the indices of the input streamlines')
        groups = [g for g in groups if g.size > 0]
        if 'group_weights_extra' in dIC:
            w = np.array(dIC['group_weights_extra'], dtype=np.float64)
            if np.any(w < 0):
                raise ValueError('All group weights must be non-negative')
            if w.size != len(groups):
                raise ValueError('Group weights and group indices must have the same size')
        else:
            w = np.ones(len(groups), dtype=np.float64)
        # re-index groups to the kept streamlines (core.pyx:1132-1157)
        if 0 in kept:
            idx_in_kept = np.full(kept.size, -1, dtype=np.int64)
            idx_in_kept[kept == 1] = np.arange(nSTR)
            new_g, new_w = [], []
            for k, g in enumerate(groups):
                g = idx_in_kept[g]
                g = g[g != -1]
                if g.size > 0:
                    new_g.append(g)
                    new_w.append(w[k])
            groups, w = new_g, np.array(new_w, dtype=np.float64)
        if dIC['group_weights_cardinality']:
            w = w * np.sqrt(np.array([g.size for g in groups], dtype=np.float64))
        if dIC['group_weights_adaptive']:
            if x_nnls is None:
                raise ValueError('Group weights cannot be computed if the fit without regularisation has not been '
                                 'performed before')
            w = w / np.array([np.linalg.norm(x_nnls[g]) + 1e-12 for g in groups], dtype=np.float64)
        arr = np.empty(len(groups), dtype=object)
        arr[:] = [g.astype(np.int32) for g in groups]
        dIC['group_idx_kept'] = arr
        dIC['group_weights'] = w
    reg['dictIC_params'] = dIC
    ones_ic = np.ones(reg['sizeIC'], dtype=np.float64)
    if rIC == 'lasso':
        wc = dIC['coeff_weights_kept'] if dIC is not None and 'coeff_weights_kept' in dIC else ones_ic
        reg['lambdaIC_max'] = lambda_max_lasso(A, y, reg['startIC'], reg['sizeIC'], wc)
        reg['lambdaIC'] = reg['lambdaIC_perc'] * reg['lambdaIC_max']
    elif rIC == 'group_lasso':
        reg['lambdaIC_max'] = lambda_max_group(A, y, dIC['group_weights'], dIC['group_idx_kept'])
        reg['lambdaIC'] = reg['lambdaIC_perc'] * reg['lambdaIC_max']
    elif rIC == 'sparse_group_lasso':
        wc = dIC['coeff_weights_kept'] if 'coeff_weights_kept' in dIC else ones_ic
        reg['lambdaIC_max'] = (lambda_max_lasso(A, y, reg['startIC'], reg['sizeIC'], wc),
                               lambda_max_group(A, y, dIC['group_weights'], dIC['group_idx_kept']))
        reg['lambdaIC'] = (reg['lambdaIC_perc'][0] * reg['lambdaIC_max'][0],
                           reg['lambdaIC_perc'][1] * reg['lambdaIC_max'][1])

    # ---- EC (core.pyx:1247-1294)
    if reg['regEC'] == 'lasso':
        if reg['sizeEC'] == 0:
            raise ValueError('No extracellular compartment found in the dictionary')
        if lambdas[1] is None or lambdas[1] < 0:
            raise ValueError('Regularisation parameter for the EC compartment must be greater than 0')
        reg['lambdaEC_perc'] = lambdas[1]
        reg['lambdaEC_max'] = lambda_max_lasso(A, y, reg['startEC'], reg['sizeEC'], np.ones(reg['sizeEC']))
        reg['lambdaEC'] = reg['lambdaEC_perc'] * reg['lambdaEC_max']
    elif reg['regEC'] is not None:
        raise ValueError('Not yet implemented')
    reg['dictEC_params'] = dEC

    # ---- ISO (core.pyx:1308-1356)
    if reg['regISO'] == 'lasso':
        if reg['sizeISO'] == 0:
            raise ValueError('No isotropic compartment found in the dictionary')
        if lambdas[2] is None or lambdas[2] < 0:
            raise ValueError('Regularisation parameter for the ISO compartment must be greater than 0')
        reg['lambdaISO_perc'] = lambdas[2]
        if dISO is not None and 'coeff_weights' in dISO:
            if np.asarray(dISO['coeff_weights']).size != reg['sizeISO']:
                raise ValueError('"coeff_weights" must have the same size as the ISO compartment')
            wc = np.asarray(dISO['coeff_weights'], dtype=np.float64)
        else:
            wc = np.ones(reg['sizeISO'])
        reg['lambdaISO_max'] = lambda_max_lasso(A, y, reg['startISO'], reg['sizeISO'], wc)
        reg['lambdaISO'] = reg['lambdaISO_perc'] * reg['lambdaISO_max']
    elif reg['regISO'] is not None:
        raise ValueError('Not yet implemented')
    reg['dictISO_params'] = dISO
    return solvers.init_regularisation(reg)


def fit(DICTIONARY, KERNELS, y, regularisation=None, tol_fun=1e-3, tol_x=1e-6, max_iter=100, x0=None,
        confidence_array=None, debias=False, nolut=False, arith='ff', A=None):
    """Evaluation.fit without I/O (core.pyx:1466-1519).  Returns (x, opt_details, A)
    where A is the operator of the final solve (the debias operator when debias=True)."""
    if A is None:
        D = dict(DICTIONARY)
        D['IC'] = dict(DICTIONARY['IC'])
        D['IC']['eval'] = np.ones(int(D['IC']['nSTR'] * KERNELS['wmr'].shape[0]), dtype=np.uint32)
        A = LinearOperator(D, KERNELS, None, nolut=nolut, arith=arith)
    x, details = solvers.solve(y, A, A.T, tol_fun=tol_fun, tol_x=tol_x, max_iter=max_iter, verbose=0, x0=x0,
                               regularisation=regularisation, confidence_array=confidence_array)
    has_reg = regularisation is not None and any(regularisation.get(k) is not None
                                                 for k in ('regIC', 'regEC', 'regISO'))
    if has_reg and debias:
        offset = int(DICTIONARY['IC']['nSTR'] * KERNELS['wmr'].shape[0])
        mask = np.ones(offset, dtype=np.uint32)
        mask[np.asarray(x)[:offset] < 0.000000000000001] = 0
        D = dict(DICTIONARY)
        D['IC'] = dict(DICTIONARY['IC'])
        D['IC']['eval'] = mask
        A = LinearOperator(D, KERNELS, None, nolut=nolut, arith=arith)
        # the regularisation is rebuilt as set_regularisation() with its defaults: no
        # regulariser, non-negative compartments (core.pyx:1488)
        rp = {'startIC': 0, 'sizeIC': offset, 'startEC': offset,
              'sizeEC': int(DICTIONARY['EC']['n'] * KERNELS['wmh'].shape[0]),
              'regIC': None, 'regEC': None, 'regISO': None, 'nnIC': True, 'nnEC': True, 'nnISO': True,
              'dictIC_params': None, 'dictEC_params': None, 'dictISO_params': None}
        rp['startISO'] = rp['sizeIC'] + rp['sizeEC']
        rp['sizeISO'] = int(DICTIONARY['ISO']['n'] * KERNELS['iso'].shape[0])
        x_debias = np.asarray(x, dtype=np.float64).copy()
        x_debias[:offset] *= mask
        x_debias[offset:] = 0
        y_mask = np.asarray(A.dot(x_debias))
        y_mask[y_mask < 0] = 0
        y_mask[y_mask > 0] = 1
        y2 = np.asarray(y, dtype=np.float64) * y_mask
        x, details = solvers.solve(y2, A, A.T, tol_fun=tol_fun, tol_x=tol_x, max_iter=max_iter, verbose=0, x0=x0,
                                   regularisation=solvers.init_regularisation(rp), confidence_array=confidence_array)
    return x, details, A
