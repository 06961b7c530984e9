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


def voxel_maps(A: LinearOperator, x, y=None, confidence=None, norm_fib=None, normalize_maps=False,
               DICTIONARY=None) -> dict:
    """The voxelwise maps of Evaluation.save_results (commit/core.pyx:1614-1750), computed on
    the device from the operator's voxel-ordered streams (``cgb_op_voxel_maps``).

    x: fitted coefficients (as save_results rescales them); y: the measured signal
    (nROWS) for the error maps; confidence: the confidence map (nROWS) for the adjusted
    error maps; norm_fib: per-IC-column weights (the reference's np.kron(ones(nIC), TRK
    norm) when kernels were normalised).  Returns float32 numpy arrays per mask voxel:
    'compartment_IC', 'compartment_EC', 'compartment_ISO' (divided by their sum + 1e-16
    when normalize_maps, as doNormalizeMaps), and with y 'fit_RMSE', 'fit_NRMSE', plus
    with confidence 'fit_RMSE_adjusted', 'fit_NRMSE_adjusted'.  With DICTIONARY (holding
    MASK and MASK_ix/iy/iz) each map is also returned as a 3-D volume under '<name>_vol'."""
    import ctypes
    from . import _lib
    dev = torch.device('cuda', A.device)

    def d(a, n):
        if a is None:
            return None
        t = torch.as_tensor(np.asarray(a, dtype=np.float64) if not isinstance(a, torch.Tensor) else a,
                            dtype=torch.float64).to(dev).contiguous()
        if t.numel() != n:
            raise RuntimeError('voxel_maps: dimensions do not match')
        return t

    nV = A.ICnVOX
    xd = d(x, A.nCOLS)
    yd = d(y, A.nROWS)
    cd = d(confidence, A.nROWS)
    nf = d(norm_fib, A.ICnSTR * A.ICnRF)
    names = ['compartment_IC', 'compartment_EC', 'compartment_ISO']
    if yd is not None:
        names += ['fit_RMSE', 'fit_NRMSE']
        if cd is not None:
            names += ['fit_RMSE_adjusted', 'fit_NRMSE_adjusted']
    out = {k: torch.zeros(nV, dtype=torch.float64, device=dev) for k in names}
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    st = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(_lib.lib().cgb_op_voxel_maps(
        A.handle, p(xd), p(yd), p(cd), p(nf), p(out['compartment_IC']), p(out['compartment_EC']),
        p(out['compartment_ISO']), p(out.get('fit_RMSE')), p(out.get('fit_NRMSE')),
        p(out.get('fit_RMSE_adjusted')), p(out.get('fit_NRMSE_adjusted')), ctypes.c_void_p(st)))
    res = {k: v.cpu().numpy().astype(np.float32) for k, v in out.items()}
    if normalize_maps:   # core.pyx:1752-1755, FP32 as the reference's float32 images
        tot = res['compartment_IC'] + res['compartment_EC'] + res['compartment_ISO']
        for k in ('compartment_IC', 'compartment_EC', 'compartment_ISO'):
            res[k] = res[k] / (tot + np.float32(1e-16))
    if DICTIONARY is not None and 'MASK' in DICTIONARY:
        dim = np.asarray(DICTIONARY['MASK']).shape
        ix, iy, iz = DICTIONARY['MASK_ix'], DICTIONARY['MASK_iy'], DICTIONARY['MASK_iz']
        for k in list(res):
            vol = np.zeros(dim, dtype=np.float32)
            vol[ix, iy, iz] = res[k]
            res[k + '_vol'] = vol
    return res
