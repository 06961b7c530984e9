"""Reader for trk2dictionary's output, producing the DICTIONARY of Evaluation.load_dictionary.

Files (written by trk2dictionary_c.cpp:473-552, 299-300, 406-431 and trk2dictionary.pyx):
``dictionary_IC_{f,v,o,len}.dict`` (u32, u32, u16, f32), ``dictionary_EC_{v,o}.dict``,
``dictionary_ISO_v.dict``, ``dictionary_TRK_{norm,kept,len,lenTot}.dict``; voxels are linear
indices x + X*(y + Y*z) of the image grid.  ``load_dictionary`` follows
commit/core.pyx:436-582: stable sort of IC / EC / ISO by voxel, division of each IC length
by its streamline's norm (doNormalizeKernels), and remapping of voxel ids to indices of the
mask voxels in Fortran order.  The mask is passed as an array (reading NIfTI is left to the
caller).  The arrays can be handed straight to ``LinearOperator`` (whose device re-layout
would accept them unsorted as well).  With ``device`` set, the raw arrays are copied to that
GPU once and the re-layout runs there (``cgb_dict_relayout``): the dictionary then holds
CUDA tensors, which ``LinearOperator`` takes without a host round trip.
"""
from __future__ import annotations

import os

import numpy as np

_FILES = {('IC', 'str'): ('dictionary_IC_f.dict', np.uint32), ('IC', 'vox'): ('dictionary_IC_v.dict', np.uint32),
          ('IC', 'dir'): ('dictionary_IC_o.dict', np.uint16), ('IC', 'len'): ('dictionary_IC_len.dict', np.float32),
          ('EC', 'vox'): ('dictionary_EC_v.dict', np.uint32), ('EC', 'dir'): ('dictionary_EC_o.dict', np.uint16),
          ('ISO', 'vox'): ('dictionary_ISO_v.dict', np.uint32),
          ('TRK', 'norm'): ('dictionary_TRK_norm.dict', np.float32),
          ('TRK', 'kept'): ('dictionary_TRK_kept.dict', np.uint8),
          ('TRK', 'len'): ('dictionary_TRK_len.dict', np.float32),
          ('TRK', 'lenTot'): ('dictionary_TRK_lenTot.dict', np.float32)}


def load_dictionary(path: str, mask: np.ndarray, normalize_kernels: bool = True, sort_kind: str = 'mergesort',
                    device=None) -> dict:
    """DICTIONARY as commit/core.pyx:436-582 builds it from the files in ``path``.

    mask: 3-D array of the fitted voxels (dictionary_tdi / dictionary_mask image data).
    device: None (numpy arrays, re-laid-out on the host) or a CUDA device index (CUDA
    tensors, re-laid-out on that device)."""
    if device is not None:
        return _load_dictionary_device(path, mask, normalize_kernels, int(device))
    mask = (np.asarray(mask) > 0).astype(np.uint8)
    D = {'IC': {}, 'EC': {}, 'ISO': {}, 'TRK': {}, 'MASK': mask}
    for (comp, key), (fname, dt) in _FILES.items():
        fp = os.path.join(path, fname)
        if os.path.exists(fp):
            D[comp][key] = np.fromfile(fp, dtype=dt)
        elif comp == 'TRK' and key in ('len', 'lenTot'):
            continue
        else:
            raise FileNotFoundError(fp)
    IC, EC, ISO = D['IC'], D['EC'], D['ISO']
    IC['n'] = IC['vox'].size
    IC['nSTR'] = D['TRK']['norm'].size
    IC['nVOX'] = int(mask.sum())
    idx = np.argsort(IC['vox'], kind=sort_kind)                     # core.pyx:508-514
    for k in ('vox', 'dir', 'str', 'len'):
        IC[k] = IC[k][idx]
    if normalize_kernels:                                           # core.pyx:516-525
        IC['len'] = (IC['len'] / D['TRK']['norm'][IC['str']]).astype(np.float32)
    EC['n'] = EC['vox'].size
    idx = np.argsort(EC['vox'], kind=sort_kind)                     # core.pyx:541-545
    EC['vox'], EC['dir'] = EC['vox'][idx], EC['dir'][idx]
    ISO['n'] = ISO['vox'].size
    ISO['vox'] = ISO['vox'][np.argsort(ISO['vox'], kind=sort_kind)]
    # voxel ids -> indices of the mask voxels in Fortran order (core.pyx:571-580)
    lin = mask.ravel(order='F').nonzero()[0]
    D['MASK_ix'], D['MASK_iy'], D['MASK_iz'] = np.unravel_index(lin, mask.shape, order='F')
    lut = np.zeros(mask.size, dtype=np.uint32)
    lut[lin] = np.arange(lin.size, dtype=np.uint32)
    IC['vox'] = lut[IC['vox']]
    EC['vox'] = lut[EC['vox']]
    ISO['vox'] = lut[ISO['vox']]
    return D


def _load_dictionary_device(path: str, mask, normalize_kernels: bool, device: int) -> dict:
    import ctypes

    import torch

    from ._lib import check, lib
    mask = (np.asarray(mask) > 0).astype(np.uint8)
    dev = torch.device('cuda', device)
    D = {'IC': {}, 'EC': {}, 'ISO': {}, 'TRK': {}, 'MASK': mask}
    tdt = {np.uint32: torch.int32, np.uint16: torch.int16, np.float32: torch.float32, np.uint8: torch.uint8}
    for (comp, key), (fname, dt) in _FILES.items():
        fp = os.path.join(path, fname)
        if not os.path.exists(fp):
            if comp == 'TRK' and key in ('len', 'lenTot'):
                continue
            raise FileNotFoundError(fp)
        a = np.fromfile(fp, dtype=dt)
        if comp == 'TRK':
            D[comp][key] = a
        else:  # the bits of the unsigned arrays, as same-width torch tensors
            D[comp][key] = torch.from_numpy(a.view(np.dtype(dt).str.replace('u', 'i'))).to(dev)
    norm = torch.from_numpy(D['TRK']['norm']).to(dev)
    maskf = torch.from_numpy(np.ascontiguousarray(mask.ravel(order='F'))).to(dev)
    IC, EC, ISO = D['IC'], D['EC'], D['ISO']
    IC['n'] = int(IC['vox'].numel())
    IC['nSTR'] = int(D['TRK']['norm'].size)
    EC['n'] = int(EC['vox'].numel())
    ISO['n'] = int(ISO['vox'].numel())
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else None  # noqa: E731
    nV = ctypes.c_int64()
    with torch.cuda.device(dev):
        st = torch.cuda.current_stream(dev).cuda_stream
        check(lib().cgb_dict_relayout(p(maskf), maskf.numel(), IC['n'], IC['nSTR'], p(IC['str']), p(IC['vox']),
                                      p(IC['dir']), p(IC['len']), p(norm), int(bool(normalize_kernels)), EC['n'],
                                      p(EC['vox']), p(EC['dir']), ISO['n'], p(ISO['vox']), ctypes.byref(nV),
                                      ctypes.c_void_p(st)))
    IC['nVOX'] = int(nV.value)
    lin = mask.ravel(order='F').nonzero()[0]
    D['MASK_ix'], D['MASK_iy'], D['MASK_iz'] = np.unravel_index(lin, mask.shape, order='F')
    return D


def to_host(D: dict) -> dict:
    """A copy of a dictionary with its CUDA tensors as numpy arrays of the reference dtypes."""
    out = {}
    for comp, d in D.items():
        if not isinstance(d, dict):
            out[comp] = d
            continue
        out[comp] = {}
        for k, v in d.items():
            if hasattr(v, 'is_cuda'):
                a = v.cpu().numpy()
                out[comp][k] = a.view(a.dtype.str.replace('i', 'u')) if a.dtype.kind == 'i' else a
            else:
                out[comp][k] = v
    return out


def write_dictionary(path: str, raw: dict) -> None:
    """Write raw trk2dictionary-style arrays (voxels as linear grid indices, lengths not
    normalised) to ``path`` in the file format load_dictionary reads."""
    os.makedirs(path, exist_ok=True)
    for (comp, key), (fname, dt) in _FILES.items():
        if comp in raw and key in raw[comp]:
            np.ascontiguousarray(raw[comp][key], dtype=dt).tofile(os.path.join(path, fname))
