"""trk2dictionary's voxelisation on the device (commit/trk2dictionary/trk2dictionary_c.cpp).

``voxelise`` turns streamlines (points in mm of the image grid, as in a .trk file) into the
arrays of the dictionary_*.dict files: IC segments (streamline, voxel, orientation,
length), per-streamline norm / length / length with blur / kept flag, EC entries from a
peaks image, ISO voxels and the track-density image.  The arithmetic follows the
reference operation by operation (FP64 geometry without fused multiply-adds, FP32 sums
per segment key), so the outputs are the reference's own.  ``write`` stores them with
``dictionary.write_dictionary`` in the file format ``dictionary.load_dictionary`` reads.

Reading .trk / .tck headers and NIfTI images is left to the caller: pass arrays.
``hash_table`` builds the (colatitude, longitude) -> direction lookup for a direction
set (the reference takes AMICO's precomputed table for its 500 directions).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check, lib


def hash_table(dirs: np.ndarray) -> np.ndarray:
    """(181*181,) int16: entry ox*181 + oy is the index of the direction (rows of dirs,
    unit vectors) closest, up to sign, to colatitude ox and longitude oy degrees."""
    d = np.asarray(dirs, dtype=np.float64)
    th = np.deg2rad(np.arange(181.0))[:, None]
    ph = np.deg2rad(np.arange(181.0))[None, :]
    v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th) + 0.0 * ph], -1).reshape(-1, 3)
    return np.abs(v @ d.T).argmax(axis=1).astype(np.int16)


def _dev(a, dtype, device):
    if a is None:
        return None
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=device, dtype=dtype).contiguous()


def voxelise(pts, offsets, dim, pixdim, hash, mask=None, fiber_shift=(0.0, 0.0, 0.0), min_seg_len=1e-3,
             min_fiber_len=0.0, max_fiber_len=250.0, do_intersect=True, blur=None, blur_apply=None, peaks=None,
             vf_thr=0.1, flip_peaks=(False, False, False), peaks_affine=None, iso_mask=None, device=0) -> dict:
    """Streamlines pts[offsets[f]:offsets[f+1]] (float32 (M, 3), mm) -> dictionary arrays
    (numpy): {'IC': {'f','v','o','len'}, 'TRK': {'norm','len','lenTot','kept'},
    'EC': {'v','o'}, 'ISO': {'v'}, 'TDI': (X, Y, Z) float64}.  mask / iso_mask: (X, Y, Z)
    arrays (non-zero = inside); peaks: (X, Y, Z, Np, 3); blur: (rho, angle, weights) of the
    replicas with blur_apply (per streamline) selecting where they are used."""
    dev = torch.device('cuda', device)
    P = _dev(np.asarray(pts, dtype=np.float32).reshape(-1, 3), torch.float32, dev)
    off = _dev(np.asarray(offsets, dtype=np.int64), torch.int64, dev)
    nfib = int(off.numel()) - 1
    H = _dev(np.asarray(hash, dtype=np.int16).ravel(), torch.int16, dev)
    if H.numel() != 181 * 181:
        raise ValueError('hash table must have 181*181 entries')
    dim = tuple(int(v) for v in dim)
    m = None if mask is None else _dev((np.asarray(mask) != 0).astype(np.uint8), torch.uint8, dev)
    im = None if iso_mask is None else _dev((np.asarray(iso_mask) != 0).astype(np.uint8), torch.uint8, dev)
    for g in (m, im):
        if g is not None and g.numel() != dim[0] * dim[1] * dim[2]:
            raise ValueError('mask size does not match the grid')
    if blur is None:
        rho, ang, w = (torch.tensor(v, dtype=torch.float64, device=dev) for v in ([0.0], [0.0], [1.0]))
    else:
        rho, ang, w = (_dev(np.asarray(v, dtype=np.float64), torch.float64, dev) for v in blur)
    ba = None if blur_apply is None else _dev(np.asarray(blur_apply).astype(np.uint8), torch.uint8, dev)
    pk = None
    npk = 0
    if peaks is not None:
        pa = np.asarray(peaks, dtype=np.float32)
        npk = int(pa.shape[-2])
        pk = _dev(pa.reshape(-1), torch.float32, dev)
    prm = _lib.CgbT2DParams()
    prm.dim[:] = dim
    prm.pixdim[:] = [float(v) for v in pixdim]
    prm.fiber_shift[:] = [float(v) for v in fiber_shift]
    prm.min_seg_len, prm.min_fiber_len, prm.max_fiber_len = float(min_seg_len), float(min_fiber_len), \
        float(max_fiber_len)
    prm.do_intersect = int(bool(do_intersect))
    prm.n_replicas = int(rho.numel())
    prm.blur_rho, prm.blur_angle, prm.blur_weights = rho.data_ptr(), ang.data_ptr(), w.data_ptr()
    prm.n_peaks = npk
    prm.vf_thr = float(vf_thr)
    prm.flip[:] = [-1 if f else 1 for f in flip_peaks]
    prm.peaks_affine[:] = [float(v) for v in np.asarray(np.eye(3) if peaks_affine is None else peaks_affine).ravel()]
    res = _lib.CgbT2DResult()
    st = torch.cuda.current_stream(dev).cuda_stream
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    check(lib().cgb_trk2dict(ctypes.byref(prm), p(P), p(off), nfib, p(ba), p(H), p(m), p(pk), p(im),
                             ctypes.byref(res), ctypes.c_void_p(st)))
    try:
        def get(ptr, n, dt):
            out = np.empty(int(n), dtype=dt)
            if n > 0:
                out.view(np.uint8)[:] = _device_bytes(ptr, out.nbytes, dev).cpu().numpy()
            return out

        ns, nk = res.n_segments, res.n_kept
        out = {'IC': {'f': get(res.ic_f, ns, np.uint32), 'v': get(res.ic_v, ns, np.uint32),
                      'o': get(res.ic_o, ns, np.uint16), 'len': get(res.ic_len, ns, np.float32)},
               'TRK': {'norm': get(res.trk_norm, nk, np.float32), 'len': get(res.trk_len, nk, np.float32),
                       'lenTot': get(res.trk_lentot, nk, np.float32), 'kept': get(res.trk_kept, nfib, np.uint8)},
               'EC': {'v': get(res.ec_v, res.n_ec, np.uint32), 'o': get(res.ec_o, res.n_ec, np.uint16)},
               'ISO': {'v': get(res.iso_v, res.n_iso, np.uint32)},
               'TDI': get(res.tdi, dim[0] * dim[1] * dim[2], np.float64).reshape(dim)}
    finally:
        lib().cgb_trk2dict_free(ctypes.byref(res))
    return out


def _device_bytes(ptr: int, n: int, dev: torch.device) -> torch.Tensor:
    """A uint8 CUDA tensor aliasing n bytes at device address ptr (no copy)."""
    class _Ary:
        __cuda_array_interface__ = {'shape': (int(n),), 'typestr': '|u1', 'data': (int(ptr), False), 'version': 3}
    return torch.as_tensor(_Ary(), device=dev)


def to_dictionary_files(res: dict) -> dict:
    """The raw arrays as ``dictionary.write_dictionary`` expects them."""
    return {'IC': {'str': res['IC']['f'], 'vox': res['IC']['v'], 'dir': res['IC']['o'], 'len': res['IC']['len']},
            'EC': {'vox': res['EC']['v'], 'dir': res['EC']['o']}, 'ISO': {'vox': res['ISO']['v']},
            'TRK': {'norm': res['TRK']['norm'], 'kept': res['TRK']['kept'], 'len': res['TRK']['len'],
                    'lenTot': res['TRK']['lenTot']}}


def write(path: str, res: dict) -> None:
    """Write the dictionary_*.dict files of a voxelisation to ``path``."""
    from .dictionary import write_dictionary
    write_dictionary(path, to_dictionary_files(res))
