"""ORACLE -- test infrastructure only.

ctypes front end of ``oracle/trk2dict_oracle.c``, the CPU restatement of trk2dictionary's
streamline voxelisation (commit/trk2dictionary/trk2dictionary_c.cpp:446-870), used by the
tests to check the device voxeliser.  The product package never imports it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD_DIR, 'libtrk2dict_oracle.so')


class Cfg(ctypes.Structure):
    _fields_ = [('dimx', ctypes.c_int), ('dimy', ctypes.c_int), ('dimz', ctypes.c_int),
                ('px', ctypes.c_float), ('py', ctypes.c_float), ('pz', ctypes.c_float),
                ('shx', ctypes.c_float), ('shy', ctypes.c_float), ('shz', ctypes.c_float),
                ('min_seg_len', ctypes.c_float), ('min_fiber_len', ctypes.c_float), ('max_fiber_len', ctypes.c_float),
                ('do_intersect', ctypes.c_int), ('n_rep', ctypes.c_int),
                ('rho', ctypes.c_void_p), ('angle', ctypes.c_void_p), ('w', ctypes.c_void_p)]


class Out(ctypes.Structure):
    _fields_ = [('trk_norm', ctypes.POINTER(ctypes.c_float)), ('trk_len', ctypes.POINTER(ctypes.c_float)),
                ('trk_lentot', ctypes.POINTER(ctypes.c_float)), ('kept', ctypes.POINTER(ctypes.c_uint8)),
                ('ic_f', ctypes.POINTER(ctypes.c_uint32)), ('ic_v', ctypes.POINTER(ctypes.c_uint32)),
                ('ic_o', ctypes.POINTER(ctypes.c_uint16)), ('ic_len', ctypes.POINTER(ctypes.c_float)),
                ('n_seg', ctypes.c_int64), ('n_kept', ctypes.c_int64), ('cap_seg', ctypes.c_int64)]


def build(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, 'trk2dict_oracle.c')
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        cmd = f'gcc -O2 -ffp-contract=off -fPIC -shared -o {LIB}.tmp {src} -lm && mv {LIB}.tmp {LIB}'
        if os.system(cmd) != 0:
            raise RuntimeError('failed to build the trk2dictionary oracle: ' + cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.t2d_run.argtypes = [ctypes.POINTER(Cfg), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Out)]
        L.t2d_free.argtypes = [ctypes.POINTER(Out)]
        _lib = L
    return _lib


def voxelise(pts, offsets, dim, pixdim, hash_table, mask=None, fiber_shift=(0.0, 0.0, 0.0), min_seg_len=1e-3,
             min_fiber_len=0.0, max_fiber_len=250.0, do_intersect=True, blur=None, blur_apply=None) -> dict:
    """Raw trk2dictionary outputs for streamlines pts[offsets[f]:offsets[f+1]] (mm)."""
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    hashv = np.ascontiguousarray(hash_table, dtype=np.int16).ravel()
    px = np.float32(pixdim[0]), np.float32(pixdim[1]), np.float32(pixdim[2])
    sh = [np.float32(np.float32(fiber_shift[i]) * px[i]) for i in range(3)]
    if blur is None:
        rho, ang, w = np.zeros(1), np.zeros(1), np.ones(1)
    else:
        rho, ang, w = (np.ascontiguousarray(a, dtype=np.float64) for a in blur)
    c = Cfg(int(dim[0]), int(dim[1]), int(dim[2]), px[0], px[1], px[2], sh[0], sh[1], sh[2],
            np.float32(min_seg_len), np.float32(min_fiber_len), np.float32(max_fiber_len), int(bool(do_intersect)),
            int(rho.size), rho.ctypes.data, ang.ctypes.data, w.ctypes.data)
    m = None if mask is None else np.ascontiguousarray(np.asarray(mask) != 0, dtype=np.uint8)
    ba = None if blur_apply is None else np.ascontiguousarray(blur_apply, dtype=np.uint8)
    o = Out()
    nfib = off.size - 1
    lib().t2d_run(ctypes.byref(c), pts.ctypes.data, off.ctypes.data, nfib,
                  ba.ctypes.data if ba is not None else None, hashv.ctypes.data,
                  m.ctypes.data if m is not None else None, ctypes.byref(o))
    ns, nk = int(o.n_seg), int(o.n_kept)

    def arr(p, n, dt):
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n > 0 else np.zeros(0, dt)

    res = {'IC': {'f': arr(o.ic_f, ns, np.uint32), 'v': arr(o.ic_v, ns, np.uint32), 'o': arr(o.ic_o, ns, np.uint16),
                  'len': arr(o.ic_len, ns, np.float32)},
           'TRK': {'norm': arr(o.trk_norm, nk, np.float32), 'len': arr(o.trk_len, nk, np.float32),
                   'lenTot': arr(o.trk_lentot, nk, np.float32), 'kept': arr(o.kept, nfib, np.uint8)}}
    lib().t2d_free(ctypes.byref(o))
    return res


REF_LIB = os.path.join(HERE, '_ref', 'libt2d_ref.so')


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def write_trk(path: str, pts, offsets) -> None:
    """A minimal .trk file: 1000-byte header (unused by the voxeliser), then per streamline
    int32 N and N float32 triplets (no scalars, no properties)."""
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    with open(path, 'wb') as f:
        f.write(b'\0' * 1000)
        for k in range(len(offsets) - 1):
            a, b = int(offsets[k]), int(offsets[k + 1])
            f.write(np.int32(b - a).tobytes())
            f.write(pts[a:b].tobytes())


def reference_voxelise(workdir, pts, offsets, dim, pixdim, hash_table, mask=None, fiber_shift=(0.0, 0.0, 0.0),
                       min_seg_len=1e-3, min_fiber_len=0.0, max_fiber_len=250.0, do_intersect=True, blur=None,
                       blur_apply=None, peaks=None, vf_thr=0.1, peaks_affine=None, iso_mask=None) -> dict:
    """Run the reference's trk2dictionary (one thread) and read back its .dict files."""
    L = ctypes.CDLL(REF_LIB)
    fp, dp, vp = ctypes.c_float, ctypes.c_double, ctypes.c_void_p
    L.t2d_ref_run.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, fp, fp,
                              fp, fp, fp, fp, fp, fp, ctypes.c_int, vp, vp, vp, ctypes.c_int, fp, vp, ctypes.c_int,
                              vp, vp, vp, vp, vp, vp, ctypes.c_char_p]
    os.makedirs(workdir, exist_ok=True)
    trk = os.path.join(workdir, 'in.trk')
    write_trk(trk, pts, offsets)
    out = os.path.join(workdir, 'out')
    nfib = len(offsets) - 1
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    im = None if iso_mask is None else np.ascontiguousarray(iso_mask, dtype=np.float32)
    pk = None if peaks is None else np.ascontiguousarray(peaks, dtype=np.float32)
    npk = 0 if peaks is None else int(pk.shape[-2])
    aff = np.ascontiguousarray(np.eye(3) if peaks_affine is None else peaks_affine, dtype=np.float64)
    if blur is None:
        rho, ang, w = np.zeros(1), np.zeros(1), np.ones(1)
    else:
        rho, ang, w = (np.ascontiguousarray(a, dtype=np.float64) for a in blur)
    ba = np.zeros(nfib, np.uint8) if blur_apply is None else np.ascontiguousarray(blur_apply, dtype=np.uint8)
    hashv = np.ascontiguousarray(hash_table, dtype=np.int16).ravel()
    tdi = np.zeros(int(np.prod(dim)), dtype=np.float64)
    rc = L.t2d_ref_run(trk.encode(), nfib, int(dim[0]), int(dim[1]), int(dim[2]), float(pixdim[0]), float(pixdim[1]),
                       float(pixdim[2]), float(fiber_shift[0]), float(fiber_shift[1]), float(fiber_shift[2]),
                       float(min_seg_len), float(min_fiber_len), float(max_fiber_len), int(bool(do_intersect)),
                       m.ctypes.data if m is not None else None, im.ctypes.data if im is not None else None,
                       pk.ctypes.data if pk is not None else None, npk, float(vf_thr), aff.ctypes.data,
                       int(rho.size), rho.ctypes.data, ang.ctypes.data, w.ctypes.data, ba.ctypes.data,
                       hashv.ctypes.data, tdi.ctypes.data, out.encode())
    if rc != 1:
        raise RuntimeError('reference trk2dictionary failed')
    t = os.path.join(out, 'temp')

    def rd(name, dt, d=t):
        return np.fromfile(os.path.join(d, name), dtype=dt)

    return {'IC': {'f': rd('dictionary_IC_f_0.dict', np.uint32), 'v': rd('dictionary_IC_v_0.dict', np.uint32),
                   'o': rd('dictionary_IC_o_0.dict', np.uint16), 'len': rd('dictionary_IC_len_0.dict', np.float32)},
            'TRK': {'norm': rd('dictionary_TRK_norm_0.dict', np.float32), 'len': rd('dictionary_TRK_len_0.dict', np.float32),
                    'lenTot': rd('dictionary_TRK_lenTot_0.dict', np.float32),
                    'kept': rd('dictionary_TRK_kept_0.dict', np.uint8)},
            'EC': {'v': rd('dictionary_EC_v.dict', np.uint32, out), 'o': rd('dictionary_EC_o.dict', np.uint16, out)},
            'ISO': {'v': rd('dictionary_ISO_v.dict', np.uint32, out)},
            'TDI': tdi.reshape(tuple(int(d) for d in dim))}


def ec_entries(tdi, peaks, hash_table, vf_thr=0.1, flip=(1, 1, 1), affine=None):
    """EC entries from a peaks image (ECSegments, trk2dictionary_c.cpp:289-398): voxels in
    x-fastest order with TDI != 0; per peak of FP32 norm >= vf_thr * the largest, the FP64
    direction through the affine and flips, folded to y >= 0, looked up in the hash."""
    X, Y, Z = tdi.shape
    Np = peaks.shape[-2]
    A = np.eye(3) if affine is None else np.asarray(affine, dtype=np.float64)
    hashv = np.asarray(hash_table).ravel()
    vs, os_ = [], []
    for iz in range(Z):
        for iy in range(Y):
            for ix in range(X):
                if tdi[ix, iy, iz] == 0:
                    continue
                pk = peaks[ix, iy, iz].astype(np.float64)
                norms = np.sqrt((pk * pk).sum(axis=1)).astype(np.float32)
                pmax = np.float32(-1) if Np == 0 else max(np.float32(-1), norms.max())
                if not pmax > 0:
                    continue
                for i in range(Np):
                    if norms[i] == 0 or norms[i] < np.float32(vf_thr) * pmax:
                        continue
                    p = pk[i]
                    d = np.array([p[0] * A[0, 0] + p[1] * A[0, 1] + p[2] * A[0, 2],
                                  p[0] * A[1, 0] + p[1] * A[1, 1] + p[2] * A[1, 2],
                                  p[0] * A[2, 0] + p[1] * A[2, 1] + p[2] * A[2, 2]]) * np.asarray(flip)
                    if d[1] < 0:
                        d = -d
                    colat = np.arctan2(np.sqrt(d[0] * d[0] + d[1] * d[1]), d[2])
                    lon = np.arctan2(d[1], d[0])
                    hi = int(round_half_away(colat / np.pi * 180.0)) * 181 + int(round_half_away(lon / np.pi * 180.0))
                    hi = min(max(hi, 0), 181 * 181 - 1)
                    vs.append(ix + X * (iy + Y * iz))
                    os_.append(hashv[hi])
    return np.array(vs, dtype=np.uint32), np.array(os_, dtype=np.uint16)


def round_half_away(v: float) -> float:
    """C's round(): halves away from zero (numpy rounds halves to even)."""
    return float(np.sign(v) * np.floor(abs(v) + 0.5))


def iso_voxels(tdi, mask=None, iso_mask=None):
    """ISO voxels (ISOcompartments, trk2dictionary_c.cpp:400-440), x-fastest order."""
    ok = tdi != 0
    if mask is not None:
        ok &= np.asarray(mask) != 0
    if iso_mask is not None:
        ok &= np.asarray(iso_mask) != 0
    return np.flatnonzero(ok.ravel(order='F')).astype(np.uint32)
