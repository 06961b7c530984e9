"""GB300 drop-in for commit/operator/operator.pyx:10-184 (``LinearOperator``).

``LinearOperator(DICTIONARY, KERNELS, THREADS, nolut=False)`` takes the same dicts the
reference takes (THREADS is accepted and ignored: the device re-layout done once at
construction replaces the CPU partitions of Evaluation.set_threads).  ``dot`` accepts a
float64 numpy vector (copied to the device and back, like the reference's host call) or
a CUDA float64 torch tensor (kept on the device, enqueued on torch's current stream).
``T`` returns the adjoint sharing the same device dictionary; ``shape``, ``nROWS``,
``nCOLS`` and ``adjoint`` are as in the reference.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check, lib


def _host(a, dtype):
    """A contiguous array of `dtype`: numpy for host data; a CUDA tensor of the same width
    (its bits) stays on the device (cgb_op_create takes device pointers as well)."""
    if isinstance(a, torch.Tensor) and a.is_cuda:
        if a.element_size() != np.dtype(dtype).itemsize:
            raise TypeError(f'CUDA dictionary array of element size {a.element_size()}, expected {np.dtype(dtype)}')
        return a.contiguous()
    a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
    return a


def _ptr(a):
    if isinstance(a, torch.Tensor):
        return ctypes.c_void_p(a.data_ptr()) if a.numel() else None
    return a.ctypes.data_as(ctypes.c_void_p) if a.size else None


def _size(a) -> int:
    return int(a.numel()) if isinstance(a, torch.Tensor) else int(a.size)


class _Handle:
    """Owns one cgb_op (device copy of the dictionary)."""

    def __init__(self, ptr, device):
        self.ptr = ptr
        self.device = device

    def __del__(self):
        try:
            if self.ptr:
                lib().cgb_op_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass


class LinearOperator:
    """Implicit COMMIT dictionary operator A (and A' via ``.T``) on a GB300."""

    def __init__(self, DICTIONARY, KERNELS, THREADS=None, nolut=False, arith: str = 'ff', device=None):
        self.DICTIONARY = DICTIONARY
        self.KERNELS = KERNELS
        self.THREADS = THREADS
        IC, EC, ISO = DICTIONARY['IC'], DICTIONARY['EC'], DICTIONARY['ISO']
        self.ICn = int(IC['n'])
        self.ICnSTR = int(IC['nSTR'])
        self.ICnRF = int(KERNELS['wmr'].shape[0])
        self.ICnVOX = int(IC['nVOX'])
        self.ECn = int(EC['n'])
        self.ECnRF = int(KERNELS['wmh'].shape[0])
        self.ISOn = int(ISO['n'])
        self.ISOnRF = int(KERNELS['iso'].shape[0])
        # number of samples and directions as operator.pyx:56-63
        if KERNELS['wmr'].size > 0:
            self.nSAMPLES = int(KERNELS['wmr'].shape[2])
        elif KERNELS['wmh'].size > 0:
            self.nSAMPLES = int(KERNELS['wmh'].shape[2])
        else:
            self.nSAMPLES = int(KERNELS['wmr'].shape[1])
        self.ndirs = int(KERNELS['wmr'].shape[1])
        self.nolut = bool(nolut)
        self.adjoint = 0
        self.nROWS = self.ICnVOX * self.nSAMPLES
        self.nCOLS = self.ICnSTR * self.ICnRF + self.ECn * self.ECnRF + self.ISOn * self.ISOnRF
        if arith not in ('ff', 'f64'):
            raise ValueError("arith must be 'ff' (float-float, FP64-accurate) or 'f64' (native FP64)")
        self.arith = arith
        if device is None:
            device = torch.cuda.current_device() if torch.cuda.is_available() else 0
        self.device = int(device)

        f = _host(IC['str'], np.uint32)
        v = _host(IC['vox'], np.uint32)
        o = _host(IC['dir'], np.uint16)
        ln = _host(IC['len'], np.float32)
        ev = IC.get('eval')
        ev = _host(ev if ev is not None else np.ones(self.ICnSTR * self.ICnRF, np.uint32), np.uint32)
        if _size(ev) < self.ICnSTR * self.ICnRF:
            raise ValueError('DICTIONARY["IC"]["eval"] is shorter than nSTR * nIC')
        ecv = _host(EC['vox'], np.uint32)
        eco = _host(EC['dir'], np.uint16)
        isov = _host(ISO['vox'], np.uint32)
        lic = _host(KERNELS['wmr'], np.float32)
        lec = _host(KERNELS['wmh'], np.float32)
        liso = _host(KERNELS['iso'], np.float32)
        if _size(f) != self.ICn or _size(v) != self.ICn or _size(ln) != self.ICn or (not nolut and _size(o) != self.ICn):
            raise ValueError('IC arrays do not match DICTIONARY["IC"]["n"]')
        if _size(ecv) != self.ECn or _size(isov) != self.ISOn:
            raise ValueError('EC/ISO arrays do not match their "n"')
        out = ctypes.c_void_p()
        check(lib().cgb_op_create(self.device, self.nSAMPLES, max(self.ndirs, 1), self.ICnSTR, self.ICn, self.ECn,
                                  self.ICnVOX, self.ISOn, _ptr(f), _ptr(ev), _ptr(v), _ptr(o), _ptr(ln), _ptr(ecv),
                                  _ptr(eco), _ptr(isov), _ptr(lic), _ptr(lec), _ptr(liso), self.ICnRF, self.ECnRF,
                                  self.ISOnRF, int(self.nolut), _lib.ARITH[arith], ctypes.byref(out)))
        self._h = _Handle(out, self.device)

    # ------------------------------------------------------------------ reference surface
    @property
    def T(self):
        """Adjoint operator (shares the device dictionary)."""
        C = object.__new__(LinearOperator)
        C.__dict__.update(self.__dict__)
        C.adjoint = 1 - self.adjoint
        return C

    @property
    def shape(self):
        return (self.nROWS, self.nCOLS) if not self.adjoint else (self.nCOLS, self.nROWS)

    @property
    def handle(self):
        return self._h.ptr

    def device_bytes(self) -> int:
        b = ctypes.c_size_t()
        check(lib().cgb_op_device_bytes(self._h.ptr, ctypes.byref(b)))
        return int(b.value)

    def dot(self, v_in, out=None, arith: str | None = None):
        """A @ v_in (or A' @ v_in for the adjoint).

        numpy float64 in -> numpy float64 out (host copies inside the call);
        torch CUDA float64 in -> torch CUDA float64 out (no host round-trip);
        torch CUDA float32 in -> float32 out through the reduced-precision kernels
        (``arith`` 'bf16' (default), 'fp16' or 'f32': LUT in that format, FP16 lengths,
        FP32 accumulation).
        """
        if isinstance(v_in, torch.Tensor) and v_in.is_cuda and v_in.dtype == torch.float32:
            ar32 = _lib.ARITH[arith or 'bf16']
            if ar32 < _lib.ARITH['bf16']:
                raise ValueError("float32 vectors need arith 'bf16', 'fp16' or 'f32'")
            v_in = v_in.contiguous()
            if v_in.numel() != self.shape[1]:
                raise RuntimeError("A.dot(): dimensions do not match")
            if out is None:
                out = torch.empty(self.shape[0], dtype=torch.float32, device=v_in.device)
            st = torch.cuda.current_stream(v_in.device).cuda_stream
            check(lib().cgb_op_apply(self._h.ptr, self.adjoint, ctypes.c_void_p(v_in.data_ptr()), v_in.numel(),
                                     ctypes.c_void_p(out.data_ptr()), out.numel(), _lib.DTYPE_F32, ar32,
                                     ctypes.c_void_p(st)))
            return out
        ar = _lib.ARITH[arith or self.arith]
        if isinstance(v_in, torch.Tensor) and v_in.is_cuda:
            if v_in.dtype != torch.float64:
                raise TypeError('LinearOperator.dot expects float64 or float32 CUDA tensors')
            v_in = v_in.contiguous()
            if v_in.numel() != self.shape[1]:
                raise RuntimeError("A.dot(): dimensions do not match")
            if out is None:
                out = torch.empty(self.shape[0], dtype=torch.float64, device=v_in.device)
            st = torch.cuda.current_stream(v_in.device).cuda_stream
            check(lib().cgb_op_apply(self._h.ptr, self.adjoint, ctypes.c_void_p(v_in.data_ptr()), v_in.numel(),
                                     ctypes.c_void_p(out.data_ptr()), out.numel(), _lib.DTYPE_F64, ar,
                                     ctypes.c_void_p(st)))
            return out
        v = np.ascontiguousarray(v_in, dtype=np.float64)
        if v.size != self.shape[1]:
            raise RuntimeError("A.dot(): dimensions do not match")
        res = np.empty(self.shape[0], dtype=np.float64) if out is None else out
        if arith is not None and ar != _lib.ARITH[self.arith]:
            check(lib().cgb_op_set_arith(self._h.ptr, ar))
        try:
            check(lib().cgb_op_apply_host(self._h.ptr, self.adjoint, _ptr(v), v.size, _ptr(res), res.size))
        finally:
            if arith is not None and ar != _lib.ARITH[self.arith]:
                check(lib().cgb_op_set_arith(self._h.ptr, _lib.ARITH[self.arith]))
        return res

    OCC_SLOTS = {'ff_forward': 0, 'ff_adjoint': 1, 'bf16_adjoint': 2, 'fp16_adjoint': 3, 'f32_adjoint': 4,
                 'bf16x2_adjoint': 5, 'bf16_forward': 6, 'fp16_forward': 7, 'f32_forward': 8,
                 'ff_fused_gradient': 9, 'bf16_fused_gradient': 10, 'fp16_fused_gradient': 11,
                 'f32_fused_gradient': 12, 'bf16x2_fused_gradient': 13, 'bf16x4_adjoint': 14,
                 'ff_forward_wide': 16, 'ff_adjoint_wide': 17, 'ff_fused_gradient_wide': 18}

    def occupancy(self, set_to: dict | None = None) -> dict:
        """Occupancy autotuning state per tuned kernel: {name: (choice, ms_build1, ms_build2)}
        (choice 0 = not tuned yet).  ``set_to`` {name: 0|1|2} fixes (or resets) choices."""
        out = {}
        for name, slot in self.OCC_SLOTS.items():
            c, a, b = ctypes.c_int32(), ctypes.c_float(), ctypes.c_float()
            st = -1 if not set_to or name not in set_to else int(set_to[name])
            check(lib().cgb_op_occupancy(self._h.ptr, slot, st, ctypes.byref(c), ctypes.byref(a), ctypes.byref(b)))
            out[name] = (int(c.value), float(a.value), float(b.value))
        return out

    def ff_shape(self, set_to: int | None = None) -> tuple:
        """Voxel shape of the float-float pair kernels (A, A'): 1 default, 2 a warp per voxel,
        0 timed on the next call; ``set_to`` sets both."""
        f, a = ctypes.c_int32(), ctypes.c_int32()
        check(lib().cgb_op_ff_shape(self._h.ptr, -1 if set_to is None else int(set_to), ctypes.byref(f),
                                    ctypes.byref(a)))
        return int(f.value), int(a.value)

    def ff_kernels(self, variant: int | None = None) -> int:
        """Float-float kernel family: 1 packed sample pairs (default), 0 one sample per lane;
        None only reads."""
        out = ctypes.c_int32()
        check(lib().cgb_op_ff_kernels(self._h.ptr, -1 if variant is None else int(variant), ctypes.byref(out)))
        return int(out.value)

    def tensor_cores(self, mode: int | None = None) -> bool:
        """Reduced-precision BF16 A*x and A'*y on the tensor cores: mode 0 (default) when the
        shape allows it and the operator has at least 32 IC segments per voxel, 1 CUDA cores
        only, 2 required; None only reads.  Returns whether it is in use."""
        out = ctypes.c_int32()
        check(lib().cgb_op_tensor_cores(self._h.ptr, -1 if mode is None else int(mode), ctypes.byref(out)))
        return bool(out.value)

    def device_status(self) -> None:
        """Synchronise and raise CgbError if a tensor-core kernel gave up a bounded wait."""
        check(lib().cgb_op_device_status(self._h.ptr))

    def host_mode(self, mode: int | None = None) -> int:
        """Host-buffer products: 0 automatic (direct row access for page-locked rows),
        1 staged copies, 2 direct; None only reads."""
        out = ctypes.c_int32()
        check(lib().cgb_op_host_mode(self._h.ptr, -1 if mode is None else int(mode), ctypes.byref(out)))
        return int(out.value)

    def set_slabs(self, nslab: int | None = 0) -> int:
        """Adjoint slab count (0: automatic, 1: off, None: only read); returns the count in use."""
        out = ctypes.c_int32()
        check(lib().cgb_op_set_slabs(self._h.ptr, -1 if nslab is None else int(nslab), ctypes.byref(out)))
        return int(out.value)

    def batch_width(self, set_to: int | None = None) -> int:
        """Vectors per multi-right-hand-side pass (0: chosen by timing on the next batched
        solve); ``set_to`` 0, 2 or 4 stores a value."""
        w = ctypes.c_int32()
        check(lib().cgb_op_batch_width(self._h.ptr, -1 if set_to is None else int(set_to), ctypes.byref(w)))
        return int(w.value)

    def batch_shape(self, set_to: int | None = None) -> int:
        """Voxel shape of the multi-vector kernels (1 default lanes per voxel, 2 a warp per
        voxel, 0 chosen by timing on the next batched solve)."""
        w = ctypes.c_int32()
        check(lib().cgb_op_batch_shape(self._h.ptr, -1 if set_to is None else int(set_to), ctypes.byref(w)))
        return int(w.value)

    def dot_batch(self, vs):
        """A @ v (or A' @ v) for a list of CUDA vectors in multi-right-hand-side passes
        (BF16 LUT, FP32 accumulation; 2 or 4 vectors per pass).  Forward: float64 columns
        in, float32 rows out; adjoint: float32 rows in, float64 columns out."""
        if not vs:
            return []
        din, dout = (torch.float32, torch.float64) if self.adjoint else (torch.float64, torch.float32)
        ins = []
        for v in vs:
            if not (isinstance(v, torch.Tensor) and v.is_cuda and v.dtype == din):
                raise TypeError(f'dot_batch expects CUDA {din} vectors')
            if v.numel() != self.shape[1]:
                raise RuntimeError("A.dot(): dimensions do not match")
            ins.append(v.contiguous())
        outs = [torch.empty(self.shape[0], dtype=dout, device=ins[0].device) for _ in ins]
        pin = (ctypes.c_void_p * len(ins))(*[t.data_ptr() for t in ins])
        pout = (ctypes.c_void_p * len(ins))(*[t.data_ptr() for t in outs])
        st = torch.cuda.current_stream(ins[0].device).cuda_stream
        check(lib().cgb_op_apply_batch(self._h.ptr, self.adjoint, len(ins), pin, pout, ctypes.c_void_p(st)))
        return outs

    def __matmul__(self, v):
        return self.dot(v)
