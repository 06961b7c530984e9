"""Differentiable COMMIT operator: ``torch.autograd.Function`` over the GB300 kernels.

``commit_apply(A, x, lut_ic=None, lut_ec=None, lut_iso=None)`` returns y = A(x) as a
CUDA float64 tensor and supports backward with respect to

* x: dLoss/dx = A' dLoss/dy (the same adjoint kernels as ``LinearOperator.T``);
* the LUTs (KERNELS['wmr'], ['wmh'], ['iso'] as float32 CUDA tensors): y is linear in
  every LUT entry, dLoss/dLUT[i,o,s] = sum over items with orientation o of
  coefficient * dLoss/dy[v,s], computed by ``cgb_op_lut_grad`` (FP64, deterministic).

When LUT tensors are passed, their current values are pushed to the operator before the
forward product (so the LUT can itself be optimised).  The reference has no gradient
path; its adjoint (commit/operator/operator.pyx:160-182) is what dLoss/dx reuses.
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import check, lib
from .operator import LinearOperator


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class CommitA(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, lut_ic, lut_ec, lut_iso, A: LinearOperator):
        if A.adjoint:
            raise ValueError('pass the forward operator')
        luts = (lut_ic, lut_ec, lut_iso)
        if any(t is not None for t in luts):
            ptrs = []
            for t in luts:
                if t is None:
                    ptrs.append(None)
                else:
                    if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
                        raise TypeError('LUT tensors must be contiguous CUDA float32')
                    ptrs.append(_vp(t))
            torch.cuda.current_stream().synchronize()
            check(lib().cgb_op_set_lut(A.handle, *ptrs))
        x64 = x.detach().to(torch.float64).contiguous()
        y = A.dot(x64)
        ctx.A = A
        ctx.x_dtype = x.dtype
        ctx.save_for_backward(x64)
        ctx.lut_shapes = [None if t is None else t.shape for t in luts]
        return y

    @staticmethod
    def backward(ctx, gy):
        A = ctx.A
        (x64,) = ctx.saved_tensors
        gy = gy.detach().to(torch.float64).contiguous()
        gx = A.T.dot(gy).to(ctx.x_dtype) if ctx.needs_input_grad[0] else None
        grads = [None, None, None]
        want = ctx.needs_input_grad[1:4]
        if any(want):
            outs = []
            for k, shp in enumerate(ctx.lut_shapes):
                outs.append(torch.zeros(shp, dtype=torch.float64, device=gy.device)
                            if (shp is not None and want[k]) else None)
            st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            check(lib().cgb_op_lut_grad(A.handle, _vp(x64), _vp(gy), _vp(outs[0]), _vp(outs[1]), _vp(outs[2]), st))
            grads = [None if o is None else o.to(torch.float32) for o in outs]
        return gx, grads[0], grads[1], grads[2], None


def commit_apply(A: LinearOperator, x: torch.Tensor, lut_ic=None, lut_ec=None, lut_iso=None) -> torch.Tensor:
    """Differentiable y = A(x) (see module docstring)."""
    return CommitA.apply(x, lut_ic, lut_ec, lut_iso, A)


def lut_gradient(A: LinearOperator, x: torch.Tensor, gy: torch.Tensor):
    """dLoss/dLUT for dLoss/dy = gy at x, as FP64 tensors (wmr, wmh, iso shapes)."""
    K = A.KERNELS
    dev = gy.device
    outs = [torch.zeros(tuple(K[k].shape), dtype=torch.float64, device=dev) if K[k].size else None
            for k in ('wmr', 'wmh', 'iso')]
    x64 = x.to(torch.float64).contiguous()
    gy = gy.to(torch.float64).contiguous()
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    check(lib().cgb_op_lut_grad(A.handle, _vp(x64), _vp(gy), _vp(outs[0]), _vp(outs[1]), _vp(outs[2]), st))
    return outs
