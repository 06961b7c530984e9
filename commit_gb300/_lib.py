"""ctypes binding of libcommit_gb300.so (declarations in include/commit_gb300.h).

The library is built in-tree by commit_gb300/build.py.  There is no fallback: if the
shared library is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libcommit_gb300.so')

CGB_OK, CGB_ERR_INVALID, CGB_ERR_CUDA, CGB_ERR_NOMEM, CGB_ERR_UNSUPPORTED, CGB_ERR_DIMENSION, CGB_ERR_BACKTRACK = range(7)
ARITH = {'f64': 0, 'ff': 1, 'bf16': 2, 'fp16': 3, 'f32': 4}
DTYPE_F64, DTYPE_F32 = 0, 1
REG = {None: 0, 'lasso': 1, 'group_lasso': 2, 'sparse_group_lasso': 3}
CRITERIA = ['Absolute tolerance on the objective', 'Relative tolerance on the objective',
            'Absolute tolerance on the unknowns', 'Relative tolerance on the unknowns',
            'Maximum number of iterations']

c_i32, c_i64, c_f64, c_vp = ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p


class CgbReg(ctypes.Structure):
    _fields_ = [('start_ic', c_i64), ('size_ic', c_i64), ('start_ec', c_i64), ('size_ec', c_i64),
                ('start_iso', c_i64), ('size_iso', c_i64),
                ('reg_ic', c_i32), ('reg_ec', c_i32), ('reg_iso', c_i32),
                ('nn_ic', c_i32), ('nn_ec', c_i32), ('nn_iso', c_i32),
                ('lambda_ic', c_f64), ('lambda_ic_group', c_f64), ('lambda_ec', c_f64), ('lambda_iso', c_f64),
                ('coeff_weights', c_vp), ('weighted_ic', c_i32), ('weighted_iso', c_i32),
                ('group_idx', c_vp), ('group_ptr', c_vp), ('group_w', c_vp), ('ngroups', c_i64),
                ('level_ptr', c_vp), ('nlevels', c_i64)]


class CgbFistaParams(ctypes.Structure):
    _fields_ = [('tol_fun', c_f64), ('tol_x', c_f64), ('max_iter', c_i32), ('verbose', c_i32),
                ('arith', c_i32), ('momentum_reuse', c_i32), ('x_ref', c_vp), ('trace', c_vp), ('trace_len', c_i32),
                ('graph', c_i32), ('max_backtracks', c_i32), ('restart', c_i32), ('trace_cost', c_i32)]


class CgbFistaResult(ctypes.Structure):
    _fields_ = [('residual', c_f64), ('regterm', c_f64), ('cost_function', c_f64), ('abs_cost', c_f64),
                ('rel_cost', c_f64), ('abs_x', c_f64), ('rel_x', c_f64), ('iterations', c_i32),
                ('stopping_criterion', c_i32), ('backtracks', c_i32), ('operator_calls', c_i32),
                ('anchors', c_i32)]


class CgbT2DParams(ctypes.Structure):
    _fields_ = [('dim', c_i32 * 3), ('pixdim', ctypes.c_float * 3), ('fiber_shift', ctypes.c_float * 3),
                ('min_seg_len', ctypes.c_float), ('min_fiber_len', ctypes.c_float), ('max_fiber_len', ctypes.c_float),
                ('do_intersect', c_i32), ('n_replicas', c_i32), ('blur_rho', c_vp), ('blur_angle', c_vp),
                ('blur_weights', c_vp), ('n_peaks', c_i32), ('vf_thr', ctypes.c_float), ('flip', c_i32 * 3),
                ('peaks_affine', c_f64 * 9)]


class CgbT2DResult(ctypes.Structure):
    _fields_ = [('n_fibers', c_i64), ('n_kept', c_i64), ('n_segments', c_i64), ('n_ec', c_i64), ('n_iso', c_i64),
                ('ic_f', c_vp), ('ic_v', c_vp), ('ic_o', c_vp), ('ic_len', c_vp), ('trk_norm', c_vp),
                ('trk_len', c_vp), ('trk_lentot', c_vp), ('trk_kept', c_vp), ('ec_v', c_vp), ('ec_o', c_vp),
                ('iso_v', c_vp), ('tdi', c_vp)]


_lib = None


class CgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def lib() -> ctypes.CDLL:
    """Load the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f'{LIB_PATH} is missing: build it with commit_gb300.build.build()')
    L = ctypes.CDLL(LIB_PATH)
    L.cgb_last_error.restype = ctypes.c_char_p
    L.cgb_version.restype = ctypes.c_char_p
    P = c_vp
    L.cgb_op_create.argtypes = [c_i32, c_i32, c_i32, c_i32, c_i64, c_i32, c_i32, c_i32,
                                P, P, P, P, P, P, P, P, P, P, P, c_i32, c_i32, c_i32, c_i32, c_i32,
                                ctypes.POINTER(c_vp)]
    L.cgb_op_destroy.argtypes = [P]
    L.cgb_op_shape.argtypes = [P, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)]
    L.cgb_op_device_bytes.argtypes = [P, ctypes.POINTER(ctypes.c_size_t)]
    L.cgb_op_set_arith.argtypes = [P, c_i32]
    L.cgb_op_set_lut.argtypes = [P, P, P, P]
    L.cgb_op_lut_grad.argtypes = [P, P, P, P, P, P, P]
    L.cgb_op_apply.argtypes = [P, c_i32, P, c_i64, P, c_i64, c_i32, c_i32, P]
    L.cgb_op_apply_host.argtypes = [P, c_i32, P, c_i64, P, c_i64]
    L.cgb_op_adjoint_noalloc.argtypes = [c_i32, c_i32, c_i32, c_i64, c_i32, c_i32, c_i32, P, P,
                                         P, P, P, P, P, P, P, P, P, P, P, c_i32, c_i32, c_i32, P, P, P]
    L.cgb_fista_run.argtypes = [P, P, P, ctypes.POINTER(CgbReg), ctypes.POINTER(CgbFistaParams), P,
                                ctypes.POINTER(CgbFistaResult), P]
    L.cgb_fista_batch_run.argtypes = [P, P, P, ctypes.POINTER(CgbReg), c_i32, ctypes.POINTER(CgbFistaParams),
                                      ctypes.POINTER(c_vp), ctypes.POINTER(CgbFistaResult), P]
    L.cgb_op_host_mode.argtypes = [P, c_i32, ctypes.POINTER(c_i32)]
    L.cgb_op_tensor_cores.argtypes = [P, c_i32, ctypes.POINTER(c_i32)]
    L.cgb_dict_relayout.argtypes = [P, c_i64, c_i64, c_i32, P, P, P, P, P, c_i32, c_i64, P, P, c_i64, P,
                                    ctypes.POINTER(c_i64), P]
    L.cgb_op_device_status.argtypes = [P]
    L.cgb_op_ff_shape.argtypes = [P, c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32)]
    L.cgb_op_ff_kernels.argtypes = [P, c_i32, ctypes.POINTER(c_i32)]
    L.cgb_op_set_slabs.argtypes = [P, c_i32, ctypes.POINTER(c_i32)]
    L.cgb_op_occupancy.argtypes = [P, c_i32, c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(ctypes.c_float),
                                   ctypes.POINTER(ctypes.c_float)]
    L.cgb_op_batch_width.argtypes = [P, c_i32, ctypes.POINTER(c_i32)]
    L.cgb_op_batch_shape.argtypes = [P, c_i32, ctypes.POINTER(c_i32)]
    L.cgb_op_apply_batch.argtypes = [P, c_i32, c_i32, ctypes.POINTER(c_vp), ctypes.POINTER(c_vp), P]
    L.cgb_op_voxel_maps.argtypes = [P, P, P, P, P, P, P, P, P, P, P, P, P]
    L.cgb_trk2dict.argtypes = [ctypes.POINTER(CgbT2DParams), P, P, c_i64, P, P, P, P, P, ctypes.POINTER(CgbT2DResult), P]
    L.cgb_trk2dict_free.argtypes = [ctypes.POINTER(CgbT2DResult)]
    L.cgb_prox_non_negativity.argtypes = [P, c_i64, c_i64, P]
    L.cgb_prox_soft_thresholding.argtypes = [P, c_f64, c_i64, c_i64, P]
    L.cgb_prox_w_soft_thresholding.argtypes = [P, P, c_f64, c_i64, c_i64, P]
    L.cgb_prox_projection_onto_l2_ball.argtypes = [P, c_f64, c_i64, c_i64, P]
    L.cgb_prox_group_lasso.argtypes = [P, c_i64, P, P, P, c_i64, P, c_i64, c_f64, P]
    L.cgb_omega_group_lasso.argtypes = [P, c_i64, P, P, P, c_i64, c_f64, ctypes.POINTER(c_f64), P]
    L.cgb_omega_sparse_group_lasso.argtypes = [P, c_i64, P, P, P, P, c_i64, c_f64, c_f64, ctypes.POINTER(c_f64), P]
    L.cgb_omega_l1.argtypes = [P, P, c_i64, c_i64, c_f64, ctypes.POINTER(c_f64), P]
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != CGB_OK:
        msg = lib().cgb_last_error().decode(errors='replace')
        if rc == CGB_ERR_DIMENSION:
            raise RuntimeError(msg)
        raise CgbError(rc, f'commit_gb300 error {rc}: {msg}')


def exported_symbols() -> list:
    """Names declared in include/commit_gb300.h (for the load test)."""
    hdr = os.path.join(os.path.dirname(HERE), 'include', 'commit_gb300.h')
    import re
    names = []
    for line in open(hdr):
        m = re.match(r'^\s*(?:int|const char \*)\s*(cgb_\w+)\s*\(', line)
        if m:
            names.append(m.group(1))
    return names
