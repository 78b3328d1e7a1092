"""ctypes binding of libgraptor_gb300.so (the C ABI in include/graptor_gb300.h).

The library is built in-tree by graptor_gb300/build.py.  There is no CPU
fallback: if the library is missing or cannot load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgraptor_gb300.so")

GT_OK, GT_ERR_OOM, GT_ERR_ARG, GT_ERR_TIMEOUT, GT_ERR_CUDA, GT_ERR_STATE = range(6)
GT_KL, GT_L2 = 0, 1
GT_TV, GT_TGV = 0, 1
GT_UNCORR, GT_FROB, GT_NUCL = 0, 1, 2
FIELDS = {"u": 0, "ubar": 1, "p": 2, "pbar": 3, "v": 4, "w": 5, "lambda": 6, "ku": 7, "data": 8, "ulo": 9}


class GraptorError(RuntimeError):
    """A library call failed (the reference raises pyopencl.Error here)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class GraptorMemoryError(GraptorError, MemoryError):
    """Device allocation failed (the reference raises pyopencl.MemoryError here,
    which Reconstruction_coupled.py:509-536 answers with a smaller slice chunk)."""


class GraptorTimeoutError(GraptorError, TimeoutError):
    pass


class GtDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("N", ctypes.c_int), ("Nz", ctypes.c_int), ("C", ctypes.c_int),
        ("nd", ctypes.c_int), ("nang", ctypes.c_int), ("angles", ctypes.POINTER(ctypes.c_double)),
        ("stepsize", ctypes.c_float), ("alpha0", ctypes.c_double), ("alpha1", ctypes.c_double),
        ("mu", ctypes.POINTER(ctypes.c_double)), ("discrepancy", ctypes.c_int), ("regularisation", ctypes.c_int),
        ("coupling", ctypes.c_int), ("normest", ctypes.c_double), ("device", ctypes.c_int),
        ("stream", ctypes.c_void_p), ("autotune", ctypes.c_int),
    ]


class GtSubsDesc(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int), ("Nz", ctypes.c_int), ("C0", ctypes.c_int), ("C1", ctypes.c_int),
        ("nang0", ctypes.c_int), ("nang1", ctypes.c_int), ("nd1", ctypes.c_int), ("Nz1", ctypes.c_int),
        ("angles0", ctypes.POINTER(ctypes.c_double)), ("angles1", ctypes.POINTER(ctypes.c_double)),
        ("stepsize", ctypes.c_float), ("alpha0", ctypes.c_double), ("alpha1", ctypes.c_double),
        ("mu", ctypes.POINTER(ctypes.c_double)), ("discrepancy", ctypes.c_int), ("regularisation", ctypes.c_int),
        ("coupling", ctypes.c_int), ("pixel_ratio", ctypes.c_double), ("refold", ctypes.c_double * 2),
        ("refnew", ctypes.c_double * 2), ("normest", ctypes.c_double), ("device", ctypes.c_int),
        ("stream", ctypes.c_void_p),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_SIGS = {
    "gt_problem_create": (ctypes.c_int, [ctypes.POINTER(GtDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "gt_problem_destroy": (None, [_P]),
    "gt_set_data": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "gt_run": (ctypes.c_int, [_P, ctypes.c_int]),
    "gt_synchronize": (ctypes.c_int, [_P]),
    "gt_get_state": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "gt_get_output_f64": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "gt_set_precise_primal": (ctypes.c_int, [_P, ctypes.c_int]),
    "gt_get_precise_primal": (ctypes.c_int, [_P]),
    "gt_set_state": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "gt_get_scalars": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double)]),
    "gt_get_tuning": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    "gt_gap": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double)]),
    "gt_gap_ex": (ctypes.c_int, [_P, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "gt_radon": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]),
    "gt_radon_ad": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]),
    "gt_launches_per_iteration": (ctypes.c_int, [_P]),
    "gt_time_kernels": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
    "gt_normest_noalloc": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P,
                                          ctypes.POINTER(ctypes.c_double)]),
    "gt_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(GtDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "gt_batch_destroy": (None, [_P]),
    "gt_batch_size": (ctypes.c_int, [_P]),
    "gt_batch_problem": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "gt_batch_run": (ctypes.c_int, [_P, ctypes.c_int]),
    "gt_batch_synchronize": (ctypes.c_int, [_P]),
    "gt_batch_invalidate": (ctypes.c_int, [_P]),
    "gt_batch_set_concurrency": (ctypes.c_int, [_P, ctypes.c_int]),
    "gt_batch_set_active": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "gt_batch_set_mode": (ctypes.c_int, [_P, _I]),
    "gt_batch_get_mode": (ctypes.c_int, [_P]),
    "gt_get_state_device": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "gt_set_state_device": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "gt_problem_stream": (ctypes.c_void_p, [_P]),
    "gt_dual_from_primal": (ctypes.c_int, [_P]),
    "gt_dual_from_primal_ex": (ctypes.c_int, [_P, _I, ctypes.c_float]),
    "gt_set_tuning": (ctypes.c_int, [_P, _I, _I]),
    "gt_set_dual_shape": (ctypes.c_int, [_P, _I]),
    "gt_get_dual_shape": (ctypes.c_int, [_P]),
    "gt_set_schedule": (ctypes.c_int, [_P, _I]),
    "gt_get_schedule": (ctypes.c_int, [_P]),
    "gt_set_primal_weight": (ctypes.c_int, [_P, ctypes.c_double]),
    "gt_get_primal_weight": (ctypes.c_double, [_P]),
    "gt_restart": (ctypes.c_int, [_P]),
    "gt_snapshot": (ctypes.c_int, [_P]),
    "gt_movement": (ctypes.c_int, [_P, _P]),
    "gt_test_bp_stall": (ctypes.c_int, [_P, _I, ctypes.c_uint]),
    "gt_nn_conv3d": (ctypes.c_int, [_P, _I, _I, _I, _I, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _P]),
    "gt_nn_flip_weights": (ctypes.c_int, [_P, _P, _I, _I, _I, _P]),
    "gt_nn_conv3d_wgrad": (ctypes.c_int, [_P, _I, _I, _I, _P, _I, _I, _I, _I, _I, _I, _I, _I, _I, _LL, _P, _P, _I,
                                          _P]),
    "gt_nn_bias_grad": (ctypes.c_int, [_P, _I, _I, _I, _I, _LL, _P, _I, _P]),
    "gt_nn_scale": (ctypes.c_int, [_P, _I, _P, _I, _I, _I, _LL, _P, _I, _P]),
    "gt_nn_relu_bwd": (ctypes.c_int, [_P, _P, _I, _I, _I, _I, _I, _LL, _P]),
    "gt_nn_pool2": (ctypes.c_int, [_P, _I, _I, _P, _I, _I, _I, _I, _I, _P]),
    "gt_nn_pool2_bwd": (ctypes.c_int, [_P, _P, _I, _I, _I, _I, _I, _I, _I, _P]),
    "gt_nn_up2": (ctypes.c_int, [_P, _P, _I, _I, _I, _I, _I, _I, _I, _P]),
    "gt_nn_up2_bwd": (ctypes.c_int, [_P, _I, _I, _P, _I, _I, _I, _I, _I, _P]),
    "gt_nn_mse": (ctypes.c_int, [_P, _P, _LL, _P, _P, _P]),
    "gt_nn_adam": (ctypes.c_int, [_P, _P, _P, _P, _P, _LL, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, _I, _P]),
    "gt_nn_cast": (ctypes.c_int, [_P, _I, _P, _LL, _P]),
    "gt_nn_set_tensor_cores": (ctypes.c_int, [_I]),
    "gt_nn_check": (ctypes.c_int, []),
    "gt_badproj_smooth": (ctypes.c_int, [_P, _I, _I, _I, _I, _P, _P]),
    "gt_badproj_wgrad": (ctypes.c_int, [_P, _I, _I, _I, _P, _P]),
    "gt_badproj_blocks": (ctypes.c_int, [_I, _I, _I]),
    "gt_badproj_compare": (ctypes.c_int, [_P, _I, _I, _I, _I, _I, _P, _P, _P, _P]),
    "gt_subs_create": (ctypes.c_int, [ctypes.POINTER(GtSubsDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "gt_subs_destroy": (None, [_P]),
    "gt_subs_set_data": (ctypes.c_int, [_P, _P, _P, _I]),
    "gt_subs_run": (ctypes.c_int, [_P, _I]),
    "gt_subs_get": (ctypes.c_int, [_P, _I, _P]),
    "gt_subs_normest": (ctypes.c_double, [_P]),
    "gt_subs_problem": (ctypes.c_void_p, [_P]),
    "gt_last_error": (ctypes.c_char_p, []),
    "gt_version": (ctypes.c_char_p, []),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load the CUDA library; raises ImportError (no fallback) if it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m graptor_gb300.build` "
                              "(graptor_gb300 has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc == GT_OK:
        return
    msg = lib().gt_last_error().decode(errors="replace")
    if rc == GT_ERR_OOM:
        raise GraptorMemoryError(rc, msg)
    if rc == GT_ERR_TIMEOUT:
        raise GraptorTimeoutError(rc, msg)
    if rc == GT_ERR_ARG:
        raise ValueError(f"[{rc}] {msg}")
    raise GraptorError(rc, msg)
