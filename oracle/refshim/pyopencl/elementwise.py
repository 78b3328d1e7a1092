"""Stand-in ``pyopencl.elementwise.ElementwiseKernel`` (oracle harness only).

The reference's one elementwise kernel is the extrapolation
``u[i] = 2.0f*u_[i] - u[i]`` (radon_tgv_primal_dual_3d.py:1075-1076); the operation
string is compiled as C++ over the arrays' memory.
"""
from __future__ import annotations

import ctypes

from . import Event, _compile
import translate as _tr


class ElementwiseKernel:
    def __init__(self, ctx, arguments, operation, name="elementwise", *_, **__):
        self._lib = _compile(_tr.translate_elementwise(arguments, operation), "ew")
        self._fn = self._lib.launch_elementwise
        self._fn.restype = None
        self._fn.argtypes = [ctypes.c_size_t, ctypes.c_void_p]

    def __call__(self, *arrays, wait_for=None, **_):
        n = arrays[0].size
        ptrs = (ctypes.c_void_p * len(arrays))(*[a.data.ptr for a in arrays])
        self._fn(n, ctypes.cast(ptrs, ctypes.c_void_p))
        return Event()
