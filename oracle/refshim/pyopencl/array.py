"""Stand-in ``pyopencl.array`` backed by NumPy (oracle harness only).

Arrays keep the memory order the reference asks for (``order='F'`` everywhere in
radon_tgv_primal_dual_{2d,3d}.py), and ``.data`` hands kernels the address of that
memory, so a translated kernel indexes exactly the bytes the OpenCL kernel would.
"""
from __future__ import annotations

import numpy as np

from . import SUM_LOG, Event


class _Data:
    def __init__(self, arr):
        self._arr = arr

    @property
    def ptr(self):
        return self._arr.ctypes.data


class Array:
    def __init__(self, queue, shape, dtype=np.float32, order="C", host=None):
        self.queue = queue
        if host is None:
            host = np.zeros(shape, dtype=dtype, order=order)
        self._a = host
        self.events = []

    # ---- attributes the reference reads
    @property
    def shape(self):
        return self._a.shape

    @property
    def dtype(self):
        return self._a.dtype

    @property
    def size(self):
        return self._a.size

    @property
    def nbytes(self):
        return self._a.nbytes

    @property
    def data(self):
        return _Data(self._a)

    def add_event(self, ev):
        self.events.append(ev)

    def finish(self):
        self.events = []

    def get(self, *_, **__):
        return self._a.copy(order="K")

    def __setitem__(self, key, value):
        self._a[key] = value

    def __itruediv__(self, other):
        # pyopencl scales by the float32-cast reciprocal for a scalar divisor
        self._a *= self._a.dtype.type(1.0 / other)
        return self

    def __imul__(self, other):
        self._a *= self._a.dtype.type(other)
        return self

    def __pow__(self, other):
        # elementwise power in the array's type (the subsampling solver's norm, U_**2)
        out = self._a ** self._a.dtype.type(other)
        order = "F" if (self._a.flags.f_contiguous and not self._a.flags.c_contiguous) else "C"
        return Array(self.queue, out.shape, out.dtype, order, host=np.asarray(out, order=order))


def to_device(queue, ary, *_, **__):
    a = np.asarray(ary)
    order = "F" if (a.flags.f_contiguous and not a.flags.c_contiguous) else "C"
    return Array(queue, a.shape, a.dtype, order, host=a.copy(order=order))


def empty(queue, shape, dtype=np.float32, order="C", *_, **__):
    return Array(queue, shape, dtype, order)


def zeros(queue, shape, dtype=np.float32, order="C", *_, **__):
    return Array(queue, shape, dtype, order)


def zeros_like(a):
    order = "F" if (a._a.flags.f_contiguous and not a._a.flags.c_contiguous) else "C"
    return Array(a.queue, a.shape, a.dtype, order)


class _Scalar:
    def __init__(self, v):
        self._v = v

    def get(self, *_, **__):
        return self._v


def sum(a, *_, **__):  # noqa: A001 - mirrors pyopencl.array.sum
    v = np.sum(a._a, dtype=a.dtype)
    SUM_LOG.append(float(v))
    return _Scalar(v)


__all__ = ["Array", "to_device", "empty", "zeros", "zeros_like", "sum", "Event"]
