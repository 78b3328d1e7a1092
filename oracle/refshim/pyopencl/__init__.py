"""Stand-in ``pyopencl`` that runs the reference's OpenCL kernels on the host CPU.

Test infrastructure only (the oracle harness): it lets the reference's own
``Reconstructionapproach2d/3d`` (radon_tgv_primal_dual_2d.py:69,
radon_tgv_primal_dual_3d.py:69) run unmodified in a container without an OpenCL
platform.  ``Program.build`` translates the kernel string (oracle/refshim/translate.py)
and compiles it with g++ into ``oracle/_ref/``; buffers are NumPy byte arrays and
the single in-order queue executes every enqueue synchronously, which is the
ordering the reference's in-order ``CommandQueue`` gives.

Only the API surface the reference touches is provided.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SHIM = os.path.dirname(_HERE)
_OUT = os.path.join(os.path.dirname(_SHIM), "_ref")

sys.path.insert(0, _SHIM)
import translate as _tr  # noqa: E402

# every float32 reduction result (clarray.sum) in call order: the power iteration
# radon_normest (radon_tgv_primal_dual_3d.py:1018-1030) is the only caller, so the
# operator-norm estimate of a run is sqrt(last entry).
SUM_LOG: list = []
# every host->device copy into a plain Buffer (the angle table of radon_struct)
COPY_LOG: list = []


class Error(Exception):
    pass


class MemoryError(Error):  # noqa: A001 - mirrors pyopencl.MemoryError
    pass


class mem_flags:  # noqa: N801
    READ_ONLY = 1 << 2
    WRITE_ONLY = 1 << 1
    READ_WRITE = 1 << 0
    COPY_HOST_PTR = 1 << 5


class device_type:  # noqa: N801
    GPU = 4
    CPU = 2


class Device:
    type = device_type.CPU
    global_mem_size = 64 << 30
    max_mem_alloc_size = 16 << 30
    name = "host CPU (reference OpenCL C via C++ translation)"


class Platform:
    def get_devices(self):
        return [Device()]


def get_platforms():
    return [Platform()]


class Context:
    def __init__(self, devices=None):
        self.devices = devices or [Device()]


def create_some_context(*_a, **_k):
    return Context()


class Event:
    def wait(self):
        return None


class CommandQueue:
    def __init__(self, ctx, *_, **__):
        self.context = ctx

    def finish(self):
        return None


class Buffer:
    """Raw device memory: a NumPy uint8 array whose address kernels receive."""

    def __init__(self, ctx, flags=0, size=0, hostbuf=None):
        self.context = ctx
        self.flags = flags
        nbytes = int(size) if hostbuf is None else np.asarray(hostbuf).nbytes
        self.host = np.zeros(max(nbytes, 1), dtype=np.uint8)
        if hostbuf is not None:
            self.host[:nbytes] = _raw_bytes(hostbuf)
        self.size = nbytes

    @property
    def ptr(self):
        return self.host.ctypes.data


def _raw_bytes(obj) -> np.ndarray:
    """Bytes of ``obj`` in MEMORY order (an F-ordered array stays F-ordered)."""
    a = np.asarray(obj)
    if a.flags.f_contiguous and not a.flags.c_contiguous:
        a = a.ravel(order="F")
    else:
        a = np.ascontiguousarray(a).ravel()
    return a.view(np.uint8)


def enqueue_copy(queue, dest, src, *_, **__):
    if isinstance(dest, Buffer):
        raw = _raw_bytes(src)
        dest.host[: raw.size] = raw
        COPY_LOG.append(raw.view(np.float32).copy() if raw.size % 4 == 0 else raw.copy())
    else:
        d = np.asarray(dest)
        raw = src.host[: d.nbytes]
        flat = d.reshape(-1, order="A")
        flat.view(np.uint8)[:] = raw
    return Event()


# ---- kernels -------------------------------------------------------------------------

def _compile(cpp: str, tag: str) -> ctypes.CDLL:
    os.makedirs(_OUT, exist_ok=True)
    h = hashlib.sha256(cpp.encode()).hexdigest()[:16]
    so = os.path.join(_OUT, f"ref_{tag}_{h}.so")
    if not os.path.exists(so):
        src = os.path.join(_OUT, f"ref_{tag}_{h}.cpp")
        with open(src, "w") as f:
            f.write(cpp)
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               f"-I{_SHIM}", src, "-o", so + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(so + ".tmp", so)
    return ctypes.CDLL(so)


def _arg_ptr(a, keep):
    if hasattr(a, "ptr"):  # Buffer, or the .data view of a pyopencl.array.Array
        return ctypes.c_void_p(a.ptr)
    if isinstance(a, (np.generic,)):
        box = np.array([a], dtype=a.dtype)
        keep.append(box)
        return ctypes.c_void_p(box.ctypes.data)
    raise TypeError(f"unsupported kernel argument {type(a)}")


class Kernel:
    def __init__(self, lib, sig):
        self.function_name = sig.name
        self._sig = sig
        self._fn = getattr(lib, "launch_" + sig.name)
        self._fn.restype = None
        self._fn.argtypes = [ctypes.c_size_t] * 3 + [ctypes.c_void_p]

    def __call__(self, queue, global_size, local_size, *args, wait_for=None, **_):
        if len(args) != len(self._sig.params):
            raise Error(f"{self.function_name}: expected {len(self._sig.params)} args, got {len(args)}")
        if len(tuple(global_size)) == 0:
            # TV mode enqueues update_w_empty over w.shape[1:] == () of a 1-element
            # buffer (radon_tgv_primal_dual_3d.py:1044-1046, :1163-1164): an empty
            # NDRange has no work-items, so nothing runs (one item would write a
            # float8 into 4 bytes).
            return Event()
        g = tuple(int(x) for x in global_size) + (1, 1, 1)
        keep: list = []
        ptrs = (ctypes.c_void_p * max(len(args), 1))(*[_arg_ptr(a, keep) for a in args])
        self._fn(g[0], g[1], g[2], ctypes.cast(ptrs, ctypes.c_void_p))
        return Event()


class Program:
    def __init__(self, ctx, src):
        self.context = ctx
        self.src = src
        self._kernels = []

    def build(self, *_, **__):
        cpp, sigs = _tr.translate(self.src)
        lib = _compile(cpp, "prog")
        self._kernels = [Kernel(lib, s) for s in sigs]
        for k in self._kernels:
            setattr(self, k.function_name, k)
        return self

    def all_kernels(self):
        return list(self._kernels)


from . import array  # noqa: E402,F401
from . import elementwise  # noqa: E402,F401
