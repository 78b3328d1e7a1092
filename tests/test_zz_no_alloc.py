"""The allocation-free operator-norm entry point, through the C ABI.

gt_normest_noalloc serves callers that cannot allocate device memory while they
run (a host framework that owns the device memory pool, or code that cannot
afford cudaFree's device-wide synchronisation).  It must give the estimate the
allocating path (gt_set_data with no supplied estimate) gives, call after call,
with its scratch in the library's fixed device array.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10  # same FP64 algorithm and reduction order on both paths


def _noalloc(angles, N, nd):
    from graptor_gb300 import _lib as L
    ang = np.ascontiguousarray(angles, np.float64)
    out = ctypes.c_double(0.0)
    rc = L.lib().gt_normest_noalloc(ctypes.c_void_p(ang.ctypes.data), N, nd, ang.size, 0, None, ctypes.byref(out))
    L.check(rc)
    return out.value


@pytest.mark.parametrize("N,nang", [(128, 60), (256, 71)])
def test_noalloc_matches_allocating_path_twice(N, nang):
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    ang = phantom.angles_deg(nang)
    with Problem(3, N, 2, 1, N, ang, (4, 1), [1.0]) as p:
        p.set_data(np.zeros((2, nang, N), np.float32))
        ref = p.scalars["normest"]
    first = _noalloc(ang, N, N)
    second = _noalloc(ang, N, N)
    assert abs(first - ref) <= TOL * ref, (first, ref)
    assert abs(second - ref) <= TOL * ref, (second, ref)


def test_noalloc_does_not_allocate_device_memory():
    torch = pytest.importorskip("torch")
    from graptor_gb300 import phantom
    ang = phantom.angles_deg(50)
    _noalloc(ang, 96, 96)  # first call on the device: scratch address set-up
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _noalloc(ang, 96, 96)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_geometry_beyond_scratch():
    from graptor_gb300 import _lib as L
    ang = np.linspace(0, np.pi, 10)
    out = ctypes.c_double(0.0)
    rc = L.lib().gt_normest_noalloc(ctypes.c_void_p(ang.ctypes.data), 1100, 1100, 10, 0, None, ctypes.byref(out))
    assert rc == L.GT_ERR_ARG
    assert b"1048576" in L.lib().gt_last_error()
