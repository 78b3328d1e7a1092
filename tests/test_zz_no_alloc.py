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


SCRATCH_DOUBLES = 1 << 20  # the library's fixed scratch array (8 MiB of doubles)


def _call(angles, N, nd, device=0):
    from graptor_gb300 import _lib as L
    ang = np.ascontiguousarray(angles, np.float64)
    out = ctypes.c_double(0.0)
    rc = L.lib().gt_normest_noalloc(ctypes.c_void_p(ang.ctypes.data), N, nd, ang.size, device, None,
                                    ctypes.byref(out))
    return rc, out.value


def _noalloc(angles, N, nd):
    from graptor_gb300 import _lib as L
    rc, value = _call(angles, N, nd)
    L.check(rc)
    return value


def _allocating(angles, N, nd):
    from graptor_gb300.solver import Problem
    nang = np.asarray(angles).size
    with Problem(3, N, 2, 1, nd, angles, (4, 1), [1.0], autotune=False) as p:
        p.set_data(np.zeros((2, nang, nd), np.float32))
        return p.scalars["normest"]


@pytest.mark.parametrize("N,nd,nang", [(128, 128, 60), (256, 256, 71), (128, 135, 60), (96, 70, 33)])
def test_noalloc_matches_allocating_path_twice(N, nd, nang):
    from graptor_gb300 import phantom
    ang = phantom.angles_deg(nang)
    ref = _allocating(ang, N, nd)
    first = _noalloc(ang, N, nd)
    second = _noalloc(ang, N, nd)
    assert abs(first - ref) <= TOL * ref, (first, ref)
    assert abs(second - ref) <= TOL * ref, (second, ref)


def test_noalloc_geometry_that_fills_the_scratch_exactly():
    # 4*nang + N*N + nd*nang + 256 == 1048576 doubles: accepted, same estimate;
    # one double more: rejected
    from graptor_gb300 import _lib as L
    N, nd, nang = 1023, 1787, 1
    assert 4 * nang + N * N + nd * nang + 256 == SCRATCH_DOUBLES
    ang = np.array([np.deg2rad(30.0) + np.pi / 2])
    ref = _allocating(ang, N, nd)
    for _ in range(2):
        got = _noalloc(ang, N, nd)
        assert abs(got - ref) <= TOL * ref, (got, ref)
    rc, _ = _call(ang, N, nd + 1)
    assert rc == L.GT_ERR_ARG
    assert b"1048576" in L.lib().gt_last_error()


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


def test_noalloc_keeps_the_callers_current_device():
    torch = pytest.importorskip("torch")
    from graptor_gb300 import _lib as L
    from graptor_gb300 import phantom
    ang = phantom.angles_deg(20)
    torch.cuda.set_device(0)
    before = torch.cuda.current_device()
    _noalloc(ang, 64, 64)
    assert torch.cuda.current_device() == before
    # an ordinal no GPU has: an error status, and the current device still unchanged
    rc, _ = _call(ang, 64, 64, device=torch.cuda.device_count() + 7)
    assert rc == L.GT_ERR_CUDA
    assert torch.cuda.current_device() == before
    # a null output pointer and non-positive sizes are argument errors
    a = np.ascontiguousarray(ang, np.float64)
    assert L.lib().gt_normest_noalloc(ctypes.c_void_p(a.ctypes.data), 64, 64, a.size, 0, None, None) == L.GT_ERR_ARG
    assert _call(ang, 0, 64)[0] == L.GT_ERR_ARG
    # and the entry point still works afterwards
    assert _noalloc(ang, 64, 64) > 0
