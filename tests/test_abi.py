"""C ABI checks that need no GPU: the library loads, exports every function the
public header declares, and rejects invalid descriptions before touching CUDA."""
import ctypes
import os
import re

import numpy as np
import pytest

from graptor_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^GT_API\s+[\w\s\*]*?\b(gt_\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_library_loads_and_exports_every_declared_symbol():
    lib = L.lib()
    names = header_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"
    assert b"sm_103a" in lib.gt_version()


def _desc(**kw):
    ang = np.linspace(0, np.pi, 8)
    mu = np.ones(2)
    d = L.GtDesc()
    d.dim, d.N, d.Nz, d.C, d.nd, d.nang = 3, 16, 4, 2, 16, ang.size
    d.angles = ang.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.stepsize, d.alpha0, d.alpha1 = 1.0, 4.0, 1.0
    d.mu = mu.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.discrepancy, d.regularisation, d.coupling = 0, 1, 1
    for k, v in kw.items():
        setattr(d, k, v)
    return d, (ang, mu)


@pytest.mark.parametrize("field,value", [("dim", 4), ("N", 0), ("C", 9), ("discrepancy", 7), ("coupling", 3),
                                         ("stepsize", 0.0), ("alpha0", -1.0), ("nang", 0)])
def test_invalid_descriptions_rejected(field, value):
    d, keep = _desc(**{field: value})
    h = ctypes.c_void_p()
    rc = L.lib().gt_problem_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == L.GT_ERR_ARG
    assert not h.value
    assert L.lib().gt_last_error()
    with pytest.raises(ValueError):
        L.check(rc)


def test_null_arguments():
    lib = L.lib()
    assert lib.gt_problem_create(None, None) == L.GT_ERR_ARG
    assert lib.gt_run(None, 1) == L.GT_ERR_ARG
    assert lib.gt_set_data(None, None, 1) == L.GT_ERR_ARG
    assert lib.gt_get_state(None, 0, None) == L.GT_ERR_ARG
    assert lib.gt_get_output_f64(None, 0, None) == L.GT_ERR_ARG
    lib.gt_problem_destroy(None)
    # bad-projection stages: rejected on the host before any launch
    assert lib.gt_badproj_smooth(None, 3, 40, 40, 3, None, None) == L.GT_ERR_ARG
    assert lib.gt_badproj_wgrad(None, 3, 40, 40, None, None) == L.GT_ERR_ARG
    assert lib.gt_badproj_compare(None, 3, 40, 40, 1, 3, None, None, None, None) == L.GT_ERR_ARG


def test_badproj_block_count():
    """Partial sums per pair: 32 x 32 interior tiles; 0 when the radius leaves no interior."""
    lib = L.lib()
    assert lib.gt_badproj_blocks(20, 30, 3) == 1
    assert lib.gt_badproj_blocks(100, 100, 2) == 9
    assert lib.gt_badproj_blocks(248, 248, 25) == 7 * 7
    assert lib.gt_badproj_blocks(20, 30, 10) == 0
    assert lib.gt_badproj_blocks(20, 30, -1) == 0


def test_error_mapping():
    with pytest.raises(MemoryError):
        L.check(L.GT_ERR_OOM)
    with pytest.raises(L.GraptorError):
        L.check(L.GT_ERR_CUDA)
    with pytest.raises(TimeoutError):
        L.check(L.GT_ERR_TIMEOUT)


def test_product_never_uses_the_oracle():
    """The package's modules never import the oracle (it is test infrastructure)."""
    pkg = os.path.join(ROOT, "graptor_gb300")
    pat = re.compile(r"^\s*(import\s+oracle\b|from\s+oracle\b|from\s+\.\.oracle\b)", re.M)
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                with open(os.path.join(dirpath, f)) as fh:
                    assert not pat.search(fh.read()), os.path.join(dirpath, f)
