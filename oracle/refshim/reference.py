"""Run the reference's own solver code on the host CPU (oracle harness only).

Imports ``radon_tgv_primal_dual_2d.py`` / ``radon_tgv_primal_dual_3d.py`` from the
reference checkout with this package's stand-in ``pyopencl`` and ``matplotlib`` on
``sys.path`` and calls the reference entry points unmodified:
``Reconstructionapproach2d`` (radon_tgv_primal_dual_2d.py:69) and
``Reconstructionapproach3d`` (radon_tgv_primal_dual_3d.py:69).

The reference draws the power-iteration start vector from the unseeded global
NumPy generator (radon_tgv_primal_dual_3d.py:1019); :func:`run_2d` / :func:`run_3d`
seed it first and return the operator-norm estimate the run used, so that the
same value can be handed to the implementation under test.

Needs the reference checkout, named by the environment variable
``GRAPTOR_REFERENCE`` (there is no default): available where fixtures are
generated, absent on GPU machines.
"""
from __future__ import annotations

import importlib.util
import math
import os
import sys

import numpy as np

_SHIM = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: required, no default path
REFERENCE_DIR = os.environ.get("GRAPTOR_REFERENCE", "")


def available() -> bool:
    return bool(REFERENCE_DIR) and os.path.isfile(os.path.join(REFERENCE_DIR, "radon_tgv_primal_dual_3d.py"))


def _ensure_path():
    if _SHIM not in sys.path:
        sys.path.insert(0, _SHIM)
    sys.dont_write_bytecode = True  # the reference checkout is read-only


_MODS: dict = {}


def load(which: str):
    """Import the reference solver module ``radon_tgv_primal_dual_<which>``."""
    if which in _MODS:
        return _MODS[which]
    _ensure_path()
    name = f"radon_tgv_primal_dual_{which}"
    spec = importlib.util.spec_from_file_location("_graptor_ref_" + which, os.path.join(REFERENCE_DIR, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    _MODS[which] = mod
    return mod


def kernel_source(which: str) -> str:
    """The reference's OpenCL C kernel string for the 2d or 3d solver."""
    _ensure_path()
    import translate
    with open(os.path.join(REFERENCE_DIR, f"radon_tgv_primal_dual_{which}.py")) as f:
        return translate.extract_kernel_source(f.read())


def program(which: str):
    """Built stand-in ``pyopencl.Program`` of the reference's kernels (per-kernel calls)."""
    _ensure_path()
    import pyopencl as cl
    return cl.Program(cl.Context(), kernel_source(which)).build()


def _run(fn, args, seed):
    _ensure_path()
    import pyopencl as cl
    cl.SUM_LOG.clear()
    cl.COPY_LOG.clear()
    np.random.seed(seed)
    import io
    import contextlib
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        out = fn(*args)
    ne = math.sqrt(cl.SUM_LOG[-1])
    ofs = cl.COPY_LOG[0].reshape(-1, 4).T.copy()  # radon_struct's float32[4, nang]
    return out, ne, ofs


def run_2d(sino, angles, alpha, mu, maxiter, discrepancy="KL",
           method="Uncorrelated 2D Reconstruction", regularisation="TGV", seed=0):
    """Reference ``Reconstructionapproach2d``; returns (Solution, Sinograms, normest, ofs)."""
    mod = load("2d")
    import pyopencl as cl
    args = (list(sino), np.asarray(angles), tuple(alpha), np.asarray(mu, dtype=np.float64), int(maxiter),
            cl.Context(), [0, 0.1], discrepancy, method, regularisation, [0.0, 1.0, 0])
    (u, sinos), ne, ofs = _run(mod.Reconstructionapproach2d, args, seed)
    return np.asarray(u), np.asarray(sinos), ne, ofs


def run_3d(sino, angles, alpha, mu, maxiter, stepsize=1, discrepancy="KL",
           method="Frobenius 3D Reconstruction", regularisation="TGV", seed=0):
    """Reference ``Reconstructionapproach3d``; returns (Solution, Sinogram, normest, ofs)."""
    mod = load("3d")
    import pyopencl as cl
    args = (list(sino), np.asarray(angles), tuple(alpha), np.asarray(mu, dtype=np.float64), int(maxiter),
            cl.Context(), [0, 0.1], int(stepsize), discrepancy, method, regularisation, [0.0, 1.0, [0]])
    (u, sinos), ne, ofs = _run(mod.Reconstructionapproach3d, args, seed)
    return np.asarray(u), np.asarray(sinos), ne, ofs


def run_subs(sino, angles, topology, alpha, mu, maxiter, stepsize=1, discrepancy="KL",
             method="Frobenius 3D Subsampling Reconstruction", regularisation="TGV", seed=0):
    """Reference ``Reconstructionapproach3dsubsmapling``
    (radon_tgv_primal_dual_3dsubsample.py:51); returns (Solution, [Sinograms0,
    Sinograms1 fine, Sinograms1 coarse], normest).

    The module does ``from numpy import *``, which shadows the built-in ``min`` /
    ``max`` that its matrix construction (Create_Matrix_Line :587-610) calls with
    two scalars; on current NumPy that raises.  The harness restores the built-ins
    in the module's namespace (the code itself is unchanged).  The operator-norm
    estimate is sqrt(sqrt(sum U^2)) of the last power-iteration round (:551, :575)."""
    import builtins
    mod = load("3dsubsample")
    mod.min, mod.max = builtins.min, builtins.max
    import pyopencl as cl
    topo = [int(topology[0]), float(topology[1]), list(topology[2]), list(topology[3])]
    args = (list(sino), list(angles), topo, tuple(alpha), np.asarray(mu, dtype=np.float64), int(maxiter),
            cl.Context(), [0, 0.1], int(stepsize), discrepancy, method, regularisation, [0.0, 1.0, [0]])
    _ensure_path()
    cl.SUM_LOG.clear()
    cl.COPY_LOG.clear()
    np.random.seed(seed)
    import io
    import contextlib
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        u, sinos = mod.Reconstructionapproach3dsubsmapling(*args)
    ne = math.sqrt(math.sqrt(cl.SUM_LOG[-1]))
    return np.asarray(u), [np.asarray(x) for x in sinos], ne
