"""Drop-in for the reference's 2-D (slice-wise) solver entry point.

``Reconstructionapproach2d`` has the signature, argument meaning and return
values of radon_tgv_primal_dual_2d.py:69 (called per slice from
Reconstruction_coupled.py:233); differences are those listed in
radon_tgv_primal_dual_3d.py of this package.  :func:`reconstruct_slices` solves
many slices of one tilt series in a single launch sequence (the reference
calls the 2-D solver once per slice).
"""
from __future__ import annotations

import numpy as np

from ._lib import GraptorError, GraptorMemoryError  # noqa: F401
from . import radon_tgv_primal_dual_3d as _r3
from .solver import METHODS, Problem


def Reconstructionapproach2d(sino, angles, Parameter, mu, maxiter, ctx, plott, discrepancy,
                             regularisationmethod, regularisation, Info, normest=None):
    """sino: list of C arrays [nang, nd]. Returns (Solution[C, N, N] float64,
    list of C float32 sinograms [nang, nd]) with N = nd (2-D :838-851)."""
    start, sectionwidth, current = Info[0], Info[1], Info[2]
    C = len(sino)
    nang, nd = np.asarray(sino[0]).shape
    dim, coupling = METHODS.get(regularisationmethod, (2, None))
    if coupling is None or dim != 2:
        raise ValueError(f"unknown 2-D regularisation method {regularisationmethod!r}")
    f = np.stack([np.asarray(s, dtype=np.float32) for s in sino])  # [C, nang, nd]
    with Problem(2, nd, 1, C, nd, angles, Parameter, np.asarray(mu, dtype=np.float64), discrepancy,
                 regularisation, coupling, 1.0, normest, _r3._device(ctx)) as prob:
        prob.set_data(f, feasible=True)
        _r3.run_with_progress(prob, int(maxiter), start, sectionwidth, str(current), "Slice")
        u = prob.get("u")    # [c, y, x]
        ku = prob.get("ku")  # [c, nang, nd]
    solution = np.transpose(u, (0, 2, 1)).astype(np.float64)
    return solution, [ku[c].copy() for c in range(C)]


def reconstruct_slices(sinos, angles, Parameter, mu, maxiter, discrepancy="KL",
                       regularisationmethod="Uncorrelated 2D Reconstruction", regularisation="TGV",
                       device=0, normest=None):
    """Many independent 2-D slices in one solve: sinos[C][nang, Nz, nd] -> u[C, Nz, N, N].

    Same per-slice problem as Reconstructionapproach2d (slices are not coupled;
    the operator norm of the shared geometry is estimated once)."""
    C = len(sinos)
    nang, Nz, nd = np.asarray(sinos[0]).shape
    dim, coupling = METHODS[regularisationmethod]
    f = np.empty((C, Nz, nang, nd), np.float32)
    for c in range(C):
        f[c] = np.transpose(np.asarray(sinos[c], dtype=np.float32), (1, 0, 2))
    with Problem(2, nd, Nz, C, nd, angles, Parameter, np.asarray(mu, dtype=np.float64), discrepancy,
                 regularisation, coupling, 1.0, normest, device) as prob:
        prob.set_data(f.reshape(C * Nz, nang, nd), feasible=True)
        prob.run(int(maxiter)).synchronize()
        return prob.get("u").reshape(C, Nz, nd, nd)
