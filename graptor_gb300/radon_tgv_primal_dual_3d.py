"""Drop-in for the reference's 3-D solver entry point.

``Reconstructionapproach3d`` has the signature, argument meaning, return values
and error behaviour of radon_tgv_primal_dual_3d.py:69 (called from
Reconstruction_coupled.py:448); the iteration runs on the GPU through the C ABI.

Differences, by design:
  * ``ctx`` is not an OpenCL context: an int selects the CUDA device, anything
    else means device 0.
  * the operator norm is an FP64 power iteration on the device (deterministic),
    instead of 10 FP32 rounds from an unseeded random image (:1018-1030); pass
    ``normest=`` to use a given value.
  * ``plott[0] == 1`` (live matplotlib plots) is not supported and is ignored.
  * out of device memory raises :class:`GraptorMemoryError` (a ``MemoryError``)
    where the reference raises ``pyopencl.MemoryError``.
"""
from __future__ import annotations

import math
import sys

import numpy as np

from ._lib import GraptorError, GraptorMemoryError  # noqa: F401  (re-exported for callers)
from .solver import METHODS, Problem

progress = True  # print the reference's progress lines (:1226-1238)


def _device(ctx) -> int:
    return int(ctx) if isinstance(ctx, (int, np.integer)) else 0


def _describe(current):
    if isinstance(current, (list, tuple, range)) and len(current) > 3:
        return f"{current[0]}, {current[1]}...{current[len(current) - 1]}"
    return str(current)


def run_with_progress(prob: Problem, maxiter: int, start, sectionwidth, label: str, what: str):
    step = max(1, math.ceil(maxiter / 100.0))
    done = 0
    while done < maxiter:
        if progress and done % step == 0:
            prob.synchronize()
            prog = start + sectionwidth * float(done) / maxiter
            print(f"Overall progress at {prog:3.0%}. Progress of current computation {done / maxiter:3.0%} "
                  f"for {what} {label}")
            sys.stdout.flush()
        n = min(step, maxiter - done) if progress else maxiter
        prob.run(n)
        done += n
    prob.synchronize()


def Reconstructionapproach3d(sino, angles, Parameter, mu, maxiter, ctx, plott, Stepsize, discrepancy,
                             regularisationmethod, regularisation, Info, normest=None):
    """sino: list of C arrays [nang, Nz, nd]. Returns (Solution[C, N, N, Nz] float64,
    Sinogram[C, nang, Nz, nd] float64) with N = nd, as the reference (:1277-1318)."""
    start, sectionwidth, current = Info[0], Info[1], Info[2]
    C = len(sino)
    nang, Nz, nd = np.asarray(sino[0]).shape
    dim, coupling = METHODS.get(regularisationmethod, (3, None))
    if coupling is None or dim != 3:
        raise ValueError(f"unknown 3-D regularisation method {regularisationmethod!r}")
    if regularisation.upper() not in ("TGV", "TV"):
        raise ValueError(f"regularisation must be 'TGV' or 'TV', got {regularisation!r}")
    f = np.empty((C, Nz, nang, nd), np.float32)  # s = c*Nz + z
    for c in range(C):
        f[c] = np.transpose(np.asarray(sino[c], dtype=np.float32), (1, 0, 2))
    if progress:
        print(f"########## Starting\t{discrepancy} {regularisation} {regularisationmethod} ############")
    with Problem(3, nd, Nz, C, nd, angles, Parameter, np.asarray(mu, dtype=np.float64), discrepancy,
                 regularisation, coupling, float(Stepsize), normest, _device(ctx)) as prob:
        prob.set_data(f.reshape(C * Nz, nang, nd), feasible=True)
        run_with_progress(prob, int(maxiter), start, sectionwidth, _describe(current), "Section")
        solution = prob.output_f64("u")     # [C, x, y, z], converted and reordered on the device
        sinogram = prob.output_f64("ku")    # [C, nang, Nz, nd]
    if progress:
        print("Progress at 100%")
        print("Iterations done for section " + _describe(current))
    return solution, sinogram
