"""Drop-in for radon_tgv_primal_dual_3dsubsample.Reconstructionapproach3dsubsmapling.

Two data sets of different resolution reconstructed jointly (the reference's
two-resolution subsampling method, radon_tgv_primal_dual_3dsubsample.py:51-1240):
channels [0, Topology[0]) have projections on the image's own detector and slice
grid, the remaining channels on a coarser grid.  The reconstruction runs in the
CUDA library (gt_subs_* in include/graptor_gb300.h): fine-grid forward and back
projection of each group with its own tilt series, the reference's area-weighting
matrix between the grids (and its transpose), the coupled TGV/TV regulariser on
the fine grid, Lsqr = 36.

Arguments and returns are the reference's:
  sino      list of C arrays [nang, Nz, nd] (fine channels first), float
  angles    list of C angle arrays in radians (+pi/2 as the callers pass them);
            the fine channels share angles[0], the coarse ones angles[Topology[0]]
  Topology  [smallerimagestart, p, Refold, Refnew]: number of fine channels, pixel
            ratio, reference point (x, z) on the coarse grid and on the fine grid
  returns   (Solution float64 [C, N, N, Nz],
             [Sinograms0 float32 [C0, nang0, Nz, N], Sinograms1 on the fine detector
              [C1, nang1, Nz, N], Sinograms1 on the coarse grid [C1, nang1, Nz1, nd1]])

Differences: the reference divides Refnew[1] by Stepsize in the caller's list
(so repeated calls compound); here the caller's list is left alone.  ``ctx`` is a
CUDA device ordinal; ``plott`` is ignored; ``normest`` may be injected.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .solver import COUPLING, DISCREPANCY, REGULARISATION

METHODS = {"Frobenius 3D Subsampling Reconstruction": "FROB", "Uncorrelated 3D Subsampling Reconstruction": "UNCORR"}


class Subsampling:
    """Owner of a gt_subs handle."""

    def __init__(self, N, Nz, C0, C1, nd1, Nz1, angles0, angles1, alpha, mu, pixel_ratio, refold, refnew,
                 discrepancy="KL", regularisation="TGV", coupling="FROB", stepsize=1.0, normest=None, device=0):
        self._h = None
        self.N, self.Nz, self.C0, self.C1, self.nd1, self.Nz1 = int(N), int(Nz), int(C0), int(C1), int(nd1), int(Nz1)
        self.angles0 = np.ascontiguousarray(angles0 if C0 else [0.0], np.float64)
        self.angles1 = np.ascontiguousarray(angles1, np.float64)
        self.nang0 = int(len(angles0)) if C0 else 0
        self.nang1 = int(self.angles1.size)
        self.mu = np.ascontiguousarray(mu, np.float64)
        d = L.GtSubsDesc()
        d.N, d.Nz, d.C0, d.C1 = self.N, self.Nz, self.C0, self.C1
        d.nang0, d.nang1, d.nd1, d.Nz1 = self.nang0, self.nang1, self.nd1, self.Nz1
        d.angles0 = self.angles0.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.angles1 = self.angles1.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.stepsize = float(stepsize)
        alpha = np.atleast_1d(np.asarray(alpha, np.float64))
        d.alpha0, d.alpha1 = float(alpha[0]), float(alpha[-1] if alpha.size > 1 else alpha[0])
        d.mu = self.mu.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.discrepancy = DISCREPANCY[discrepancy.upper()]
        d.regularisation = REGULARISATION[regularisation.upper()]
        d.coupling = COUPLING[coupling.upper()]
        d.pixel_ratio = float(pixel_ratio)
        d.refold[0], d.refold[1] = float(refold[0]), float(refold[1])
        d.refnew[0], d.refnew[1] = float(refnew[0]), float(refnew[1])
        d.normest = float(normest) if normest else 0.0
        d.device = int(device)
        h = ctypes.c_void_p()
        L.check(L.lib().gt_subs_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h is not None and self._h.value:
            L.lib().gt_subs_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_data(self, f0, f1, feasible=True):
        """f0 [C0*Nz, nang0, N], f1 [C1*Nz1, nang1, nd1] (s = c*Nz + z)."""
        a0 = np.ascontiguousarray(f0, np.float32) if self.C0 else np.zeros(1, np.float32)
        a1 = np.ascontiguousarray(f1, np.float32)
        L.check(L.lib().gt_subs_set_data(self._h, ctypes.c_void_p(a0.ctypes.data), ctypes.c_void_p(a1.ctypes.data),
                                         int(bool(feasible))))
        return self

    def run(self, iters):
        L.check(L.lib().gt_subs_run(self._h, int(iters)))
        return self

    @property
    def normest(self):
        return float(L.lib().gt_subs_normest(self._h))

    def get(self, which):
        shapes = {"u": (0, ((self.C0 + self.C1) * self.Nz, self.N, self.N)),
                  "ku0": (1, (self.C0 * self.Nz, self.nang0, self.N)),
                  "ku1": (2, (self.C1 * self.Nz, self.nang1, self.N)),
                  "kulo": (3, (self.C1 * self.Nz1, self.nang1, self.nd1))}
        code, shape = shapes[which]
        out = np.empty(shape, np.float32)
        if out.size:
            L.check(L.lib().gt_subs_get(self._h, code, ctypes.c_void_p(out.ctypes.data)))
        return out


def Reconstructionapproach3dsubsmapling(sino, angles, Topology, Parameter, mu, maxiter, ctx, plott, Stepsize,
                                        discrepancy, regularisationmethod, regularisation, Info, normest=None):
    """Drop-in for the reference entry point (radon_tgv_primal_dual_3dsubsample.py:51)."""
    C0, p, refold, refnew = int(Topology[0]), float(Topology[1]), list(Topology[2]), list(Topology[3])
    C = len(sino)
    C1 = C - C0
    nang0, Nz, N = np.asarray(sino[0]).shape if C0 else (0,) + np.asarray(sino[C0]).shape[1:]
    nang1, Nz1, nd1 = np.asarray(sino[C0]).shape
    if C0 == 0:
        raise ValueError("the fine channels (Topology[0] >= 1) set the image size")
    # [nang, Nz, nd] per channel -> [c*Nz + z, nang, nd]
    f0 = np.stack([np.transpose(np.asarray(sino[c], np.float32), (1, 0, 2)) for c in range(C0)]).reshape(C0 * Nz, nang0, N)
    f1 = np.stack([np.transpose(np.asarray(sino[c], np.float32), (1, 0, 2)) for c in range(C0, C)]).reshape(C1 * Nz1, nang1, nd1)
    ctx = ctx if isinstance(ctx, int) else 0
    with Subsampling(N, Nz, C0, C1, nd1, Nz1, angles[0], angles[C0], Parameter, np.asarray(mu)[:C], p, refold, refnew,
                     discrepancy, regularisation, METHODS[regularisationmethod], Stepsize, normest, ctx) as s:
        s.set_data(f0, f1).run(maxiter)
        u = s.get("u").reshape(C, Nz, N, N)
        k0, k1, klo = s.get("ku0"), s.get("ku1"), s.get("kulo")
    solution = np.transpose(u, (0, 2, 3, 1)).astype(np.float64)  # [C, N(y), N(x), Nz]
    # the reference's Solution[j,:,:,i] = U[:,:,i+Nz*j] with U F-ordered [x, y, s]: first index x
    solution = np.transpose(solution, (0, 2, 1, 3)).copy()
    sino0 = np.transpose(k0.reshape(C0, Nz, nang0, N), (0, 2, 1, 3)).astype(np.float32)
    sino1 = np.transpose(k1.reshape(C1, Nz, nang1, N), (0, 2, 1, 3)).astype(np.float32)
    sino1lo = np.transpose(klo.reshape(C1, Nz1, nang1, nd1), (0, 2, 1, 3)).astype(np.float32)
    return solution, [sino0, sino1, sino1lo]
