"""Python front end of the CPU oracle (test infrastructure only).

Wraps ``oracle/tgv_oracle.c`` (an FP32 restatement of the reference's kernels,
compiled with gcc) and restates the reference's host logic around it:

* ``radon_struct``            radon_tgv_primal_dual_3d.py:947-979
* ``Make_function_feasible``  radon_tgv_primal_dual_3d.py:860-870
* step sizes and scalings     radon_tgv_primal_dual_3d.py:1178-1189 (2-D :753-762)
* the iteration               radon_tgv_primal_dual_3d.py:1194-1221 (2-D :767-799)
* input / output reordering   radon_tgv_primal_dual_3d.py:1277-1316 (2-D :838-874)

Only tests, the package smoke check and bench.py's CPU-baseline leg use this
module, as the checker or as the timed CPU baseline; the product never does.
The reference's power iteration starts from an unseeded random vector, so the
operator-norm estimate ``normest`` is an explicit argument here.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "tgv_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

KL, L2 = 0, 1
TV, TGV = 0, 1
UNCORR, FROB, NUCL = 0, 1, 2


class Desc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("N", ctypes.c_int), ("Nz", ctypes.c_int), ("C", ctypes.c_int),
                ("nd", ctypes.c_int), ("nang", ctypes.c_int), ("discrepancy", ctypes.c_int),
                ("regularisation", ctypes.c_int), ("coupling", ctypes.c_int), ("stepsize", ctypes.c_float)]


class State(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("u", "ubar", "p", "pbar", "v", "w", "lam")]


def build(force: bool = False) -> str:
    """Compile the oracle library (gcc, OpenMP, no fused multiply-add)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + f".{os.getpid()}.tmp"
        subprocess.run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", SRC, "-o", tmp, "-lm"],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


# ---------------------------------------------------------------- geometry / projectors
def radon_struct(angles, N: int, nd: int) -> np.ndarray:
    """Angle table float32[nang, 4] = (X, Y, offset, Xinv) per angle."""
    ang = np.ascontiguousarray(angles, dtype=np.float64)
    ofs = np.zeros((ang.size, 4), np.float32)
    lib().or_radon_struct(N, nd, ang.size, _p(ang), _p(ofs))
    return ofs


def radon(img, ofs, nd: int) -> np.ndarray:
    """Forward projection of img[S, N, N] (x fastest) -> sino[S, nang, nd]."""
    img = _f32(img)
    S, N = img.shape[0], img.shape[-1]
    sino = np.zeros((S, ofs.shape[0], nd), np.float32)
    lib().or_radon(_p(sino), _p(img), _p(_f32(ofs)), N, nd, ofs.shape[0], S)
    return sino


def radon_ad(sino, ofs, N: int) -> np.ndarray:
    """Back projection of sino[S, nang, nd] -> img[S, N, N]."""
    sino = _f32(sino)
    S, nang, nd = sino.shape
    img = np.zeros((S, N, N), np.float32)
    lib().or_radon_ad(_p(img), _p(sino), _p(_f32(ofs)), N, nd, nang, S)
    return img


def make_feasible(f, ofs, N: int) -> np.ndarray:
    f = _f32(f).copy()
    S, nang, nd = f.shape
    lib().or_make_feasible(_p(f), _p(_f32(ofs)), N, nd, nang, S)
    return f


# ---------------------------------------------------------------- solver
def lsqr(dim: int) -> float:
    """Step-size bound: 17 in 3-D (:1180), (18 + sqrt 33)/2 in 2-D (2-D :754)."""
    return 17.0 if dim == 3 else 0.5 * (18.0 + math.sqrt(33.0))


def scalars(dim, alpha, mu, ne, discrepancy):
    """The float32 kernel arguments tgv_radon derives on the host (:1178-1189, :1079-1130)."""
    sigma = 1.0 / math.sqrt(lsqr(dim))
    tau = sigma
    a = np.asarray(alpha, dtype=np.float64) / (ne ** 2)
    mu = np.asarray(mu, dtype=np.float64)
    mu_eff = (mu if discrepancy == KL else mu / (sigma + mu)).astype(np.float32)
    return dict(sigma=np.float32(sigma), tau=np.float32(tau), sigma_data=np.float32(sigma / ne),
                norming=np.float32(1.0 / ne), alphainv0=np.float32(1.0 / a[0]), alphainv1=np.float32(1.0 / a[1]),
                mu_eff=mu_eff)


class Solver:
    """The reference iteration on CPU for one problem, state in the oracle layout."""

    def __init__(self, dim, N, Nz, C, nd, ofs, f, alpha, mu, ne, discrepancy=KL, regularisation=TGV,
                 coupling=FROB, stepsize=1.0, feasible=True):
        self.desc = Desc(dim, N, Nz, C, nd, ofs.shape[0], discrepancy, regularisation, coupling, float(stepsize))
        self.ofs = _f32(ofs)
        f = _f32(f).reshape(Nz * C, ofs.shape[0], nd)
        self.f = make_feasible(f, ofs, N) if feasible else f.copy()
        self.sc = scalars(dim, alpha, mu, ne, discrepancy)
        S, K, KW = Nz * C, dim, (6 if dim == 3 else 3)
        z = lambda *sh: np.zeros(sh, np.float32)  # noqa: E731
        self.u, self.ubar = z(S, N, N), z(S, N, N)
        self.p, self.pbar, self.v = z(K, S, N, N), z(K, S, N, N), z(K, S, N, N)
        self.w, self.lam = z(KW, S, N, N), z(S, ofs.shape[0], nd)
        self.ku = z(S, ofs.shape[0], nd)
        self.iterations = 0

    def run(self, iters: int):
        st = State(*[_p(a) for a in (self.u, self.ubar, self.p, self.pbar, self.v, self.w, self.lam)])
        sc = self.sc
        rc = lib().or_iterate(ctypes.byref(self.desc), _p(self.ofs), _p(self.f), ctypes.byref(st), int(iters),
                              ctypes.c_float(sc["sigma"]), ctypes.c_float(sc["tau"]), ctypes.c_float(sc["sigma_data"]),
                              ctypes.c_float(sc["norming"]), ctypes.c_float(sc["alphainv0"]),
                              ctypes.c_float(sc["alphainv1"]), _p(sc["mu_eff"]), _p(self.ku))
        if rc:
            raise MemoryError("oracle: allocation failed")
        self.iterations += iters
        return self


# ---------------------------------------------------------------- reference-shaped entry points
_METHODS = {
    "Uncorrelated 2D Reconstruction": (2, UNCORR), "Frobenius 2D Reconstruction": (2, FROB),
    "Nuclear 2D Reconstruction": (2, NUCL), "Uncorrelated 3D Reconstruction": (3, UNCORR),
    "Frobenius 3D Reconstruction": (3, FROB), "Nuclear 3D Reconstruction": (3, NUCL),
}


def reconstruct_2d(sino, angles, Parameter, mu, maxiter, discrepancy, method, regularisation, normest):
    """Reference ``Reconstructionapproach2d`` (2-D :69) with an explicit normest."""
    C = len(sino)
    nang, nd = np.asarray(sino[0]).shape
    f = np.stack([np.asarray(s, np.float32) for s in sino])  # [C, nang, nd]
    ofs = radon_struct(angles, nd, nd)
    coupling = _METHODS[method][1]
    s = Solver(2, nd, 1, C, nd, ofs, f, Parameter, mu, normest, KL if discrepancy == "KL" else L2,
               TGV if regularisation.upper() == "TGV" else TV, coupling).run(maxiter)
    sol = np.transpose(s.u, (0, 2, 1)).astype(np.float64)  # [C, x, y]
    return sol, s.ku.copy()  # sinograms [C, nang, nd]


def reconstruct_3d(sino, angles, Parameter, mu, maxiter, Stepsize, discrepancy, method, regularisation, normest):
    """Reference ``Reconstructionapproach3d`` (3-D :69) with an explicit normest."""
    C = len(sino)
    nang, Nz, nd = np.asarray(sino[0]).shape
    f = np.stack([np.transpose(np.asarray(s, np.float32), (1, 0, 2)) for s in sino])  # [C, Nz, nang, nd]
    ofs = radon_struct(angles, nd, nd)
    coupling = _METHODS[method][1]
    s = Solver(3, nd, Nz, C, nd, ofs, f.reshape(C * Nz, nang, nd), Parameter, mu, normest,
               KL if discrepancy == "KL" else L2, TGV if regularisation.upper() == "TGV" else TV, coupling,
               stepsize=Stepsize).run(maxiter)
    u = s.u.reshape(C, Nz, nd, nd)  # [c, z, y, x]
    sol = np.transpose(u, (0, 3, 2, 1)).astype(np.float64)  # [C, x, y, z]
    ku = s.ku.reshape(C, Nz, nang, nd)
    sino_out = np.transpose(ku, (0, 2, 1, 3)).astype(np.float64)  # [C, nang, Nz, nd]
    return sol, sino_out
