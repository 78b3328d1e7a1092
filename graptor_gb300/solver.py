"""Host-side problem handle over the C ABI.

:class:`Problem` is one reconstruction problem resident on one GPU: it owns the
device state of the reference's tgv_radon (U, U_, P, P_, V, W, Lamb, F;
radon_tgv_primal_dual_3d.py:1160-1176) and runs graph-captured iterations.
Host arrays use the reference solver's layouts (see include/graptor_gb300.h).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib as L

DISCREPANCY = {"KL": L.GT_KL, "L2": L.GT_L2}
REGULARISATION = {"TV": L.GT_TV, "TGV": L.GT_TGV}
COUPLING = {"UNCORR": L.GT_UNCORR, "FROB": L.GT_FROB, "NUCL": L.GT_NUCL}

# Reconstruction_coupled.py:971-995 method strings -> (dim, coupling)
METHODS = {
    "Uncorrelated 2D Reconstruction": (2, "UNCORR"), "Frobenius 2D Reconstruction": (2, "FROB"),
    "Nuclear 2D Reconstruction": (2, "NUCL"), "Uncorrelated 3D Reconstruction": (3, "UNCORR"),
    "Frobenius 3D Reconstruction": (3, "FROB"), "Nuclear 3D Reconstruction": (3, "NUCL"),
}


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


class Problem:
    """One TGV/TV primal-dual problem on the GPU.

    Parameters mirror Reconstructionapproach2d/3d: ``angles`` in radians already
    shifted by +pi/2, ``alpha = (alpha0, alpha1)``, ``mu`` per channel,
    ``stepsize`` the slice step.  ``normest=None`` estimates the operator norm by
    an FP64 power iteration on the device; a positive value is used as given.
    """

    def __init__(self, dim, N, Nz, C, nd, angles, alpha=(4.0, 1.0), mu=None, discrepancy="KL",
                 regularisation="TGV", coupling="FROB", stepsize=1.0, normest=None, device=0, stream=None,
                 autotune=True, _handle=None):
        self._h = None
        self._owner = _handle is None
        self.dim, self.N, self.Nz, self.C, self.nd = int(dim), int(N), int(Nz), int(C), int(nd)
        self.angles = np.ascontiguousarray(angles, dtype=np.float64)
        self.nang = int(self.angles.size)
        self.S = self.Nz * self.C
        self.K = self.dim
        self.KW = 6 if self.dim == 3 else 3
        alpha = np.atleast_1d(np.asarray(alpha, dtype=np.float64))
        if alpha.size == 1:
            alpha = np.array([alpha[0], alpha[0]])
        self.alpha = alpha
        self.mu = np.ascontiguousarray(np.ones(self.C) if mu is None else mu, dtype=np.float64)
        if self.mu.size != self.C:
            raise ValueError(f"mu has {self.mu.size} entries for {self.C} channels")
        self.regularisation = regularisation.upper()
        self.discrepancy, self.coupling = discrepancy.upper(), coupling.upper()
        self.stepsize, self.normest_in, self.device = float(stepsize), normest, int(device)
        self._stream, self._autotune = stream, bool(autotune)
        if _handle is not None:
            self._h = _handle
            return
        h = ctypes.c_void_p()
        L.check(L.lib().gt_problem_create(ctypes.byref(self.desc()), ctypes.byref(h)))
        self._h = h

    def desc(self) -> L.GtDesc:
        """The C description of this problem (arrays stay owned by self)."""
        d = L.GtDesc()
        d.dim, d.N, d.Nz, d.C, d.nd, d.nang = self.dim, self.N, self.Nz, self.C, self.nd, self.nang
        d.angles = self.angles.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.stepsize = self.stepsize
        d.alpha0, d.alpha1 = float(self.alpha[0]), float(self.alpha[1])
        d.mu = self.mu.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.discrepancy = DISCREPANCY[self.discrepancy]
        d.regularisation = REGULARISATION[self.regularisation]
        d.coupling = COUPLING[self.coupling]
        d.normest = float(self.normest_in) if self.normest_in else 0.0
        d.device = self.device
        d.stream = self._stream
        d.autotune = int(self._autotune)
        return d

    # ------------------------------------------------------------------ lifecycle
    def close(self):
        if self._owner and self._h is not None and self._h.value:
            L.lib().gt_problem_destroy(self._h)
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

    # ------------------------------------------------------------------ data / iteration
    def set_data(self, f, feasible: bool = True):
        """Sinogram data ``f[S, nang, nd]`` (s = c*Nz + z); resets the iterates."""
        f = np.ascontiguousarray(f, dtype=np.float32).reshape(self.S, self.nang, self.nd)
        L.check(L.lib().gt_set_data(self._h, _ptr(f), int(bool(feasible))))
        return self

    def run(self, iters: int):
        L.check(L.lib().gt_run(self._h, int(iters)))
        return self

    def synchronize(self):
        L.check(L.lib().gt_synchronize(self._h))
        return self

    def _shape(self, field):
        img, sino = (self.S, self.N, self.N), (self.S, self.nang, self.nd)
        return {"u": img, "ubar": img, "p": (self.K,) + img, "pbar": (self.K,) + img, "v": (self.K,) + img,
                "w": (self.KW,) + img, "lambda": sino, "ku": sino, "data": sino, "ulo": img}[field]

    def get(self, field: str) -> np.ndarray:
        out = np.empty(self._shape(field), np.float32)
        L.check(L.lib().gt_get_state(self._h, L.FIELDS[field], _ptr(out)))
        return out

    def output_f64(self, field: str) -> np.ndarray:
        """The 3-D entry point's float64 return values, reordered on the device:
        "u" as Solution [C, N, N, Nz] (x, y, z), "ku" as Sinogram [C, nang, Nz, nd]."""
        if field == "u":
            out = np.empty((self.C, self.N, self.N, self.Nz), np.float64)
        elif field == "ku":
            out = np.empty((self.C, self.nang, self.Nz, self.nd), np.float64)
        else:
            raise ValueError("output_f64: 'u' or 'ku'")
        L.check(L.lib().gt_get_output_f64(self._h, L.FIELDS[field], _ptr(out)))
        return out

    def set(self, field: str, value) -> None:
        a = np.ascontiguousarray(value, dtype=np.float32).reshape(self._shape(field))
        L.check(L.lib().gt_set_state(self._h, L.FIELDS[field], _ptr(a)))

    def set_tuning(self, fwd: int, bp: int):
        """Force the projector launch configurations (see gt_set_tuning)."""
        L.check(L.lib().gt_set_tuning(self._h, int(fwd), int(bp)))
        return self

    def set_dual_shape(self, cfg: int):
        """Force the dual kernel's launch shape (see gt_set_dual_shape)."""
        L.check(L.lib().gt_set_dual_shape(self._h, int(cfg)))
        return self

    def set_primal_weight(self, w: float):
        """Primal weight of the step pair: sigma = w / sqrt(Lsqr), tau = 1 / (w sqrt(Lsqr))
        (1 = the reference's steps, the default; see gt_set_primal_weight)."""
        L.check(L.lib().gt_set_primal_weight(self._h, float(w)))
        return self

    @property
    def primal_weight(self) -> float:
        return float(L.lib().gt_get_primal_weight(self._h))

    def restart(self):
        """Restart the extrapolation from the current point (ubar = u, pbar = p)."""
        L.check(L.lib().gt_restart(self._h))
        return self

    def snapshot(self):
        """Keep a copy of (u, p, v, w, lambda) for :meth:`movement`."""
        L.check(L.lib().gt_snapshot(self._h))
        return self

    def movement(self) -> tuple:
        """L2 distances of the primal (u, p) and dual (v, w, lambda) parts from the snapshot."""
        out = (ctypes.c_double * 2)()
        L.check(L.lib().gt_movement(self._h, out))
        return float(out[0]), float(out[1])

    def set_schedule(self, schedule: int):
        """1: the p / pbar half of the primal update beside the projectors (default);
        0: the whole primal update after them; 2: the p / pbar half fused into the
        next iteration's dual kernel (3-D TGV; see gt_set_schedule)."""
        L.check(L.lib().gt_set_schedule(self._h, int(schedule)))
        return self

    def set_precise_primal(self, on: bool = True):
        """Hold u as two floats so that steps below half an ulp of u are kept (the
        relative gap then falls below the float32 plateau; see gt_set_precise_primal)."""
        L.check(L.lib().gt_set_precise_primal(self._h, int(bool(on))))
        return self

    @property
    def precise_primal(self) -> bool:
        return bool(L.lib().gt_get_precise_primal(self._h))

    def dual_from_primal(self, empty_weight: float = 1.0, cap: int = 0, repair: bool = False):
        """Set lambda consistent with the current u (for warm starts); bins
        without data move empty_weight of the way to their fixed point; cap 10
        or 100 sets lambda = mu (1 - cap) where f > 10 K u; repair first lifts u
        along rays with data that it misses (gt_dual_from_primal_ex)."""
        flags = {0: 0, 10: 2, 100: 4}[int(cap)] | (8 if repair else 0)
        L.check(L.lib().gt_dual_from_primal_ex(self._h, flags, float(empty_weight)))
        return self

    def repair_missed_rays(self):
        """Lift u (and ubar) along rays with data that the image misses (K u = 0
        < f, KL), leaving lambda: the primal value becomes finite again."""
        L.check(L.lib().gt_dual_from_primal_ex(self._h, 8 | 16, 1.0))
        return self

    @property
    def scalars(self) -> dict:
        out = (ctypes.c_double * 4)()
        L.check(L.lib().gt_get_scalars(self._h, out))
        return {"normest": out[0], "sigma": out[1], "tau": out[2], "iterations": int(out[3])}

    @property
    def tuning(self) -> dict:
        """Launch shapes and iteration schedule the autotuner chose (see launch_fwd /
        launch_bp / gt_set_schedule)."""
        out = (ctypes.c_int * 2)()
        L.check(L.lib().gt_get_tuning(self._h, out))
        return {"fwd_cfg": out[0], "bp_cfg": out[1], "dual_cfg": L.lib().gt_get_dual_shape(self._h),
                "schedule": L.lib().gt_get_schedule(self._h)}

    def gap(self, U: float = 0.0) -> dict:
        """FP64 primal-dual gap of the current iterate on the box u in [0, U] (U <= 0: 2 max u)."""
        out = (ctypes.c_double * 8)()
        L.check(L.lib().gt_gap_ex(self._h, float(U), out))
        return {"primal": out[0], "dual": out[1], "gap": out[2], "relative": out[3], "theta": out[4], "U": out[5],
                "data": out[6], "fstar": out[7]}

    def solve_to_gap(self, tol: float = 1e-4, check_every: int = 50, max_iters: int = 100000) -> dict:
        """Iterate until the relative gap is finite and <= tol (checked every
        `check_every` iterations).  The gap is not finite while K u = 0 on a bin
        with data (infinite KL primal value), e.g. before the first iteration."""
        done = 0
        g = self.gap()
        while not (math.isfinite(g["relative"]) and g["relative"] <= tol) and done < max_iters:
            n = min(check_every, max_iters - done)
            self.run(n)
            done += n
            g = self.gap()
        g["iterations"] = done
        return g

    # ------------------------------------------------------------------ checkpoint / resume
    def _state_fields(self):
        f = ("u", "ubar", "p", "pbar", "v", "w", "lambda") if self.regularisation == "TGV" else \
            ("u", "ubar", "v", "lambda")
        return f + ("ulo",) if self.precise_primal else f  # the low part after u (setting u clears it)

    def save(self, path: str) -> None:
        """Checkpoint the solve to ``path`` (.npz): the problem description, the
        data, the step-size scalars (operator-norm estimate and primal weight
        included), the precise primal mode and every iterate (the low part of u
        with it), so that :meth:`load` continues the iteration exactly."""
        self.synchronize()
        sc = self.scalars
        fields = {k: self.get(k) for k in self._state_fields()}
        np.savez(path, dim=self.dim, N=self.N, Nz=self.Nz, C=self.C, nd=self.nd, angles=self.angles,
                 alpha=self.alpha, mu=self.mu, discrepancy=self.discrepancy, regularisation=self.regularisation,
                 coupling=self.coupling, stepsize=self.stepsize, normest=sc["normest"],
                 iterations=sc["iterations"] + getattr(self, "iteration_offset", 0), data=self.get("data"),
                 primal_weight=self.primal_weight, precise_primal=self.precise_primal,
                 **{"state_" + k: v for k, v in fields.items()})

    @classmethod
    def load(cls, path: str, device: int = 0, stream=None, autotune: bool = True) -> "Problem":
        """A problem restored from a :meth:`save` checkpoint on ``device``; its
        next iterations equal those the saved problem would have run."""
        z = np.load(path, allow_pickle=False)
        p = cls(int(z["dim"]), int(z["N"]), int(z["Nz"]), int(z["C"]), int(z["nd"]), z["angles"], z["alpha"],
                z["mu"], str(z["discrepancy"]), str(z["regularisation"]), str(z["coupling"]), float(z["stepsize"]),
                float(z["normest"]), device, stream, autotune)
        p.set_data(z["data"], feasible=False)  # stored after the feasibility mask
        if "primal_weight" in z.files and float(z["primal_weight"]) != 1.0:
            p.set_primal_weight(float(z["primal_weight"]))
        if "precise_primal" in z.files and bool(z["precise_primal"]):
            p.set_precise_primal(True)
        for k in p._state_fields():
            p.set(k, z["state_" + k])
        p.iteration_offset = int(z["iterations"])
        return p

    def time_kernels(self, reps: int = 5) -> dict:
        """Mean CUDA-event duration (ms) of each kernel of one iteration; the
        primal update as a whole (k_update) and as its u / ubar and p / pbar halves;
        k_dual_fused: the fused dual kernel of schedule 2 where that schedule is set
        (absent otherwise)."""
        out = (ctypes.c_float * 7)()
        L.check(L.lib().gt_time_kernels(self._h, int(reps), out, 7))
        r = {"k_dual": out[0], "k_fwd": out[1], "k_bp": out[2], "k_update": out[3], "k_update_u": out[4],
             "k_update_p": out[5]}
        if out[6] > 0:
            r["k_dual_fused"] = out[6]
        return r

    @property
    def launches_per_iteration(self) -> int:
        return int(L.lib().gt_launches_per_iteration(self._h))


class Batch:
    """Independent problems advanced together by one graph launch per chunk.

    ``specs`` are keyword dicts of :class:`Problem` (dim, N, Nz, C, nd, angles, ...).
    Members are :class:`Problem` views (``batch[k]``) for data and results; the
    batch owns them."""

    def __init__(self, specs, device=0):
        self._b = None
        self._views = [Problem(**{**sp, "device": device}, _handle=ctypes.c_void_p(0)) for sp in specs]
        descs = (L.GtDesc * len(self._views))(*[v.desc() for v in self._views])
        b = ctypes.c_void_p()
        L.check(L.lib().gt_batch_create(len(self._views), descs, ctypes.byref(b)))
        self._b = b
        for k, v in enumerate(self._views):
            h = ctypes.c_void_p()
            L.check(L.lib().gt_batch_problem(self._b, k, ctypes.byref(h)))
            v._h = h

    def __len__(self):
        return len(self._views)

    def __getitem__(self, k) -> Problem:
        return self._views[k]

    def run(self, iters: int):
        L.check(L.lib().gt_batch_run(self._b, int(iters)))
        return self

    def synchronize(self):
        L.check(L.lib().gt_batch_synchronize(self._b))
        return self

    def invalidate(self):
        L.check(L.lib().gt_batch_invalidate(self._b))

    def set_active(self, k: int, active: bool = True):
        """Leave problem k out of (or bring it back into) the following runs."""
        L.check(L.lib().gt_batch_set_active(self._b, int(k), int(bool(active))))
        return self

    def set_mode(self, mode: int):
        """0: a graph of the members' own iterations on concurrent chains (default);
        1: fused launches, each over the work units of every active member
        (see gt_batch_set_mode)."""
        L.check(L.lib().gt_batch_set_mode(self._b, int(mode)))
        return self

    @property
    def mode(self) -> int:
        return int(L.lib().gt_batch_get_mode(self._b))

    def set_concurrency(self, chains: int):
        """Spread the problems over `chains` concurrent chains (default 8)."""
        L.check(L.lib().gt_batch_set_concurrency(self._b, int(chains)))
        return self

    def close(self):
        if self._b is not None and self._b.value:
            for v in self._views:
                v._h = None
            L.lib().gt_batch_destroy(self._b)
        self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def radon(img_dev, sino_dev, angles, N, nd, S, stream=None):
    """Forward projection of device tensors (device layout [N*N][S] -> [nang*nd][S])."""
    ang = np.ascontiguousarray(angles, dtype=np.float64)
    L.check(L.lib().gt_radon(ctypes.c_void_p(img_dev), ctypes.c_void_p(sino_dev), _ptr(ang), int(N), int(nd),
                             int(ang.size), int(S), stream))


def radon_ad(sino_dev, img_dev, angles, N, nd, S, stream=None):
    """Back projection of device tensors (device layout [nang*nd][S] -> [N*N][S])."""
    ang = np.ascontiguousarray(angles, dtype=np.float64)
    L.check(L.lib().gt_radon_ad(ctypes.c_void_p(sino_dev), ctypes.c_void_p(img_dev), _ptr(ang), int(N), int(nd),
                                int(ang.size), int(S), stream))
