"""Seeded synthetic inputs with the shapes and value distributions of the workloads.

No public dataset is used: the workloads are synthetic phantoms.

* :func:`ellipses_2d` -- image of random ellipses, intensities U[0.1, 1], background 0
  (the 2-D single-channel workload, 128x128 with 10 ellipses).
* :func:`ellipsoids_3d` -- multi-channel volume whose channels share one label map
  of random ellipsoids, so edges coincide across channels; channel 0 is dense,
  the other channels are sparse (each covers a drawn 5-20 % of the voxels).
* :func:`poisson` -- Poisson counts at a given peak, rescaled so the noiseless
  peak maps to 1 (data of order one, like the reference's percentile scaling,
  Reconstruction_coupled.py:348-351).
* :func:`angles_deg` -- uniform tilt series in degrees, converted to the solver's
  convention (radians + pi/2, as the reference CLI passes them,
  Reconstruction_coupled.py:233, :448).
"""
from __future__ import annotations

import numpy as np


def angles_deg(n: int, lo: float = -70.0, hi: float = 70.0) -> np.ndarray:
    return np.linspace(lo, hi, n) * np.pi / 180.0 + np.pi / 2.0


def _grid(N):
    c = (np.arange(N) - (N - 1) / 2.0) / (N / 2.0)
    return c


def ellipses_2d(N: int, n_ellipses: int = 10, seed: int = 0) -> np.ndarray:
    """float32[N, N] indexed [y, x]."""
    rng = np.random.default_rng(seed)
    g = _grid(N)
    X, Y = np.meshgrid(g, g)  # [y, x]
    img = np.zeros((N, N), np.float32)
    for _ in range(n_ellipses):
        cx, cy = rng.uniform(-0.55, 0.55, 2)
        a, b = rng.uniform(0.06, 0.35, 2)
        th = rng.uniform(0, np.pi)
        val = rng.uniform(0.1, 1.0)
        xr = (X - cx) * np.cos(th) + (Y - cy) * np.sin(th)
        yr = -(X - cx) * np.sin(th) + (Y - cy) * np.cos(th)
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1.0] = val
    return img


def label_volume(N: int, Nz: int, n_ellipsoids: int, seed: int) -> np.ndarray:
    """int16[Nz, N, N] label map ([z, y, x]); 0 is background."""
    rng = np.random.default_rng(seed)
    g = _grid(N)
    gz = (np.arange(Nz) - (Nz - 1) / 2.0) / max(Nz / 2.0, 1.0)
    lab = np.zeros((Nz, N, N), np.int16)
    Y, X = np.meshgrid(g, g, indexing="ij")
    for k in range(1, n_ellipsoids + 1):
        cx, cy = rng.uniform(-0.5, 0.5, 2)
        cz = rng.uniform(-0.4, 0.4)
        a, b = rng.uniform(0.08, 0.4, 2)
        cc = rng.uniform(0.3, 0.9)
        th = rng.uniform(0, np.pi)
        xr = (X - cx) * np.cos(th) + (Y - cy) * np.sin(th)
        yr = -(X - cx) * np.sin(th) + (Y - cy) * np.cos(th)
        r2 = (xr / a) ** 2 + (yr / b) ** 2
        for z in range(Nz):
            m = r2 + ((gz[z] - cz) / cc) ** 2 <= 1.0
            lab[z][m] = k
    return lab


def ellipsoids_3d(N: int, Nz: int, C: int, n_ellipsoids: int = 12, seed: int = 0) -> np.ndarray:
    """float32[C, Nz, N, N] ([c, z, y, x]); channels share the label map."""
    rng = np.random.default_rng(seed + 7919)
    lab = label_volume(N, Nz, n_ellipsoids, seed)
    vol = np.zeros((C, Nz, N, N), np.float32)
    labels = np.arange(1, n_ellipsoids + 1)
    frac = np.array([(lab == k).mean() for k in labels])
    for c in range(C):
        val = np.zeros(n_ellipsoids + 1, np.float32)
        if c == 0:
            val[1:] = rng.uniform(0.1, 1.0, n_ellipsoids)
        else:
            target = rng.uniform(0.05, 0.20)
            order = rng.permutation(labels)
            cover = 0.0
            for k in order:
                if cover >= target:
                    break
                if cover + frac[k - 1] <= max(target, 0.2) or cover == 0.0:
                    val[k] = rng.uniform(0.1, 1.0)
                    cover += frac[k - 1]
        vol[c] = val[lab]
    return vol


def poisson(sino: np.ndarray, peak: float, seed: int = 0) -> np.ndarray:
    """Poisson counts with the noiseless maximum at ``peak`` counts, divided by ``peak``."""
    rng = np.random.default_rng(seed + 104729)
    m = float(np.max(sino))
    lam = np.clip(sino, 0, None) * (peak / m if m > 0 else 0.0)
    return (rng.poisson(lam) / peak).astype(np.float32)
