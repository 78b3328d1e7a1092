"""Detection of unsuitable projections (find_bad_ele.py:139-230), in NumPy.

Restatement of ``Find_Bad_projections``: brightness-corrected data, subsampled to
about 250 detector columns, smoothed by a box filter (``reduce_noise``), turned into
a weighted gradient magnitude per projection (``weighted_gradient``); consecutive
projections (and projections two apart, with 1.5x the search radius) are compared
by the smallest absolute difference over shifts within the search radius
(``compare_shift_twosided``); each projection's error is the smaller of its two
combined neighbour errors, and the largest errors are reported (1-based numbers).

Differences: the reference's subsampling step uses true division for a ``range``
step (a TypeError on Python 3 once the detector is wider than 250); here it is the
integer step it means.  The reference's ``E**(0.5)`` in the two-sided comparison
discards its result, so the comparison uses E itself, as the reference does.
"""
from __future__ import annotations

import numpy as np

from .preprocess import brightness_correction


def reduce_noise(U: np.ndarray, steps: int) -> np.ndarray:
    """Box sum over a (2 steps + 1)^2 window divided by 4 steps^2 (find_bad_ele.py:69-75)."""
    Nx, Ny = U.shape
    E = np.zeros([Nx - 2 * steps, Ny - 2 * steps])
    for k in range(-steps, steps + 1):
        for l in range(-steps, steps + 1):
            E += U[steps + k:Nx - steps + k, steps + l:Ny - steps + l]
    return E / (4 * steps ** 2)


def compare_shift(U: np.ndarray, V: np.ndarray, steps: int):
    """min over shifts |(k, l)| <= steps of |U - V shifted| on the interior (:76-100)."""
    Nx0, Ny0 = U.shape
    Ui = U[steps:Nx0 - steps, steps:Ny0 - steps]
    E = None
    for k in range(-steps, steps + 1):
        for l in range(-steps, steps + 1):
            D = np.abs(Ui - V[steps + k:Nx0 - steps + k, steps + l:Ny0 - steps + l])
            E = D if E is None else np.minimum(E, D)
    return np.linalg.norm(E), E


def compare_shift_twosided(U: np.ndarray, V: np.ndarray, steps: int):
    """Elementwise max of the two one-sided comparisons, 1-norm (:55-67)."""
    _, E1 = compare_shift(U, V, steps)
    _, E2 = compare_shift(V, U, steps)
    E = np.maximum(E1, E2)
    return np.linalg.norm(E.reshape(E.size), 1), E


def weighted_gradient(u: np.ndarray):
    """Largest neighbour difference (diagonals divided by sqrt 2) times the smallest
    neighbour magnitude, on the interior (:103-136)."""
    Nx, Ny = u.shape
    c = u[1:Nx - 1, 1:Ny - 1]
    E, Nb = [], []
    for i, j in [(-1, -1), (-1, 1), (0, -1), (0, 1), (1, -1), (1, 1), (-1, 0), (1, 0)]:
        nb = u[1 + i:Nx - 1 + i, 1 + j:Ny - 1 + j]
        E.append(np.abs(c - nb) / np.sqrt(i * i + j * j))
        Nb.append(np.abs(nb))
    value = np.max(E, axis=0) * np.min(Nb, axis=0)
    return np.linalg.norm(value), value


def find_bad_projections(name: str, searchradius=None, prozent_to_reduce=0.1, data=None):
    """1-based numbers of the projections judged unsuitable (largest combined
    neighbour error first).  ``prozent_to_reduce`` is a fraction (< 1) or a count
    (>= 1); -1 means 0.1.  ``data`` may supply the brightness-corrected stack
    [n_projections][n_slices][n_detectors] instead of reading ``name``."""
    print("###### Determining Bad Projections ######")
    if data is None:
        data, _, _ = brightness_correction(name, "", 0.0, [])
    NA, Nz, Nx = data.shape
    if prozent_to_reduce == -1:
        prozent_to_reduce = 0.1
    smoothing = 3
    Nx_new = 250
    Nz_new = int(Nx_new * Nz / float(Nx))
    if Nx > Nx_new:
        data = data[:, ::max(Nz // max(Nz_new, 1), 1)][:, :, ::max(Nx // Nx_new, 1)]
    data = np.stack([reduce_noise(data[i], smoothing) for i in range(data.shape[0])]).astype(np.float32)
    NA, Nz, Nx = data.shape
    if searchradius is None:
        searchradius = min(Nx, Nz) / 10
    searchradius = int(searchradius)
    W = np.stack([weighted_gradient(data[i].astype(np.float64))[1] for i in range(NA)]).astype(np.float32)
    err1 = [compare_shift_twosided(W[i].astype(np.float64), W[i + 1].astype(np.float64), searchradius)[0]
            for i in range(NA - 1)]
    err2 = [compare_shift_twosided(W[i].astype(np.float64), W[i + 2].astype(np.float64), int(searchradius * 1.5))[0]
            for i in range(NA - 2)]
    N = len(err1) + 1
    combined = []
    for i in range(N):
        j, jj = np.clip(i, 0, N - 2), np.clip(i - 1, 0, N - 2)
        jjj, jjjj = np.clip(i, 0, N - 3), np.clip(i - 2, 0, N - 3)
        a = err1[j] + 0.5 * err2[jjj]
        b = err1[jj] + 0.5 * err2[jjjj]
        combined.append(min(a, b))
    if prozent_to_reduce >= 1:
        prozent_to_reduce = float(prozent_to_reduce) / N
    order = []
    err = list(combined)
    for _ in range(len(err)):
        m = max(err)
        k = err.index(m)
        err[k] = -1
        order.append(k + 1)
    bad = order[:int(round(N * prozent_to_reduce))]
    print("badprojections found", bad)
    return bad
