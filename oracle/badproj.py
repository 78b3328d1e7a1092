"""NumPy oracle of the bad-projection detector (test infrastructure only).

Restates ``Find_Bad_projections`` and its helpers (find_bad_ele.py:55-230) with the
reference's array types, so that the device stages (gt_badproj_*) can be checked
value for value:

* ``reduce_noise``            :69-75   box sum in float64, /(4 s^2); the stack stores it as float32 (:152-155)
* ``weighted_gradient``       :103-136 differences in the input's type (float32 inside the detector:
                                        ``abs(a - b) * 1 / 2 ** 0.5`` stays float32), product in float64
* ``compare_shift``           :76-100  ``abs(U - V_)`` in the input's type (float32 inside the detector),
                                        minimum over shifts, as float64
* ``compare_shift_twosided``  :55-67   elementwise maximum of both directions, 1-norm
* ``find_bad_projections``    :139-230 the pipeline on a brightness-corrected stack

Pinned against the reference's own outputs in ``tests/golden/badproj.npz``
(``tests/golden/make_badproj_golden.py``).  Differences from the reference: the
subsampling step (:148-151) divides with ``/`` inside ``range`` (a TypeError on
Python 3 once the detector is wider than 250 columns) -- here it is the integer step
it means; the default search radius (:162-163) calls NumPy's ``min`` on two
scalars (it raises) -- here it is Python's ``min``.  The reference's ``E**(0.5)`` in
the two-sided comparison discards its result, so the comparison uses E itself, as
the reference does.  Only tests and the benchmark's CPU baseline use this module.
"""
from __future__ import annotations

import numpy as np


def reduce_noise(U: np.ndarray, steps: int) -> np.ndarray:
    Nx, Ny = U.shape
    E = np.zeros([Nx - 2 * steps, Ny - 2 * steps])
    for k in range(-steps, steps + 1):
        for l in range(-steps, steps + 1):
            E += U[steps + k:Nx - steps + k, steps + l:Ny - steps + l]
    return E / (4 * steps ** 2)


def weighted_gradient(u: np.ndarray):
    Nx, Ny = u.shape
    c = u[1:Nx - 1, 1:Ny - 1]
    E, Nb = [], []
    for i, j in [(-1, -1), (-1, 1), (0, -1), (0, 1), (1, -1), (1, 1), (-1, 0), (1, 0)]:
        nb = u[1 + i:Nx - 1 + i, 1 + j:Ny - 1 + j]
        E.append(np.abs(c - nb) * 1 / ((i * i + j * j) ** 0.5))  # Python float: keeps u's type
        Nb.append(np.abs(nb))
    value = np.max(E, axis=0).astype(np.float64) * np.min(Nb, axis=0).astype(np.float64)
    return np.linalg.norm(value), value


def compare_shift(U: np.ndarray, V: np.ndarray, steps: int):
    Nx0, Ny0 = U.shape
    Ui = U[steps:Nx0 - steps, steps:Ny0 - steps]
    E = None
    for k in range(-steps, steps + 1):
        for l in range(-steps, steps + 1):
            D = np.abs(Ui - V[steps + k:Nx0 - steps + k, steps + l:Ny0 - steps + l])
            E = D if E is None else np.minimum(E, D)
    E = E.astype(np.float64)
    return np.linalg.norm(E), E


def compare_shift_twosided(U: np.ndarray, V: np.ndarray, steps: int):
    _, E1 = compare_shift(U, V, steps)
    _, E2 = compare_shift(V, U, steps)
    E = np.maximum(E1, E2)
    return np.linalg.norm(E.reshape(E.size), 1), E


def subsample(data: np.ndarray) -> np.ndarray:
    """The reduction to about 250 detector columns (:148-151)."""
    NA, Nz, Nx = data.shape
    Nx_new = 250
    Nz_new = int(Nx_new * Nz / float(Nx))
    if Nx > Nx_new:
        data = data[:, ::max(Nz // max(Nz_new, 1), 1)][:, :, ::max(Nx // Nx_new, 1)]
    return data


def stages(data: np.ndarray, smoothing: int = 3):
    """(smoothed stack float32, weighted gradients float32) of a brightness-corrected stack."""
    data = subsample(data)
    S = np.stack([reduce_noise(data[i], smoothing) for i in range(data.shape[0])]).astype(np.float32)
    W = np.stack([weighted_gradient(S[i])[1] for i in range(S.shape[0])]).astype(np.float32)
    return S, W


def pair_errors(W: np.ndarray, offset: int, radius: int):
    return [compare_shift_twosided(W[i], W[i + offset], radius)[0] for i in range(W.shape[0] - offset)]


def select(err1, err2, prozent_to_reduce):
    """Combined neighbour errors and the ranking (:192-228); 1-based numbers."""
    N = len(err1) + 1
    combined = []
    for i in range(N):
        j, jj = np.clip(i, 0, N - 2), np.clip(i - 1, 0, N - 2)
        jjj, jjjj = np.clip(i, 0, N - 3), np.clip(i - 2, 0, N - 3)
        combined.append(min(err1[j] + 0.5 * err2[jjj], err1[jj] + 0.5 * err2[jjjj]))
    if prozent_to_reduce == -1:
        prozent_to_reduce = 0.1
    if prozent_to_reduce >= 1:
        prozent_to_reduce = float(prozent_to_reduce) / N
    err, order = list(combined), []
    for _ in range(len(err)):
        m = max(err)
        k = err.index(m)
        err[k] = -1
        order.append(k + 1)
    return order[:int(round(N * prozent_to_reduce))], combined


def find_bad_projections(data: np.ndarray, searchradius=None, prozent_to_reduce=0.1):
    """Oracle of the whole detector on a brightness-corrected stack [NA][Nz][Nx]."""
    S, W = stages(data)
    if searchradius is None:
        searchradius = min(S.shape[1], S.shape[2]) / 10
    r = int(searchradius)
    err1 = pair_errors(W, 1, r)
    err2 = pair_errors(W, 2, int(r * 1.5))
    return select(err1, err2, prozent_to_reduce)[0]
