"""Detection of unsuitable projections (find_bad_ele.py:139-230) on the GPU.

``find_bad_projections`` keeps the reference's host steps -- brightness-corrected
data (h5utilities ``Brightness_correction``), subsampling to about 250 detector
columns, the default search radius, combining each projection's neighbour errors,
ranking -- and runs the array stages on the device through the C ABI
(include/graptor_gb300.h, ``gt_badproj_*``):

  * gt_badproj_smooth   reduce_noise (:69-75), box sums in float64 stored as float32 (:152-155)
  * gt_badproj_wgrad    weighted_gradient (:103-136) in float32, as on the reference's float32 stack
  * gt_badproj_compare  compare_shift_twosided (:55-100) for projections one apart with the search
                        radius and two apart with 1.5 times it (:177-190)

Every stored value equals the reference's; the neighbour errors are float64 sums of
the same terms in another order.  The device stack stays in HBM for the whole
detection; only the stack goes up and the 2 NA neighbour errors come back.

Differences from the reference: its subsampling step (:148-151) divides with ``/``
inside ``range`` (a TypeError on Python 3 once the detector is wider than 250
columns) -- here it is the integer step it means; its default radius calls NumPy's
``min`` on two scalars (which raises) -- here it is Python's ``min``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .preprocess import brightness_correction

SMOOTHING = 3


def _torch():
    import torch
    return torch


def _p(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _stream(dev):
    return ctypes.c_void_p(_torch().cuda.current_stream(dev).cuda_stream)


def subsample(data: np.ndarray) -> np.ndarray:
    """The reduction to about 250 detector columns (:148-151)."""
    NA, Nz, Nx = data.shape
    Nx_new = 250
    Nz_new = int(Nx_new * Nz / float(Nx))
    if Nx > Nx_new:
        data = data[:, ::max(Nz // max(Nz_new, 1), 1)][:, :, ::max(Nx // Nx_new, 1)]
    return data


def upload(data: np.ndarray, device=0):
    """The subsampled stack as a float64 device tensor [NA][Nz][Nx]."""
    torch = _torch()
    dev = torch.device("cuda", device) if isinstance(device, int) else torch.device(device)
    host = np.ascontiguousarray(subsample(np.asarray(data)), dtype=np.float64)
    return torch.from_numpy(host).to(dev)


def stages(d):
    """(smoothed stack, weighted gradients) of a device stack, both float32 device tensors."""
    torch = _torch()
    NA, Nz, Nx = d.shape
    s = SMOOTHING
    if Nz - 2 * s < 3 or Nx - 2 * s < 3:
        raise ValueError(f"projections of {Nz} x {Nx} pixels are too small for the detector")
    S = torch.empty((NA, Nz - 2 * s, Nx - 2 * s), dtype=torch.float32, device=d.device)
    W = torch.empty((NA, Nz - 2 * s - 2, Nx - 2 * s - 2), dtype=torch.float32, device=d.device)
    st = _stream(d.device)
    L.check(L.lib().gt_badproj_smooth(_p(d), NA, Nz, Nx, s, _p(S), st))
    L.check(L.lib().gt_badproj_wgrad(_p(S), NA, S.shape[1], S.shape[2], _p(W), st))
    return S, W


def pair_errors(W, offset: int, radius: int, want_pixels: bool = False):
    """Neighbour errors of projections (q, q + offset) as a float64 device tensor
    (and the per-pixel maxima [pairs][Nz-2r][Nx-2r] when ``want_pixels``)."""
    torch = _torch()
    NA, nz, nx = W.shape
    npairs = max(NA - offset, 0)
    err = torch.zeros(npairs, dtype=torch.float64, device=W.device)
    mz, mx = nz - 2 * radius, nx - 2 * radius
    if radius < 0 or mz < 0 or mx < 0:
        raise ValueError(f"search radius {radius} does not fit projections of {nz} x {nx} pixels")
    E = torch.zeros((npairs, mz, mx), dtype=torch.float32, device=W.device) if want_pixels else None
    if npairs == 0 or mz == 0 or mx == 0:  # empty interior: the reference's norm of nothing
        return (err, E) if want_pixels else err
    blocks = L.lib().gt_badproj_blocks(nz, nx, radius)
    part = torch.empty(npairs * blocks, dtype=torch.float64, device=W.device)
    L.check(L.lib().gt_badproj_compare(_p(W), NA, nz, nx, offset, radius, _p(part), _p(err),
                                       _p(E) if want_pixels else None, _stream(W.device)))
    return (err, E) if want_pixels else err


def compare_shift_twosided(U: np.ndarray, V: np.ndarray, steps: int, device=0):
    """compare_shift_twosided (:55-67) of two images as the detector stores them
    (float32): (1-norm, per-pixel maxima as float64)."""
    torch = _torch()
    W = torch.from_numpy(np.ascontiguousarray(np.stack([U, V]), dtype=np.float32)).to(torch.device("cuda", device))
    err, E = pair_errors(W, 1, int(steps), want_pixels=True)
    return float(err.cpu()[0]), E[0].cpu().numpy().astype(np.float64)


def select(err1, err2, prozent_to_reduce):
    """Each projection's error is the smaller of its two combined neighbour errors;
    the largest are reported, 1-based (:192-228).  Returns (numbers, combined)."""
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


def detect(d, searchradius=None):
    """Neighbour errors (err1, err2) of a device stack: float64 device tensors."""
    S, W = stages(d)
    if searchradius is None:
        searchradius = min(S.shape[1], S.shape[2]) / 10
    r = int(searchradius)
    return pair_errors(W, 1, r), pair_errors(W, 2, int(r * 1.5))


def find_bad_projections(name: str, searchradius=None, prozent_to_reduce=0.1, data=None, device=0):
    """1-based numbers of the projections judged unsuitable (largest combined
    neighbour error first).  ``prozent_to_reduce`` is a fraction (< 1) or a count
    (>= 1); -1 means 0.1.  ``data`` may supply the brightness-corrected stack
    [n_projections][n_slices][n_detectors] instead of reading ``name``."""
    print("###### Determining Bad Projections ######")
    if data is None:
        data, _, _ = brightness_correction(name, "", 0.0, [])
    e1, e2 = detect(upload(data, device), searchradius)
    bad = select(e1.cpu().tolist(), e2.cpu().tolist(), prozent_to_reduce)[0]
    print("badprojections found", bad)
    return bad
