"""Projection-data preprocessing of the reference CLI, in NumPy.

Restates h5utilities.py's loaders that the command line uses:

* :func:`brightness_correction` -- ``Brightness_correction`` (h5utilities.py:144-198):
  drop bad projections (1-based numbers from a file and a list), cut a fraction of
  the detector on both sides, subtract the background measured in the cut-off
  band, rescale every projection to the common mean brightness.
* :func:`global_rescaling` -- ``global_rescaling`` (:273-312): drop bad
  projections, shift the minimum to zero, cut the sides; returns the background
  level for the ``mean`` baseline option.
* :func:`brightness_correction2` -- ``Brightness_correction2`` (:256-269) on one
  sinogram.
* :func:`read_bad_projection_file` -- the bad-projection text file (one number per
  entry).  The reference builds this list with ``map(int, ...) + list``, which
  fails on Python 3; here it is a list of ints, which is what the code means.

Arrays are [n_projections][n_slices][n_detectors] (the reference's ``np_data``).
"""
from __future__ import annotations

import math

import numpy as np

from .mrc import read_projections


def read_bad_projection_file(path: str):
    if not path:
        return []
    with open(path) as fh:
        return [int(t) for t in fh.read().split()]


def _drop(data, angles, bad):
    keep = [i for i in range(data.shape[0]) if (i + 1) not in bad]
    return data[keep], np.asarray(angles)[keep]


def _cut_background(data, cutedges):
    """Cut ceil(Nx*cutedges) detector columns on both sides; the background is the
    mean of the inner halves of the cut bands (h5utilities.py:167-177)."""
    Nx = data.shape[2]
    cut = int(math.ceil(Nx * cutedges))
    if cut > 0:
        bg = 0.5 * (np.mean(data[:, :, cut // 2:cut]) + np.mean(data[:, :, Nx - cut // 2:Nx]))
    else:
        bg = 0.0
    return data[:, :, cut:Nx - cut], bg


def brightness_correction(name: str, badname: str, cutedges: float, bad_projections):
    data, angles = read_projections(name)
    bad = read_bad_projection_file(badname) + list(bad_projections)
    data, angles = _drop(data, angles, bad)
    data, bg = _cut_background(data, float(cutedges))
    data = data - bg
    means = data.reshape(data.shape[0], -1).mean(axis=1)
    W = means.mean()
    data = data * (W / means)[:, None, None]
    return data, angles, 0


def global_rescaling(name: str, badname: str, cutedges: float, bad_projections):
    data, angles = read_projections(name)
    bad = read_bad_projection_file(badname) + list(bad_projections)
    data = data - np.min(data)
    data, angles = _drop(data, angles, bad)
    data = data - np.min(data)
    data, bg = _cut_background(data, float(cutedges))
    return data, angles, bg


def brightness_correction2(sino: np.ndarray) -> np.ndarray:
    means = sino.reshape(sino.shape[0], -1).mean(axis=1)
    W = means.mean()
    return sino * (W / means)[:, None]


def pixel_size(name: str) -> float:
    """Detector pixel size recorded with a projection stack (``readh5alternative``,
    h5utilities.py:421-475): ``Info/Dimensions/2`` second entry in HDF5 files,
    -1 (unknown) for MRC stacks and when h5py is missing."""
    if ".h5" not in name:
        return -1.0
    try:
        import h5py
    except ImportError:
        return -1.0
    with h5py.File(name, "r") as hf:
        return float(np.array(hf.get("Info").get("Dimensions").get("2"))[1])


def load_channel(name: str, brightness: str, badname: str, cutedges: float, bad_projections):
    """The loader the CLI picks by the brightness option (Reconstruction_coupled.py:148-155)."""
    if brightness.upper() == "BRIGHT":
        return brightness_correction(name, badname, cutedges, bad_projections)
    if brightness.upper() == "BASIC":
        return global_rescaling(name, badname, cutedges, bad_projections)
    data, angles = read_projections(name)
    return data, angles, 0
