"""MRC volumes and tilt-angle files, in NumPy.

The reference reads and writes projection stacks and reconstructions with the
``mrcfile`` package (h5utilities.py:358-419 reads, Reconstruction_coupled.py:263-290
and :471-495 write) and reads the tilt angles from a ``.rawtlt`` text file (one
angle in degrees per entry) or, failing that, a ``.csv`` file (first column).
``mrcfile`` is not a dependency here; this module reads and writes the MRC2014
layout directly: a 1024-byte little- or big-endian header (sizes, data mode,
cell, axis order, density statistics, ``MAP `` stamp, machine stamp, labels), an
optional extended header, then the data in C order [nz][ny][nx].
"""
from __future__ import annotations

import os
import sys

import numpy as np

# MRC2014 data modes
_MODES = {0: np.int8, 1: np.int16, 2: np.float32, 4: np.complex64, 6: np.uint16, 12: np.float16}
_MODE_OF = {np.dtype(np.int8): 0, np.dtype(np.int16): 1, np.dtype(np.float32): 2, np.dtype(np.complex64): 4,
            np.dtype(np.uint16): 6, np.dtype(np.float16): 12}


def _eprint(*a):
    print(*a, file=sys.stderr)


def read_mrc(path: str) -> np.ndarray:
    """The data of an MRC file as an array [nz][ny][nx] (native byte order).

    Reads permissively like the reference (``mrcfile.open(..., permissive=True)``):
    a missing ``MAP `` stamp or an unknown machine stamp only decides the byte
    order from the header's sizes."""
    with open(path, "rb") as fh:
        head = fh.read(1024)
        if len(head) < 1024:
            raise IOError(f"{path}: shorter than an MRC header")
        order = "<"
        if head[212:214] == b"\x11\x11":
            order = ">"
        elif head[212:214] != b"\x44\x44" and head[212:214] != b"\x44\x41":
            nx_le = np.frombuffer(head[0:4], "<i4")[0]
            mode_le = np.frombuffer(head[12:16], "<i4")[0]
            if not (0 < nx_le < 1 << 24 and mode_le in _MODES):
                order = ">"
        ints = np.frombuffer(head[:56], order + "i4")
        nx, ny, nz, mode = (int(v) for v in ints[:4])
        if mode not in _MODES:
            raise IOError(f"{path}: unsupported MRC data mode {mode}")
        if min(nx, ny, nz) < 0:
            raise IOError(f"{path}: negative dimensions {nx} x {ny} x {nz}")
        nsymbt = int(np.frombuffer(head[92:96], order + "i4")[0])
        fh.seek(1024 + max(nsymbt, 0))
        dt = np.dtype(_MODES[mode]).newbyteorder(order)
        count = nx * ny * nz
        data = np.fromfile(fh, dtype=dt, count=count)
        if data.size != count:
            raise IOError(f"{path}: expected {count} values, found {data.size}")
    return data.reshape(nz, ny, nx).astype(dt.newbyteorder("="), copy=False)


def write_mrc(path: str, data, overwrite: bool = True, voxel_size: float = 1.0) -> None:
    """Write a 2-D or 3-D array as MRC2014 (little-endian), mode from the dtype
    (float64 is stored as float32, as ``mrcfile`` does for the reference's
    float32 results)."""
    if os.path.exists(path) and not overwrite:
        raise IOError(f"{path} exists")
    a = np.asarray(data)
    if a.dtype == np.float64:
        a = a.astype(np.float32)
    if a.dtype not in _MODE_OF:
        raise ValueError(f"dtype {a.dtype} has no MRC mode")
    if a.ndim == 2:
        a = a[None]
    if a.ndim != 3:
        raise ValueError("MRC data must be 2-D or 3-D")
    a = np.ascontiguousarray(a.astype(a.dtype.newbyteorder("<"), copy=False))
    nz, ny, nx = a.shape
    head = np.zeros(256, "<i4")
    head[0:3] = (nx, ny, nz)
    head[3] = _MODE_OF[np.dtype(a.dtype.newbyteorder("="))]
    head[7:10] = (nx, ny, nz)  # mx, my, mz
    fl = head.view("<f4")
    fl[10:13] = (nx * voxel_size, ny * voxel_size, nz * voxel_size)  # cell lengths
    fl[13:16] = (90.0, 90.0, 90.0)
    head[16:19] = (1, 2, 3)  # mapc, mapr, maps
    if a.size and not np.iscomplexobj(a):
        vals = a.astype(np.float64)
        fl[19], fl[20], fl[21] = vals.min(), vals.max(), vals.mean()
        fl[54] = vals.std()
    head[22] = 1 if nz == 1 else 401  # ispg: image stack / volume
    head[23] = 0  # no extended header
    b = bytearray(head.tobytes())
    b[104:108] = b"MRCO"  # exttyp
    b[108:112] = np.int32(20140).tobytes()  # nversion
    b[208:212] = b"MAP "
    b[212:216] = b"\x44\x44\x00\x00"  # little-endian machine stamp
    with open(path, "wb") as fh:
        fh.write(bytes(b))
        fh.write(a.tobytes())


def read_angles(mrc_path: str) -> np.ndarray:
    """Tilt angles (radians) for a projection stack, from ``<name>.rawtlt``
    (whitespace-separated degrees) or else ``<name>.csv`` (first column), as
    h5utilities.py:373-405; warns when both exist and uses ``.rawtlt``."""
    raw = mrc_path.replace(".mrc", ".rawtlt")
    csv = mrc_path.replace(".mrc", ".csv")
    if os.path.isfile(raw):
        if os.path.isfile(csv):
            _eprint(f"Warning, two candidates for angle files {raw} and {csv}. By default rawtlt information is used")
        ang = []
        with open(raw) as fh:
            for entry in fh.read().split():
                try:
                    ang.append(float(entry) / 180 * np.pi)
                except ValueError:
                    raise ValueError(f'Numbers "{entry}" in the angle file {raw} could not be interpreted correctly')
        return np.array(ang)
    if os.path.isfile(csv):
        import csv as _csv
        ang = []
        with open(csv) as fh:
            for row in _csv.reader(fh, delimiter=","):
                if not row:
                    continue
                try:
                    ang.append(float(row[0]) / 180 * np.pi)
                except ValueError:
                    raise ValueError(f'Number "{row[0]}" in the angle file {csv} could not be interpreted correctly')
        return np.array(ang)
    raise IOError(f"Could not find angle files {csv} or {raw}")


def read_projections(path: str):
    """Projection stack and angles like ``readh5`` (h5utilities.py:358-419):
    data float64 [n_projections][n_slices][n_detectors], angles in radians.
    HDF5 input needs ``h5py``, which is optional."""
    if ".h5" in path:
        try:
            import h5py
        except ImportError as e:
            raise IOError(f"{path}: reading .h5 needs h5py, which is not installed") from e
        with h5py.File(path, "r") as hf:
            data = np.array(hf.get("data"), dtype=np.float64)
            angles = np.array(hf.get("Info").get("Dimensions").get("3"))
        return data, angles
    if ".mrc" in path:
        return read_mrc(path).astype(np.float64), read_angles(path)
    raise IOError(f"Could not interpret datatype of {path}, aborting process")
