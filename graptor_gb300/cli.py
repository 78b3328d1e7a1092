"""Command-line reconstruction, mirroring Reconstruction_coupled.py.

    python -m graptor_gb300.cli example/Al_EDXsino.mrc example/HAADF_lrsino.mrc \\
        --SliceLevels 50 55 1 --Coupling frob3d --Outfile Result/results --Discrepancy KL \\
        --Maxiter 2000 --alpha 4 1 --Channelnames Alum HAADF --mu 0.008 0.5 --Regularisation TGV

Same options, defaults, preprocessing and outputs as the reference's ``main``
(Reconstruction_coupled.py:871-1146) with its drivers ``Coupled_Reconstruction2d``
(:109-295) and ``Coupled_Reconstruction3d`` (:297-539): load each channel with the
brightness option, percentile scaling (``--Scalepars``), baseline handling,
slice selection, reconstruction through the drop-in
``Reconstructionapproach2d/3d`` (CUDA), rescaling by the data/sinogram ratio, and
MRC output (``<prefix>_<channel>.mrc``, ``_sinogram.mrc``, ``_all_channels.mrc``,
``_all_channels_normalized.mrc``) plus the ``.config`` record of the arguments.

Differences: ``--GPU_Choice -1`` (the reference asks interactively) selects CUDA
device 0; live plotting is not supported (``--Plot`` is accepted and ignored);
HDF5 input needs ``h5py``.  The two-resolution couplings (FrobSubs / UncorrSubs)
run ``Coupled_Reconstruction3dbigresu`` (:542-873) through the drop-in
``Reconstructionapproach3dsubsmapling``.
"""
from __future__ import annotations

import argparse
import math
import os
import sys
import time

import numpy as np

from . import mrc, preprocess
from ._lib import GraptorError, GraptorMemoryError


def eprint(*a):
    print(*a, file=sys.stderr)
    sys.stderr.flush()


METHODS_2D = {
    "FROB2D": "Frobenius 2D Reconstruction", "FROBENIUS2D": "Frobenius 2D Reconstruction",
    "FROBENIUS": "Frobenius 2D Reconstruction", "FROB": "Frobenius 2D Reconstruction",
    "NUCL2D": "Nuclear 2D Reconstruction", "NUCLEAR2D": "Nuclear 2D Reconstruction",
    "NUCLEAR": "Nuclear 2D Reconstruction", "NUC2D": "Nuclear 2D Reconstruction",
    "UNCORRELATED": "Uncorrelated 2D Reconstruction", "UNCORRELATED2D": "Uncorrelated 2D Reconstruction",
    "UNCORR": "Uncorrelated 2D Reconstruction", "UNCORR2D": "Uncorrelated 2D Reconstruction",
    "UNCOR": "Uncorrelated 2D Reconstruction", "UNCOR2D": "Uncorrelated 2D Reconstruction",
}
METHODS_3D = {
    "NUCL3D": "Nuclear 3D Reconstruction", "NUCLEAR3D": "Nuclear 3D Reconstruction",
    "NUC3D": "Nuclear 3D Reconstruction", "NUCLE3D": "Nuclear 3D Reconstruction",
    "FROBENIUS3D": "Frobenius 3D Reconstruction", "3D": "Frobenius 3D Reconstruction",
    "FROB3D": "Frobenius 3D Reconstruction",
    "UNCORRELATED3D": "Uncorrelated 3D Reconstruction", "UNCOR3D": "Uncorrelated 3D Reconstruction",
    "UNCORR3D": "Uncorrelated 3D Reconstruction",
}
METHODS_SUBS = {k: "Frobenius 3D Subsampling Reconstruction" for k in (
    "FROBENIUS_SUBSAMPLING", "SUBSAMPLING_FROBENIUS", "FROSUBS", "SUBS", "SUB", "FROBSUBS", "FROBSUB", "FROSUB")}
METHODS_SUBS.update({k: "Uncorrelated 3D Subsampling Reconstruction" for k in (
    "UNCORRELATED_SUBSAMPLING", "SUBSAMPLING_UNCORRELATED", "UNCORSUBS", "UNCORRSUBS", "UNCORSUB", "UNSUB", "UNSUBS")})


def parse_method(coupling: str):
    """(method string, setting) as Reconstruction_coupled.py:958-992; setting
    0 = 2-D, 1 = 3-D, 2 = subsampling; unknown names fall back to Frobenius 2-D."""
    m = coupling.upper()
    if m in METHODS_2D:
        return METHODS_2D[m], 0
    if m in METHODS_3D:
        return METHODS_3D[m], 1
    if m in METHODS_SUBS:
        return METHODS_SUBS[m], 2
    eprint(f"!!!!!!!!!!!! Warning: method {m}is not known, setting method to 'Frobenius 2D Reconstruction'.")
    return "Frobenius 2D Reconstruction", 0


def resolve_names(names):
    """Append .h5 / .mrc where the name has neither (Reconstruction_coupled.py:1005-1026)."""
    out = []
    for n in names:
        if ".h5" not in n and ".mrc" not in n:
            if n.endswith("."):
                n = n[:-1]
            if os.path.isfile(n + ".h5"):
                n = n + ".h5"
            elif os.path.isfile(n + ".mrc"):
                n = n + ".mrc"
            else:
                raise IOError(f"The file with name {n} has not been found. Operation aborted.")
        if not os.path.isfile(n):
            raise IOError(f"The file with name {n} has not been found. Operation aborted.")
        out.append(n)
    return out


def _baseline(sino, baseline, threshold, averagenoise, dims3):
    """Baseline options (2-D: :184-201; 3-D: :357-374)."""
    b = baseline.upper()
    if b == ("MEAN1" if dims3 else "MEAN"):
        sino = sino - averagenoise
    if b == ("MEAN2" if dims3 else "MEANTHRES"):
        sino = sino - np.mean(sino[np.where(sino < threshold)])
    if b == "THRESHOLDING":
        sino = sino.copy()
        sino[np.where(sino < threshold)] = 0
    return sino


def _save(result, channelnames, solution, sino):
    """MRC outputs of :263-290 / :471-495 (solution [C][Nz][N][N], sino [C][nang][Nz][nd])."""
    C = solution.shape[0]
    for i in range(C):
        mrc.write_mrc(f"{result}_{channelnames[i]}.mrc", solution[i].astype(np.float32))
        mrc.write_mrc(f"{result}_{channelnames[i]}_sinogram.mrc", sino[i].astype(np.float32))
    if C > 1:
        Nz, Nx, Ny = solution.shape[1:]
        coll = np.zeros([Nz, Nx, C * Ny], np.float32)
        for j in range(C):
            coll[:, :, j * Ny:(j + 1) * Ny] = solution[j]
        mrc.write_mrc(f"{result}_all_channels.mrc", coll)
        coll = np.zeros([Nz, Nx, C * Ny], np.float32)
        for j in range(C):
            coll[:, :, j * Ny:(j + 1) * Ny] = solution[j] / np.max(solution[j])
        mrc.write_mrc(f"{result}_all_channels_normalized.mrc", coll)


def _load(names, datahandling, badprojections, find_bad, scalepars, section, dims3, device=0, apply_found=False):
    """Load, clean and scale every channel (2-D: :129-170; 3-D: :320-345).

    The projections ``--Find_Bad_Projections`` finds are reported but, as in the
    reference, not removed: it appends the list as one entry of ``Badprojections``
    (:138, :328), and the loader's ``i+1 in text`` test (h5utilities.py:144-165)
    never matches a list.  ``apply_found`` (``--Apply_Found_Projections``) removes
    them."""
    brightness, baseline, cutedges, badfile, threshold = datahandling[:5]
    cutedges, threshold = float(cutedges), float(threshold)
    bad = list(badprojections)
    if find_bad[0] not in (0, 0.0):
        from .badproj import find_bad_projections
        found = find_bad_projections(names[0], find_bad[1], find_bad[0], device=device)
        if apply_found:
            bad.extend(found)
        else:
            eprint("Note: as in the reference, the projections found are not removed "
                   "(--Apply_Found_Projections removes them).")
    data, ratio, noise, angles = [], [], [], None
    for n in names:
        d, angles, avg = preprocess.load_channel(n, brightness, badfile, cutedges, bad)
        Ny = d.shape[1]
        if min(section[0], section[-1]) < 0 or max(section[0], section[-1]) >= Ny:
            raise IndexError(f"Slice levels are not in a suitable scope. Must lie between 0 and Ny={Ny - 1}. "
                             "Aborting operation!")
        if dims3:  # ratio before the percentile scaling (:330-333)
            ratio.append(np.sum(d[:, list(section)]) / len(angles))
            d = d - np.percentile(d, scalepars[0])
        else:  # ratio after the shift (:159-162)
            d = d - np.percentile(d, scalepars[0])
            ratio.append(np.sum(d[:, list(section)]) / len(angles))
        d = d / np.percentile(d, scalepars[1])
        data.append(d)
        noise.append(avg)
    return data, ratio, noise, angles, baseline, threshold


def reconstruct_2d(names, result, mu, alpha, maxiter, method, levels, datahandling, badprojections, find_bad,
                   channelnames, regularisation, discrepancy, scalepars, device=0, apply_found=False):
    """Slice-by-slice 2-D reconstruction (Coupled_Reconstruction2d)."""
    from .radon_tgv_primal_dual_2d import Reconstructionapproach2d
    section = range(levels[0], levels[1] + 1, levels[2])
    data, ratio, noise, angles, baseline, threshold = _load(names, datahandling, badprojections, find_bad, scalepars,
                                                            section, False, device, apply_found)
    C = len(names)
    nang, _, Nx = data[0].shape
    Nz = len(section)
    U = np.zeros([C, Nz, Nx, Nx], np.float32)
    sinos = np.zeros([C, nang, Nz, Nx], np.float32)
    meth = method if C > 1 else "Uncorrelated 2D Reconstruction"
    t0 = time.time()
    for j, lev in enumerate(section):
        coll = [_baseline(np.array(data[i][:, lev, :]), baseline, threshold, noise[i], False) for i in range(C)]
        info = [j / float(Nz), 1 / float(Nz), lev]
        u, sn = Reconstructionapproach2d(coll, angles + np.pi / 2, (alpha[0], alpha[1]), mu, maxiter, device,
                                         [0, 0.1], discrepancy, meth, regularisation, info)
        U[:, j] = u
        sinos[:, :, j, :] = np.asarray(sn)
    sol, nsino = U.copy(), sinos.copy()
    for i in range(C):
        fak = np.sum(nsino[i]) / ratio[i]
        sol[i] /= fak / nang
        nsino[i] /= fak / nang
    _save(result, channelnames, sol, nsino)
    print("\nTime required for reconstruction:", int(10.0 * (time.time() - t0)) / 10.0, " seconds.\n")
    return sol


def reconstruct_3d(names, result, mu, alpha, maxiter, method, levels, datahandling, badprojections, find_bad,
                   channelnames, regularisation, discrepancy, overlay, chunksize, scalepars, device=0,
                   apply_found=False):
    """Volumetric reconstruction in slice chunks with overlap (Coupled_Reconstruction3d):
    chunks of at most ``chunksize`` slices (all of them when <= 0), shrunk by 0.7 and
    retried when the device runs out of memory."""
    from .radon_tgv_primal_dual_3d import Reconstructionapproach3d
    section = list(range(levels[0], levels[1] + 1, levels[2]))
    data, ratio, noise, angles, baseline, threshold = _load(names, datahandling, badprojections, find_bad, scalepars,
                                                            section, True, device, apply_found)
    C = len(names)
    coll = []
    for i in range(C):
        s = _baseline(data[i], baseline, threshold, noise[-1], True)
        coll.append(s[:, section, :])
    nang, nsec, nd = coll[0].shape
    possible = nsec if chunksize < 1 else min(nsec, chunksize)
    U = np.zeros([C, nd, nd, nsec])
    new_sino = np.zeros([C, nang, nsec, nd])
    remaining = section[:]
    t0 = time.time()
    while remaining:
        if overlay > possible / 4.0:
            overlay = int(possible / 4)
            eprint(f"Overlap is too large for possible split size, reducing overlap to {overlay} which is a fourth "
                   "of the possible splits.")
        current = remaining[:min(possible, len(remaining))]
        sp, ep = section.index(current[0]), section.index(current[-1])
        cur = [c[:, sp:ep + 1, :] for c in coll]
        localending = possible - 2 * overlay if possible < len(remaining) else len(remaining)
        ov_s = 0 if len(remaining) == len(section) else overlay
        ov_e = len(current) - len(remaining) if possible >= len(remaining) else overlay
        info = [sp / float(nsec), (len(current) - ov_e) / float(nsec), current]
        try:
            u_loc, s_loc = Reconstructionapproach3d(cur, angles + np.pi / 2, (alpha[0], alpha[1]), mu, maxiter, device,
                                                    [0, 0.1], levels[2], discrepancy, method, regularisation, info)
        except GraptorMemoryError:
            possible = int(possible * 0.7)
            eprint(f"Warning: Computation requires too much memory, the problem is split, trying to compute "
                   f"{possible} slices at once.")
            if possible < 1:
                raise MemoryError("Even a single slice requires too much memory.")
            continue
        except GraptorError as err:
            possible = int(possible * 0.7)
            eprint(f"An exception of type {type(err).__name__} occurred. Arguments:\n{err.args!r}")
            if possible < 1:
                raise
            continue
        remaining = remaining[localending:]
        U[:, :, :, sp + ov_s:ep + 1 - ov_e] = u_loc[:, :, :, ov_s:len(current) - ov_e]
        new_sino[:, :, sp + ov_s:ep + 1 - ov_e, :] = s_loc[:, :, ov_s:len(current) - ov_e, :]
    sol = np.zeros([C, nsec, nd, nd], np.float32)
    for i in range(nsec):
        sol[:, i] = U[:, :, :, i]
    ns = new_sino.astype(np.float32)
    for i in range(C):
        fak = np.sum(new_sino[i]) / ratio[i]
        sol[i] /= fak / nang
        ns[i] /= fak / nang
    _save(result, channelnames, sol, ns)
    print("\nTime required for reconstruction:", int(10.0 * (time.time() - t0)) / 10.0, " seconds.\n")
    return U


def pixel_ratio(sizes, C0, given):
    """Coarse/fine pixel ratio p (Reconstruction_coupled.py:590-611): from the pixel
    sizes stored with the data when both resolutions have one (a different
    ``--Pixelratio`` then aborts), else the ``--Pixelratio`` input; sizes within one
    resolution must agree."""
    jj = sizes.index(max(sizes[:C0]))
    for i in range(C0):
        if sizes[i] != sizes[jj] and sizes[i] > 0 and sizes[jj] > 0:
            raise ValueError(f"Warning: no uniform Pixelsize in the high resolution data with sizes {sizes[i]} and "
                             f"{sizes[jj]}. Aborting computations.")
    j = sizes.index(max(sizes[C0:]))
    if sizes[j] > 0 and sizes[jj] > 0:
        p = sizes[j] / sizes[jj]
        if abs(p - given) > 0.001 and given > 0:
            raise ValueError(f"Warning: the Pixelratio given as input ({given}) does not coincide with the pixel ratio "
                             f"obtained in the data({p}). Aborting computations.")
        return p
    if given > 0:
        return given
    raise ValueError("Warning: no suitable information concerning Pixelsize was given in input or in data. Aborting "
                     "computations.")


def coarse_section(levels_lo, levels_hi, p, refnew_y, refold_y, ny1, rounding):
    """Coarse slices covering fine slices [levels_lo, levels_hi]: the fine slice index
    mapped through the common centre, y1 = (y0 - refnew_y)/p + refold_y, clipped to
    [0, ny1-1]; the whole section uses floor/ceil (:619-621), each chunk round (:715-717)."""
    lo_f, hi_f = (math.floor, math.ceil) if rounding == "cover" else (round, round)
    z_ = int(np.clip(lo_f(1 / p * (levels_lo - refnew_y) + refold_y), 0, ny1 - 1))
    zu = int(np.clip(hi_f(1 / p * (levels_hi - refnew_y) + refold_y), 0, ny1 - 1))
    return z_, zu


def subs_bad_projections(names, C0, badprojections, find_bad, device=0, apply_found=False):
    """Per-resolution lists of projections to drop in the two-resolution driver:
    ``badprojections[r]`` (r = 0 fine, 1 coarse), plus, with ``apply_found``, what
    ``--Find_Bad_Projections`` finds in the first channel of that resolution."""
    out = [list(b) for b in badprojections]
    if find_bad[0] not in (0, 0.0):
        if apply_found:
            from . import badproj
            for r, first in ((0, names[0]), (1, names[C0])):
                out[r].extend(badproj.find_bad_projections(first, find_bad[1], find_bad[0], device=device))
        else:
            eprint("Warning: bad projections found by --Find_Bad_Projections are not applied in the subsampling "
                   "reconstruction (--Apply_Found_Projections applies them).")
    return out


def reconstruct_subs(names, C0, result, mu, alpha, maxiter, method, levels, datahandling, badprojections, find_bad,
                     channelnames, regularisation, discrepancy, pixelratio, overlay, chunksize, scalepars, device=0,
                     apply_found=False):
    """Joint reconstruction from fine (``names[:C0]``) and coarse (``names[C0:]``)
    projection data (Coupled_Reconstruction3dbigresu, Reconstruction_coupled.py:542-873).

    Per resolution its own data handling (``datahandling[k][r]``, r = 0 fine, 1 coarse)
    and bad projections; the coarse/fine pixel ratio from the data or ``--Pixelratio``;
    the fine slices ``levels`` and the coarse slices that cover them; slice chunks with
    overlap, each reconstructed by the drop-in ``Reconstructionapproach3dsubsmapling``
    (CUDA); per-channel rescaling by the data/sinogram ratio; MRC outputs (fine
    reconstruction of every channel, fine sinograms, and for the coarse channels the
    coarse ``_sinogram_smallresu.mrc`` and fine-grid ``_sinogram.mrc`` projections).

    As in the reference, bad projections found by ``--Find_Bad_Projections`` are not
    applied here (the reference appends them as a third, unread entry of the
    per-resolution list), and the coarse channels' fine-grid sinograms are all divided
    by the last coarse channel's factor.  ``apply_found`` (``--Apply_Found_Projections``)
    searches the first channel of each resolution and removes the projections found
    from that resolution's channels."""
    from .radon_tgv_primal_dual_3dsubsample import Reconstructionapproach3dsubsmapling
    brightness, baseline, cutedges, badfile, threshold = datahandling[:5]
    C = len(names)
    C1 = C - C0
    if C0 < 1 or C1 < 1:
        raise ValueError("subsampling needs at least one fine and one coarse channel")
    badprojections = subs_bad_projections(names, C0, badprojections, find_bad, device, apply_found)
    data, angles, noise, sizes = [], [], [], []
    for n in names:
        r = int(n in names[C0:])
        d, a, avg = preprocess.load_channel(n, brightness[r], badfile[r], float(cutedges[r]), badprojections[r])
        data.append(d)
        angles.append(np.asarray(a, np.float64) + np.pi / 2)
        noise.append(avg)
        sizes.append(preprocess.pixel_size(n))
    _, ny0, nx0 = data[0].shape
    _, ny1, nx1 = data[C0].shape
    p = pixel_ratio(sizes, C0, pixelratio)
    refnew = [(nx0 - 1) / 2.0, (ny0 - 1) / 2.0]
    refold = [(nx1 - 1) / 2.0, (ny1 - 1) / 2.0]
    section0 = list(range(levels[0], levels[1] + 1, levels[2]))
    if min(section0) < 0 or max(section0) >= ny0:
        raise IndexError(f"Slice levels are not in a suitable scope. Must lie between 0 and Ny={ny0 - 1}. "
                         "Aborting operation!")
    z_, zu = coarse_section(min(section0), max(section0), p, refnew[1], refold[1], ny1, "cover")
    section1 = list(range(z_, zu + 1))
    print("Computing the Sinogram_levels:", section0)
    print("Corresponds in the Lowresolution Sinograms to ", section1)
    if zu < 1 or z_ > ny1:
        eprint("!!!!!!!!!!! Warning: Section in lowresolution can not cover corresponding Section in High-resolution "
               "data!!!!!!")
    ratio = []
    for i in range(C):  # ratio before the percentile scaling (:636-643)
        sec = section1 if i >= C0 else section0
        d = data[i]
        ratio.append(np.sum(d[:, sec] / len(angles[i])))
        d = d - np.percentile(d, scalepars[0])
        data[i] = d / np.percentile(d, scalepars[1])
    coll = []
    for i in range(C):  # baseline per resolution (:646-664), then the slice selection (:666-669)
        r = int(i >= C0)
        s = _baseline(data[i], baseline[r], float(threshold[r]), noise[i], True)
        coll.append(s[:, section1 if r else section0, :])
    nd, nang0 = coll[0].shape[2], coll[0].shape[0]
    nang1, nd1 = coll[C0].shape[0], coll[C0].shape[2]
    possible = len(section0) if chunksize < 1 else min(len(section0), chunksize)
    U = np.zeros([C, nx0, nx0, len(section0)])
    new_sino = np.zeros([C0, nang0, len(section0), nd], np.float32)
    new_sino_small = np.zeros([C1, nang1, len(section1), nd1], np.float32)
    new_sino_high = np.zeros([C1, nang1, len(section0), nd], np.float32)
    remaining = section0[:]
    t0 = time.time()
    while remaining:
        if overlay > possible / 4.0:
            overlay = int(possible / 4)
            eprint(f"Overlap is too large for possible split size, reducing overlap to {overlay} which is a fourth "
                   "of the possible splits.")
        current = remaining[:min(possible, len(remaining))]
        sp, ep = section0.index(current[0]), section0.index(current[-1])
        cz_, czu = coarse_section(min(current), max(current), p, refnew[1], refold[1], ny1, "round")
        sec1 = list(range(cz_, czu + 1))
        a = possible - 2 * overlay if possible < len(remaining) else len(remaining)
        ov_s = 0 if len(remaining) == len(section0) else overlay
        ov_e = len(current) - len(remaining) if possible >= len(remaining) else overlay
        sps, eps = section1.index(sec1[0]), section1.index(sec1[-1])
        cur = [coll[i][:, sp:ep + 1, :] for i in range(C0)] + [coll[i][:, sps:eps + 1, :] for i in range(C0, C)]
        topology = [C0, p, [refold[0], refold[1] - cz_], [refnew[0], refnew[1] - min(current)]]
        info = [sp / float(len(section0)), len(current) / float(len(section0)), current]
        try:
            u_loc, s_loc = Reconstructionapproach3dsubsmapling(cur, angles, topology, (alpha[0], alpha[1]), mu,
                                                               maxiter, device, [0, 0.1], levels[2], discrepancy,
                                                               method, regularisation, info)
        except GraptorMemoryError:
            possible = int(possible * 0.7)
            eprint(f"Warning: Computation requires too much memory, the problem is split, trying to compute "
                   f"{possible} slices at once.")
            if possible < 1:
                raise MemoryError("Even a single slice requires too much memory.")
            continue
        except GraptorError as err:
            possible = int(possible * 0.7)
            eprint(f"An exception of type {type(err).__name__} occurred. Arguments:\n{err.args!r}")
            if possible < 1:
                raise
            continue
        remaining = remaining[a:]
        U[:, :, :, sp + ov_s:ep + 1 - ov_e] = u_loc[:, :, :, ov_s:len(current) - ov_e]
        new_sino[:, :, sp + ov_s:ep + 1 - ov_e, :] = s_loc[0][:, :, ov_s:len(current) - ov_e, :]
        new_sino_high[:, :, sp + ov_s:ep + 1 - ov_e, :] = s_loc[1][:, :, ov_s:len(current) - ov_e, :]
        new_sino_small[:, :, sps:eps + 1, :] = s_loc[2]
    nz = len(section0)
    sol = np.zeros([C, nz, nx0, nx0], np.float32)
    for i in range(nz):
        sol[:, i] = U[:, :, :, i]
    ns, nsh, nss = new_sino.copy(), new_sino_high.copy(), new_sino_small.copy()
    for i in range(C0):
        fak = np.sum(ns[i]) / ratio[i]
        sol[i] /= fak / len(angles[i])
        ns[i] /= fak / len(angles[i])
    for i in range(C1):
        fak = np.sum(nss[i]) / ratio[i + C0]
        sol[i + C0] /= fak / len(angles[i + C0])
        nss[i] /= fak / len(angles[i + C0])
        nsh /= fak / len(angles[i + C0])
    for i in range(C):
        mrc.write_mrc(f"{result}_{channelnames[i]}.mrc", sol[i])
    for i in range(C1):
        mrc.write_mrc(f"{result}_{channelnames[i + C0]}_sinogram_smallresu.mrc", nss[i])
        mrc.write_mrc(f"{result}_{channelnames[i + C0]}_sinogram.mrc", nsh[i])
    for i in range(C0):
        mrc.write_mrc(f"{result}_{channelnames[i]}_sinogram.mrc", ns[i])
    coll_u = np.zeros([nz, nx0, C * nx0], np.float32)
    coll_n = np.zeros([nz, nx0, C * nx0], np.float32)
    for j in range(C):
        coll_u[:, :, j * nx0:(j + 1) * nx0] = np.transpose(U[j], (2, 0, 1))
        coll_n[:, :, j * nx0:(j + 1) * nx0] = sol[j] / np.max(sol[j])
    mrc.write_mrc(f"{result}_all_channels.mrc", coll_u)
    mrc.write_mrc(f"{result}_all_channels_normalized.mrc", coll_n)
    print("\nTime required for reconstruction:", int(10.0 * (time.time() - t0)) / 10.0, " seconds.\n")
    return U


def build_parser():
    p = argparse.ArgumentParser(prog="python -m graptor_gb300.cli",
                                description="Multi-channel TV/TGV tomographic reconstruction (CUDA), with the options "
                                            "of Reconstruction_coupled.py.")
    p.add_argument("Infiles", type=str, nargs="+")
    p.add_argument("--Infiles_Smallresolution", default=[], type=str, nargs="+")
    p.add_argument("-o", "--Outfile", default="reconstruction")
    p.add_argument("--SliceLevels", type=int, default=[0], nargs="+")
    p.add_argument("-m", "--Maxiter", type=int, default=2000)
    p.add_argument("--Regularisation", default="TGV", type=str)
    p.add_argument("--Coupling", type=str, default="")
    p.add_argument("--Discrepancy", default="KL", type=str)
    p.add_argument("--mu", type=float, default=[], nargs="+")
    p.add_argument("--alpha", type=float, default=[4, 1.0], nargs="+")
    p.add_argument("--Plot", nargs="+", default=[0])
    p.add_argument("--Pixelratio", type=float, nargs="+", default=[-1])
    p.add_argument("--Datahandling", nargs="+", default=["bright", "thresholding", "0.0", "", "0.05"])
    p.add_argument("--GPU_Choice", type=int, default=-1)
    p.add_argument("--Channelnames", default=[], type=str, nargs="+")
    p.add_argument("--Badprojections", default=[], type=int, nargs="+")
    p.add_argument("--Datahandling2", nargs="+", default=["bright", "thresholding", "0.0", "", "0.05"])
    p.add_argument("--Badprojections2", default=[], type=int, nargs="+")
    p.add_argument("--Find_Bad_Projections", nargs="+", default=[], type=float)
    p.add_argument("--Apply_Found_Projections", action="store_true",
                   help="remove the projections --Find_Bad_Projections finds (the reference reports them only)")
    p.add_argument("--Overlapping", default=1, type=int)
    p.add_argument("--Chunksize", default=-1, type=int)
    p.add_argument("--Scalepars", default=[1, 98], type=int, nargs="+")
    return p


def main(argv=None):
    args = build_parser().parse_args(argv)
    outdir = os.path.split(args.Outfile)[0]
    print("Output will be written to " + outdir)
    if outdir and not os.path.exists(outdir):
        os.makedirs(outdir)
    find_bad = list(args.Find_Bad_Projections) or [0]
    while len(find_bad) < 2:
        find_bad.append(None)
    reg = args.Regularisation.upper()
    if reg not in ("TGV", "TV"):
        eprint(f"Regularisation {reg} not recognised, changed to TGV")
        reg = "TGV"
    alpha = list(args.alpha)
    if len(alpha) == 1:
        alpha.append(1.0)
        eprint(f'Warning: not sufficiently many regularization parameters "alpha" are given, setting second entry '
               f"to one resulting in {alpha}.")
    alpha = alpha[:2]
    method, setting = parse_method(args.Coupling)
    if setting == 2 and not args.Infiles_Smallresolution:
        eprint("Warning !!!! Only one type of data is given, changing method to 'Frobenius 3D Reconstruction'.")
        method, setting = "Frobenius 3D Reconstruction", 1
    names = resolve_names(list(args.Infiles))
    C0 = len(names)
    if setting == 2:  # the coarse channels follow the fine ones (:1005-1009)
        names = names + resolve_names(list(args.Infiles_Smallresolution))
    disc = args.Discrepancy.upper()
    if disc not in ("KL", "L2"):
        eprint("Warning!!!!!! Discrepancy input not understood, set to KL (Kullback-Leibler). Possible choices are "
               "KL or L2.")
        disc = "KL"
    dh = list(args.Datahandling)
    defaults = ["bright", "thresholding", "0.000001", "", "0.05"]
    dh = (dh + defaults[len(dh):])[:5]
    dh2 = list(args.Datahandling2)
    dh2 = (dh2 + dh[len(dh2):])[:5]
    mu = list(np.ones(len(names)))
    for i in range(min(len(args.mu), len(names))):
        mu[i] = args.mu[i]
    chn = [f"Channel{i}" for i in range(len(names))]
    for i in range(min(len(args.Channelnames), len(names))):
        chn[i] = args.Channelnames[i]
    levels = list(args.SliceLevels)
    if len(levels) == 1:
        levels.append(levels[0])
    if len(levels) == 2:
        levels.append(1)
    if (levels[1] + 1 - levels[0]) * levels[2] <= 0:
        raise ValueError("Slice instructions are not usable, as entries are non consistent (start needs to be smaller "
                         "or equal than end and step size needs to be larger or equal to 1). Aborting operation!")
    device = max(args.GPU_Choice, 0)
    cfg = f"{args.Outfile}{method}_{mu}{alpha}_{args.Maxiter}Layer{levels}"
    with open(cfg + ".config", "w") as fh:
        fh.write(" " + str(args) + "\n")
    pr = list(args.Pixelratio)
    pr = pr[0] if len(pr) == 1 else pr[0] / pr[1]
    if setting == 2:
        handling = [[dh[k], dh2[k]] for k in range(5)]
        u = reconstruct_subs(names, C0, args.Outfile, mu, alpha, args.Maxiter, method, levels, handling,
                             [list(args.Badprojections), list(args.Badprojections2)], find_bad, chn, reg, disc, pr,
                             args.Overlapping, args.Chunksize, args.Scalepars, device, args.Apply_Found_Projections)
    elif setting == 1:
        u = reconstruct_3d(names, args.Outfile, mu, alpha, args.Maxiter, method, levels, dh, args.Badprojections,
                           find_bad, chn, reg, disc, args.Overlapping, args.Chunksize, args.Scalepars, device,
                           args.Apply_Found_Projections)
    else:
        u = reconstruct_2d(names, args.Outfile, mu, alpha, args.Maxiter, method, levels, dh, args.Badprojections,
                           find_bad, chn, reg, disc, args.Scalepars, device, args.Apply_Found_Projections)
    print("\nAlgorithm completed, results are written in " + outdir + ".")
    return u


if __name__ == "__main__":
    main()
