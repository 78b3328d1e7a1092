"""Generate the golden fixtures by running the REFERENCE's own code.

Run in a checkout that has the reference available (``GRAPTOR_REFERENCE``):

    python tests/golden/make_golden.py

Every output comes from the reference itself, executed on the CPU through the
oracle harness (oracle/refshim): the reference's OpenCL C kernels translated to
C++ and its Python host code (``Reconstructionapproach2d/3d``) run unmodified.
Inputs are seeded synthetic phantoms (graptor_gb300/phantom.py) and seeded
random fields; nothing is copied from the reference's example data.

Fixtures (NumPy .npz, float32 unless noted):
  projectors.npz   radon / radon_ad on random slices for several geometries,
                   with the reference's angle table
  kernels_2d.npz   one call of every 2-D dual/primal kernel on random inputs
  kernels_3d.npz   one call of every 3-D dual/primal kernel on random inputs
  solve_*.npz      full solver runs: inputs, the normest the run used, and the
                   reference's returned (Solution, Sinogram) at several counts
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "refshim"))
sys.path.insert(0, ROOT)

import reference as R  # noqa: E402
from graptor_gb300 import phantom  # noqa: E402

F32 = np.float32


def fbuf(shape):
    """Zeroed float32 buffer in the reference's F-ordered device layout."""
    return np.zeros(shape, F32, order="F")


class KernelRunner:
    """Call single reference kernels through the stand-in pyopencl."""

    def __init__(self, which):
        import pyopencl as cl
        self.cl = cl
        self.prg = R.program(which)
        self.q = cl.CommandQueue(cl.Context())

    def __call__(self, name, gsize, *args):
        from pyopencl.array import _Data
        conv = []
        for a in args:
            conv.append(_Data(a) if isinstance(a, np.ndarray) and a.ndim > 0 else a)
        getattr(self.prg, name)(self.q, gsize, None, *conv)


# ------------------------------------------------------------------ projectors
def geometry_cases():
    deg = np.pi / 180.0
    return [
        # name, N(=image side), nd, angles (solver convention, radians)
        ("tilt15", 17, 17, phantom.angles_deg(15)),
        ("edges", 16, 16, np.array([0.0, 90.0, 180.0, 45.0, 135.0, -45.0, 89.99, 90.01, 30.0]) * deg),
        ("wide_det", 12, 19, phantom.angles_deg(7, -80, 80)),
        ("one_angle", 9, 9, np.array([0.3])),
    ]


def make_projectors(out):
    rng = np.random.default_rng(11)
    kr = KernelRunner("3d")
    d = {}
    for name, N, nd, ang in geometry_cases():
        S = 3
        # angle table exactly as radon_struct builds it (:947-979)
        X = np.cos(ang); Y = np.sin(ang); Xinv = 1.0 / X
        mask = np.abs(Xinv) > 10 * nd
        X[mask] = 0; Y[mask] = np.sin(ang[mask]).round(); Xinv[mask] = 0
        off = (nd - 1.0) / 2.0 - X * (N - 1) / 2.0 - Y * (N - 1) / 2.0
        ofs = np.zeros((4, ang.size), F32, order="F")
        ofs[0], ofs[1], ofs[2], ofs[3] = X, Y, off, Xinv
        img = rng.standard_normal((S, N, N)).astype(F32)  # [s, y, x]
        img_dev = fbuf((N, N, S)); img_dev[...] = np.transpose(img, (2, 1, 0))
        sino_dev = fbuf((nd, ang.size, S))
        kr("radon", (nd, ang.size, S), sino_dev, img_dev, ofs, np.int32(N), np.int32(N))
        lam = rng.standard_normal((S, ang.size, nd)).astype(F32)
        lam_dev = fbuf((nd, ang.size, S)); lam_dev[...] = np.transpose(lam, (2, 1, 0))
        bp_dev = fbuf((N, N, S))
        kr("radon_ad", (N, N, S), bp_dev, lam_dev, ofs, np.int32(nd), np.int32(ang.size))
        d[f"{name}/angles"] = ang
        d[f"{name}/N"] = np.int32(N)
        d[f"{name}/nd"] = np.int32(nd)
        d[f"{name}/ofs"] = np.ascontiguousarray(ofs.T)
        d[f"{name}/img"] = img
        d[f"{name}/sino"] = np.transpose(sino_dev, (2, 1, 0)).copy()
        d[f"{name}/lam"] = lam
        d[f"{name}/bp"] = np.transpose(bp_dev, (2, 1, 0)).copy()
    np.savez_compressed(out, **d)


# ------------------------------------------------------------------ per-kernel fixtures
def _vec_dev(a, width):
    """oracle SoA [K, S, y, x] -> reference AoS (width, x, y, S) F-order."""
    K, S, Ny, Nx = a.shape
    dev = fbuf((width, Nx, Ny, S))
    dev[:K] = np.transpose(a, (0, 3, 2, 1))
    return dev


def _vec_host(dev, K):
    return np.ascontiguousarray(np.transpose(dev[:K], (0, 3, 2, 1)))


def _sc_dev(a):
    dev = fbuf(a.shape[::-1]); dev[...] = np.transpose(a, tuple(range(a.ndim))[::-1]); return dev


def _sc_host(dev):
    return np.ascontiguousarray(np.transpose(dev, tuple(range(dev.ndim))[::-1]))


def make_kernels(out, dim):
    rng = np.random.default_rng(20 + dim)
    kr = KernelRunner(f"{dim}d")
    N, Nz, C, nd, nang = (10, 4, 3, 10, 6) if dim == 3 else (12, 1, 3, 12, 7)
    S = Nz * C
    K, KW = (3, 6) if dim == 3 else (2, 3)
    VW, WW = (4, 8) if dim == 3 else (2, 4)  # AoS widths (float3 padded to 4 / float8; float2 / float3->4)
    r = lambda *sh: rng.standard_normal(sh).astype(F32)  # noqa: E731
    d = {"N": np.int32(N), "Nz": np.int32(Nz), "C": np.int32(C), "nd": np.int32(nd), "nang": np.int32(nang)}
    sigma, tau, step = F32(0.24), F32(0.23), F32(2.0 if dim == 3 else 1.0)
    d.update(sigma=sigma, tau=tau, stepsize=step)
    u, ubar, p, pbar, v, w = r(S, N, N), r(S, N, N), r(K, S, N, N), r(K, S, N, N), r(K, S, N, N), r(KW, S, N, N)
    d.update(u=u, ubar=ubar, p=p, pbar=pbar, v=v, w=w)
    g3 = (N, N, S)
    ex = (F32(sigma), F32(1.0), F32(step), F32(C)) if dim == 3 else (F32(sigma), F32(1.0))
    # update_v
    vd = _vec_dev(v, VW)
    kr("update_v", g3, vd, _sc_dev(ubar), _vec_dev(pbar, VW), *ex)
    d["out/update_v"] = _vec_host(vd, K)
    # update_w
    wd = _vec_dev(w, WW)
    kr("update_w", g3, wd, _vec_dev(pbar, VW), *ex)
    d["out/update_w"] = _vec_host(wd, KW)
    # ball projections (scaled so that some points project and some do not)
    ainv = F32(0.8)
    for meth in ("frob", "unchor", "Nucl"):
        vd = _vec_dev(v, VW); nv = fbuf((N, N, Nz))
        gs = (N, N, Nz) if meth != "unchor" else g3
        kr(f"update_NormV_{meth}", gs, vd, nv, ainv, F32(C))
        d[f"out/normv_{meth}"] = _vec_host(vd, K)
        if meth == "Nucl":
            continue
        wd = _vec_dev(w, WW); nw = fbuf((N, N, Nz))
        kr(f"update_NormW_{meth}", gs, wd, nw, ainv, F32(C))
        d[f"out/normw_{meth}"] = _vec_host(wd, KW)
    d["alphainv"] = ainv
    # data prox
    lam, ku, f = r(S, nang, nd), r(S, nang, nd), np.abs(r(S, nang, nd))
    mu = np.abs(r(C)) + F32(0.1)
    d.update(lam=lam, ku=ku, f=f, mu=mu)
    for disc in ("KL", "L2"):
        ld = _sc_dev(lam)
        args = (ld, _sc_dev(ku), _sc_dev(f), F32(0.05), mu.copy())
        if dim == 3:
            args = args + (F32(C),)
        kr(f"update_lambda_{disc}", (nd, nang, S), *args)
        d[f"out/lambda_{disc}"] = _sc_host(ld)
    # update_u
    kstar = r(S, N, N)
    d["kstar"] = kstar
    ud = fbuf(g3)
    ex_u = (F32(tau), F32(0.125), F32(step), F32(C)) if dim == 3 else (F32(tau), F32(0.125))
    kr("update_u", g3, ud, _sc_dev(u), _vec_dev(v, VW), _sc_dev(kstar), *ex_u)
    d["out/update_u"] = _sc_host(ud)
    # update_p
    pd = fbuf((VW, N, N, S))
    ex_p = (F32(tau), F32(step), F32(C)) if dim == 3 else (F32(tau),)
    kr("update_p", g3, pd, _vec_dev(p, VW), _vec_dev(v, VW), _vec_dev(w, WW), *ex_p)
    d["out/update_p"] = _vec_host(pd, K)
    np.savez_compressed(out, **d)


# ------------------------------------------------------------------ full solver runs
def sino_2d(N, nang, seed, peak):
    from oracle import oracle as O
    img = phantom.ellipses_2d(N, 10, seed)
    ang = phantom.angles_deg(nang)
    ofs = O.radon_struct(ang, N, N)
    g = O.radon(img[None], ofs, N)[0]  # [nang, nd]
    return phantom.poisson(g, peak, seed), ang


def sino_3d(N, Nz, C, nang, seed, peaks):
    from oracle import oracle as O
    vol = phantom.ellipsoids_3d(N, Nz, C, 8, seed)  # [c, z, y, x]
    ang = phantom.angles_deg(nang)
    ofs = O.radon_struct(ang, N, N)
    out = []
    for c in range(C):
        g = O.radon(vol[c], ofs, N)  # [z, nang, nd]
        out.append(np.transpose(phantom.poisson(g, peaks[c], seed + c), (1, 0, 2)).copy())  # [nang, Nz, nd]
    return out, ang


def make_solve_2d(out, N, nang, C, method, reg, disc, iters, seed, mu, peak=1e3):
    sinos, ang = [], None
    for c in range(C):
        s, ang = sino_2d(N, nang, seed + 31 * c, peak)
        sinos.append(s)
    d = {"sino": np.stack(sinos), "angles": ang, "alpha": np.array([4.0, 1.0]), "mu": np.array(mu, np.float64),
         "method": method, "regularisation": reg, "discrepancy": disc, "iters": np.array(iters, np.int32)}
    for it in iters:
        u, s, ne, _ = R.run_2d(sinos, ang, (4.0, 1.0), mu, it, disc, method, reg, seed=seed)
        d[f"u/{it}"] = u.astype(F32)
        d[f"sinogram/{it}"] = s.astype(F32)
        d["normest"] = np.float64(ne)
    np.savez_compressed(out, **d)


def make_solve_3d(out, N, Nz, C, nang, method, reg, disc, iters, seed, mu, stepsize=1, peaks=None):
    peaks = peaks or [1e4] + [20.0] * (C - 1)
    sinos, ang = sino_3d(N, Nz, C, nang, seed, peaks)
    d = {"sino": np.stack(sinos), "angles": ang, "alpha": np.array([4.0, 1.0]), "mu": np.array(mu, np.float64),
         "method": method, "regularisation": reg, "discrepancy": disc, "iters": np.array(iters, np.int32),
         "stepsize": np.int32(stepsize)}
    for it in iters:
        u, s, ne, _ = R.run_3d(sinos, ang, (4.0, 1.0), mu, it, stepsize, disc, method, reg, seed=seed)
        d[f"u/{it}"] = u.astype(F32)
        d[f"sinogram/{it}"] = s.astype(F32)
        d["normest"] = np.float64(ne)
    np.savez_compressed(out, **d)


def main():
    if not R.available():
        raise SystemExit("reference checkout not found; set GRAPTOR_REFERENCE")
    j = lambda n: os.path.join(HERE, n)  # noqa: E731
    make_projectors(j("projectors.npz"))
    make_kernels(j("kernels_2d.npz"), 2)
    make_kernels(j("kernels_3d.npz"), 3)
    # 2-D single-channel TGV-KL at the full 2-D workload size and count (128^2, 60 angles, 500 it)
    make_solve_2d(j("solve_2d_tgv_kl_128.npz"), 128, 60, 1, "Uncorrelated 2D Reconstruction", "TGV", "KL",
                  [1, 10, 100, 500], seed=1, mu=[0.2])
    make_solve_2d(j("solve_2d_frob_tgv_l2.npz"), 40, 24, 2, "Frobenius 2D Reconstruction", "TGV", "L2",
                  [1, 50], seed=2, mu=[0.2, 0.05])
    make_solve_2d(j("solve_2d_nucl_tv_kl.npz"), 40, 24, 2, "Nuclear 2D Reconstruction", "TV", "KL",
                  [1, 50], seed=3, mu=[0.2, 0.05])
    # 3-D coupled 4-channel FROB3D-KL with the workload's 71 angles and mu, reduced volume
    make_solve_3d(j("solve_3d_frob_tgv_kl.npz"), 48, 6, 4, 71, "Frobenius 3D Reconstruction", "TGV", "KL",
                  [1, 10, 200, 2500], seed=4, mu=[0.2, 5e-4, 4e-3, 5e-4])
    make_solve_3d(j("solve_3d_uncorr_tv_l2.npz"), 24, 5, 2, 20, "Uncorrelated 3D Reconstruction", "TV", "L2",
                  [1, 40], seed=5, mu=[0.2, 0.1], stepsize=2)
    make_solve_3d(j("solve_3d_nucl_tgv_l2.npz"), 24, 5, 3, 20, "Nuclear 3D Reconstruction", "TGV", "L2",
                  [1, 40], seed=6, mu=[0.2, 0.1, 0.05])


if __name__ == "__main__":
    main()
