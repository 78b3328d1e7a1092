"""Golden fixtures of the two-resolution subsampling method, from the REFERENCE's
own code (radon_tgv_primal_dual_3dsubsample.py) run through the oracle harness
(oracle/refshim, see ``reference.run_subs``).

    python tests/golden/make_subs_golden.py

Inputs are seeded synthetic phantoms: the fine channels are projections of a
seeded ellipsoid volume on the fine detector, the coarse channel the projection
of the same object on a grid coarser by the pixel ratio, with Poisson noise.
Output: tests/golden/solve_subs_*.npz (inputs, the normest the run used, the
reference's Solution and sinograms after 1 and 30 iterations).
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
from oracle import oracle as O  # noqa: E402


def project(vol, ang, nd):
    """[S, N, N] -> [S, nang, nd] with the CPU oracle's projector (bit-exact with the reference)."""
    S, N, _ = vol.shape
    ofs = O.radon_struct(ang, N, nd)
    return O.radon(vol.astype(np.float32), ofs, nd)


CASES = {
    "frob_tgv_kl": dict(N=16, Nz=6, C0=1, C1=1, nang0=11, nang1=7, p=2.0, stepsize=1, disc="KL", reg="TGV",
                        method="Frobenius 3D Subsampling Reconstruction", mu=[0.3, 0.2]),
    "uncorr_tgv_l2": dict(N=20, Nz=4, C0=2, C1=1, nang0=9, nang1=8, p=2.0, stepsize=1, disc="L2", reg="TGV",
                          method="Uncorrelated 3D Subsampling Reconstruction", mu=[0.5, 0.4, 0.2]),
    "frob_tv_kl": dict(N=16, Nz=8, C0=1, C1=2, nang0=10, nang1=6, p=2.0, stepsize=2, disc="KL", reg="TV",
                       method="Frobenius 3D Subsampling Reconstruction", mu=[0.3, 0.1, 0.2]),
}


def make(name, c, seed):
    N, Nz, C0, C1 = c["N"], c["Nz"], c["C0"], c["C1"]
    p = c["p"]
    N1, Nz1 = int(N / p), max(1, int(Nz / p))
    vol = phantom.ellipsoids_3d(N, Nz, C0 + C1, 6, seed)  # [c, z, y, x]
    ang0 = phantom.angles_deg(c["nang0"])
    ang1 = phantom.angles_deg(c["nang1"], -60, 60)
    sino = []
    for ch in range(C0):
        g = project(vol[ch], ang0, N)  # [Nz, nang, nd]
        sino.append(np.transpose(phantom.poisson(g, 200.0, seed + ch), (1, 0, 2)).astype(np.float32))
    for ch in range(C0, C0 + C1):
        # the coarse object: 2x2(x z) block averages of the fine one (p = 2), projected on the coarse grid
        v = vol[ch]
        vz = v[: Nz1 * int(p)].reshape(Nz1, int(p), N, N).mean(1)
        vc = vz.reshape(Nz1, N1, int(p), N1, int(p)).mean((2, 4))
        g = project(vc, ang1, N1)
        sino.append(np.transpose(phantom.poisson(g, 200.0, seed + ch), (1, 0, 2)).astype(np.float32))
    angles = [ang0] * C0 + [ang1] * C1
    topo = [C0, p, [(N1 - 1) / 2.0, (Nz1 - 1) / 2.0], [(N - 1) / 2.0, (Nz - 1) / 2.0]]
    out = {"sino_" + str(k): s for k, s in enumerate(sino)}
    out.update(angles0=ang0, angles1=ang1, C0=C0, C1=C1, p=p, stepsize=c["stepsize"], N=N, Nz=Nz, N1=N1, Nz1=Nz1,
               refold=np.array(topo[2]), refnew=np.array(topo[3]), mu=np.array(c["mu"]),
               alpha=np.array([4.0, 1.0]))
    for iters in (1, 30):
        u, sinos, ne = R.run_subs(sino, angles, topo, (4.0, 1.0), c["mu"], iters, c["stepsize"], c["disc"],
                                  c["method"], c["reg"], seed=seed)
        out[f"u_{iters}"] = u.astype(np.float32)
        out[f"ku0_{iters}"], out[f"ku1_{iters}"], out[f"kulo_{iters}"] = sinos
        out[f"normest_{iters}"] = np.array(ne)
    np.savez_compressed(os.path.join(HERE, f"solve_subs_{name}.npz"), **out)
    print(name, {k: v.shape for k, v in out.items() if hasattr(v, "shape") and v.ndim > 1}, "normest", ne)


if __name__ == "__main__":
    O.build()
    for k, (name, c) in enumerate(CASES.items()):
        make(name, c, 100 + k)
