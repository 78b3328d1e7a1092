"""GPU parity at full geometries: the CUDA path against the CPU oracle
(oracle/tgv_oracle.c, which reproduces the reference's own kernels bit for bit)
on the benchmarked problem itself and on the detector / angle geometry of the
large 768-bin run.

* 3-D coupled 4-channel FROB3D TGV-KL, 256x256 x 60 slices, 256 bins x 71 angles
  in [-70, 70] degrees (the workload bench.py times), 10 iterations;
* 768x768 pixels, 768 bins x 141 angles, 2 slices x 2 channels (the in-plane
  geometry of the 768x768x384x4 run), 5 iterations.

Bar: relative L2 <= 1e-5 on u, lambda and K ubar after those iterations (the
reference kernels are radon_tgv_primal_dual_3d.py:773-844; the loop :1194-1221).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0))


def _compare(N, Nz, C, nang, mu, peaks, iters, seed, parity_report, case):
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    from oracle import oracle as O
    vol = phantom.ellipsoids_3d(N, Nz, C, 12, seed)  # [c, z, y, x]
    ang = phantom.angles_deg(nang)
    ofs = O.radon_struct(ang, N, N)
    clean = O.radon(vol.reshape(C * Nz, N, N), ofs, N).reshape(C, Nz, nang, N)
    f = np.concatenate([phantom.poisson(clean[c], peaks[c], seed + c) for c in range(C)])  # [S, nang, nd]
    with Problem(3, N, Nz, C, N, ang, (4.0, 1.0), mu, "KL", "TGV", "FROB") as p:
        p.set_data(f).run(iters).synchronize()
        ne = p.scalars["normest"]
        got = {k: p.get(k) for k in ("u", "lambda", "ku")}
    ref = O.Solver(3, N, Nz, C, N, ofs, f, (4.0, 1.0), mu, ne, O.KL, O.TGV, O.FROB).run(iters)
    want = {"u": ref.u, "lambda": ref.lam, "ku": ref.ku}
    errs = {k: rel(got[k], want[k]) for k in got}
    parity_report({"case": case, "iterations": iters, **errs})
    for k, e in errs.items():
        assert np.isfinite(got[k]).all(), k
        assert e <= TOL, f"{case} {k}: {e:.3e} > {TOL:.0e}"


def test_benched_problem_matches_oracle(parity_report):
    # the bench workload: 256^2 x 60 x 4 channels, 71 angles, mu of the coupled data set
    _compare(256, 60, 4, 71, [0.2, 5e-4, 4e-3, 5e-4], [1e4, 20.0, 20.0, 20.0], 10, 0, parity_report,
             "3d_frob_tgv_kl_256x256x60x4_71ang")


def test_large_detector_geometry_matches_oracle(parity_report):
    # 768 bins x 141 angles on a 768^2 image: the geometry of the 768^2 x 384 x 4 run
    _compare(768, 2, 2, 141, [0.2, 4e-3], [1e4, 20.0], 5, 3, parity_report, "3d_frob_tgv_kl_768x768x2x2_141ang")
