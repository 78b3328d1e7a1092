"""Two-resolution subsampling (gt_subs_*, graptor_gb300/radon_tgv_primal_dual_3dsubsample.py)
against the reference's own solver run on the same inputs (tests/golden/solve_subs_*.npz,
made by tests/golden/make_subs_golden.py through the oracle harness).  The
reference's operator-norm estimate (random start) is injected; results after 1 and
30 iterations must agree within 1e-4 relative L2 (after one iteration, to rounding)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = ["frob_tgv_kl", "uncorr_tgv_l2", "frob_tv_kl"]
META = {"frob_tgv_kl": ("KL", "TGV", "Frobenius 3D Subsampling Reconstruction"),
        "uncorr_tgv_l2": ("L2", "TGV", "Uncorrelated 3D Subsampling Reconstruction"),
        "frob_tv_kl": ("KL", "TV", "Frobenius 3D Subsampling Reconstruction")}


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0))


@pytest.mark.parametrize("name", CASES)
def test_subsampling_matches_reference(golden, name, parity_report):
    from graptor_gb300.radon_tgv_primal_dual_3dsubsample import Reconstructionapproach3dsubsmapling
    g = golden(f"solve_subs_{name}.npz")
    C0, C1 = int(g["C0"]), int(g["C1"])
    sino = [g[f"sino_{k}"] for k in range(C0 + C1)]
    angles = [g["angles0"]] * C0 + [g["angles1"]] * C1
    topo = [C0, float(g["p"]), list(g["refold"]), list(g["refnew"])]
    disc, reg, method = META[name]
    for iters, tol in ((1, 1e-6), (30, 1e-4)):
        u, sinos = Reconstructionapproach3dsubsmapling(sino, angles, topo, tuple(g["alpha"]), g["mu"], iters, 0,
                                                       [0, 0.1], int(g["stepsize"]), disc, method, reg, [0, 1, [0]],
                                                       normest=float(g[f"normest_{iters}"]))
        errs = {"u": rel(u, g[f"u_{iters}"]), "ku0": rel(sinos[0], g[f"ku0_{iters}"]),
                "ku1": rel(sinos[1], g[f"ku1_{iters}"]), "kulo": rel(sinos[2], g[f"kulo_{iters}"])}
        parity_report({"case": f"subsampling {name}", "iterations": iters, **errs})
        assert u.shape == g[f"u_{iters}"].shape
        for k, e in errs.items():
            assert e <= tol, (name, iters, k, e)


def test_subsampling_own_normest_is_close_to_the_reference_estimate(golden):
    from graptor_gb300.radon_tgv_primal_dual_3dsubsample import Subsampling
    g = golden("solve_subs_frob_tgv_kl.npz")
    C0, C1 = int(g["C0"]), int(g["C1"])
    N, Nz, N1, Nz1 = int(g["N"]), int(g["Nz"]), int(g["N1"]), int(g["Nz1"])
    f0 = np.transpose(g["sino_0"], (1, 0, 2)).reshape(C0 * Nz, -1, N)
    f1 = np.transpose(g["sino_1"], (1, 0, 2)).reshape(C1 * Nz1, -1, N1)
    with Subsampling(N, Nz, C0, C1, N1, Nz1, g["angles0"], g["angles1"], (4, 1), g["mu"], float(g["p"]),
                     g["refold"], g["refnew"]) as s:
        s.set_data(f0, f1)
        ne = s.normest
    # the reference's 25 FP32 rounds from a random image against 30 rounds from ones
    assert abs(ne - float(g["normest_30"])) / float(g["normest_30"]) < 1e-3, (ne, float(g["normest_30"]))
