"""FP64 primal-dual gap (no counterpart in the reference's loop; its draft energy
code is radon_tgv_primal_dual_3d.py:882-927): the device gap of a state equals
the FP64 NumPy evaluation (oracle/fp64.py) of the same state, and it decreases
toward zero as the iteration converges."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # dim, N, Nz, C, nang, disc, reg, coupling
    (3, 24, 4, 2, 20, "KL", "TGV", "FROB"),
    (3, 20, 3, 3, 16, "L2", "TGV", "UNCORR"),
    (3, 20, 4, 2, 18, "KL", "TV", "FROB"),
    (2, 28, 3, 2, 20, "L2", "TGV", "FROB"),
    (2, 24, 2, 1, 18, "KL", "TGV", "UNCORR"),
    (3, 16, 3, 3, 12, "L2", "TGV", "NUCL"),
]


def _problem(case, iters):
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    from oracle import oracle as O
    dim, N, Nz, C, nang, disc, reg, cpl = case
    rng = np.random.default_rng(7)
    ang = phantom.angles_deg(nang)
    ofs = O.radon_struct(ang, N, N)
    img = np.abs(rng.standard_normal((C * Nz, N, N))).astype(np.float32)
    f = phantom.poisson(O.radon(img, ofs, N), 300.0, 2)
    mu = rng.uniform(0.1, 0.5, C)
    p = Problem(dim, N, Nz, C, N, ang, (4.0, 1.0), mu, disc, reg, cpl, 1.0, 15.0)
    p.set_data(f).run(iters).synchronize()
    return p, ang, mu


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(map(str, c)))
def test_gap_matches_fp64_evaluation_of_same_state(case):
    from oracle import fp64 as F
    dim, N, Nz, C, nang, disc, reg, cpl = case
    p, ang, mu = _problem(case, 150)
    g = p.gap()
    st = {k: p.get(k).astype(np.float64) for k in ("u", "v", "lambda", "data")}
    st["p"] = p.get("p").astype(np.float64) if reg == "TGV" else np.zeros((dim, C * Nz, N, N))
    st["w"] = p.get("w").astype(np.float64) if reg == "TGV" else np.zeros((6 if dim == 3 else 3, C * Nz, N, N))
    p.close()
    o = F.Solver64(dim, N, Nz, C, N, ang, st["data"], (4.0, 1.0), mu, 15.0, disc, reg, cpl, feasible=False)
    e = o.energies(st["u"], st["p"], st["v"], st["w"], st["lambda"], U=g["U"])
    assert abs(g["primal"] - e["primal"]) <= 1e-5 * abs(e["primal"]), (g, e)
    assert abs(g["dual"] - e["dual"]) <= 1e-5 * abs(e["primal"]), (g, e)
    assert abs(g["theta"] - e["theta"]) <= 1e-6
    assert abs(g["relative"] - e["relative"]) <= 1e-4 * max(1.0, abs(e["relative"]))


def test_gap_decreases_and_weak_duality():
    p, _, _ = _problem((3, 24, 4, 2, 20, "KL", "TGV", "FROB"), 20)
    rel = []
    for _ in range(5):
        p.run(400).synchronize()
        g = p.gap()
        assert g["primal"] >= g["dual"] - 1e-12 * abs(g["primal"])  # weak duality on the box
        rel.append(g["relative"])
    p.close()
    assert rel[-1] < 0.5 * rel[0], rel


# Nuclear coupling is left out: the reference's 3-D nuclear projection can return
# NaN and its 2-D one is chaotic under rounding, both reproduced bit for bit by the
# device (against the reference's own kernels); an FP64 restatement cannot follow them.
FP64_CASES = [
    (3, 24, 4, 2, 20, "KL", "TGV", "FROB"),
    (2, 32, 2, 1, 24, "L2", "TGV", "UNCORR"),
    (3, 20, 3, 2, 16, "KL", "TV", "FROB"),
    (3, 16, 3, 3, 12, "L2", "TGV", "UNCORR"),
]


@pytest.mark.parametrize("case", FP64_CASES, ids=lambda c: "-".join(map(str, c)))
def test_iterates_match_fp64_oracle_of_the_same_iteration(case):
    """The FP32 device iteration against the FP64 NumPy restatement of the same
    iteration (oracle/fp64.py, exact hat weights, double precision throughout)
    after 300 iterations: relative L2 error of u, v and lambda <= 1e-4."""
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    from oracle import fp64 as F
    from oracle import oracle as O
    dim, N, Nz, C, nang, disc, reg, cpl = case
    rng = np.random.default_rng(17)
    ang = phantom.angles_deg(nang)
    ofs = O.radon_struct(ang, N, N)
    img = np.abs(rng.standard_normal((C * Nz, N, N))).astype(np.float32)
    f = phantom.poisson(O.radon(img, ofs, N), 300.0, 3)
    mu = rng.uniform(0.1, 0.5, C)
    iters = 300
    with Problem(dim, N, Nz, C, N, ang, (4.0, 1.0), mu, disc, reg, cpl, 1.0, 15.0) as p:
        p.set_data(f, feasible=False).run(iters).synchronize()
        got = {k: p.get(k).astype(np.float64) for k in ("u", "v", "lambda")}
    o = F.Solver64(dim, N, Nz, C, N, ang, f, (4.0, 1.0), mu, 15.0, disc, reg, cpl, feasible=False).run(iters)
    want = {"u": o.u, "v": o.v, "lambda": o.lam}
    errs = {k: float(np.linalg.norm(got[k] - want[k]) / np.linalg.norm(want[k])) for k in got}
    print(case, {k: f"{v:.2e}" for k, v in errs.items()})
    for k, e in errs.items():
        assert e <= 1e-4, (k, errs)
