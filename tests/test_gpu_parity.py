"""GPU parity: the CUDA path (through the C ABI) against the reference's own
outputs (tests/golden, produced by the reference code) and against the CPU oracle.

Bars: the standalone projectors reproduce the reference bit for bit (same FP32
operation order); full solves match within the 1e-4 relative L2 the
specification sets (inside the solver the projector sums use fused multiply-add
and the coupled ball projections evaluate the norm as sqrt of a sum of squares
where the reference nests hypot, so they differ in the last bits).
"""
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4  # relative L2 after the stated iteration count


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def to_dev(torch, host_sx):
    """host [S, X...] -> device layout [X, S] (slice fastest)."""
    a = np.ascontiguousarray(host_sx, np.float32)
    S = a.shape[0]
    return torch.from_numpy(a.reshape(S, -1).T.copy()).cuda()


def from_dev(t, shape):
    S = shape[0]
    return t.cpu().numpy().T.reshape(shape)


def test_projectors_bitexact(golden, torch_cuda):
    from graptor_gb300 import solver
    torch = torch_cuda
    g = golden("projectors.npz")
    for n in sorted({k.split("/")[0] for k in g}):
        N, nd, ang = int(g[f"{n}/N"]), int(g[f"{n}/nd"]), g[f"{n}/angles"]
        img, lam = g[f"{n}/img"], g[f"{n}/lam"]
        S = img.shape[0]
        d_img, d_lam = to_dev(torch, img), to_dev(torch, lam)
        d_sino = torch.zeros(ang.size * nd, S, device="cuda")
        d_bp = torch.zeros(N * N, S, device="cuda")
        solver.radon(d_img.data_ptr(), d_sino.data_ptr(), ang, N, nd, S)
        solver.radon_ad(d_lam.data_ptr(), d_bp.data_ptr(), ang, N, nd, S)
        np.testing.assert_array_equal(from_dev(d_sino, (S, ang.size, nd)), g[f"{n}/sino"], err_msg=n)
        np.testing.assert_array_equal(from_dev(d_bp, (S, N, N)), g[f"{n}/bp"], err_msg=n)


def test_projector_adjointness(torch_cuda):
    from graptor_gb300 import phantom, solver
    torch = torch_cuda
    rng = np.random.default_rng(5)
    N, S = 96, 40
    ang = phantom.angles_deg(45)
    x = rng.standard_normal((S, N, N)).astype(np.float32)
    y = rng.standard_normal((S, ang.size, N)).astype(np.float32)
    dx, dy = to_dev(torch, x), to_dev(torch, y)
    Rx = torch.zeros(ang.size * N, S, device="cuda")
    Rty = torch.zeros(N * N, S, device="cuda")
    solver.radon(dx.data_ptr(), Rx.data_ptr(), ang, N, N, S)
    solver.radon_ad(dy.data_ptr(), Rty.data_ptr(), ang, N, N, S)
    a = float((Rx.double() * dy.double()).sum())
    b = float((dx.double() * Rty.double()).sum())
    assert abs(a - b) / abs(a) < 1e-5


SOLVES = ["solve_2d_tgv_kl_128.npz", "solve_2d_frob_tgv_l2.npz", "solve_2d_nucl_tv_kl.npz",
          "solve_3d_frob_tgv_kl.npz", "solve_3d_uncorr_tv_l2.npz", "solve_3d_nucl_tgv_l2.npz"]


def oracle_sensitivity(g, it):
    """How far the REFERENCE's own result moves when the data change by one ulp.

    The 2-D nuclear projection (radon_tgv_primal_dual_2d.py:124-204) switches
    between an eigen-decomposition and a diagonal shortcut on a threshold, and
    its eigenvector formulas cancel catastrophically; iterated, last-bit
    differences grow (1 ulp of data -> ~1e-2 after 50 iterations).  The oracle
    reproduces the reference bit for bit, so it measures that growth."""
    from oracle import oracle as O
    sino = [s for s in g["sino"]]
    pert = [np.nextafter(s, np.float32(np.inf)) if k == 0 else s for k, s in enumerate(sino)]
    args = (g["angles"], tuple(g["alpha"]), g["mu"], it, str(g["discrepancy"]), str(g["method"]),
            str(g["regularisation"]), float(g["normest"]))
    a = O.reconstruct_2d(sino, *args)[0]
    b = O.reconstruct_2d(pert, *args)[0]
    return rel(b, a)


@pytest.mark.parametrize("name", SOLVES)
def test_solver_matches_reference_outputs(golden, name, parity_report):
    """Reference-produced Solution and Sinogram at every stored iteration count."""
    from graptor_gb300 import radon_tgv_primal_dual_2d as r2
    from graptor_gb300 import radon_tgv_primal_dual_3d as r3
    r3.progress = False
    g = golden(name)
    sino = [s for s in g["sino"]]
    kw = dict(normest=float(g["normest"]))
    for it in [int(i) for i in g["iters"]]:
        if "stepsize" in g:
            u, s = r3.Reconstructionapproach3d(sino, g["angles"], tuple(g["alpha"]), g["mu"], it, 0, [0, 0.1],
                                               int(g["stepsize"]), str(g["discrepancy"]), str(g["method"]),
                                               str(g["regularisation"]), [0, 1, [0]], **kw)
        else:
            u, s = r2.Reconstructionapproach2d(sino, g["angles"], tuple(g["alpha"]), g["mu"], it, 0, [0, 0.1],
                                               str(g["discrepancy"]), str(g["method"]), str(g["regularisation"]),
                                               [0, 1, 0], **kw)
            s = np.stack(s)
        ref_u, ref_s = g[f"u/{it}"], g[f"sinogram/{it}"]
        assert u.shape == ref_u.shape and u.dtype == np.float64
        if np.isnan(ref_u).any():
            pytest.fail(f"{name}: reference output has NaN at {it}")
        eu, es = rel(u, ref_u), rel(s, ref_s)
        parity_report({"case": name, "iterations": it, "u": eu, "sinogram": es})
        if str(g["method"]).startswith("Nuclear 2D"):
            # chaotic under rounding: the first step agrees to rounding, later steps
            # stay within the reference's own one-ulp sensitivity
            if it == 1:
                assert eu <= 1e-6 and es <= 1e-6, (eu, es)
            else:
                bound = max(TOL, 4.0 * oracle_sensitivity(g, it))
                parity_report({"case": name, "iterations": it, "reference_1ulp_sensitivity": bound / 4})
                assert eu <= bound, f"{name} u@{it}: {eu:.3e} > {bound:.3e}"
            continue
        assert eu <= TOL, f"{name} u@{it}: {eu:.3e}"
        assert es <= TOL, f"{name} sinogram@{it}: {es:.3e}"


CASES = [
    # dim, N, Nz, C, nang, disc, reg, coupling, stepsize
    (3, 40, 6, 4, 30, "KL", "TGV", "FROB", 1.0),
    (3, 33, 5, 3, 17, "L2", "TGV", "UNCORR", 2.0),
    (3, 24, 4, 2, 20, "KL", "TV", "FROB", 1.0),
    (3, 20, 3, 10, 12, "L2", "TGV", "UNCORR", 1.0),   # more than 8 uncoupled channels
    (3, 24, 4, 5, 16, "L2", "TGV", "FROB", 1.0),      # 5 channels: the 8-wide register path
    (2, 48, 7, 3, 25, "KL", "TGV", "FROB", 1.0),      # batched independent 2-D slices
    (2, 37, 1, 1, 29, "L2", "TV", "UNCORR", 1.0),
    (2, 30, 3, 2, 19, "KL", "TGV", "NUCL", 1.0),
    (3, 20, 4, 3, 15, "L2", "TGV", "NUCL", 1.0),
    (3, 1, 1, 1, 3, "KL", "TGV", "FROB", 1.0),        # 1x1 image
    (3, 16, 1, 2, 1, "L2", "TGV", "FROB", 1.0),       # one slice, one angle
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(map(str, c)))
def test_solver_matches_oracle(case, parity_report):
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    from oracle import oracle as O
    dim, N, Nz, C, nang, disc, reg, cpl, step = case
    rng = np.random.default_rng(zlib.crc32(repr(case).encode()))
    ang = phantom.angles_deg(nang, -75, 75)
    ofs = O.radon_struct(ang, N, N)
    img = np.abs(rng.standard_normal((C * Nz, N, N))).astype(np.float32)
    f = phantom.poisson(O.radon(img, ofs, N), 200.0, 1) + 0.01
    mu = rng.uniform(0.05, 0.5, C)
    ne = 17.0
    iters = 25
    with Problem(dim, N, Nz, C, N, ang, (3.0, 1.5), mu, disc, reg, cpl, step, ne) as p:
        p.set_data(f).run(iters).synchronize()
        u, ku, lam, v = p.get("u"), p.get("ku"), p.get("lambda"), p.get("v")
        ubar = p.get("ubar")
    def oracle(fdata, n):
        return O.Solver(dim, N, Nz, C, N, ofs, fdata, (3.0, 1.5), mu, ne, O.KL if disc == "KL" else O.L2,
                        O.TGV if reg == "TGV" else O.TV, {"UNCORR": O.UNCORR, "FROB": O.FROB, "NUCL": O.NUCL}[cpl],
                        stepsize=step).run(n)
    o = oracle(f, iters)
    o2 = oracle(np.nextafter(f, np.float32(np.inf)), iters) if (dim == 2 and cpl == "NUCL") else None
    for name, a, b in (("u", u, o.u), ("ubar", ubar, o.ubar), ("ku", ku, o.ku), ("lambda", lam, o.lam),
                       ("v", v, o.v)):
        e = rel(a, b)
        bound = 1e-5
        if o2 is not None:  # chaotic method: the reference's own one-ulp sensitivity, see oracle_sensitivity
            bound = max(bound, 4.0 * rel(getattr(o2, {"lambda": "lam"}.get(name, name)), b))
        parity_report({"case": "oracle:" + "-".join(map(str, case)), "iterations": iters, name: e, "bound": bound})
        assert e <= bound, f"{case} {name}: {e:.3e} > {bound:.1e}"


def test_state_roundtrip_and_warm_start():
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    rng = np.random.default_rng(3)
    N, Nz, C, nang = 24, 3, 2, 10
    ang = phantom.angles_deg(nang)
    f = np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32)
    with Problem(3, N, Nz, C, N, ang, (4, 1), [0.2, 0.1], normest=15.0) as p:
        p.set_data(f).run(7).synchronize()
        snap = {k: p.get(k) for k in ("u", "ubar", "p", "pbar", "v", "w", "lambda")}
        p.run(5).synchronize()
        after = p.get("u")
        p.set_data(f)  # resets
        for k, a in snap.items():
            p.set(k, a)
        np.testing.assert_array_equal(p.get("w"), snap["w"])
        p.run(5).synchronize()
        np.testing.assert_array_equal(p.get("u"), after)
        assert p.scalars["normest"] == 15.0


@pytest.mark.parametrize("S_case", [(40, 3, 2, 21, 40), (36, 16, 1, 17, 36), (41, 4, 2, 19, 41), (38, 2, 2, 23, 45),
                                    (27, 8, 1, 13, 22), (9, 4, 1, 31, 2)],
                         ids=["S6", "S16", "S8odd", "S4nd45", "S8nd22", "S4nd2"])
def test_projector_launch_shapes_give_identical_iterates(S_case):
    """Every forward / back projection launch shape the autotuner can pick sums the
    same terms in the same order, so the iterates agree bit for bit; this includes
    the register-blocked row-tile back projector (18, 19), whose zero-weight
    pairings leave every sum unchanged."""
    from graptor_gb300 import _lib as L
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    N, Nz, C, nang, nd = S_case
    rng = np.random.default_rng(zlib.crc32(repr(S_case).encode()))
    ang = phantom.angles_deg(nang, -85, 95)
    f = np.abs(rng.standard_normal((C * Nz, nang, nd))).astype(np.float32)
    ref = None
    with Problem(3, N, Nz, C, nd, ang, (4, 1), [0.2] * C, normest=17.0) as p:
        p.set_data(f)
        nf = L.lib().gt_set_tuning(p._h, 99, 0)
        assert nf != 0  # out of range is refused
        configs = [(fc, 0) for fc in range(20)] + [(0, bc) for bc in range(1, 20)] if (C * Nz) % 4 == 0 else [(0, 0)]
        for fc, bc in configs:
            p.set_data(f)
            try:
                p.set_tuning(fc, bc)
            except ValueError:
                continue  # configuration not offered for this slice count
            p.run(6).synchronize()
            got = {k: p.get(k) for k in ("u", "ku", "lambda", "v")}
            if ref is None:
                ref = got
                continue
            for k in got:
                np.testing.assert_array_equal(got[k], ref[k], err_msg=f"fwd {fc} bp {bc} field {k}")


@pytest.mark.parametrize("stepsize", [2.0, 1.0])
@pytest.mark.parametrize("dim,C,cpl,reg", [(3, 1, "FROB", "TGV"), (3, 2, "FROB", "TGV"), (3, 3, "UNCORR", "TGV"),
                                           (3, 4, "FROB", "TGV"), (3, 3, "FROB", "TGV"), (3, 2, "NUCL", "TGV"),
                                           (3, 4, "FROB", "TV"), (2, 4, "FROB", "TGV"), (2, 2, "NUCL", "TGV")])
def test_dual_launch_shapes_give_identical_iterates(dim, C, cpl, reg, stepsize):
    """The two-slice float2 dual kernel, the register-capped one and the kernels that
    load every operand before the arithmetic compute every value with the same
    operations as the one-slice kernel: identical iterates (step size 1: shape 9
    leaves out the divisions by it, x / 1 = x)."""
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    N, Nz, nang = 28, 6, 15
    rng = np.random.default_rng(40 + C)
    ang = phantom.angles_deg(nang)
    f = np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32)
    got = []
    z2 = dim == 3 and reg == "TGV" and cpl != "NUCL"
    if cpl == "NUCL":
        shapes = (0, 2, 3, 4, 5)
    elif dim == 2:
        shapes = (0, 2, 3, 4, 5, 6, 8)
    else:
        shapes = (0, 1, 2, 3, 4, 5, 6, 7, 8, 9) if z2 else (0, 2, 3, 4, 5, 6, 7, 8, 9)
    fields = ("u", "ubar", "v", "w", "p", "pbar", "lambda") if reg == "TGV" else ("u", "ubar", "v", "lambda")
    with Problem(dim, N, Nz, C, N, ang, (4, 1), [0.3] * C, regularisation=reg, coupling=cpl, normest=17.0,
                 stepsize=stepsize) as p:
        for shape in shapes:
            # the primal update as one launch after the projectors (schedule 0), as its
            # p / pbar half beside them (schedule 1) or inside the next dual kernel
            # (schedule 2, where it applies): the same values
            last = ((0, 1, 2) if z2 else (0, 1))
            for schedule in (last if shape == shapes[-1] else (1,)):
                p.set_schedule(schedule)
                p.set_data(f)
                p.set_dual_shape(shape)
                p.run(9).synchronize()
                got.append({k: p.get(k) for k in fields})
        if not z2:
            with pytest.raises(ValueError):
                p.set_schedule(2)
        with pytest.raises(ValueError):
            p.set_schedule(3)
        with pytest.raises(ValueError):
            p.set_dual_shape(10)
        if not z2:
            with pytest.raises(ValueError):
                p.set_dual_shape(1)
        if cpl == "NUCL":
            for sh in (6, 8):
                with pytest.raises(ValueError):
                    p.set_dual_shape(sh)
        if cpl == "NUCL" or dim == 2:
            for sh in (7, 9):
                with pytest.raises(ValueError):
                    p.set_dual_shape(sh)
    for g in got[1:]:
        for k in got[0]:
            np.testing.assert_array_equal(g[k], got[0][k], err_msg=k)
    with Problem(3, N, 5, C, N, ang, (4, 1), [0.3] * C, normest=17.0) as q:  # odd Nz: no two-slice shapes
        with pytest.raises(ValueError):
            q.set_dual_shape(1)
        if C <= 4:
            for sh in (7, 9):
                with pytest.raises(ValueError):
                    q.set_dual_shape(sh)


@pytest.mark.parametrize("C,cpl,Nz", [(1, "FROB", 8), (2, "UNCORR", 6), (4, "FROB", 10), (3, "FROB", 4)])
def test_fused_schedule_gives_the_iterates_of_plain_iterations(C, cpl, Nz):
    """Schedule 2 (the p / pbar half of each primal update computed inside the next
    dual kernel, p / v / w alternating between two buffer sets) over runs that end
    inside and across a 32-iteration graph chunk, and split into several gt_run
    calls: every field equals that of plain iterations (schedule 0) bit for bit,
    and the fused kernel's own timing leaves the state unchanged."""
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    N, nang = 36, 17
    rng = np.random.default_rng(60 + C)
    ang = phantom.angles_deg(nang)
    f = np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32)
    fields = ("u", "ubar", "v", "w", "p", "pbar", "lambda", "ku")
    with Problem(3, N, Nz, C, N, ang, (4, 1), [0.3] * C, coupling=cpl, normest=17.0, stepsize=1.5) as p:
        ref = {}
        p.set_schedule(0)
        p.set_data(f)
        for n in (3, 9, 45, 70):  # cumulative 3, 12, 57, 127 iterations
            p.run(n).synchronize()
            ref[n] = {k: p.get(k) for k in fields}
        p.set_schedule(2)
        assert p.tuning["schedule"] == 2
        p.set_data(f)
        for n in (3, 9, 45, 70):
            p.run(n).synchronize()
            for k in fields:
                np.testing.assert_array_equal(p.get(k), ref[n][k], err_msg=f"{k} after run({n})")
        before = {k: p.get(k) for k in fields}
        t = p.time_kernels(reps=1)
        assert t.get("k_dual_fused", 0) > 0, t
        # time_kernels advanced the state by one plain iteration; the fused timing
        # itself wrote only the second buffer set: one more plain iteration from
        # `before` gives the same state
        after = {k: p.get(k) for k in fields}
        p.set_schedule(0)
        p.set_data(f)
        p.run(3 + 9 + 45 + 70 + 1).synchronize()
        for k in fields:
            np.testing.assert_array_equal(after[k], p.get(k), err_msg=k)
        assert any(not np.array_equal(before[k], after[k]) for k in fields)


def test_float64_outputs_are_the_reordered_state():
    """gt_get_output_f64 (the drop-in entry point's return values, converted and
    reordered on the device) equals the float32 state reordered on the host:
    Solution [C, x, y, z] and Sinogram [C, nang, Nz, nd], value for value; other
    fields and 2-D problems are refused."""
    from graptor_gb300 import _lib as L
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    N, Nz, C, nang, nd = 20, 3, 2, 11, 23
    rng = np.random.default_rng(77)
    ang = phantom.angles_deg(nang)
    f = np.abs(rng.standard_normal((C * Nz, nang, nd))).astype(np.float32)
    with Problem(3, N, Nz, C, nd, ang, (4, 1), [0.3] * C, normest=17.0) as p:
        p.set_data(f).run(7).synchronize()
        u = p.get("u").reshape(C, Nz, N, N)
        ku = p.get("ku").reshape(C, Nz, nang, nd)
        np.testing.assert_array_equal(p.output_f64("u"), np.transpose(u, (0, 3, 2, 1)).astype(np.float64))
        np.testing.assert_array_equal(p.output_f64("ku"), np.transpose(ku, (0, 2, 1, 3)).astype(np.float64))
        out = np.empty(8)
        assert L.lib().gt_get_output_f64(p._h, L.FIELDS["v"], out.ctypes.data) == L.GT_ERR_ARG
    with Problem(2, N, 1, C, nd, ang, (4, 1), [0.3] * C, normest=17.0) as q:
        with pytest.raises(ValueError):
            q.output_f64("u")


@pytest.mark.parametrize("disc", ["KL", "L2"])
def test_dual_from_primal_is_a_fixed_point(disc):
    """lambda from gt_dual_from_primal equals the fixed point of the lambda update
    for K u (KL: mu (1 - f / K u), kept where f > 10 K u; L2: mu (K u - f)),
    checked in float64 on the host."""
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    rng = np.random.default_rng(5 if disc == "KL" else 6)
    N, Nz, C, nang = 24, 4, 2, 13
    ang = phantom.angles_deg(nang)
    f = np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32)
    mu = np.array([0.2, 0.05])
    with Problem(3, N, Nz, C, N, ang, (4, 1), mu, discrepancy=disc, normest=17.0) as p:
        p.set_data(f).run(30).synchronize()
        lam0 = p.get("lambda")
        p.dual_from_primal().synchronize()
        ku, lam, u = p.get("ku").astype(np.float64), p.get("lambda").astype(np.float64), p.get("u")
        fd = p.get("data").astype(np.float64)
        m = np.repeat(mu, Nz)[:, None, None]
        if disc == "KL":
            pos = (ku > 0) & (fd <= 10 * ku)
            expect = np.where(pos, m * (1 - fd / np.where(ku > 0, ku, 1)), lam0)
        else:
            expect = m * (ku - fd)
        assert rel(lam, expect) < 1e-6
        # ku is the projection of the current u
        assert np.abs(u).sum() > 0


def test_dual_reset_repairs_missed_rays():
    """With repair, an image that misses rays carrying data (K u = 0 < f) is
    lifted along them first: afterwards K u > 0 wherever f > 0, so the KL primal
    value (and the gap) is finite, and lambda is finite."""
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    rng = np.random.default_rng(77)
    N, Nz, C, nang = 24, 4, 2, 13
    ang = phantom.angles_deg(nang)
    f = np.zeros((C * Nz, nang, N), np.float32)
    f[:, :, 8:14] = np.abs(rng.standard_normal((C * Nz, nang, 6))).astype(np.float32) + 0.1
    with Problem(3, N, Nz, C, N, ang, (4, 1), [0.2, 0.05], normest=17.0) as p:
        p.set_data(f, feasible=False)
        zero = np.zeros((C * Nz, N, N), np.float32)
        p.set("u", zero)
        p.set("ubar", zero)
        p.dual_from_primal(repair=True).synchronize()
        ku, fd, u, lam = p.get("ku"), p.get("data"), p.get("u"), p.get("lambda")
        assert (ku[fd > 0] > 0).all()
        assert np.isfinite(lam).all() and (u >= 0).all() and u.max() > 0
        assert np.array_equal(p.get("ubar"), u)
        assert np.isfinite(p.gap()["primal"])


def test_fp64_normest_matches_reference_estimate(golden):
    """The FP64 power iteration agrees with the reference's FP32 estimate."""
    from graptor_gb300.solver import Problem
    for name in ("solve_2d_tgv_kl_128.npz", "solve_3d_frob_tgv_kl.npz"):
        g = golden(name)
        sino = g["sino"]
        C = sino.shape[0]
        if sino.ndim == 3:
            nang, nd = sino.shape[1:]
            p = Problem(2, nd, 1, C, nd, g["angles"], (4, 1), g["mu"])
            p.set_data(sino)
        else:
            nang, Nz, nd = sino.shape[1:]
            p = Problem(3, nd, Nz, C, nd, g["angles"], (4, 1), g["mu"])
            p.set_data(np.transpose(sino, (0, 2, 1, 3)).reshape(C * Nz, nang, nd))
        ne = p.scalars["normest"]
        p.close()
        assert abs(ne - float(g["normest"])) / float(g["normest"]) < 1e-4, (name, ne, float(g["normest"]))


def test_batch_matches_individual_problems():
    """A batch of uneven problems (sizes, channels, angle sets, KL/L2, 2-D/3-D)
    gives each member the result it gets when solved alone."""
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Batch, Problem
    rng = np.random.default_rng(11)
    specs, datas = [], []
    for k, (dim, N, Nz, C, nang, disc) in enumerate([(3, 24, 5, 2, 20, "KL"), (3, 17, 3, 1, 13, "L2"),
                                                     (2, 30, 4, 3, 25, "KL"), (3, 20, 6, 4, 30, "L2")]):
        ang = phantom.angles_deg(nang, -75, 75)
        specs.append(dict(dim=dim, N=N, Nz=Nz, C=C, nd=N, angles=ang, alpha=(4.0, 1.0), mu=rng.uniform(0.1, 0.4, C),
                          discrepancy=disc, regularisation="TGV", coupling="FROB", normest=12.0 + k))
        datas.append(np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32))
    with Batch(specs) as b:
        for k in range(len(b)):
            b[k].set_data(datas[k])
        b.run(37).synchronize()
        got = [b[k].get("u") for k in range(len(b))]
    for k, sp in enumerate(specs):
        with Problem(**sp) as p:
            p.set_data(datas[k]).run(37).synchronize()
            np.testing.assert_array_equal(got[k], p.get("u"), err_msg=f"member {k}")
    # members left out of some runs keep their state and resume exactly
    with Batch(specs) as b:
        for k in range(len(b)):
            b[k].set_data(datas[k])
        b.run(20)
        b.set_active(1, False).set_active(3, False)
        b.run(17).synchronize()
        held = [b[k].get("u") for k in (1, 3)]
        b.set_active(1, True).set_active(3, True)
        b.run(17).synchronize()
        out = [b[k].get("u") for k in range(len(b))]
    its = {0: 54, 1: 37, 2: 54, 3: 37}
    for k, sp in enumerate(specs):
        with Problem(**sp) as p:
            p.set_data(datas[k]).run(its[k]).synchronize()
            np.testing.assert_array_equal(out[k], p.get("u"), err_msg=f"member {k} after pause")
            if k in (1, 3):
                p.set_data(datas[k]).run(20).synchronize()
                np.testing.assert_array_equal(held[(k - 1) // 2], p.get("u"), err_msg=f"member {k} paused")


def test_out_of_memory_is_a_memory_error():
    """An allocation the device cannot hold fails cleanly as GraptorMemoryError (the
    reference's pyopencl.MemoryError, which Reconstruction_coupled.py:509-536
    answers by shrinking the slice chunk); the device stays usable."""
    from graptor_gb300 import GraptorMemoryError, phantom
    from graptor_gb300.solver import Problem
    ang = phantom.angles_deg(30)
    with pytest.raises(GraptorMemoryError):
        Problem(3, 4096, 256, 8, 4096, ang, (4, 1), np.ones(8))   # ~18 TB of state
    with Problem(3, 16, 2, 1, 16, ang, (4, 1), [0.2], normest=10.0) as p:  # still usable
        p.set_data(np.ones((2, 30, 16), np.float32)).run(2).synchronize()


@pytest.mark.parametrize("reg,mode", [("TGV", "plain"), ("TV", "plain"), ("TGV", "precise")])
def test_checkpoint_resume_continues_exactly(tmp_path, reg, mode):
    """save() after 20 iterations, load() into a new problem: its next 10 iterations
    equal those of the saved problem, bit for bit (with primal weight 7 and the
    precise primal mode: both restored, the low part of u included)."""
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Problem
    rng = np.random.default_rng(91)
    N, Nz, C, nang = 24, 4, 2, 13
    ang = phantom.angles_deg(nang)
    f = np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32)
    path = str(tmp_path / "ckpt.npz")
    with Problem(3, N, Nz, C, N, ang, (4, 1), [0.2, 0.05], regularisation=reg) as p:
        p.set_data(f)
        if mode == "precise":
            p.set_primal_weight(7.0).set_precise_primal()
        p.run(20)
        p.save(path)
        p.run(10).synchronize()
        want = {k: p.get(k) for k in p._state_fields()}
        if mode == "precise":
            assert "ulo" in want and np.abs(want["ulo"]).max() > 0
        else:
            with pytest.raises(ValueError):
                p.get("ulo")
    with Problem.load(path) as q:
        assert q.iteration_offset == 20
        assert q.precise_primal == (mode == "precise")
        assert q.primal_weight == (7.0 if mode == "precise" else 1.0)
        q.run(10).synchronize()
        for k, v in want.items():
            np.testing.assert_array_equal(q.get(k), v, err_msg=k)


def test_bounded_wait_of_tma_back_projection_reports_timeout():
    """Failure detection without a GPU fault: the TMA back projector is made to wait
    for a copy that is never issued; every block gives up after a short bounded
    wait, flags it and returns, gt_synchronize reports GT_ERR_TIMEOUT, and the
    same problem then runs normally again (the context stays usable)."""
    from graptor_gb300 import _lib as L
    from graptor_gb300 import GraptorTimeoutError, phantom
    from graptor_gb300.solver import Problem
    rng = np.random.default_rng(92)
    N, Nz, C, nang = 32, 64, 2, 11  # S = 128: one box width
    ang = phantom.angles_deg(nang)
    f = np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32)
    with Problem(3, N, Nz, C, N, ang, (4, 1), [0.2, 0.2], normest=15.0, autotune=False) as p:
        p.set_data(f)
        p.set_tuning(0, 14)
        L.check(L.lib().gt_test_bp_stall(p._h, 5, 4096))
        p.run(2)
        with pytest.raises(GraptorTimeoutError):
            p.synchronize()
        p.synchronize()  # the flag was cleared
        L.check(L.lib().gt_test_bp_stall(p._h, -1, 1 << 22))
        p.set_data(f).run(4).synchronize()
        got = p.get("u")
        p.set_tuning(0, 4)
        p.set_data(f).run(4).synchronize()
        np.testing.assert_array_equal(got, p.get("u"))


def test_fused_batch_matches_individual_problems():
    """The fused batch mode (one launch per phase over every member's work
    units) gives each member the result it gets alone: uneven sizes, channel
    counts (S odd, even, a multiple of 4; one, four and eight slices per thread),
    angle sets and KL/L2, members paused
    and resumed.  Mixed couplings are refused."""
    from graptor_gb300 import phantom
    from graptor_gb300.solver import Batch, Problem
    rng = np.random.default_rng(23)
    specs, datas = [], []
    for k, (N, Nz, C, nang, disc) in enumerate([(24, 5, 2, 20, "KL"), (17, 3, 1, 13, "L2"), (30, 4, 3, 25, "KL"),
                                                (20, 6, 4, 30, "L2"), (9, 1, 1, 7, "KL"), (41, 2, 2, 33, "L2"),
                                                (19, 24, 4, 11, "KL"), (13, 50, 4, 9, "L2"), (16, 17, 3, 12, "KL")]):
        ang = phantom.angles_deg(nang, -75, 75)
        specs.append(dict(dim=3, N=N, Nz=Nz, C=C, nd=N, angles=ang, alpha=(4.0, 1.0), mu=rng.uniform(0.1, 0.4, C),
                          discrepancy=disc, regularisation="TGV", coupling="FROB", normest=12.0 + k))
        datas.append(np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32))
    with Batch(specs) as b:
        for k in range(len(b)):
            b[k].set_data(datas[k])
        b.set_mode(1)
        assert b.mode == 1
        b.run(21)
        b.set_active(2, False)
        b.run(9)
        b.set_active(2, True)
        b.run(10).synchronize()
        got = [{f: b[k].get(f) for f in ("u", "lambda", "w")} for k in range(len(b))]
    for k, sp in enumerate(specs):
        with Problem(**sp) as p:
            p.set_data(datas[k]).run(31 if k == 2 else 40).synchronize()
            for f in got[k]:
                np.testing.assert_array_equal(got[k][f], p.get(f), err_msg=f"member {k} field {f}")
    mixed = [dict(specs[0]), dict(specs[1], coupling="UNCORR")]
    with Batch(mixed) as b:
        with pytest.raises(ValueError):
            b.set_mode(1)
        assert b.mode == 0
