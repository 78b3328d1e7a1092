"""Pin the CPU oracle to the reference: every fixture under tests/golden/ was
produced by the reference's own code (tests/golden/make_golden.py), and the
oracle must reproduce each one bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden.make_golden import geometry_cases  # noqa: F401  (documents the cases)


def test_projectors_bitexact(golden):
    g = golden("projectors.npz")
    names = sorted({k.split("/")[0] for k in g})
    assert names
    for n in names:
        N, nd = int(g[f"{n}/N"]), int(g[f"{n}/nd"])
        ofs = O.radon_struct(g[f"{n}/angles"], N, nd)
        np.testing.assert_array_equal(ofs, g[f"{n}/ofs"], err_msg=n)
        np.testing.assert_array_equal(O.radon(g[f"{n}/img"], ofs, nd), g[f"{n}/sino"], err_msg=n)
        np.testing.assert_array_equal(O.radon_ad(g[f"{n}/lam"], ofs, N), g[f"{n}/bp"], err_msg=n)


@pytest.mark.parametrize("dim", [2, 3])
def test_kernels_bitexact(golden, dim):
    import ctypes
    g = golden(f"kernels_{dim}d.npz")
    N, Nz, C, nd, nang = (int(g[k]) for k in ("N", "Nz", "C", "nd", "nang"))
    lib = O.lib()
    P = O._p

    def desc(coupling=O.FROB, disc=O.KL):
        return O.Desc(dim, N, Nz, C, nd, nang, disc, O.TGV, coupling, float(g["stepsize"]))

    d = desc()
    sig, tau = ctypes.c_float(g["sigma"]), ctypes.c_float(g["tau"])
    v = g["v"].copy(); lib.or_update_v(ctypes.byref(d), P(v), P(g["ubar"]), P(g["pbar"]), sig)
    np.testing.assert_array_equal(v, g["out/update_v"])
    w = g["w"].copy(); lib.or_update_w(ctypes.byref(d), P(w), P(g["pbar"]), sig)
    np.testing.assert_array_equal(w, g["out/update_w"])
    ainv = ctypes.c_float(g["alphainv"])
    for meth, cpl in (("frob", O.FROB), ("unchor", O.UNCORR), ("Nucl", O.NUCL)):
        dd = desc(cpl)
        v = g["v"].copy(); lib.or_norm_v(ctypes.byref(dd), P(v), ainv)
        np.testing.assert_array_equal(v, g[f"out/normv_{meth}"], err_msg=meth)
        if meth != "Nucl":
            w = g["w"].copy(); lib.or_norm_w(ctypes.byref(dd), P(w), ainv)
            np.testing.assert_array_equal(w, g[f"out/normw_{meth}"], err_msg=meth)
    for disc, dc in (("KL", O.KL), ("L2", O.L2)):
        dd = desc(disc=dc)
        lam = g["lam"].copy()
        lib.or_update_lambda(ctypes.byref(dd), P(lam), P(g["ku"]), P(g["f"]), ctypes.c_float(0.05), P(g["mu"]))
        np.testing.assert_array_equal(lam, g[f"out/lambda_{disc}"], err_msg=disc)
    un = np.zeros_like(g["u"])
    lib.or_update_u(ctypes.byref(d), P(un), P(g["u"]), P(g["v"]), P(g["kstar"]), tau, ctypes.c_float(0.125))
    np.testing.assert_array_equal(un, g["out/update_u"])
    pn = np.zeros_like(g["p"])
    lib.or_update_p(ctypes.byref(d), P(pn), P(g["p"]), P(g["v"]), P(g["w"]), tau)
    np.testing.assert_array_equal(pn, g["out/update_p"])


SOLVES = ["solve_2d_tgv_kl_128.npz", "solve_2d_frob_tgv_l2.npz", "solve_2d_nucl_tv_kl.npz",
          "solve_3d_frob_tgv_kl.npz", "solve_3d_uncorr_tv_l2.npz", "solve_3d_nucl_tgv_l2.npz"]


def run_oracle(g, iters):
    sino = [s for s in g["sino"]]
    args = (sino, g["angles"], tuple(g["alpha"]), g["mu"], iters)
    kw = (str(g["discrepancy"]), str(g["method"]), str(g["regularisation"]), float(g["normest"]))
    if "stepsize" in g:
        return O.reconstruct_3d(*args, int(g["stepsize"]), *kw)
    return O.reconstruct_2d(*args, *kw)


@pytest.mark.parametrize("name", SOLVES)
def test_solver_bitexact(golden, name):
    g = golden(name)
    iters = [int(i) for i in g["iters"]]
    for it in iters:
        if it > 500 and "3d" in name:
            continue  # the 2500-iteration 3-D case runs in test_solver_bitexact_long
        u, s = run_oracle(g, it)
        np.testing.assert_array_equal(u.astype(np.float32), g[f"u/{it}"], err_msg=f"{name} u@{it}")
        np.testing.assert_array_equal(np.asarray(s, np.float32), g[f"sinogram/{it}"], err_msg=f"{name} sino@{it}")


@pytest.mark.slow
def test_solver_bitexact_long(golden):
    g = golden("solve_3d_frob_tgv_kl.npz")
    u, s = run_oracle(g, 2500)
    np.testing.assert_array_equal(u.astype(np.float32), g["u/2500"])
