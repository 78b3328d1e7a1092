"""CPU tests of the command-line path: MRC / angle-file I/O, preprocessing, the
option handling of the reference CLI, and the bad-projection detector's oracle and
host steps against golden vectors produced by the reference's own find_bad_ele.py
(tests/golden/make_badproj_golden.py)."""
import os

import numpy as np
import pytest

from graptor_gb300 import badproj, cli, mrc, preprocess
from oracle import badproj as obad


def test_mrc_roundtrip_modes(tmp_path):
    rng = np.random.default_rng(1)
    for dt in (np.float32, np.int16, np.uint16, np.int8, np.float16):
        a = (rng.standard_normal((3, 5, 7)) * 20).astype(dt)
        p = str(tmp_path / f"a_{np.dtype(dt).name}.mrc")
        mrc.write_mrc(p, a)
        b = mrc.read_mrc(p)
        assert b.dtype == np.dtype(dt) and np.array_equal(a, b)
    # 2-D input is stored as one section; float64 as float32
    p = str(tmp_path / "two.mrc")
    mrc.write_mrc(p, rng.standard_normal((4, 6)))
    assert mrc.read_mrc(p).shape == (1, 4, 6) and mrc.read_mrc(p).dtype == np.float32


def test_mrc_big_endian_and_extended_header(tmp_path):
    a = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4)
    head = np.zeros(256, ">i4")
    head[0:4] = (4, 3, 2, 2)
    head[23] = 64  # extended header bytes
    b = bytearray(head.tobytes())
    b[208:212] = b"MAP "
    b[212:214] = b"\x11\x11"
    p = str(tmp_path / "be.mrc")
    with open(p, "wb") as fh:
        fh.write(bytes(b) + b"\0" * 64 + a.astype(">f4").tobytes())
    assert np.array_equal(mrc.read_mrc(p), a)


def test_angle_files(tmp_path):
    p = str(tmp_path / "s.mrc")
    mrc.write_mrc(p, np.zeros((3, 2, 4), np.float32))
    with pytest.raises(IOError):
        mrc.read_angles(p)
    with open(p.replace(".mrc", ".csv"), "w") as fh:
        fh.write("-60,a\n0,b\n60,c\n")
    assert np.allclose(mrc.read_angles(p), np.array([-60, 0, 60]) / 180 * np.pi)
    with open(p.replace(".mrc", ".rawtlt"), "w") as fh:
        fh.write("-30\n 0\n30\n")
    assert np.allclose(mrc.read_angles(p), np.array([-30, 0, 30]) / 180 * np.pi)  # rawtlt wins
    d, ang = mrc.read_projections(p)
    assert d.dtype == np.float64 and d.shape == (3, 2, 4) and ang.size == 3


def _stack(tmp_path, data, angles_deg, name="st"):
    p = str(tmp_path / f"{name}.mrc")
    mrc.write_mrc(p, data.astype(np.float32))
    with open(p.replace(".mrc", ".rawtlt"), "w") as fh:
        fh.write("\n".join(str(a) for a in angles_deg))
    return p


def test_brightness_correction_and_rescaling(tmp_path):
    rng = np.random.default_rng(2)
    data = rng.random((6, 5, 20)) + 1.0
    p = _stack(tmp_path, data, np.linspace(-60, 60, 6))
    data = data.astype(np.float32).astype(np.float64)
    bad = [2, 5]  # 1-based
    d, ang, _ = preprocess.brightness_correction(p, "", 0.1, bad)
    keep = [0, 2, 3, 5]
    ref = data[keep]
    cut = 2
    bg = 0.5 * (ref[:, :, 1:2].mean() + ref[:, :, 19:20].mean())
    ref = ref[:, :, cut:20 - cut] - bg
    m = ref.reshape(4, -1).mean(1)
    ref = ref * (m.mean() / m)[:, None, None]
    assert np.allclose(d, ref) and ang.size == 4
    g, _, bgo = preprocess.global_rescaling(p, "", 0.1, bad)
    r2 = data - data.min()
    r2 = r2[keep]
    r2 = r2 - r2.min()
    assert np.isclose(bgo, 0.5 * (r2[:, :, 1:2].mean() + r2[:, :, 19:20].mean()))
    assert np.allclose(g, r2[:, :, 2:18])
    badfile = str(tmp_path / "bad.txt")
    with open(badfile, "w") as fh:
        fh.write("2\n")
    d2, _, _ = preprocess.brightness_correction(p, badfile, 0.1, [5])
    assert np.allclose(d2, d)


def test_found_projections_reported_not_removed(tmp_path, monkeypatch):
    """The reference appends the detector's list as one entry of Badprojections
    (Reconstruction_coupled.py:138, :328); its loader's ``i+1 in text`` never matches
    a list, so nothing found is removed.  The CLI does the same by default and
    removes them with --Apply_Found_Projections.  The detector is a host fake here."""
    rng = np.random.default_rng(4)
    p = _stack(tmp_path, rng.random((6, 5, 20)) + 1.0, np.linspace(-60, 60, 6))
    calls = []

    def fake(name, searchradius, prozent, device=0):
        calls.append((name, searchradius, prozent, device))
        return [3, 6]

    monkeypatch.setattr(badproj, "find_bad_projections", fake)
    dh = ["bright", "thresholding", "0.0", "", "0.05"]
    common = (dh, [1], [0.1, 2.0], [1, 98], range(0, 5), True)
    kept = cli._load([p], *common, device=0)
    assert calls == [(p, 2.0, 0.1, 0)]
    assert kept[0][0].shape[0] == 5 and len(kept[3]) == 5  # only --Badprojections 1 removed
    dropped = cli._load([p], *common, device=0, apply_found=True)
    assert dropped[0][0].shape[0] == 3 and len(dropped[3]) == 3  # 1, 3 and 6 removed
    assert cli.build_parser().parse_args([p, "--Apply_Found_Projections"]).Apply_Found_Projections
    assert not cli.build_parser().parse_args([p]).Apply_Found_Projections


def test_subsampling_driver_applies_found_projections_on_request(monkeypatch):
    """Two-resolution driver: found projections are left in by default (as in the
    reference) and added per resolution with --Apply_Found_Projections."""
    calls = []

    def fake(name, searchradius, prozent, device=0):
        calls.append(name)
        return [2] if name == "fine0" else [4, 5]

    monkeypatch.setattr(badproj, "find_bad_projections", fake)
    names, bad = ["fine0", "fine1", "coarse0"], [[1], [7]]
    assert cli.subs_bad_projections(names, 2, bad, [0, 2.0]) == [[1], [7]] and calls == []
    assert cli.subs_bad_projections(names, 2, bad, [0.1, 2.0]) == [[1], [7]] and calls == []
    assert cli.subs_bad_projections(names, 2, bad, [0.1, 2.0], apply_found=True) == [[1, 2], [7, 4, 5]]
    assert calls == ["fine0", "coarse0"]
    assert bad == [[1], [7]]  # the caller's lists are not modified


def test_cli_option_handling(tmp_path):
    assert cli.parse_method("frob3d") == ("Frobenius 3D Reconstruction", 1)
    assert cli.parse_method("Uncorr2d") == ("Uncorrelated 2D Reconstruction", 0)
    assert cli.parse_method("nucl3d") == ("Nuclear 3D Reconstruction", 1)
    assert cli.parse_method("frobsubs")[1] == 2
    assert cli.parse_method("whatever") == ("Frobenius 2D Reconstruction", 0)
    p = _stack(tmp_path, np.ones((2, 2, 4)), [0, 10])
    assert cli.resolve_names([p[:-4]]) == [p]
    assert cli.resolve_names([p[:-4] + "."]) == [p]
    with pytest.raises(IOError):
        cli.resolve_names([str(tmp_path / "missing")])
    a = cli.build_parser().parse_args([p])
    assert a.Maxiter == 2000 and a.alpha == [4, 1.0] and a.Scalepars == [1, 98] and a.Overlapping == 1
    with pytest.raises(ValueError):
        cli.main([p, "--SliceLevels", "3", "1", "--Outfile", str(tmp_path / "o")])


def test_bad_projection_oracle_matches_reference(golden):
    """The detector's oracle against the reference's own helpers and pipeline: the
    helpers on float64 and on float32 arrays, every stage of Find_Bad_projections
    (smoothed stack, weighted gradients, neighbour errors) and the selections, all
    bit-exact."""
    g = golden("badproj.npz")
    for n in sorted({k.split("/")[0] for k in g}):
        data = g[f"{n}/data"]
        sm = obad.reduce_noise(data[0], 3)
        np.testing.assert_array_equal(sm, g[f"{n}/reduce_noise0"])
        w0 = obad.weighted_gradient(sm)[1]
        np.testing.assert_array_equal(w0, g[f"{n}/wgrad0"])
        w1 = obad.weighted_gradient(obad.reduce_noise(data[1], 3))[1]
        nrm, E = obad.compare_shift_twosided(w0, w1, 4)
        np.testing.assert_array_equal(E, g[f"{n}/shift_E"])
        assert nrm == float(g[f"{n}/shift_norm"])
        # float32, as the detector stores its stacks
        w0f = obad.weighted_gradient(sm.astype(np.float32))[1]
        np.testing.assert_array_equal(w0f, g[f"{n}/wgrad0_f32"])
        w1f = obad.weighted_gradient(obad.reduce_noise(data[1], 3).astype(np.float32))[1]
        nrm, E = obad.compare_shift_twosided(w0f.astype(np.float32), w1f.astype(np.float32), 4)
        np.testing.assert_array_equal(E, g[f"{n}/shift_E_f32"])
        assert nrm == float(g[f"{n}/shift_norm_f32"])
        S, W = obad.stages(data)
        np.testing.assert_array_equal(S, g[f"{n}/pipe_smooth"])
        np.testing.assert_array_equal(W, g[f"{n}/pipe_wgrad"])
        assert obad.pair_errors(W, 1, 4) == list(g[f"{n}/pipe_err1"])
        assert obad.pair_errors(W, 2, 6) == list(g[f"{n}/pipe_err2"])
        for frac in ("0.15", "3"):
            got = obad.find_bad_projections(data, 4, float(frac) if "." in frac else int(frac))
            assert list(got) == list(g[f"{n}/bad_{frac}"]), (n, frac)


def test_bad_projection_host_selection_matches_oracle():
    """The product's host step (combining neighbour errors and ranking) is the
    oracle's, including count-style fractions, -1 and ties (first index wins)."""
    rng = np.random.default_rng(5)
    for NA in (3, 4, 9, 30):
        e1 = list(rng.random(NA - 1))
        e2 = list(rng.random(NA - 2))
        for frac in (0.1, 0.5, -1, 2, 1):
            assert badproj.select(e1, e2, frac) == obad.select(e1, e2, frac)
    tie = [1.0, 1.0, 1.0, 1.0]
    assert badproj.select(tie, tie[:3], 3)[0] == obad.select(tie, tie[:3], 3)[0] == [1, 2, 3]


def test_subsampling_geometry_helpers():
    # sizes from the data win; a matching --Pixelratio is accepted, a different one aborts
    assert cli.pixel_ratio([1.0, 1.0, 2.5], 2, -1) == 2.5
    assert cli.pixel_ratio([1.0, 2.5], 1, 2.5004) == 2.5
    with pytest.raises(ValueError):
        cli.pixel_ratio([1.0, 2.5], 1, 3.0)
    with pytest.raises(ValueError):
        cli.pixel_ratio([1.0, 2.0, 2.5], 2, -1)
    # MRC data carries no size: the input decides, and no input aborts
    assert cli.pixel_ratio([-1.0, -1.0], 1, 2.0) == 2.0
    with pytest.raises(ValueError):
        cli.pixel_ratio([-1.0, -1.0], 1, -1)
    # whole section covers with floor/ceil, a chunk rounds; both clip to the coarse stack
    assert cli.coarse_section(2, 9, 2.0, 5.5, 2.5, 6, "cover") == (0, 5)
    assert cli.coarse_section(2, 3, 2.0, 5.5, 2.5, 6, "cover") == (0, 2)
    assert cli.coarse_section(2, 3, 2.0, 5.5, 2.5, 6, "round") == (1, 1)
    assert cli.coarse_section(0, 40, 2.0, 5.5, 2.5, 6, "cover") == (0, 5)
    assert preprocess.pixel_size("x.mrc") == -1.0


def test_chunk_shrinks_and_retries_after_out_of_memory(tmp_path, monkeypatch):
    """Host fault injection: the volume solver reports out-of-memory for chunks of
    more than 3 slices; the driver shrinks the chunk by 0.7 and retries
    (Reconstruction_coupled.py:509-536) until every slice is reconstructed."""
    from graptor_gb300 import GraptorMemoryError
    from graptor_gb300 import radon_tgv_primal_dual_3d as r3
    calls = []

    def fake(sino, angles, Parameter, mu, maxiter, ctx, plott, Stepsize, discrepancy, method, reg, Info):
        nang, nz, nd = np.asarray(sino[0]).shape
        calls.append(nz)
        if nz > 3:
            raise GraptorMemoryError(1, "forced allocation failure")
        u = np.stack([np.full((nd, nd, nz), 1.0 + c) for c in range(len(sino))])
        return u, np.ones((len(sino), nang, nz, nd))

    monkeypatch.setattr(r3, "Reconstructionapproach3d", fake)
    p = _stack(tmp_path, np.abs(np.random.default_rng(3).standard_normal((5, 12, 8))) + 1.0, np.linspace(-60, 60, 5))
    out = str(tmp_path / "r" / "x")
    u = cli.main([p, "--SliceLevels", "0", "9", "--Coupling", "frob3d", "--Outfile", out, "--Chunksize", "8",
                  "--Overlapping", "0", "--Datahandling", "basic", "none", "0.0", "", "0.0"])
    assert calls[0] == 8 and calls[1] == 5 and max(calls[2:]) <= 3  # 8 -> 5 -> 3 slices at once
    assert u.shape == (1, 8, 8, 10) and np.all(u == 1.0)
