"""Bad-projection detection on the GPU (gt_badproj_*, graptor_gb300/badproj.py)
against the reference's own pipeline (tests/golden/badproj.npz, recorded from
find_bad_ele.py by tests/golden/make_badproj_golden.py) and against the oracle
(oracle/badproj.py) on larger seeded stacks.

Every stored array -- smoothed stack, weighted gradients, per-pixel maxima of the
shifted comparison -- must be bit-identical; the neighbour errors are float64 sums of
identical terms in another order (relative difference <= 1e-12); the selected
projections must be the same."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _stack(NA, Nz, Nx, seed, corrupt=2):
    """Seeded projection stack with blobs, small shifts, noise and corrupted projections."""
    rng = np.random.default_rng(seed)
    zz, xx = np.meshgrid(np.arange(Nz), np.arange(Nx), indexing="ij")
    base = np.zeros((Nz, Nx))
    for _ in range(8):
        cz, cx, r = rng.uniform(0.2, 0.8) * Nz, rng.uniform(0.2, 0.8) * Nx, rng.uniform(0.04, 0.12) * min(Nz, Nx)
        base += rng.uniform(0.5, 2.0) * ((zz - cz) ** 2 + (xx - cx) ** 2 < r * r)
    data = np.stack([np.roll(base, int(rng.integers(-2, 3)), axis=1) for _ in range(NA)])
    data += 0.05 * rng.random(data.shape)
    for k in rng.choice(NA, corrupt, replace=False):
        data[k] = np.roll(data[k], Nz // 5, axis=0) + 0.8 * rng.random((Nz, Nx))
    return data


def test_pipeline_matches_reference(golden):
    from graptor_gb300 import badproj
    g = golden("badproj.npz")
    for n in sorted({k.split("/")[0] for k in g}):
        data = g[f"{n}/data"]
        S, W = badproj.stages(badproj.upload(data))
        np.testing.assert_array_equal(S.cpu().numpy(), g[f"{n}/pipe_smooth"])
        np.testing.assert_array_equal(W.cpu().numpy(), g[f"{n}/pipe_wgrad"])
        e1 = badproj.pair_errors(W, 1, 4).cpu().numpy()
        e2 = badproj.pair_errors(W, 2, 6).cpu().numpy()
        np.testing.assert_allclose(e1, g[f"{n}/pipe_err1"], rtol=RTOL, atol=0)
        np.testing.assert_allclose(e2, g[f"{n}/pipe_err2"], rtol=RTOL, atol=0)
        for frac in ("0.15", "3"):
            got = badproj.find_bad_projections("stack", 4, float(frac) if "." in frac else int(frac), data=data)
            assert list(got) == list(g[f"{n}/bad_{frac}"]), (n, frac)
        # the helper on the two float32 gradient images the reference compared
        W0, W1 = W[0].cpu().numpy(), W[1].cpu().numpy()
        nrm, E = badproj.compare_shift_twosided(W0, W1, 4)
        np.testing.assert_array_equal(E, g[f"{n}/shift_E_f32"])
        assert abs(nrm / float(g[f"{n}/shift_norm_f32"]) - 1) <= RTOL


@pytest.mark.parametrize("shape,seed", [((24, 120, 140), 11), ((9, 64, 520), 12), ((3, 40, 37), 13)])
def test_detector_matches_oracle(shape, seed):
    """Default search radius; (9, 64, 520) takes the subsampling branch (step 2 in both
    directions, 26 smoothed rows: every block is at the bottom edge); NA = 3 is the
    fewest projections the ranking accepts."""
    from graptor_gb300 import badproj
    from oracle import badproj as obad
    data = _stack(*shape, seed)
    S0, W0 = obad.stages(data)
    S, W = badproj.stages(badproj.upload(data))
    np.testing.assert_array_equal(S.cpu().numpy(), S0)
    np.testing.assert_array_equal(W.cpu().numpy(), W0)
    r = int(min(S0.shape[1], S0.shape[2]) / 10)
    e1, e2 = badproj.detect(badproj.upload(data))
    np.testing.assert_allclose(e1.cpu().numpy(), obad.pair_errors(W0, 1, r), rtol=RTOL, atol=0)
    np.testing.assert_allclose(e2.cpu().numpy(), obad.pair_errors(W0, 2, int(r * 1.5)), rtol=RTOL, atol=0)
    for frac in (0.1, 2, -1):
        assert badproj.find_bad_projections("stack", None, frac, data=data) == \
            obad.find_bad_projections(data, None, frac)


@pytest.mark.parametrize("radius", [0, 1, 2, 5, 9])
def test_pair_errors_per_pixel_match_oracle(radius):
    """Per-pixel maxima bit-identical for radii 0 (no shift), 1 and 2 (the smallest
    sliding windows) up to the one that leaves a single interior row (19 rows)."""
    from graptor_gb300 import badproj
    from oracle import badproj as obad
    import torch
    rng = np.random.default_rng(100 + radius)
    Wh = rng.random((4, 19, 70)).astype(np.float32)
    W = torch.from_numpy(Wh).cuda()
    for offset in (1, 2):
        err, E = badproj.pair_errors(W, offset, radius, want_pixels=True)
        for q in range(4 - offset):
            nrm, E0 = obad.compare_shift_twosided(Wh[q], Wh[q + offset], radius)
            np.testing.assert_array_equal(E[q].cpu().numpy().astype(np.float64), E0)
            assert abs(float(err[q]) / nrm - 1) <= RTOL


def test_edge_cases_and_determinism():
    from graptor_gb300 import badproj
    import torch
    W = torch.from_numpy(np.random.default_rng(7).random((5, 20, 30)).astype(np.float32)).cuda()
    a = badproj.pair_errors(W, 1, 3).cpu().numpy()
    b = badproj.pair_errors(W, 1, 3).cpu().numpy()
    assert np.array_equal(a, b)  # fixed summation order
    assert np.array_equal(badproj.pair_errors(W, 1, 10).cpu().numpy(), np.zeros(4))  # no interior row: 0
    with pytest.raises(ValueError):
        badproj.pair_errors(W, 1, 11)  # the reference cannot shape its arrays either
    assert badproj.pair_errors(W, 5, 3).numel() == 0
    with pytest.raises(ValueError):
        badproj.stages(badproj.upload(np.ones((3, 8, 40))))  # 2 rows left after smoothing
