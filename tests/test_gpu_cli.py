"""The command-line path end to end on the GPU: synthetic MRC projection stacks
with .rawtlt angles -> graptor_gb300.cli (the options of Reconstruction_coupled.py)
-> MRC reconstructions, for the 3-D and the 2-D couplings, with and without
slice chunking."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _write_stacks(tmp, N=32, Nz=12, C=2, nang=25):
    import torch

    from graptor_gb300 import mrc, phantom, solver
    vol = phantom.ellipsoids_3d(N, Nz, C, 8, seed=4)  # [c, z, y, x]
    ang = phantom.angles_deg(nang)
    S = C * Nz
    img = torch.from_numpy(vol.reshape(S, N * N).T.copy()).cuda()
    sino = torch.zeros(nang * N, S, device="cuda")
    solver.radon(img.data_ptr(), sino.data_ptr(), ang, N, N, S)
    g = sino.cpu().numpy().T.reshape(C, Nz, nang, N)
    names = []
    deg = np.linspace(-70, 70, nang)
    for c in range(C):
        stack = np.transpose(phantom.poisson(g[c], 500.0, c), (1, 0, 2)) + 0.01  # [nang, Nz, nd]
        p = os.path.join(tmp, f"ch{c}.mrc")
        mrc.write_mrc(p, stack.astype(np.float32))
        with open(p.replace(".mrc", ".rawtlt"), "w") as fh:
            fh.write("\n".join(f"{a:.6f}" for a in deg))
        names.append(p)
    return names, N, Nz, nang


@pytest.mark.parametrize("coupling,extra", [("frob3d", []), ("frob3d", ["--Chunksize", "5", "--Overlapping", "1"]),
                                            ("uncorr2d", []), ("frob2d", [])])
def test_cli_reconstructs_mrc_stacks(tmp_path, coupling, extra):
    from graptor_gb300 import cli, mrc
    names, N, Nz, nang = _write_stacks(str(tmp_path))
    out = str(tmp_path / "res" / "rec")
    cli.main(names + ["--SliceLevels", "2", "9", "--Coupling", coupling, "--Maxiter", "40", "--Outfile", out,
                      "--mu", "0.2", "0.2", "--Channelnames", "A", "B", "--Datahandling", "basic", "none", "0.0", "",
                      "0.0", "--GPU_Choice", "0"] + extra)
    nz = 8
    a = mrc.read_mrc(out + "_A.mrc")
    s = mrc.read_mrc(out + "_B_sinogram.mrc")
    allc = mrc.read_mrc(out + "_all_channels.mrc")
    norm = mrc.read_mrc(out + "_all_channels_normalized.mrc")
    assert a.shape == (nz, N, N) and s.shape == (nang, nz, N) and allc.shape == (nz, N, 2 * N)
    assert np.isfinite(a).all() and a.max() > 0
    assert np.isclose(norm[:, :, :N].max(), 1.0, atol=1e-6)
    assert any(f.endswith(".config") for f in os.listdir(tmp_path / "res"))


@pytest.mark.parametrize("coupling,extra", [("frobsubs", []), ("uncorrsubs", ["--Chunksize", "5"])])
def test_cli_two_resolution(tmp_path, coupling, extra):
    """Fine 32-pixel stacks of channel 0 plus a coarse 16-pixel stack of channel 1
    (2x2 detector/slice binning, pixel ratio 2) through the subsampling driver."""
    from graptor_gb300 import cli, mrc
    names, N, Nz, nang = _write_stacks(str(tmp_path))
    fine1 = mrc.read_mrc(names[1]).astype(np.float64)  # [nang, Nz, N]
    coarse = 0.25 * (fine1[:, 0::2, 0::2] + fine1[:, 1::2, 0::2] + fine1[:, 0::2, 1::2] + fine1[:, 1::2, 1::2])
    lo = os.path.join(str(tmp_path), "lo.mrc")
    mrc.write_mrc(lo, coarse.astype(np.float32))
    with open(lo.replace(".mrc", ".rawtlt"), "w") as fh:
        fh.write("\n".join(f"{a:.6f}" for a in np.linspace(-70, 70, nang)))
    out = str(tmp_path / "res" / "rec")
    cli.main([names[0], "--Infiles_Smallresolution", lo, "--SliceLevels", "2", "9", "--Coupling", coupling,
              "--Maxiter", "40", "--Outfile", out, "--mu", "0.2", "0.2", "--Channelnames", "A", "B", "--Pixelratio",
              "2", "--Datahandling", "basic", "none", "0.0", "", "0.0", "--GPU_Choice", "0"] + extra)
    nz = 8
    a, b = mrc.read_mrc(out + "_A.mrc"), mrc.read_mrc(out + "_B.mrc")
    s_small = mrc.read_mrc(out + "_B_sinogram_smallresu.mrc")
    s_high = mrc.read_mrc(out + "_B_sinogram.mrc")
    s_a = mrc.read_mrc(out + "_A_sinogram.mrc")
    # fine slices 2..9 map to coarse slices floor((2-5.5)/2+2.5)=0 .. ceil((9-5.5)/2+2.5)=5, six slices
    assert a.shape == b.shape == (nz, N, N)
    assert s_a.shape == (nang, nz, N) and s_high.shape == (nang, nz, N) and s_small.shape == (nang, 6, N // 2)
    for x in (a, b, s_small, s_high, s_a):
        assert np.isfinite(x).all()
    assert a.max() > 0 and b.max() > 0
    norm = mrc.read_mrc(out + "_all_channels_normalized.mrc")
    assert norm.shape == (nz, N, 2 * N) and np.isclose(norm[:, :, N:].max(), 1.0, atol=1e-6)
