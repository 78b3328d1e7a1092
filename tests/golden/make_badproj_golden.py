"""Golden vectors for the bad-projection detector, from the REFERENCE's own code.

    python tests/golden/make_badproj_golden.py

Imports the reference's ``find_bad_ele.py`` from the checkout that the environment
variable ``GRAPTOR_REFERENCE`` names (required) with stand-ins for the modules it imports but does not use on
this path (``h5utilities`` -- only its ``Brightness_correction`` is called, and it
is replaced by a function returning the seeded input stack -- ``mrcfile``,
``scipy.misc`` and ``matplotlib``), then records its helper outputs and
``Find_Bad_projections`` on seeded synthetic projection stacks narrower than 250
detector columns (the reference's subsampling branch does not run on Python 3)
and an explicit search radius (its default, ``min(Nx, Nz)/10``, calls NumPy's ``min``
through ``from numpy import *`` and raises).
Besides the helpers' outputs on float64 and float32 arrays and the selections, it
records every stage of ``Find_Bad_projections`` as the reference's helpers returned
it inside the pipeline (smoothed stack, weighted gradients, the neighbour errors of
projections one and two apart).
Output: tests/golden/badproj.npz.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("GRAPTOR_REFERENCE", "")
if not REF or not os.path.isfile(os.path.join(REF, "find_bad_ele.py")):
    raise SystemExit("set GRAPTOR_REFERENCE to the reference checkout (the directory holding find_bad_ele.py)")


def stacks():
    rng = np.random.default_rng(20240607)
    out = []
    for NA, Nz, Nx in ((14, 40, 56), (11, 33, 48)):
        base = np.zeros((Nz, Nx))
        zz, xx = np.meshgrid(np.arange(Nz), np.arange(Nx), indexing="ij")
        for _ in range(5):
            cz, cx, r = rng.uniform(8, Nz - 8), rng.uniform(8, Nx - 8), rng.uniform(3, 9)
            base += rng.uniform(0.5, 2.0) * ((zz - cz) ** 2 + (xx - cx) ** 2 < r * r)
        data = np.stack([np.roll(base, int(rng.integers(-2, 3)), axis=1) for _ in range(NA)])
        data += 0.05 * rng.random(data.shape)
        for k in rng.choice(NA, 2, replace=False):  # two corrupted projections
            data[k] = np.roll(data[k], 9, axis=0) + 0.8 * rng.random((Nz, Nx))
        out.append(data)
    return out


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "refshim"))  # matplotlib stand-in
    current = {}
    h5 = types.ModuleType("h5utilities")
    h5.Brightness_correction = lambda name, badname, cutedges, bad: (current["data"].copy(), None, 0)
    sys.modules["h5utilities"] = h5
    sys.modules["mrcfile"] = types.ModuleType("mrcfile")
    misc = types.ModuleType("scipy.misc")
    sys.modules["scipy.misc"] = misc
    import scipy
    scipy.misc = misc
    sys.path.insert(0, REF)
    import find_bad_ele as fb

    res = {}
    for n, data in enumerate(stacks()):
        res[f"{n}/data"] = data
        sm = fb.reduce_noise(data[0], 3)
        res[f"{n}/reduce_noise0"] = sm
        res[f"{n}/wgrad0"] = fb.weighted_gradient(sm)[1]
        w1 = fb.weighted_gradient(fb.reduce_noise(data[1], 3))[1]
        nrm, E = fb.compare_shift_twosided(res[f"{n}/wgrad0"], w1, 4)
        res[f"{n}/shift_norm"] = np.array(nrm)
        res[f"{n}/shift_E"] = E
        # the helpers on the float32 arrays Find_Bad_projections stores (:152-175)
        w0f = fb.weighted_gradient(sm.astype(np.float32))[1]
        res[f"{n}/wgrad0_f32"] = w0f
        w1f = fb.weighted_gradient(fb.reduce_noise(data[1], 3).astype(np.float32))[1]
        nrm, E = fb.compare_shift_twosided(w0f.astype(np.float32), w1f.astype(np.float32), 4)
        res[f"{n}/shift_norm_f32"] = np.array(nrm)
        res[f"{n}/shift_E_f32"] = E
        for frac in (0.15, 3):
            current["data"] = data
            rec = {"rn": [], "wg": [], "cmp": []}
            helpers = (fb.reduce_noise, fb.weighted_gradient, fb.compare_shift_twosided)

            def recorder(key, fn):
                def call(*a):
                    out = fn(*a)
                    rec[key].append(out)
                    return out
                return call

            fb.reduce_noise, fb.weighted_gradient, fb.compare_shift_twosided = (
                recorder("rn", helpers[0]), recorder("wg", helpers[1]), recorder("cmp", helpers[2]))
            try:
                res[f"{n}/bad_{frac}"] = np.array(fb.Find_Bad_projections("stack", 4, frac))
            finally:
                fb.reduce_noise, fb.weighted_gradient, fb.compare_shift_twosided = helpers
            if frac == 3:  # every stage of the pipeline, as the reference's helpers returned it
                NA = data.shape[0]
                res[f"{n}/pipe_smooth"] = np.stack(rec["rn"]).astype(np.float32)
                res[f"{n}/pipe_wgrad"] = np.stack([w for _, w in rec["wg"]]).astype(np.float32)
                norms = np.array([c[0] for c in rec["cmp"]])
                res[f"{n}/pipe_err1"], res[f"{n}/pipe_err2"] = norms[:NA - 1], norms[NA - 1:]
    np.savez_compressed(os.path.join(HERE, "badproj.npz"), **res)
    print("wrote", os.path.join(HERE, "badproj.npz"), {k: v.shape for k, v in res.items() if "bad_" in k})


if __name__ == "__main__":
    main()
