#!/usr/bin/env python
"""Benchmark of the plain primal-dual solver on the 3-D coupled workload.

Workload (one "step" = one primal-dual iteration over the whole problem):
  3-D coupled 4-channel Frobenius TGV with KL discrepancy, 256x256 in-plane x 60
  slices, 256 detector bins x 71 angles in [-70, 70] degrees, mu = (0.2, 5e-4,
  4e-3, 5e-4), alpha = (4, 1); seeded synthetic ellipsoid phantoms (channel 0
  dense with Poisson noise at peak 1e4, channels 1-3 sparse at peak 20).
Metric: voxel-iterations per second (voxel-channels x iterations / s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's algorithm on the host CPU: the oracle
(oracle/tgv_oracle.c), an FP32 restatement that reproduces the reference's own
kernels bit for bit (tests/test_oracle_golden.py), on all host threads, each step
one iteration over a slab of slices sized to keep the run within minutes.
Multi-GPU: one independent replica per rank (the problems are independent), no
collective on the data path; the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import contextlib
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W = dict(N=256, Nz=60, C=4, nang=71, alpha=(4.0, 1.0), mu=[0.2, 5e-4, 4e-3, 5e-4], peaks=[1e4, 20.0, 20.0, 20.0],
         stated_iterations=2500, coupling="FROB")
METRIC = "voxel-iter/s"
WORKLOAD_NAME = "3D {cpl}3D TGV-KL {N}x{N}x{Nz}, 4 channels, {N} bins x {nang} angles"
COUPLING_METHOD = {"FROB": "Frobenius 3D Reconstruction", "UNCORR": "Uncorrelated 3D Reconstruction",
                   "NUCL": "Nuclear 3D Reconstruction"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def algorithmic_bytes(V, Sb):
    """Bytes one iteration must move (3-D TGV): 172 per voxel-channel + 16 per bin.

    Per kernel (what each launch must read and write at least once):
    k_dual   reads ubar 4, pbar 12, v 12, w 24; writes v 12, w 24          (88 B/voxel-ch)
    k_fwd    reads ubar 4 B/voxel-ch, f 4, lambda 4; writes lambda 4, K ubar 4 (16 B/bin)
    k_bp     reads lambda 4 B/bin; writes K* lambda 4 B/voxel-ch
    k_update reads u 4, p 12, v 12, w 24, K* lambda 4; writes u 4, ubar 4, p 12, pbar 12 (88 B/voxel-ch)
      launched as two halves (the iteration's schedule):
      k_update_u reads u 4, v 12, K* lambda 4; writes u 4, ubar 4                  (28 B/voxel-ch)
      k_update_p reads p 12, v 12, w 24; writes p 12, pbar 12                      (72 B/voxel-ch)
    k_dual_fused (schedule 2: the p half of the previous iteration inside the dual kernel)
             reads ubar 4, p 12, v 12, w 24; writes p 12, v 12, w 24                 (100 B/voxel-ch)
    The iteration figure stays the unfused one (the algorithm's own traffic); schedule 2
    moves 100 + 28 + 8 B/voxel-ch + 20 B/bin per iteration.
    """
    return {"iteration": 172 * V + 16 * Sb, "k_dual": 88 * V, "k_fwd": 4 * V + 16 * Sb,
            "k_bp": 4 * V + 4 * Sb, "k_update": 88 * V, "k_update_u": 28 * V, "k_update_p": 72 * V,
            "k_dual_fused": 100 * V}


def gather_bytes(N, nang, S):
    """Bytes a projector moves through L1 per launch: every (pixel, angle) pair
    has two interpolation taps of S floats (k_bp reads two sinogram bins per pixel
    and angle; k_fwd reads two image pixels per ray and row, about as many pairs).
    The model counts every pair as inside the detector, an upper bound."""
    return 2 * 4 * N * N * nang * S


# L1 data path: 128 B per clock per SM, 152 SMs, 2.07 GHz maximum SM clock (nominal)
L1_NOMINAL_GBS = 128 * 152 * 2.07


def workload_config(world):
    """The workload's description, identical in both arms' lines."""
    N, Nz, C, nang = W["N"], W["Nz"], W["C"], W["nang"]
    V = N * N * Nz * C
    return {"workload": WORKLOAD_NAME.format(N=N, Nz=Nz, nang=nang, cpl=W["coupling"]), "voxel_channels": V,
            "sinogram_bins": N * nang * Nz * C, "dim": 3, "N": N, "Nz": Nz, "C": C, "nang": nang,
            "coupling": W["coupling"], "discrepancy": "KL", "regularisation": "TGV",
            "stated_iterations": W["stated_iterations"],
            "l2": f"inputs larger than L2 (solver state {V * 76 / 1e9:.1f} GB per replica)",
            "parallelism": f"replicas x{world}"}


def make_problem_data(seed=0):
    """Host sinograms [C][nang, Nz, nd] of the seeded phantom, projected on the GPU."""
    import torch

    from graptor_gb300 import phantom, solver
    N, Nz, C, nang = W["N"], W["Nz"], W["C"], W["nang"]
    vol = phantom.ellipsoids_3d(N, Nz, C, 12, seed)  # [c, z, y, x]
    ang = phantom.angles_deg(nang)
    S = C * Nz
    img = torch.from_numpy(vol.reshape(S, N * N).T.copy()).cuda()
    sino = torch.zeros(nang * N, S, device="cuda")
    solver.radon(img.data_ptr(), sino.data_ptr(), ang, N, N, S)
    g = sino.cpu().numpy().T.reshape(C, Nz, nang, N)
    out = []
    for c in range(C):
        noisy = phantom.poisson(g[c], W["peaks"][c], seed + c)  # [z, nang, nd]
        out.append(np.ascontiguousarray(np.transpose(noisy, (1, 0, 2))))  # [nang, Nz, nd]
    del img, sino
    return out, ang


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v for v in vis.split(",") if v.strip().isdigit()]
        self.index = int(ids[index]) if index < len(ids) else index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.proc or not self.path:
            return None
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        load = [s for s in sm if s > 0.5 * smax] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": smax, "reasons": reasons, "samples": len(rows)}


def cpu_baseline(seconds=15.0):
    """The oracle (reference-exact FP32 port) on all host threads, bounded sample."""
    from graptor_gb300 import phantom
    from oracle import oracle as O
    N, C, nang = W["N"], W["C"], W["nang"]
    Nz = 8
    rng = np.random.default_rng(0)
    ang = phantom.angles_deg(nang)
    ofs = O.radon_struct(ang, N, N)
    f = np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32)
    s = O.Solver(3, N, Nz, C, N, ofs, f, W["alpha"], W["mu"], 100.0, O.KL, O.TGV, getattr(O, W["coupling"]))
    s.run(1)
    t0 = time.perf_counter()
    it = 0
    while time.perf_counter() - t0 < seconds or it < 2:
        s.run(1)
        it += 1
    dt = time.perf_counter() - t0
    V = N * N * Nz * C
    return {"value": V * it / dt, "unit": METRIC, "cores": os.cpu_count(), "kind": "port",
            "sample": f"{it} iterations of the same problem at 256x256x{Nz} slices x 4 channels, 71 angles "
                      f"(oracle/tgv_oracle.c, OpenMP {os.cpu_count()} threads, {dt:.1f} s)"}


def dist_setup(n):
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, world):
    """Reference arm: the reference algorithm on the host CPU (oracle port), rank 0 only."""
    if rank != 0:
        return None
    from graptor_gb300 import phantom
    from oracle import oracle as O
    N, C, nang = W["N"], W["C"], W["nang"]
    ang = phantom.angles_deg(nang)
    ofs = O.radon_struct(ang, N, N)
    rng = np.random.default_rng(0)

    def solver(Nz):
        f = np.abs(rng.standard_normal((C * Nz, nang, N))).astype(np.float32)
        return O.Solver(3, N, Nz, C, N, ofs, f, W["alpha"], W["mu"], 100.0, O.KL, O.TGV, getattr(O, W["coupling"]))

    probe = solver(2)
    t0 = time.perf_counter()
    probe.run(1)
    per_slice = (time.perf_counter() - t0) / 2
    budget = 150.0 / max(1, args.steps + args.warmup)
    Nz = int(max(2, min(W["Nz"], budget / max(per_slice, 1e-6))))
    s = solver(Nz)
    s.run(args.warmup)
    t0 = time.perf_counter()
    s.run(args.steps)
    dt = time.perf_counter() - t0
    V = N * N * Nz * C
    value = V * args.steps / dt
    sample = (f"each step one iteration over 256x256x{Nz} slices x 4 channels, 71 angles (oracle/tgv_oracle.c, "
              f"bit-exact with the reference kernels, OpenMP {os.cpu_count()} threads)")
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(world), "sample_slices": Nz,
            "time_for_stated_iterations_s": W["stated_iterations"] * (N * N * W["Nz"] * C) / value,
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": os.cpu_count(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_ours(args, rank, world, local):
    import torch

    from graptor_gb300 import radon_tgv_primal_dual_3d as r3
    from graptor_gb300.solver import Problem
    torch.cuda.set_device(local)
    N, Nz, C, nang = W["N"], W["Nz"], W["C"], W["nang"]
    sino, ang = make_problem_data(seed=rank)
    S = C * Nz
    V = N * N * S
    Sb = N * nang * S
    f = np.concatenate([np.transpose(s, (1, 0, 2)) for s in sino])  # [S, nang, nd]
    stream = torch.cuda.Stream()
    forced = args.fwd_shape is not None or args.bp_shape is not None or args.dual_shape is not None
    prob = Problem(3, N, Nz, C, N, ang, W["alpha"], W["mu"], "KL", "TGV", W["coupling"], 1.0, None, local,
                   stream.cuda_stream, autotune=not forced)
    prob.set_data(f)
    if forced:  # launch shapes given on the command line (profiler captures): no tuning launches
        prob.set_tuning(args.fwd_shape or 0, args.bp_shape or 0)
        prob.set_dual_shape(args.dual_shape or 0)
    if args.schedule is not None:
        prob.set_schedule(args.schedule)
    prob.run(args.warmup).synchronize()

    # ---- device-timed region: K iterations, inputs resident in HBM
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        prob.run(args.steps)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    clocks = clk.summary()
    value = world * V * args.steps / (ms / 1e3)
    if args.quick:
        prob.close()
        return {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "config": {"workload": WORKLOAD_NAME.format(N=W["N"], Nz=W["Nz"], nang=W["nang"], cpl=W["coupling"]), "Nz": Nz, "quick": True}, "clocks": clocks}

    # ---- per-kernel durations (CUDA events on the launching stream) for the roofline
    kms = prob.time_kernels(reps=5)
    kms.pop("k_update")  # the iteration launches the update as its two halves
    alg = algorithmic_bytes(V, Sb)
    top = max(kms, key=kms.get)
    hbm, peak_kind = peaks()
    achieved = alg[top] / (kms[top] / 1e3) / 1e9
    traffic = ncu_traffic(top)
    it_ms = ms / args.steps
    solver_gbs = alg["iteration"] / (it_ms / 1e3) / 1e9
    launches = prob.launches_per_iteration * args.steps
    roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": alg[top], "ms_per_launch": kms[top]}
    if top in ("k_fwd", "k_bp"):
        # a projector gathers from L2-resident operands: its limit is the L1 data path
        gb = gather_bytes(N, nang, S)
        roof["l1"] = {"achieved": gb / (kms[top] / 1e3) / 1e9, "peak": L1_NOMINAL_GBS, "unit": "GB/s",
                      "frac": gb / (kms[top] / 1e3) / 1e9 / L1_NOMINAL_GBS, "peak_source": "nominal",
                      "gather_bytes_per_launch": gb}
    ne = prob.scalars["normest"]
    tuning = prob.tuning
    prob.close()

    # ---- end to end through the reference-facing entry point, host buffers
    r3.progress = False
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    u, s_out = r3.Reconstructionapproach3d(sino, ang, W["alpha"], np.array(W["mu"]), args.steps, local, [0, 0.1], 1,
                                           "KL", COUPLING_METHOD[W["coupling"]], "TGV", [0.0, 1.0, [0]])
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    h2d = 4 * Sb
    d2h = 8 * V + 8 * Sb  # the float64 Solution and Sinogram the entry point returns
    e2e = {"value": world * V * args.steps / e2e_s, "unit": METRIC,
           "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
           "seconds": e2e_s, "includes": "problem setup, H2D of the sinograms, FP64 operator-norm estimate, "
                                         "K iterations, D2H of Solution and Sinogram (one call)"}
    # time to relative gap: cold plain solver vs learned warm start + batch (the
    # metric's first quantity), at the tolerance both reach in bounded time (every rank)
    # at the metric's tolerance 1e-4 (u held as two floats: with float32 u the gap stalls at a few 1e-4;
    # primal weight 10 after the warm arm's cold pre-iterations) on 64^2 x 16 x 2, and at 1e-2 on
    # 128^2 x 32 x 2 with the reference's steps and float32 u
    ttg = ttg2 = None
    if args.ttg_seeds > 0:
        ttg = time_to_gap_compare(rank, world, local, args.ttg_seeds, weights=WARM["weights_1e4"], N=64, Nz=16,
                                  tol=1e-4, pweight=10.0, precise=True, check_every=1000, max_iters=200000)
        ttg2 = time_to_gap_compare(rank, world, local, args.ttg_seeds)
    if rank != 0:
        return None
    out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": it_ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ellipsoid phantoms, Poisson noise)",
           "config": workload_config(world),
           "time_for_stated_iterations_s": it_ms * W["stated_iterations"] / 1e3, "normest": ne, "autotuned": tuning,
           "roofline": roof,
           "kernels_ms": kms,
           "hbm_kernels": {k: {"achieved": alg[k] / (kms[k] / 1e3) / 1e9, "frac": alg[k] / (kms[k] / 1e3) / 1e9 / hbm}
                           for k in ("k_dual", "k_update_u", "k_update_p", "k_dual_fused") if k in kms},
           "solver_roofline": {"achieved": solver_gbs, "peak": hbm, "unit": "GB/s", "frac": solver_gbs / hbm,
                               "algorithmic_bytes_per_iteration": alg["iteration"]},
           "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline()
    if ttg is not None:
        out["time_to_gap"] = ttg
        out["time_to_gap_1e-2"] = ttg2
    return out


BATCH_SIZES = {"uneven": dict(N=(96, 512), nang=(30, 180), Nz=(1, 64)),   # the 64-problem batch (config 3)
               "small": dict(N=(32, 128), nang=(30, 90), Nz=(1, 8))}     # many small problems


def batched_specs(n=64, seed=0, sizes="uneven"):
    """n independent problems: N, angles (over [-75, 75] deg) and slices uniform over
    the ranges of BATCH_SIZES[sizes] ("uneven": N U{96..512}, angles U{30..180},
    slices U{1..64}; "small": N U{32..128}, angles U{30..90}, slices U{1..8}),
    channels U{1..4}, alternating KL / L2, TGV with Frobenius coupling."""
    from graptor_gb300 import phantom
    rng = np.random.default_rng(seed)
    rg = BATCH_SIZES[sizes]
    specs = []
    for k in range(n):
        N = int(rng.integers(rg["N"][0], rg["N"][1] + 1))
        nang = int(rng.integers(rg["nang"][0], rg["nang"][1] + 1))
        C = int(rng.integers(1, 5))
        Nz = int(rng.integers(rg["Nz"][0], rg["Nz"][1] + 1))
        disc = "KL" if k % 2 == 0 else "L2"
        mu = [0.2] + [0.05] * (C - 1)
        specs.append(dict(dim=3, N=N, Nz=Nz, C=C, nd=N, angles=phantom.angles_deg(nang, -75, 75), alpha=(4.0, 1.0),
                          mu=mu, discrepancy=disc, regularisation="TGV", coupling="FROB"))
    return specs


def batched_data(spec, seed):
    """Sinograms [S, nang, nd] of a 10-ellipse phantom per channel (slices scaled copies),
    projected on the GPU, Poisson noise at a peak of 1e3 counts."""
    import torch

    from graptor_gb300 import phantom, solver
    N, Nz, C, ang = spec["N"], spec["Nz"], spec["C"], spec["angles"]
    S = Nz * C
    base = np.stack([phantom.ellipses_2d(N, 10, seed * 7 + c) for c in range(C)])  # [C, y, x]
    scale = 0.6 + 0.4 * np.cos(np.linspace(0, np.pi, Nz))
    vol = (base[:, None] * scale[None, :, None, None]).astype(np.float32).reshape(S, N * N)
    img = torch.from_numpy(vol.T.copy()).cuda()
    sino = torch.zeros(len(ang) * N, S, device="cuda")
    solver.radon(img.data_ptr(), sino.data_ptr(), ang, N, N, S)
    g = sino.cpu().numpy().T.reshape(S, len(ang), N)
    return phantom.poisson(g, 1e3, seed)


def run_batched(args, rank, world, local):
    """Config-3 workload (or --batch-sizes small): every rank advances its own batch
    of independent problems, timed four ways: a graph of the members' own tuned
    iterations on concurrent chains, the same with one fixed launch shape, the
    fused mode (one launch per phase over every member's work units, fixed shapes),
    and the problems one after another.  The autotuner's share is its set-up time
    (gt_set_data with tuning minus without) against the tuned batch's run."""
    import torch

    from graptor_gb300.solver import Batch, Problem
    torch.cuda.set_device(local)
    specs = batched_specs(args.batch, seed=rank, sizes=args.batch_sizes)
    datas = [batched_data(sp, k) for k, sp in enumerate(specs)]
    V = sum(sp["N"] ** 2 * sp["Nz"] * sp["C"] for sp in specs)
    out = {}
    setup_s = {}
    for label, tune, mode in (("autotuned", True, 0), ("fixed_shape", False, 0), ("fused", False, 1)):
        with Batch([{**sp, "autotune": tune} for sp in specs], device=local) as b:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for k in range(len(b)):
                b[k].set_data(datas[k])
            torch.cuda.synchronize()
            setup_s[label] = time.perf_counter() - t0
            b.set_mode(mode)
            chains_s = {}
            for chains in (((1, 2, 4, 8, 64) if tune else (8,)) if mode == 0 else (1,)):
                b.set_concurrency(chains)
                b.run(args.warmup).synchronize()
                barrier(world)
                t0 = time.perf_counter()
                b.run(args.steps).synchronize()
                chains_s[chains] = max_over_ranks(time.perf_counter() - t0, world)
            best = min(chains_s, key=chains_s.get)
            dt = chains_s[best]
            out[label] = {"seconds": dt, "voxel_iter_per_s": world * V * args.steps / dt, "chains": best,
                          "seconds_by_chains": chains_s, "shapes": [b[k].tuning for k in range(len(b))][:8]}
    # the same problems one after another (each alone on the GPU, tuned shapes)
    seq = 0.0
    for k, sp in enumerate(specs):
        with Problem(**sp, device=local) as p:
            p.set_data(datas[k]).run(args.warmup).synchronize()
            t0 = time.perf_counter()
            p.run(args.steps).synchronize()
            seq += time.perf_counter() - t0
    seq = max_over_ranks(seq, world)
    out["sequential"] = {"seconds": seq, "voxel_iter_per_s": world * V * args.steps / seq}
    tuning_s = max(0.0, setup_s["autotuned"] - setup_s["fixed_shape"])
    out["tuning"] = {"seconds": tuning_s, "share_of_tuned_batch": tuning_s / (tuning_s + out["autotuned"]["seconds"]),
                     "setup_seconds": setup_s}
    if rank != 0:
        return None
    best_label = min(("autotuned", "fixed_shape", "fused"), key=lambda k: out[k]["seconds"])
    best = out[best_label]
    rg = BATCH_SIZES[args.batch_sizes]
    return {"metric": METRIC, "value": best["voxel_iter_per_s"], "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * best["seconds"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 10-ellipse phantoms, Poisson peak 1e3)",
            "config": {"workload": f"batched: {args.batch} independent 3D FROB TGV problems, N U{{{rg['N'][0]}.."
                                   f"{rg['N'][1]}}}, angles U{{{rg['nang'][0]}..{rg['nang'][1]}}} over [-75,75] deg, "
                                   f"C U{{1..4}}, Nz U{{{rg['Nz'][0]}..{rg['Nz'][1]}}}, KL/L2 alternating",
                       "voxel_channels_total": V, "sizes": [(sp["N"], sp["Nz"], sp["C"], len(sp["angles"]),
                                                             sp["discrepancy"]) for sp in specs]},
            "best": best_label, "batch": out,
            "speedup_vs_sequential": out["sequential"]["seconds"] / best["seconds"],
            "speedup_fused_vs_graph": out["autotuned"]["seconds"] / out["fused"]["seconds"],
            "speedup_tuned_vs_fixed_shape": out["fixed_shape"]["seconds"] / out["autotuned"]["seconds"]}


WARM = dict(N=128, Nz=32, C=2, nang=71, pre=500, tol=1e-2, check_every=100, max_iters=40000, fallback_after=10000,
            weights=os.path.join(ROOT, "graptor_gb300", "weights", "unet_tgv_kl_c2_p500.npz"),
            # trained on targets of the precise primal mode with primal weight 10 (the 1e-4 solver)
            weights_1e4=os.path.join(ROOT, "graptor_gb300", "weights", "unet_tgv_kl_c2_p500_w10.npz"))


def run_unet(args, rank, world, local):
    """The warm-start network's forward pass (3-level 3-D U-Net 16-32-64, 2 channels in
    and out, batch 2 of 32x128x128, bfloat16 activations): convolutions with
    16k input and output channels on the tensor cores (tcgen05; 3x3x3 ones by the
    kernel that stages input halos and weights in shared memory), the others on
    the CUDA cores; beside it the same pass with the tensor-core kernel that gathers
    every tap from global memory, and with every convolution on the CUDA cores."""
    import torch

    from graptor_gb300 import _lib as L
    from graptor_gb300.warmstart import UNet3D, unet_layers
    torch.cuda.set_device(local)
    B, C, D, H, Wd = 2, 2, 32, 128, 128
    net = UNet3D(C, C, residual=C, device=local)
    net.refresh()
    x = torch.randn((B, C, D, H, Wd), device="cuda", generator=torch.Generator("cuda").manual_seed(rank)).to(
        torch.bfloat16)
    out = torch.zeros((B, C, D, H, Wd), device="cuda")
    # algorithmic FLOPs of the convolutions (2 per multiply-add), by level
    flops = tc_flops = 0.0
    levels = {"enc1a": 0, "enc1b": 0, "enc2a": 1, "enc2b": 1, "bota": 2, "botb": 2, "dec2a": 1, "dec2b": 1,
              "dec1a": 0, "dec1b": 0, "head": 0}
    for name, ci, co, k in unet_layers(C, C):
        vox = B * D * H * Wd / 8 ** levels[name]
        fl = 2.0 * vox * ci * co * k ** 3
        flops += fl
        if ci % 16 == 0 and co % 16 == 0:
            tc_flops += fl
    times = {}
    for tc in (0, 2, 1):  # CUDA cores, tensor cores gathering every tap, tensor cores with staged halos
        L.check(L.lib().gt_nn_set_tensor_cores(tc))
        for _ in range(args.warmup):
            net.forward(x, out)
        torch.cuda.synchronize()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            net.forward(x, out)
        e1.record()
        e1.synchronize()
        L.check(L.lib().gt_nn_check())
        times[tc] = max_over_ranks(e0.elapsed_time(e1) / args.steps, world)
    L.check(L.lib().gt_nn_set_tensor_cores(1))
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peak, kind = float(json.load(fh)["bf16_tflops"]), "measured"
    except Exception:
        peak, kind = 1900.0, "fallback"
    if rank != 0:
        return None
    ms = times[1]
    return {"metric": "unet-forward/s", "value": world * 1e3 / ms, "unit": "forward/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)", "data": "synthetic",
            "config": {"workload": "warm-start U-Net 16-32-64 forward, batch 2 x 2 channels x 32x128x128",
                       "conv_gflop": flops / 1e9, "tensor_core_gflop": tc_flops / 1e9},
            "cuda_cores_only_ms": times[0], "tensor_cores_gather_ms": times[2],
            "roofline": {"bound": "tensor", "achieved": flops / (ms / 1e3) / 1e12, "peak": peak, "unit": "TFLOP/s",
                         "frac": flops / (ms / 1e3) / 1e12 / peak, "peak_source": kind, "traffic": None}}


def run_subsample(args, rank, world, local):
    """The two-resolution solver (radon_tgv_primal_dual_3dsubsample.py): channel 0 measured
    on the fine grid (N bins x Nz slices), channel 1 on a grid twice as coarse (N/2 bins x
    Nz/2 slices, pixel ratio 2, 2x2 binning of its fine projections), 71 angles each, TGV-KL
    with Frobenius coupling of both channels on the fine grid.  value = fine-grid
    voxel-channel iterations per second."""
    import torch

    from graptor_gb300 import _lib as L
    from graptor_gb300 import phantom, solver
    from graptor_gb300.radon_tgv_primal_dual_3dsubsample import Subsampling
    torch.cuda.set_device(local)
    N, Nz, nang = W["N"], W["Nz"], W["nang"]
    if N % 2 or Nz % 2:
        raise ValueError("the two-resolution workload needs even N and Nz")
    vol = phantom.ellipsoids_3d(N, Nz, 2, 12, seed=rank)  # [c, z, y, x]
    ang = phantom.angles_deg(nang)
    img = torch.from_numpy(vol.reshape(2 * Nz, N * N).T.copy()).cuda()
    sino = torch.zeros(nang * N, 2 * Nz, device="cuda")
    solver.radon(img.data_ptr(), sino.data_ptr(), ang, N, N, 2 * Nz)
    g = sino.cpu().numpy().T.reshape(2, Nz, nang, N)
    f0 = phantom.poisson(g[0], 1e4, rank)                                  # [Nz, nang, N]
    fine1 = phantom.poisson(g[1], 20.0, rank + 1)
    f1 = 0.25 * (fine1[0::2, :, 0::2] + fine1[1::2, :, 0::2] + fine1[0::2, :, 1::2] + fine1[1::2, :, 1::2])
    refnew, refold = [(N - 1) / 2.0, (Nz - 1) / 2.0], [(N / 2 - 1) / 2.0, (Nz / 2 - 1) / 2.0]
    with Subsampling(N, Nz, 1, 1, N // 2, Nz // 2, ang, ang, W["alpha"], [0.2, 4e-3], 2.0, refold, refnew,
                     device=local) as s:
        s.set_data(f0, f1)
        p = L.lib().gt_subs_problem(s._h)
        s.run(args.warmup)
        L.check(L.lib().gt_synchronize(p))
        barrier(world)
        t0 = time.perf_counter()
        s.run(args.steps)
        L.check(L.lib().gt_synchronize(p))
        dt = max_over_ranks(time.perf_counter() - t0, world)
    V = N * N * Nz * 2
    if rank != 0:
        return None
    return {"metric": METRIC, "value": world * V * args.steps / dt, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 2-channel ellipsoid phantoms, Poisson peaks 1e4 / 20)",
            "config": {"workload": f"two-resolution TGV-KL FROB: channel 0 {N}x{N}x{Nz} ({N} bins), channel 1 "
                                   f"{N // 2} bins x {Nz // 2} slices (pixel ratio 2), {nang} angles each",
                       "voxel_channels_fine_grid": V}}


def time_to_gap_compare(rank, world, local, nseeds, weights=None, N=None, Nz=None, tol=None, fields=("u",),
                        pweight=1.0, precise=False, check_every=None, max_iters=None):
    """Time to relative primal-dual gap <= tol on held-out seeded problems
    (3-D TGV-KL, FROB, 2 channels, 128^2 x 32 unless N / Nz given, 71 angles): the
    plain solver cold-started, problems one after another, against the learned
    warm start (pre cold iterations, U-Net prediction of u, lambda from K u; at a
    check that finds a problem's gap infinite, u is lifted along the rays with data
    it misses; a problem whose gap is still infinite fallback_after iterations after
    the prediction goes back to its cold iterate) with all problems advanced
    together as one Batch; converged problems leave the batch.  Set-up (buffers,
    data upload, operator norm, autotuning) is outside both timed regions; gap
    checks every check_every iterations are inside both.  pweight / precise: the
    solver settings of both arms after the warm arm's cold pre-iterations (those
    keep the reference's steps and float32 u, the regime the network was trained
    on): the primal weight of the step pair and u held as two floats (needed below
    the float32 plateau of the gap, a few 1e-4)."""
    import math

    import torch

    from graptor_gb300 import warmstart as WS
    from graptor_gb300.solver import Batch, Problem
    torch.cuda.set_device(local)
    N, Nz, C = N or WARM["N"], Nz or WARM["Nz"], WARM["C"]
    tol = tol or WARM["tol"]
    check_every = check_every or WARM["check_every"]
    max_iters = max_iters or WARM["max_iters"]
    seeds = [9000 + 1000 * rank + k for k in range(nseeds)]
    cases = [WS.phantom_case(s, N, Nz, C, WARM["nang"], device=local) for s in seeds]
    specs = [WS.problem_spec(N, Nz, C, ang) for _, ang in cases]
    wpath = weights or WARM["weights"]
    net = WS.UNet3D.load(wpath, device=local)

    def done(g):
        return math.isfinite(g) and g <= tol

    # plain cold start, one problem after another
    cold_its, cold_s, lpi = [], 0.0, 4
    for (f, _), sp in zip(cases, specs):
        with Problem(**sp, device=local) as p:
            p.set_data(f)
            if pweight != 1.0:
                p.set_primal_weight(pweight)
            if precise:
                p.set_precise_primal()
            p.synchronize()
            lpi = p.launches_per_iteration
            t0 = time.perf_counter()
            it, g = WS.iterations_to_gap(p, tol, check_every, max_iters)
            p.synchronize()
            cold_s += time.perf_counter() - t0
            cold_its.append(it)
    # warm start + batch
    warm_its = [None] * len(cases)
    with Batch(specs, device=local) as b:
        for k, (f, _) in enumerate(cases):
            b[k].set_data(f)
        b.invalidate()
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        b.run(WARM["pre"]).synchronize()
        ws = WS.WarmStarter(net, tuple(fields), pre_iters=0)
        snaps = [ws.apply(b[k], f, keep_snapshot=True) for k, (f, _) in enumerate(cases)]
        if pweight != 1.0 or precise:
            for k in range(len(cases)):
                if pweight != 1.0:
                    b[k].set_primal_weight(pweight)
                if precise:
                    b[k].set_precise_primal()
            b.invalidate()
        its = WARM["pre"]
        fell_back = [False] * len(cases)
        while any(w is None for w in warm_its) and its < max_iters:
            b.run(check_every).synchronize()  # the members' gap evaluations run on their own streams
            its += check_every
            for k in range(len(cases)):
                if warm_its[k] is not None:
                    continue
                g = b[k].gap()["relative"]
                if not math.isfinite(g):
                    b[k].repair_missed_rays()  # the iterate misses a ray with data: lift u along it
                    g = b[k].gap()["relative"]
                if done(g):
                    warm_its[k] = its
                    b.set_active(k, False)  # converged: the batch goes on without it
                elif not fell_back[k] and not math.isfinite(g) and its - WARM["pre"] >= WARM["fallback_after"]:
                    ws.restore(b[k], snaps[k])  # back to the cold iterate (the plain solver is the fallback)
                    fell_back[k] = True
        b.synchronize()
        warm_s = time.perf_counter() - t0
    cold_s = max_over_ranks(cold_s, world)
    warm_s = max_over_ranks(warm_s, world)
    return {"tolerance": tol, "seeds": seeds, "size": [N, N, Nz, C], "cold_seconds": cold_s,
            "warm_batched_seconds": warm_s, "ratio": cold_s / warm_s, "cold_iterations": cold_its,
            "warm_iterations": warm_its, "fell_back_to_cold": fell_back, "pre_iterations": WARM["pre"],
            "check_every": check_every, "max_iterations": max_iters, "primal_weight": pweight,
            "precise_primal": bool(precise), "weights": os.path.relpath(wpath, ROOT), "fields": list(fields),
            "gpu_launches": lpi * (sum(cold_its) + len(cases) * its)}


def run_gapsweep(args, rank, world, local):
    """Relative primal-dual gap and distance moved against iterations for a list of
    primal weights (--primal-weights; sigma = w/sqrt(Lsqr), tau = 1/(w sqrt(Lsqr)),
    w = 1 the reference's pair), cold start, one held-out problem (seed 9000) of
    the time-to-gap workload (3-D TGV-KL, FROB, 2 channels, 71 angles; --n / --nz);
    --steps iterations, a record every 5000: gap, its box term U sum min(0, K^T
    lambda - div v~) (the dual's bound for u in [0, U], U = 2 max u), the primal
    distance moved relative to ||u|| and the dual distance moved."""
    import math

    import torch

    from graptor_gb300 import warmstart as WS
    from graptor_gb300.solver import Problem
    torch.cuda.set_device(local)
    N, Nz = args.n or WARM["N"], args.nz or WARM["Nz"]
    f, ang = WS.phantom_case(9000 + rank, N, Nz, WARM["C"], WARM["nang"], device=local)
    rows = []
    for w in [float(x) for x in args.primal_weights.split(",")]:
        with Problem(**WS.problem_spec(N, Nz, WARM["C"], ang), device=local) as p:
            p.set_data(f).set_primal_weight(w).snapshot()
            if args.precise:
                p.set_precise_primal()
            t0 = time.perf_counter()
            hist, done = [], 0
            while done < args.steps:
                p.run(5000)
                done += 5000
                g = p.gap()
                mx, my = p.movement()
                un = float(np.linalg.norm(p.get("u")))
                hist.append({"iterations": done, "relative_gap": g["relative"], "box_term": g["dual"] + g["fstar"],
                             "gap": g["gap"], "primal_moved_rel": mx / max(un, 1e-30), "dual_moved": my})
                p.snapshot()
                if math.isfinite(g["relative"]) and g["relative"] <= 1e-4:
                    break
            rows.append({"primal_weight": w, "seconds": time.perf_counter() - t0, "history": hist})
    if rank != 0:
        return None
    best = min(rows, key=lambda r: r["history"][-1]["relative_gap"])
    return {"metric": "relative-gap", "value": best["history"][-1]["relative_gap"], "unit": "relative gap",
            "n_gpus": world, "steps": args.steps, "warmup": 0, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded 2-channel ellipsoid phantom)",
            "config": {"workload": f"primal-weight sweep: 3D TGV-KL FROB {N}x{N}x{Nz}, 2 channels, "
                                   f"{WARM['nang']} angles, cold start", "precise_primal": bool(args.precise)},
            "sweep": rows}


def run_warmstart(args, rank, world, local):
    """The time-to-gap comparison (time_to_gap_compare) as its own bench line."""
    r = time_to_gap_compare(rank, world, local, args.seeds, args.weights, args.n, args.nz, args.tol,
                            tuple(args.fields.split(",")), args.pweight, args.precise, args.check_every,
                            args.max_iters)
    if rank != 0:
        return None
    N, _, Nz, C = r["size"]
    return {"metric": "time-to-gap", "value": r["warm_batched_seconds"], "unit": "s", "n_gpus": world,
            "steps": len(r["seeds"]), "warmup": 0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded 2-channel ellipsoid phantoms, Poisson peaks 1e4 / 20)",
            "config": {"workload": f"time to relative gap <= {r['tolerance']}: {len(r['seeds'])} held-out 3D TGV-KL "
                                   f"FROB problems {N}x{N}x{Nz}, {C} channels, {WARM['nang']} angles",
                       "pre_iterations": r["pre_iterations"], "check_every": r["check_every"],
                       "max_iterations": r["max_iterations"], "primal_weight": r["primal_weight"],
                       "precise_primal": r["precise_primal"], "weights": r["weights"]},
            "cold_seconds": r["cold_seconds"], "warm_batched_seconds": r["warm_batched_seconds"],
            "speedup": r["ratio"], "cold_iterations": r["cold_iterations"], "warm_iterations": r["warm_iterations"],
            "fell_back_to_cold": r["fell_back_to_cold"], "gpu_launches": r["gpu_launches"]}


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel and not line.startswith("#"):
                return float(parts[1])
    except OSError:
        pass
    return None


def badproj_lane_ops(nz, nx, radius, pairs):
    """FP32 lane operations of gt_badproj_compare: per interior pixel and shift, one
    subtraction and one minimum in each of the two directions."""
    mz, mx = nz - 2 * radius, nx - 2 * radius
    return pairs * mz * mx * (2 * radius + 1) ** 2 * 4


def run_badproj(args, rank, world, local):
    """Bad-projection detection (find_bad_ele.py Find_Bad_projections) on a stack of
    nang projections x N slices x N detector columns, default search radius.  A step is
    one whole detection of the device-resident stack (smoothing, weighted gradients,
    shifted comparisons of neighbours one and two apart, pair sums); value =
    projections examined per second.  e2e = the public call with the host stack
    (upload, detection, errors back, ranking)."""
    import torch

    from graptor_gb300 import badproj
    torch.cuda.set_device(local)
    NA, Nz, Nx = W["nang"], W["N"], W["N"]
    rng = np.random.default_rng(rank)
    zz, xx = np.meshgrid(np.arange(Nz), np.arange(Nx), indexing="ij")
    base = np.zeros((Nz, Nx))
    for _ in range(12):
        cz, cx, r = rng.uniform(0.2, 0.8) * Nz, rng.uniform(0.2, 0.8) * Nx, rng.uniform(0.04, 0.12) * Nx
        base += rng.uniform(0.5, 2.0) * ((zz - cz) ** 2 + (xx - cx) ** 2 < r * r)
    data = np.stack([np.roll(base, int(rng.integers(-3, 4)), axis=1) for _ in range(NA)])
    data += 0.05 * rng.random(data.shape)
    for k in rng.choice(NA, 4, replace=False):
        data[k] = np.roll(data[k], Nz // 5, axis=0) + 0.8 * rng.random((Nz, Nx))
    d = badproj.upload(data, local)
    S, Wg = badproj.stages(d)
    r1 = int(min(S.shape[1], S.shape[2]) / 10)
    r2 = int(r1 * 1.5)
    nz, nx = Wg.shape[1], Wg.shape[2]
    for _ in range(args.warmup):
        badproj.detect(d)
    torch.cuda.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # 256 MB > L2, between steps
    st = torch.cuda.current_stream()
    step_ms, cmp_ms = [], []
    barrier(world)
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(st)
            S, Wg = badproj.stages(d)
            e[1].record(st)
            badproj.pair_errors(Wg, 1, r1)
            badproj.pair_errors(Wg, 2, r2)
            e[2].record(st)
            e[2].synchronize()
            step_ms.append(e[0].elapsed_time(e[2]))
            cmp_ms.append(e[1].elapsed_time(e[2]))
    torch.cuda.synchronize()
    ms = max_over_ranks(sum(step_ms), world)
    clocks = clk.summary()
    if rank != 0:
        return None
    value = world * NA * args.steps / (ms / 1e3)
    # e2e: the public call with the host stack
    badproj.find_bad_projections("stack", None, 0.1, data=data, device=local)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(e2e_steps):
        with contextlib.redirect_stdout(io.StringIO()):
            badproj.find_bad_projections("stack", None, 0.1, data=data, device=local)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    # roofline of the comparison kernel: FP32 issue (subtract + minimum per shift and direction)
    ops = badproj_lane_ops(nz, nx, r1, NA - 1) + badproj_lane_ops(nz, nx, r2, NA - 2)
    cmp = statistics.median(cmp_ms)
    nominal = 152 * 128 * 2.07e9  # lanes x maximum SM clock
    roof = {"bound": "fp32-issue", "kernel": "k_compare", "achieved": ops / (cmp / 1e3), "peak": nominal,
            "unit": "lane-op/s", "frac": ops / (cmp / 1e3) / nominal, "peak_source": "nominal (152 SMs x 128 lanes x 2.07 GHz)",
            "traffic": None, "algorithmic_ops_per_step": ops, "ms_per_step": cmp}
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import badproj as obad
        t0 = time.perf_counter()
        Sh, Wh = obad.stages(data[:8])
        t_stage = (time.perf_counter() - t0) / 8
        k = 3
        t0 = time.perf_counter()
        obad.pair_errors(Wh[:k + 1], 1, r1)
        t1 = (time.perf_counter() - t0) / k
        t0 = time.perf_counter()
        obad.pair_errors(Wh[:k + 2], 2, r2)
        t2 = (time.perf_counter() - t0) / k
        est = t_stage * NA + t1 * (NA - 1) + t2 * (NA - 2)
        cpu = {"value": NA / est, "unit": "projections/s", "cores": 1, "kind": "port",
               "sample": f"oracle (NumPy) stages of 8 projections and {k} pairs at each offset, scaled to {NA} projections"}
    return {"metric": "projections/s", "value": value, "unit": "projections/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (box sums f64)",
            "data": "synthetic (seeded blobs, shifts, noise, 4 corrupted projections)",
            "config": {"workload": f"bad-projection detection: {NA} projections x {Nz} slices x {Nx} detector columns, "
                                   f"search radius {r1} / {r2}",
                       "l2": "256 MB written between steps (L2 flushed)"},
            "e2e": {"value": NA / e2e_s, "unit": "projections/s", "h2d_bytes_per_step": int(data.nbytes),
                    "d2h_bytes_per_step": 8 * (2 * NA - 3)},
            "gpu_launches": 6 * args.steps, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--nz", type=int, default=None,
                    help="slices per channel (default 60); smaller cases for profiler captures")
    ap.add_argument("--n", type=int, default=None, help="image side (default 256); profiler captures")
    ap.add_argument("--nang", type=int, default=None,
                    help="projection angles (default 71; the 768^2 x 384 large run uses 141)")
    ap.add_argument("--workload", default="coupled3d", choices=["coupled3d", "batched", "warmstart", "gapsweep", "unet", "subsample", "badproj"],
                    help="coupled3d: the 3-D 4-channel workload (default); batched: 64 uneven problems; "
                         "warmstart: time to gap, cold start against learned warm start + batch; gapsweep: gap "
                         "against iterations for several primal weights; unet: the "
                         "warm-start network's forward pass; subsample: the two-resolution solver; badproj: "
                         "bad-projection detection on nang projections x N x N")
    ap.add_argument("--batch", type=int, default=64, help="problems per rank for --workload batched")
    ap.add_argument("--batch-sizes", default="uneven", choices=sorted(BATCH_SIZES),
                    help="--workload batched: the uneven config-3 sizes or many small problems")
    ap.add_argument("--seeds", type=int, default=8, help="held-out problems per rank for --workload warmstart")
    ap.add_argument("--primal-weights", default="1,3,10", help="--workload gapsweep: primal weights to sweep")
    ap.add_argument("--pweight", type=float, default=1.0,
                    help="--workload warmstart: primal weight of both arms after the pre-iterations")
    ap.add_argument("--check-every", type=int, default=None, help="--workload warmstart: iterations between gap checks")
    ap.add_argument("--max-iters", type=int, default=None, help="--workload warmstart: iteration cap per problem")
    ap.add_argument("--precise", action="store_true",
                    help="--workload gapsweep / warmstart: u held as two floats (gt_set_precise_primal)")
    ap.add_argument("--fields", default="u", help="--workload warmstart: the fields the network predicts (u or u,v)")
    ap.add_argument("--tol", type=float, default=None, help="--workload warmstart: relative gap tolerance (1e-2)")
    ap.add_argument("--ttg-seeds", type=int, default=4,
                    help="held-out problems of the time-to-gap object in the default line (0: leave it out)")
    ap.add_argument("--weights", default=None, help="network weights for --workload warmstart")
    ap.add_argument("--coupling", default="FROB", choices=["FROB", "UNCORR", "NUCL"],
                    help="channel coupling of the coupled3d workload (default FROB, the headline)")
    ap.add_argument("--fwd-shape", type=int, default=None,
                    help="force the forward projector's launch shape (no autotuning); profiler captures")
    ap.add_argument("--bp-shape", type=int, default=None, help="force the back projector's launch shape")
    ap.add_argument("--dual-shape", type=int, default=None, help="force the dual kernel's launch shape")
    ap.add_argument("--schedule", type=int, default=None, choices=[0, 1, 2],
                    help="force the iteration schedule (0: primal update after the projectors, 1: its p half beside "
                         "them, 2: its p half fused into the next dual kernel)")
    ap.add_argument("--quick", action="store_true",
                    help="only the device-timed region (no e2e, kernel timing or CPU baseline): profiler runs")
    args = ap.parse_args()
    if args.workload == "warmstart":  # --n / --nz size the warm-start problems instead
        if args.nz:
            WARM["Nz"] = int(args.nz)
        if args.n:
            WARM["N"] = int(args.n)
        args.nz = args.n = None
    if args.nz:
        W["Nz"] = int(args.nz)
    if args.n:
        W["N"] = int(args.n)
    W["coupling"] = args.coupling
    if args.nang:
        W["nang"] = int(args.nang)
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == "batched":
        out = run_batched(args, rank, world, local)
    elif args.workload == "warmstart":
        out = run_warmstart(args, rank, world, local)
    elif args.workload == "gapsweep":
        out = run_gapsweep(args, rank, world, local)
    elif args.workload == "unet":
        out = run_unet(args, rank, world, local)
    elif args.workload == "subsample":
        out = run_subsample(args, rank, world, local)
    elif args.workload == "badproj":
        out = run_badproj(args, rank, world, local)
    else:
        from oracle import oracle as O
        O.build()  # the CPU-baseline leg needs the oracle library (built before any GPU work)
        out = run_ours(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
