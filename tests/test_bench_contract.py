"""The bench JSON contract on the CPU: the reference arm's line (the oracle on the
host cores) carries the keys the harness reads, at a tiny size."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    sys.path.insert(0, ROOT)
    import bench
    saved = dict(bench.W)
    try:
        bench.W.update(N=16, Nz=4, nang=8)

        class A:
            steps, warmup = 2, 1
        out = bench.run_reference(A(), 0, 1)
    finally:
        bench.W.clear()
        bench.W.update(saved)
    json.dumps(out)  # serialisable
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in out, k
    assert out["impl"] == "reference" and out["value"] > 0 and out["steps"] == 2
    assert out["cpu_baseline"]["kind"] == "port" and out["cpu_baseline"]["cores"] >= 1
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["value"] == out["value"]
    assert "workload" in out["config"]


def test_bench_cli_options():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0
    for opt in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--coupling", "--fwd-shape", "--quick"):
        assert opt in r.stdout, opt


def test_badproj_work_count():
    """The comparison kernel's algorithmic count (roofline numerator) against a
    direct count of (pixel, shift, direction) triples times two operations."""
    sys.path.insert(0, ROOT)
    import bench
    for nz, nx, r, pairs in ((20, 30, 3, 4), (9, 33, 4, 1), (40, 40, 0, 2)):
        direct = 0
        for y in range(r, nz - r):
            for x in range(r, nx - r):
                direct += sum(1 for k in range(-r, r + 1) for l in range(-r, r + 1)) * 2 * 2
        assert bench.badproj_lane_ops(nz, nx, r, pairs) == pairs * direct
