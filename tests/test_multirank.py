"""Multi-process path of bench.py on CPU ranks (gloo, world size 2).

The solver shards only as independent replicas (each rank its own problems, no
collective on the data path); the harness's host logic -- rendezvous, barrier,
max-over-ranks timing, rank-0-only reference arm -- is what these tests cover."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    r, w, local = bench.dist_setup(world)
    assert (r, w) == (rank, world) and dist.get_backend() == "gloo"
    bench.barrier(w)
    t = bench.max_over_ranks(float(rank + 1) * 0.5, w)
    # each rank solves its own replica on the CPU oracle: no data-path collective
    import numpy as np
    from oracle import oracle as O
    ofs = O.radon_struct(np.linspace(0.3, 2.8, 6), 8, 8)
    f = np.full((2, 6, 8), 1.0 + rank, np.float32)
    u = O.Solver(3, 8, 2, 1, 8, ofs, f, (4, 1), [0.2], 10.0).run(3).u
    total = bench.max_over_ranks(float(u.sum()), w)
    q.put((rank, t, float(u.sum()), total))
    dist.destroy_process_group()


def test_two_gloo_ranks_replicas_and_max_timing():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    assert [r[1] for r in res] == [1.0, 1.0]          # max over ranks of 0.5, 1.0
    assert res[0][2] != res[1][2]                      # independent replicas
    assert res[0][3] == res[1][3] == max(res[0][2], res[1][2])


def _ref_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    bench.W.update(N=16, Nz=4, nang=8)
    r, w, _ = bench.dist_setup(world)

    class A:
        steps, warmup = 2, 1
    out = bench.run_reference(A(), r, w)
    q.put((rank, out is None, None if out is None else out["impl"]))
    dist.destroy_process_group()


def test_reference_arm_runs_on_rank_zero_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ref_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    assert res[0] == (0, False, "reference")
    assert res[1] == (1, True, None)
