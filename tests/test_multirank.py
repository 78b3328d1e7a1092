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


def _zext(a, lower, upper, rank, world):
    """a[..., C, nz, N, N] with a plane below / above where this slab has a neighbour:
    the neighbour's plane where the stencil reads it, zeros where it only keeps the
    array's boundary rule off the slab's own first / last plane.  Returns (ext, offset)."""
    import numpy as np
    parts, off = [], 0
    if rank > 0:
        parts.append(lower[..., None, :, :] if lower is not None else np.zeros_like(a[..., :1, :, :]))
        off = 1
    parts.append(a)
    if rank < world - 1:
        parts.append(upper[..., None, :, :] if upper is not None else np.zeros_like(a[..., :1, :, :]))
    return np.concatenate(parts, axis=-3), off


def _slab_worker(rank, world, port, q, iters):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import numpy as np
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from graptor_gb300 import slabs
    from oracle import fp64 as F
    dim, N, Nz, C, nang, step = 3, 10, 7, 2, 9, 2.0
    rng = np.random.default_rng(5)
    ang = np.linspace(0.2, 2.9, nang)
    f = rng.uniform(0.0, 3.0, (C * Nz, nang, N))
    mu, ne, alpha, cpl = np.array([0.3, 0.1]), 12.0, (4.0, 1.0), "FROB"
    full = F.Solver64(dim, N, Nz, C, N, ang, f, alpha, mu, ne, "KL", "TGV", cpl, step, feasible=False)
    z0, z1 = slabs.slab_ranges(Nz, world)[rank]
    nz = z1 - z0
    sg, tau, a0, a1, R = full.sigma, full.tau, full.a0, full.a1, full.R
    wb, _ = F.w_weights(dim, cpl)
    fl = f.reshape(C, Nz, nang, N)[:, z0:z1]
    m = np.repeat(mu, nz).reshape(C, nz, 1, 1)
    u, ubar = np.zeros((C, nz, N, N)), np.zeros((C, nz, N, N))
    p, pbar, v = (np.zeros((3, C, nz, N, N)) for _ in range(3))
    w = np.zeros((6, C, nz, N, N))
    lam = np.zeros((C, nz, nang, N))
    K = lambda x: (R @ x.reshape(C * nz, N * N).T).T.reshape(C, nz, nang, N) / ne  # noqa: E731
    KT = lambda y: (R.T @ y.reshape(C * nz, -1).T).T.reshape(C, nz, N, N) / ne  # noqa: E731
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a))  # noqa: E731
    flat = lambda a, n: a.reshape(a.shape[:-4] + (C * n, N, N))  # noqa: E731
    for _ in range(iters):
        # v: grad(ubar) reads ubar(z+1)
        up = slabs.fetch_upper(T(ubar[:, 0]), rank, world)
        e, o = _zext(ubar, None, None if up is None else up.numpy(), rank, world)
        n = e.shape[-3]
        g = F.grad(flat(e, n), dim, n, step).reshape(3, C, n, N, N)[:, :, o:o + nz]
        v = F.project(flat(v + sg * (g - pbar), nz), a1, C, nz, cpl).reshape(3, C, nz, N, N)
        # w: E(pbar) reads pbar(z-1)
        lo = slabs.fetch_lower(T(pbar[:, :, -1]), rank, world)
        e, o = _zext(pbar, None if lo is None else lo.numpy(), None, rank, world)
        n = e.shape[-3]
        eg = F.sym_grad(flat(e, n), dim, n, step).reshape(6, C, n, N, N)[:, :, o:o + nz]
        w = F.project(flat(w + sg * eg, nz), a0, C, nz, cpl, wb).reshape(6, C, nz, N, N)
        # lambda: slice-local
        s = lam + sg * K(ubar)
        wv = s - m
        lam = s - 0.5 * (wv + np.sqrt(wv * wv + 4 * (sg / ne) * fl * m))
        # u: div(v) reads v(z-1)
        lo = slabs.fetch_lower(T(v[:, :, -1]), rank, world)
        e, o = _zext(v, None if lo is None else lo.numpy(), None, rank, world)
        n = e.shape[-3]
        d = F.div(flat(e, n), dim, n, step).reshape(C, n, N, N)[:, o:o + nz]
        un = np.maximum(0.0, u + tau * (d - KT(lam)))
        ubar, u = 2 * un - u, un
        # p: div_sym(w) reads w(z+1)
        up = slabs.fetch_upper(T(w[:, :, 0]), rank, world)
        e, o = _zext(w, None, None if up is None else up.numpy(), rank, world)
        n = e.shape[-3]
        ds = F.div_sym(flat(e, n), dim, n, step).reshape(3, C, n, N, N)[:, :, o:o + nz]
        pn = p + tau * (v + ds)
        pbar, p = 2 * pn - p, pn
    parts = [None] * world
    dist.all_gather_object(parts, u)
    if rank == 0:
        whole = np.concatenate(parts, axis=1).reshape(C * Nz, N, N)
        ref = full.run(iters).u
        q.put((float(np.abs(whole - ref).max()), float(np.abs(ref).max())))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_z_slab_split_matches_single_process(world):
    """One 3-D TGV-KL volume (2 channels, 7 planes) split into z-slabs over gloo
    ranks, each iteration exchanging one plane of ubar, pbar, v and w with the
    neighbouring slabs (graptor_gb300.slabs), reproduces the single-process FP64
    iteration (oracle/fp64.py) bit for bit after 25 iterations."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_slab_worker, args=(r, world, port, q, 25)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    diff, scale = q.get()
    assert scale > 0 and diff == 0.0, (diff, scale)  # the same operations on the same values: bit for bit


def test_slab_ranges():
    from graptor_gb300.slabs import slab_ranges
    assert slab_ranges(7, 2) == [(0, 4), (4, 7)]
    assert slab_ranges(7, 3) == [(0, 3), (3, 5), (5, 7)]
    assert slab_ranges(384, 8)[-1] == (336, 384)
    with pytest.raises(ValueError):
        slab_ranges(2, 3)
