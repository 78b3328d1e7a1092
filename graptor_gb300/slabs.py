"""Z-slab decomposition of one volume over ranks, and its halo exchange.

The solver's work shards across GPUs in two ways.  Independent problems (batches,
warm-start seeds) need no communication: each rank runs its own (``bench.py``
runs such replicas).  One large volume splits into slabs of whole z-planes, every
channel of a plane on the same rank: the projectors act slice by slice (parallel
beam) and the channel coupling is per voxel, so both stay local, and only the
z-stencils reach across a slab boundary -- one plane of four fields per
iteration, in the order the iteration uses them:

  * ubar at z + 1  for the forward z-difference of grad  (update_v, 3-D :615-634)
  * pbar at z - 1  for the backward z-difference of E   (update_w, :637-660)
  * v at z - 1     for the backward z-difference of div (update_u, :706-729)
  * w at z + 1     for the forward z-difference of div_sym (update_p, :734-757)

(radon_tgv_primal_dual_3d.py).  :func:`fetch_upper` / :func:`fetch_lower` are
those exchanges over ``torch.distributed`` point-to-point (gloo on host tensors,
NCCL on device tensors); the slab plan is :func:`slab_ranges`.  One box of this
build has one GPU, so the decomposition runs on CPU ranks in the tests, where a
slab-split iteration reproduces the single-process iteration exactly.
"""
from __future__ import annotations


def slab_ranges(Nz: int, world: int):
    """[(z0, z1)] per rank: consecutive, as even as possible, every rank at least one plane."""
    if world < 1 or Nz < world:
        raise ValueError(f"cannot split {Nz} planes over {world} ranks")
    base, extra = divmod(Nz, world)
    out, z = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append((z, z + n))
        z += n
    return out


def _exchange(send, to_rank, from_rank):
    import torch
    import torch.distributed as dist
    reqs = []
    recv = None
    if to_rank is not None:
        reqs.append(dist.isend(send.contiguous(), to_rank))
    if from_rank is not None:
        recv = torch.empty_like(send)
        reqs.append(dist.irecv(recv, from_rank))
    for q in reqs:
        q.wait()
    return recv


def fetch_upper(first_plane, rank: int, world: int):
    """Send this slab's first plane to the rank below and return the first plane of
    the rank above (None on the last rank): the z + 1 halo."""
    return _exchange(first_plane, rank - 1 if rank > 0 else None, rank + 1 if rank < world - 1 else None)


def fetch_lower(last_plane, rank: int, world: int):
    """Send this slab's last plane to the rank above and return the last plane of the
    rank below (None on rank 0): the z - 1 halo."""
    return _exchange(last_plane, rank + 1 if rank < world - 1 else None, rank - 1 if rank > 0 else None)
