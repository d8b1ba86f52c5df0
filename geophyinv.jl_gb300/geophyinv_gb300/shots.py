"""Shot (supersource) partitioning over ranks and the gradient sum.

The reference splits the supersources over Distributed workers in
contiguous chunks (`sschunks`, src/fdtd/fdtd.jl:246-255) and sums the
per-worker gradients into a SharedArray (`sum_grads!`,
src/fdtd/gradient.jl:2-14).  Here one rank drives one GPU; shots are
independent, so the forward path needs no communication and a gradient is
summed once per `gradient!` call.
"""
from fractions import Fraction


def sschunks(nss, nworker):
    """Contiguous 0-based [start, stop) ranges of supersources per worker:
    the bounds round(range(0, nss, length = nworker + 1)) with ties to even,
    as Julia's round(Int, x)."""
    if nss < 1 or nworker < 1:
        raise ValueError("nss and nworker must be positive")
    nworker = min(nss, nworker)
    ssi = [round(Fraction(nss * i, nworker)) for i in range(nworker + 1)]
    return [(ssi[i], ssi[i + 1]) for i in range(nworker)]


def my_shots(nss, rank, world):
    """The supersources of `rank` among `world` ranks (empty when the rank has
    none)."""
    chunks = sschunks(nss, world)
    return range(*chunks[rank]) if rank < len(chunks) else range(0)


def rank_world(group=None):
    """(rank, world size) of an initialised torch.distributed group, else
    (0, 1)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def reduce_scalar(x, group=None, op="sum"):
    """Sum (or max) of a per-rank float (a misfit) over the ranks, in
    float64."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return x
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM if op == "sum" else dist.ReduceOp.MAX, group=group)
    return float(t.item())


def reduce_gradient(g, group=None):
    """Sum a per-rank gradient (numpy array or torch tensor) over the ranks of
    `group` in place and return it; a no-op without an initialised process
    group."""
    import numpy as np
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return g
    t = torch.from_numpy(np.ascontiguousarray(g)) if isinstance(g, np.ndarray) else g
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    if isinstance(g, np.ndarray):
        g[...] = t.numpy().reshape(g.shape)
    return g
