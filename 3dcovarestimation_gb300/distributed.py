"""Data-parallel helpers: the path shards by images, one process per GPU.

cov-SGD: every rank runs the fused step on its own image batch; the gradient of the Covar
parameters (r * L^3 + r floats) is averaged once per step before identical optimizer updates
(the reference's DDP step, ``covar_distributed.py:100-105``).  Mean: every rank backprojects
its images into partial rhs / lhs grids, which are summed once before a replicated CG (the
reference's ``reconstruct_mean_from_halfsets_DDP``, ``mean.py:294-356``, sums them the same
way).  With one process these are no-ops.
"""

import torch
import torch.distributed as dist


def world():
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def shard(n_items: int, rank: int, world_size: int):
    """Contiguous [lo, hi) share of n_items for rank (sizes differ by at most one)."""
    base, extra = divmod(n_items, world_size)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def allreduce_mean_(tensors):
    """Average tensors across ranks in place (gradients)."""
    w = world()
    if w == 1:
        return tensors
    for t in tensors:
        dist.all_reduce(t)
        t /= w
    return tensors


def allreduce_sum_(tensors):
    """Sum tensors across ranks in place (partial mean grids).  Complex tensors are reduced
    through their real view."""
    if world() == 1:
        return tensors
    for t in tensors:
        dist.all_reduce(torch.view_as_real(t) if t.is_complex() else t)
    return tensors
