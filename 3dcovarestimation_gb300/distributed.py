"""Data-parallel helpers: the path shards by images, one process per GPU.

cov-SGD: every rank runs the fused step on its own image shard; the gradient of the Covar
parameters (r * L^3 + r floats) is averaged once per step before identical optimizer updates
(the reference's DDP step, ``covar_distributed.py:100-105``).  The costs are means over each
rank's images, so ranks with unequal shards weight their contribution by their image count.
Mean: every rank backprojects its images into partial rhs / lhs grids, which are summed once
before a replicated CG; with half-sets, the ranks split into two groups whose sums are the two
half-set backprojections (``reconstruct_mean_from_halfsets_DDP``, ``mean.py:294-356``).  With
one process these are no-ops.
"""

from typing import List, Optional, Sequence

import torch
import torch.distributed as dist


def world():
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def shard(n_items: int, rank: int, world_size: int):
    """Contiguous [lo, hi) share of n_items for rank (sizes differ by at most one)."""
    base, extra = divmod(n_items, world_size)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _real_view(t):
    return torch.view_as_real(t) if t.is_complex() else t


def allreduce_mean_(tensors: Sequence[torch.Tensor], count: Optional[float] = None, group=None):
    """Average tensors across ranks in place.  Without ``count`` every rank weighs the same; with
    ``count`` (the number of items this rank's tensors average over) the result is
    sum_i count_i t_i / sum_i count_i, the mean over all items when shards are unequal."""
    if world() == 1:
        return tensors
    if count is None:
        w = dist.get_world_size(group)
        for t in tensors:
            dist.all_reduce(_real_view(t), group=group)
            t /= w
        return tensors
    total = torch.tensor([float(count)], dtype=torch.float64, device=tensors[0].device)
    dist.all_reduce(total, group=group)
    for t in tensors:
        t *= float(count)
        dist.all_reduce(_real_view(t), group=group)
        t /= float(total)
    return tensors


def allreduce_sum_(tensors: Sequence[torch.Tensor], group=None):
    """Sum tensors across ranks in place (partial mean grids).  Complex tensors are reduced
    through their real view."""
    if world() == 1:
        return tensors
    for t in tensors:
        dist.all_reduce(_real_view(t), group=group)
    return tensors


def halfset_groups(ranks: Optional[List[int]] = None):
    """The two half-set process groups: the first and second half of ``ranks`` (all ranks by
    default), as ``mean.py:325-327`` forms them.  Returns (group1, group2, ranks)."""
    if ranks is None:
        ranks = list(range(dist.get_world_size()))
    h = len(ranks) // 2
    return dist.new_group(ranks=ranks[:h]), dist.new_group(ranks=ranks[h:]), ranks


def reduce_halfset_backprojections(rhs: torch.Tensor, lhs: torch.Tensor, L: int, ranks: Optional[List[int]] = None):
    """Sum each half-set group's partial backprojections (rhs, lhs on the fine grid), form the
    group's quick mean crop(ifft(rhs / (lhs + 0.1))) as ``mean.py:333-334`` does, and give every
    rank both halves: returns ((mean1, rhs1, lhs1), (mean2, rhs2, lhs2)).  ``rhs`` / ``lhs`` are
    reduced in place."""
    from .projection_funcs import centered_ifft3

    g1, g2, ranks = halfset_groups(ranks)
    rank = dist.get_rank()
    grp = g1 if rank in ranks[: len(ranks) // 2] else g2
    allreduce_sum_([rhs, lhs], group=grp)
    mean = centered_ifft3(rhs / (lhs + 1e-1), cropping_size=(L,) * 3).real.contiguous()
    halves = ([], [])
    for t in (mean, rhs, lhs):
        parts = [torch.zeros_like(t) for _ in range(dist.get_world_size())]
        dist.all_gather([_real_view(p) for p in parts], _real_view(t.contiguous()))
        halves[0].append(parts[ranks[0]])
        halves[1].append(parts[ranks[-1]])
    dist.destroy_process_group(g1)
    dist.destroy_process_group(g2)
    return tuple(halves[0]), tuple(halves[1])
