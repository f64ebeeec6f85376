"""Small helpers of the reference's ``cov3d/utils.py`` that the hot path's callers use: the
soft-edged kernel of the image preprocessing (``utils.py:258-300``) and the subspace metrics
used to validate the BF16 path (principal angles, ``utils.py:152-162``)."""

import math

import torch

from .projection_funcs import centered_fft2, centered_fft3


def _grid_radius(L: int, dim: int, shifted: bool) -> torch.Tensor:
    """Radius on the unnormalised grid ceil(arange(-L/2, L/2)) (shifted by 1/2 for even L when
    ``shifted``), the definition of ASPIRE's ``grid_2d`` / ``grid_3d``, in their default float32."""
    g = torch.ceil(torch.arange(-L / 2, L / 2, dtype=torch.float64))
    if shifted and L % 2 == 0:
        g = torch.arange(-L / 2 + 0.5, L / 2 + 0.5, dtype=torch.float64)
    axes = torch.meshgrid(*([g.to(torch.float32)] * dim), indexing="ij")
    return torch.sqrt(sum(a * a for a in axes)).to(torch.float64)


def soft_edged_kernel(radius: float, L: int, dim: int, radius_backoff: int = 2, in_fourier: bool = False):
    """Normalised disc (dim 2) or ball (dim 3) of the given radius with a raised-cosine edge of
    width ``radius_backoff`` (reference ``utils.py:258-300``; radius below 3 is raised to 3)."""
    radius = max(radius, 3)
    r = _grid_radius(L, dim, shifted=True)
    r0 = radius - radius_backoff
    k = torch.zeros_like(r)
    k[r < r0] = 1
    edge = (r >= r0) & (r < radius)
    r32 = r.to(torch.float32)  # the edge profile in float32, as the reference evaluates it
    k = torch.where(edge, ((1 + torch.cos(math.pi * (r32 - r0) / (radius - r0))) / 2).to(torch.float64), k)
    k = k / k.sum()
    if in_fourier:
        k = centered_fft2(k) if dim == 2 else centered_fft3(k)
    return k


def principal_angles(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Principal angles (radians, ascending) between the column spans of a (n, k) and b (n, k)
    (the metric of the reference's ``utils.py:152-162``)."""
    qa, _ = torch.linalg.qr(a.to(torch.float64))
    qb, _ = torch.linalg.qr(b.to(torch.float64))
    s = torch.linalg.svdvals(qa.T @ qb).clamp(-1.0, 1.0)
    return torch.arccos(s).flip(0)
