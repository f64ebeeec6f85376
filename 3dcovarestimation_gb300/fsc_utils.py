"""Fourier-shell statistics on the GPU: drop-in for ``cov3d.fsc_utils`` (reference
``fsc_utils.py``), used by the half-set regularisers of the covariance and the mean.

Shell i of an L^d grid holds the radii in (i - 1/2, i + 1/2) of the centered integer grid
ceil(k - L/2), the last shell (i - 1/2, i + 1) (``FourierShell.radial_avg_interval``); no radius
is a half integer, so shell = round(radius) capped at the last one.  Averages are scatter-adds
over a cached shell-index map; every function takes CUDA tensors (there is no CPU path).
"""

import math
from functools import lru_cache
from typing import Tuple, Union

import torch

from .projection_funcs import centered_fft3


@lru_cache(maxsize=32)
def _shells(L: int, dim: int, device_str: str):
    dev = torch.device(device_str)
    g = torch.ceil(torch.arange(-L / 2, L / 2, dtype=torch.float64))
    grids = torch.meshgrid(*([g] * dim), indexing="ij")
    rad = torch.sqrt(sum(x * x for x in grids))
    ns = int(math.ceil(rad.max().item()))
    idx = torch.clamp(torch.floor(rad + 0.5), max=ns - 1).to(torch.int64).reshape(-1)
    size = torch.bincount(idx, minlength=ns).to(torch.float64)
    return idx.to(dev), size.to(dev), ns


def _require_cuda(t):
    if not t.is_cuda:
        raise ValueError("fsc_utils takes CUDA tensors (no CPU path)")


def shell_index(L: int, dim: int = 3, device=None):
    """(shell of every grid point, flattened; shell sizes; number of shells)."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    return _shells(int(L), int(dim), str(dev))


def _average(x: torch.Tensor, dim: int) -> torch.Tensor:
    """Shell averages over the last ``dim`` axes of x: (..., S)."""
    _require_cuda(x)
    L = x.shape[-1]
    idx, size, ns = shell_index(L, dim, x.device)
    flat = x.reshape(x.shape[:-dim] + (-1,))
    out = torch.zeros(flat.shape[:-1] + (ns,), dtype=x.dtype, device=x.device)
    out.index_add_(-1, idx, flat)
    return out / size.to(out.real.dtype if out.is_complex() else out.dtype)


def average_fourier_shell(*spectrum_signals: torch.Tensor) -> torch.Tensor:
    """Shell average of each signal (fsc_utils.py:116-135, 199-208): (S,) for one signal,
    (n, S) for several (or for one batched signal)."""
    s = spectrum_signals[0]
    dim = s.ndim
    x = torch.stack(spectrum_signals) if len(spectrum_signals) > 1 else s.unsqueeze(0)
    out = _average(x, dim)
    return out[0] if out.shape[0] == 1 else out


def rpsd(*signals: torch.Tensor) -> torch.Tensor:
    """Radial power spectral density (fsc_utils.py:137-147, 211-220)."""
    x = torch.stack(signals) if len(signals) > 1 else signals[0].unsqueeze(0)
    out = _average(torch.abs(centered_fft3(x)) ** 2, 3)
    return out[0] if out.shape[0] == 1 else out


def expand_fourier_shell(shells: torch.Tensor, L: int, dim: int) -> torch.Tensor:
    """Shell values -> full grid (fsc_utils.py:166-184, 223-234)."""
    _require_cuda(shells)
    idx, _, ns = shell_index(L, dim, shells.device)
    sh = shells.unsqueeze(0) if shells.ndim == 1 else shells
    pad = torch.zeros(sh.shape[:-1] + (max(ns, sh.shape[-1]),), dtype=sh.dtype, device=sh.device)
    pad[..., : min(ns, sh.shape[-1])] = sh[..., :ns]
    out = pad[..., idx].reshape(sh.shape[:-1] + (L,) * dim)
    return out[0] if out.shape[0] == 1 else out


def upsample_and_expand_fourier_shell(shells: torch.Tensor, L: int, dim: int) -> torch.Tensor:
    """Linear resampling (align_corners=False) of the shell profile to the shell count of an
    L^dim grid, then expansion (fsc_utils.py:237-255)."""
    ns = shell_index(L, dim, shells.device)[2]
    x = shells.unsqueeze(0).unsqueeze(0) if shells.ndim == 1 else shells.unsqueeze(0)
    up = torch.nn.functional.interpolate(x, size=ns, mode="linear", align_corners=False).squeeze()
    return expand_fourier_shell(up, L, dim)


def sum_over_shell(shell: torch.Tensor, L: int, dim: int) -> torch.Tensor:
    """Sum of shell values weighted by shell sizes (fsc_utils.py:149-164, 258-269)."""
    size = shell_index(L, dim, shell.device)[1].to(shell.dtype)
    return torch.sum(shell * size, dim=-1)


def vol_fsc(signal1: torch.Tensor, signal2: torch.Tensor) -> torch.Tensor:
    """Fourier shell correlation of two volumes (fsc_utils.py:272-291)."""
    f1, f2 = centered_fft3(signal1), centered_fft3(signal2)
    c, p1, p2 = _average(torch.stack([torch.real(f1 * torch.conj(f2)), torch.abs(f1) ** 2, torch.abs(f2) ** 2]), 3)
    return c / torch.sqrt(p1 * p2)


def covar_correlate(fourier_eigenvecs1: torch.Tensor, fourier_eigenvecs2: torch.Tensor,
                    return_shell_size: bool = False) -> Union[torch.Tensor, Tuple[torch.Tensor, torch.Tensor]]:
    """sum_i s_i^T conj(s_i), s_i the shell averages of eigvec1[i] * conj(eigvec2)
    (fsc_utils.py:312-340)."""
    _, size, ns = shell_index(fourier_eigenvecs1.shape[-1], 3, fourier_eigenvecs1.device)
    out = torch.zeros((ns, ns), dtype=fourier_eigenvecs1.dtype, device=fourier_eigenvecs1.device)
    for i in range(fourier_eigenvecs1.shape[0]):
        s = _average(fourier_eigenvecs1[i].unsqueeze(0) * torch.conj(fourier_eigenvecs2), 3)
        out += s.T @ s.conj()
    if return_shell_size:
        return out, size.to(out.real.dtype)
    return out


def covar_rpsd(eigenvectors: torch.Tensor, from_fourier: bool = False) -> torch.Tensor:
    """Radial PSD of a covariance given by its eigenvectors (fsc_utils.py:294-309)."""
    f = eigenvectors if from_fourier else centered_fft3(eigenvectors)
    c, size = covar_correlate(f, f, return_shell_size=True)
    return c.real * torch.outer(size, size)


def covar_fsc(eigenvecs1: torch.Tensor, eigenvecs2: torch.Tensor) -> torch.Tensor:
    """Fourier shell correlation of two covariances (fsc_utils.py:343-367)."""
    f1, f2 = centered_fft3(eigenvecs1), centered_fft3(eigenvecs2)
    c = covar_correlate(f1, f2).real
    r1 = covar_correlate(f1, f1).real
    r2 = covar_correlate(f2, f2).real
    bottom = torch.sqrt((r1 / r1[0, 0]) * (r2 / r2[0, 0])) * torch.sqrt(r1[0, 0]) * torch.sqrt(r2[0, 0])
    return c / bottom
