"""Dataset gains on the GPU (reference ``CovarDataset.get_total_gain`` /
``get_total_covar_gain``, ``dataset.py:322-421``): the diagonal of sum_i P_i^T P_i on the
Fourier grid and its Fourier-shell-pair version used by the half-set covariance regulariser.

``dataset`` is anything the reference's CovarDataset contract covers for these two methods:
``dataset[i:j]`` returns ``(images, pts_rot, filters, idx)`` and ``dataset.resolution`` is L.
The backprojections run in the library's spreading kernels (nearest plan, upsampling 1).
"""

from typing import Optional

import torch

from .fsc_utils import average_fourier_shell
from .nufft_plan import NufftPlanDiscretized
from .projection_funcs import im_backward


def _device(device):
    return torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())


def get_total_gain(dataset, batch_size: int = 1024, device: Optional[torch.device] = None) -> torch.Tensor:
    """|sum_i im_backward(ctf_i, ctf_i)| per batch, summed, / L: the total gain of every
    frequency (reference ``dataset.py:322-356``)."""
    L = dataset.resolution
    dev = _device(device)
    plan = NufftPlanDiscretized((L,) * 3, upsample_factor=1, mode="nearest", use_half_grid=False)
    gain = torch.zeros((L,) * 3, device=dev, dtype=torch.float32)
    for i in range(0, len(dataset), batch_size):
        _, pts, filters, _ = dataset[i: min(i + batch_size, len(dataset))]
        pts = pts.to(device=dev, dtype=torch.float32)
        filters = filters.to(device=dev, dtype=torch.float32)
        plan.setpts(pts)
        gain += im_backward(torch.complex(filters, torch.zeros_like(filters)), plan, filters,
                            fourier_domain=True).squeeze().abs()
    return gain / L


def get_total_covar_gain(dataset, batch_size: Optional[int] = None,
                         device: Optional[torch.device] = None) -> torch.Tensor:
    """sum_i s_i^T s_i with s_i the Fourier-shell averages of |P_i^T (ctf_i^2)| / L^2 (the
    per-image adjoint, Nyquist row/column zeroed): the gain of every shell pair in the
    covariance least-squares problem (reference ``dataset.py:358-421``)."""
    L = dataset.resolution
    dev = _device(device)
    plan = NufftPlanDiscretized((L,) * 3, upsample_factor=1, mode="nearest", use_half_grid=False)
    batch_size = batch_size or 256
    out = None
    for i in range(0, len(dataset), batch_size):
        _, pts, filters, _ = dataset[i: min(i + batch_size, len(dataset))]
        pts = pts.to(device=dev, dtype=torch.float32)
        filters = filters.to(device=dev, dtype=torch.float32).clone()
        plan.setpts(pts)
        if L % 2 == 0:
            filters[:, 0, :] = 0
            filters[:, :, 0] = 0
        g = plan.execute_adjoint_unaggregated(torch.complex(filters**2, torch.zeros_like(filters))).abs() / L**2
        s = average_fourier_shell(*g)
        s = s.unsqueeze(0) if s.ndim == 1 else s
        out = s.T @ s if out is None else out + s.T @ s
    return out
