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


def _set_poses(plan, poses, L):
    """Rotation matrices (B, 3, 3) are generated into points by the kernels; reference-style
    points (B, 3, L^2) are used as given."""
    if poses.ndim == 3 and tuple(poses.shape[-2:]) == (3, 3):
        plan.setrot(poses, L)
    else:
        plan.setpts(poses)


def get_total_gain(dataset, batch_size: int = 1024, device: Optional[torch.device] = None) -> torch.Tensor:
    """|sum_i im_backward(ctf_i, ctf_i)| per batch, summed, / L: the total gain of every
    frequency (reference ``dataset.py:322-356``)."""
    L = dataset.resolution
    dev = _device(device)
    plan = NufftPlanDiscretized((L,) * 3, upsample_factor=1, mode="nearest", use_half_grid=False)
    gain = torch.zeros((L,) * 3, device=dev, dtype=torch.float32)
    for i in range(0, len(dataset), batch_size):
        _, pts, filters, _ = dataset[i: min(i + batch_size, len(dataset))]
        filters = filters.to(device=dev, dtype=torch.float32)
        _set_poses(plan, pts.to(device=dev, dtype=torch.float32), L)
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
        filters = filters.to(device=dev, dtype=torch.float32).clone()
        _set_poses(plan, pts.to(device=dev, dtype=torch.float32), L)
        if L % 2 == 0:
            filters[:, 0, :] = 0
            filters[:, :, 0] = 0
        g = plan.execute_adjoint_unaggregated(torch.complex(filters**2, torch.zeros_like(filters))).abs() / L**2
        s = average_fourier_shell(*g)
        s = s.unsqueeze(0) if s.ndim == 1 else s
        out = s.T @ s if out is None else out + s.T @ s
    return out


# ----------------------------------------------------------------------------- residency


class ResidentDataset:
    """A covariance dataset held in device memory for the whole training run (the reference
    keeps ``CovarDataset`` on the host and copies every batch, ``dataset.py:135-164`` and
    ``covar_sgd.py:231-244``; its ``pts_rot`` alone is (N, 3, L^2) floats).

    Per image it holds the image (Fourier or spatial domain, like ``CovarDataset``), the
    rotation matrix (3, 3) -- points are generated inside the kernels, so nothing of size
    (N, 3, L^2) exists -- and the CTF (L, L).  ``dataset[i:j]`` returns ``(images, rotations,
    filters, idx)`` like ``CovarDataset.__getitem__`` with rotations in place of ``pts_rot``;
    every consumer here (``CovarTrainer``, ``latentMAP``, the gains) accepts either.
    ``to_fourier_domain`` / ``to_spatial_domain`` and ``half_split`` follow
    ``dataset.py:426-433`` and ``dataset.py:302-320``."""

    def __init__(self, images: torch.Tensor, rotations: torch.Tensor, filters: torch.Tensor, noise_var: float,
                 fourier_domain: bool = False, mask: Optional[torch.Tensor] = None,
                 device: Optional[torch.device] = None) -> None:
        dev = _device(device) if device is not None else images.device
        if dev.type != "cuda":
            raise ValueError("ResidentDataset keeps its data on a CUDA device")
        self.images = images.to(dev)
        self.rotations = rotations.to(device=dev, dtype=torch.float32).contiguous()
        self.filters = filters.to(device=dev, dtype=torch.float32)
        self.noise_var = float(noise_var)
        self.resolution = int(self.images.shape[-1])
        self._in_spatial_domain = not fourier_domain
        self.mask = mask
        self.device = dev

    def __len__(self) -> int:
        return int(self.images.shape[0])

    def __getitem__(self, idx):
        return self.images[idx], self.rotations[idx], self.filters[idx], idx

    def get_subset(self, idx: torch.Tensor) -> "ResidentDataset":
        idx = torch.as_tensor(idx, device=self.device)
        sub = ResidentDataset(self.images[idx], self.rotations[idx], self.filters[idx], self.noise_var,
                              fourier_domain=not self._in_spatial_domain, mask=self.mask, device=self.device)
        return sub

    def half_split(self, permute: bool = True):
        """Two halves (a random permutation when ``permute``) and the permutation."""
        n = len(self)
        perm = torch.randperm(n) if permute else torch.arange(n)
        return self.get_subset(perm[: n // 2]), self.get_subset(perm[n // 2:]), perm

    def to_fourier_domain(self) -> None:
        if self._in_spatial_domain:
            from .projection_funcs import centered_fft2

            self.images = centered_fft2(self.images)
            self.noise_var *= self.resolution**2
            self._in_spatial_domain = False

    def to_spatial_domain(self) -> None:
        if not self._in_spatial_domain:
            from .projection_funcs import centered_ifft2

            self.images = centered_ifft2(self.images).real
            self.noise_var /= self.resolution**2
            self._in_spatial_domain = True

    def get_total_gain(self, batch_size: int = 1024, device=None) -> torch.Tensor:
        return get_total_gain(self, batch_size, device or self.device)

    def get_total_covar_gain(self, batch_size: Optional[int] = None, device=None) -> torch.Tensor:
        return get_total_covar_gain(self, batch_size, device or self.device)


class ResidentLoader:
    """Batches of a :class:`ResidentDataset` as device views, in order (the reference's
    ``create_dataloader`` with ``BatchIndexSampler(shuffle=False)``, ``dataset.py:798-895``,
    without worker processes or host-to-device copies)."""

    def __init__(self, dataset: ResidentDataset, batch_size: int) -> None:
        self.dataset = dataset
        self.batch_size = int(batch_size)

    def __len__(self) -> int:
        return (len(self.dataset) + self.batch_size - 1) // self.batch_size

    def __iter__(self):
        n = len(self.dataset)
        for i in range(0, n, self.batch_size):
            yield self.dataset[i: min(i + self.batch_size, n)]
