"""Covariance / mean parametrisation (drop-in for ``cov3d.covar``).

``Covar`` keeps the reference's parameters (``vectors`` of unit norm and
``log_sqrt_eigenvals``, ``covar.py:278-458``) and ``state_dict`` layout, so checkpoints load in
either implementation.  ``init_grid_correction`` additionally accepts ``"nufft"`` together
with a :class:`NufftPlan`, whose ES deapodisation then plays the role of the sinc^2 factor.
"""

from typing import Any, Dict, List, Optional, Tuple, Union

import torch

from .projection_funcs import centered_fft3, centered_ifft3, crop_tensor


def sinc_grid_correction(resolution: int, upsampling_factor: int, nufft_disc: str) -> torch.Tensor:
    """sinc (nearest) or sinc^2 (bilinear) per axis, outer product (reference ``covar.py:45-65``)."""
    pos = torch.arange(-(resolution // 2), (resolution - 1) // 2 + 1) / resolution
    pos = torch.pi * pos / upsampling_factor
    s = torch.sin(pos) / pos
    s[pos == 0] = 1
    s[s < 1e-6] = 1
    if nufft_disc == "bilinear":
        s = s**2
    return torch.einsum("i,j,k->ijk", s, s, s)


class VolumeBase(torch.nn.Module):
    """Common domain / grid-correction handling (reference ``covar.py:9-112``)."""

    def __init__(self, resolution: int, dtype: torch.dtype = torch.float32, fourier_domain: bool = False,
                 upsampling_factor: int = 2) -> None:
        super().__init__()
        self.resolution = resolution
        self.dtype = dtype
        self._in_spatial_domain = not fourier_domain
        self.upsampling_factor = upsampling_factor
        self.grid_correction = None

    def init_grid_correction(self, nufft_disc: str, plan=None) -> None:
        if nufft_disc in ("bilinear", "nearest"):
            self.grid_correction = sinc_grid_correction(self.resolution, self.upsampling_factor, nufft_disc).to(
                self.device)
        elif nufft_disc == "nufft" and plan is not None:
            self.grid_correction = plan.grid_correction.to(self.device)
        else:
            self.grid_correction = None

    def to(self, *args: Any, **kwargs: Any) -> "VolumeBase":
        super().to(*args, **kwargs)
        if self.grid_correction is not None:
            self.grid_correction = self.grid_correction.to(*args, **kwargs)
        return self

    def state_dict(self, *args: Any, **kwargs: Any) -> dict:
        sd = super().state_dict(*args, **kwargs)
        sd.update({"_in_spatial_domain": self._in_spatial_domain,
                   "grid_correction": self.grid_correction.to("cpu") if self.grid_correction is not None else None})
        return sd

    def load_state_dict(self, state_dict: dict, *args: Any, **kwargs: Any) -> None:
        state_dict = dict(state_dict)
        self._in_spatial_domain = state_dict.pop("_in_spatial_domain")
        self.grid_correction = state_dict.pop("grid_correction")
        super().load_state_dict(state_dict, *args, **kwargs)


class Mean(VolumeBase):
    """Mean volume as unit-norm shape times exp(log amplitude) (reference ``covar.py:115-275``)."""

    def __init__(self, volume_init: torch.Tensor, resolution: int, dtype: torch.dtype = torch.float32,
                 fourier_domain: bool = False, volume_mask: Optional[torch.Tensor] = None,
                 upsampling_factor: int = 2) -> None:
        super().__init__(resolution, dtype, fourier_domain, upsampling_factor)
        v = volume_init.squeeze(0).unsqueeze(0)
        amp = v.reshape(v.shape[0], -1).norm(dim=1)
        self.volume = torch.nn.Parameter(v / amp)
        self.log_volume_amplitude = torch.nn.Parameter(torch.log(amp))
        self.volume_mask = volume_mask

    @property
    def device(self) -> torch.device:
        return self.volume.device

    def get_volume_spatial_domain(self) -> torch.Tensor:
        return self.volume * torch.exp(self.log_volume_amplitude)

    def get_volume_fourier_domain(self) -> torch.Tensor:
        v = self.get_volume_spatial_domain()
        if self.grid_correction is not None:
            v = v / self.grid_correction
        return centered_fft3(v, padding_size=(self.resolution * self.upsampling_factor,) * 3)

    def forward(self, dummy_var: Optional[Any] = None) -> torch.Tensor:
        return self.get_volume_spatial_domain() if self._in_spatial_domain else self.get_volume_fourier_domain()

    def state_dict(self, *args: Any, **kwargs: Any) -> dict:
        sd = super().state_dict(*args, **kwargs)
        sd.update({"volume_mask": self.volume_mask.to("cpu") if self.volume_mask is not None else None})
        return sd

    def load_state_dict(self, state_dict: dict, *args: Any, **kwargs: Any) -> None:
        state_dict = dict(state_dict)
        self.volume_mask = state_dict.pop("volume_mask")
        super().load_state_dict(state_dict, *args, **kwargs)


class Covar(VolumeBase):
    """Low-rank covariance: r eigen-volumes as unit-norm ``vectors`` times exp(``log_sqrt_eigenvals``)
    (reference ``covar.py:278-458``)."""

    def __init__(self, resolution: int, rank: int, dtype: torch.dtype = torch.float32,
                 pixel_var_estimate: Union[float, torch.Tensor] = 1, fourier_domain: bool = False,
                 upsampling_factor: int = 2, vectors: Optional[torch.Tensor] = None) -> None:
        super().__init__(resolution, dtype, fourier_domain, upsampling_factor)
        self.rank = rank
        self.pixel_var_estimate = pixel_var_estimate
        if vectors is None:
            vectors = torch.randn((rank,) + (resolution,) * 3, dtype=dtype) * (float(pixel_var_estimate) ** 0.5)
        else:
            vectors = torch.clone(vectors).to(dtype)
        v, s = self._get_eigenvecs_representation(vectors)
        self.vectors = torch.nn.Parameter(v)
        self.log_sqrt_eigenvals = torch.nn.Parameter(s)

    @staticmethod
    def _get_eigenvecs_representation(vectors: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
        norms = vectors.reshape(vectors.shape[0], -1).norm(dim=1)
        return vectors / norms.reshape(-1, 1, 1, 1), torch.log(norms)

    @property
    def device(self) -> torch.device:
        return self.vectors.device

    def set_vectors(self, new_vectors: torch.Tensor) -> None:
        v, s = self._get_eigenvecs_representation(new_vectors)
        self.vectors.data.copy_(v)
        self.log_sqrt_eigenvals.data.copy_(s)

    def init_random_vectors(self, num_vectors: int) -> torch.Tensor:
        return torch.randn((num_vectors,) + (self.resolution,) * 3, dtype=self.dtype) * (
            float(self.pixel_var_estimate) ** 0.5)

    def get_vectors_spatial_domain(self) -> torch.Tensor:
        return self.vectors * torch.exp(self.log_sqrt_eigenvals).reshape(-1, 1, 1, 1)

    def get_vectors_fourier_domain(self) -> torch.Tensor:
        v = self.get_vectors_spatial_domain()
        if self.grid_correction is not None:
            v = v / self.grid_correction
        return centered_fft3(v, padding_size=(self.resolution * self.upsampling_factor,) * 3)

    def get_vectors(self) -> torch.Tensor:
        return self.get_vectors_spatial_domain() if self._in_spatial_domain else self.get_vectors_fourier_domain()

    def forward(self, dummy_var: Optional[Any] = None) -> torch.Tensor:
        return self.get_vectors()

    @property
    def eigenvecs(self) -> Tuple[torch.Tensor, torch.Tensor]:
        """Orthonormal eigenvectors and eigenvalues from an SVD of the factor (``covar.py:418-430``)."""
        with torch.no_grad():
            v = self.get_vectors_spatial_domain().reshape(self.rank, -1)
            _, S, Vh = torch.linalg.svd(v, full_matrices=False)
            return Vh.reshape((self.rank,) + (self.resolution,) * 3), S**2

    def grad_lr_factor(self) -> List[Dict[str, Union[torch.nn.Parameter, float]]]:
        """Parameter groups: eigenvalues learn 100x faster (``covar.py:432-438``)."""
        return [{"params": self.vectors, "lr": 1}, {"params": self.log_sqrt_eigenvals, "lr": 100}]

    def orthogonal_projection(self) -> None:
        with torch.no_grad():
            v = self.get_vectors_spatial_domain().reshape(self.rank, -1)
            _, S, Vh = torch.linalg.svd(v, full_matrices=False)
            self.set_vectors((S.reshape(-1, 1) * Vh).reshape((self.rank,) + (self.resolution,) * 3))
