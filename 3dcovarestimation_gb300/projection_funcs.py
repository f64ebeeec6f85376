"""Projection operators (drop-in for ``cov3d.projection_funcs``).

``vol_forward`` / ``im_backward`` keep the reference's signatures and results
(``projection_funcs.py:321-399``).  With a :class:`NufftPlanDiscretized` the whole operator
(interpolation + Nyquist zeroing + CTF multiply + 1/L, and its adjoint) is one fused kernel
launch; with a :class:`NufftPlan` the exact ES NUFFT runs and the epilogue follows in torch.
The centered FFT helpers are thin torch.fft (cuFFT) wrappers with the reference's pad/crop
conventions.
"""

import math
from typing import List, Optional, Tuple, Union

import torch

from . import _lib
from .nufft_plan import (BaseNufftPlan, NufftPlan, NufftPlanDiscretized, NufftSpec, _BackprojectFn, _InterpFn,
                         _ProjectFn, _SpreadFn, nufft_adjoint, nufft_forward)


def pad_tensor(tensor: torch.Tensor, size: List[int], dims: Optional[List[int]] = None) -> torch.Tensor:
    """Centered zero padding (reference ``projection_funcs.py:11-38``)."""
    if dims is None:
        dims = [(-1 - i) % tensor.ndim for i in range(len(size))]
    dims = [d % tensor.ndim for d in dims]
    shape = list(tensor.shape)
    index = [slice(None)] * tensor.ndim
    for d, s in zip(dims, size):
        start = s // 2 - tensor.shape[d] // 2
        index[d] = slice(start, start + tensor.shape[d])
        shape[d] = s
    out = torch.zeros(shape, dtype=tensor.dtype, device=tensor.device)
    out[tuple(index)] = tensor
    return out


def crop_tensor(tensor: torch.Tensor, size: List[int], dims: Optional[List[int]] = None) -> torch.Tensor:
    """Centered crop (reference ``projection_funcs.py:41-64``)."""
    if dims is None:
        dims = [(-1 - i) % tensor.ndim for i in range(len(size))]
    dims = [d % tensor.ndim for d in dims]
    index = [slice(None)] * tensor.ndim
    for d, s in zip(dims, size):
        start = tensor.shape[d] // 2 - s // 2
        index[d] = slice(start, start + s)
    return tensor[tuple(index)]


def crop_image(images: torch.Tensor, L_crop: int) -> torch.Tensor:
    """Central crop of the last two axes (reference ``projection_funcs.py:67-79``)."""
    L = images.shape[-1]
    idx = torch.arange(-(L_crop // 2), L_crop // 2 + L_crop % 2, device=images.device) + L // 2
    return images[..., idx, :][..., idx].reshape(*images.shape[:-2], L_crop, L_crop)


def _centered_fft(fft_func, tensor, dim, size=None):
    if size is not None:
        tensor = pad_tensor(tensor, size, dim)
    return torch.fft.fftshift(fft_func(torch.fft.ifftshift(tensor, dim=dim), dim=dim), dim=dim)


def centered_fft2(image: torch.Tensor, im_dim: List[int] = [-1, -2], padding_size=None) -> torch.Tensor:
    return _centered_fft(torch.fft.fft2, image, im_dim, padding_size)


def centered_ifft2(image: torch.Tensor, im_dim: List[int] = [-1, -2], cropping_size=None) -> torch.Tensor:
    t = _centered_fft(torch.fft.ifft2, image, im_dim)
    return crop_tensor(t, cropping_size, im_dim) if cropping_size is not None else t


def centered_fft3(image: torch.Tensor, im_dim: List[int] = [-1, -2, -3], padding_size=None) -> torch.Tensor:
    return _centered_fft(torch.fft.fftn, image, im_dim, padding_size)


def centered_ifft3(image: torch.Tensor, im_dim: List[int] = [-1, -2, -3], cropping_size=None) -> torch.Tensor:
    t = _centered_fft(torch.fft.ifftn, image, im_dim)
    return crop_tensor(t, cropping_size, im_dim) if cropping_size is not None else t


def make_nufft_plan(spec: NufftSpec, input: Optional[torch.Tensor] = None):
    """Build a plan from a spec; optionally move ``input`` to the domain the plan expects
    (reference ``projection_funcs.py:168-196``)."""
    plan = spec.nufft_type(**spec.get_nufft_kwargs())
    if input is None:
        return plan
    if spec.input_in_fourier:
        input = centered_fft3(input, padding_size=tuple(v * spec.upsample_factor for v in input.shape[-3:]))
    return plan, input


def _nyquist_zero(x):
    if x.shape[-1] % 2 == 0:
        x = x.clone()
        x[..., 0, :] = 0
        x[..., :, 0] = 0
    return x


def vol_forward(volume: torch.Tensor, plan: Union[BaseNufftPlan, List[BaseNufftPlan]],
                filters: Optional[torch.Tensor] = None, fourier_domain: bool = False) -> torch.Tensor:
    """Project volumes to images (reference ``projection_funcs.py:321-370``): plan forward,
    (N, r, L, L) layout, zero Nyquist row/column, x CTF, optional centered iFFT2, / L."""
    L = plan.sz[-1] if not isinstance(plan, (list, tuple)) else plan[0].sz[-1]
    if isinstance(plan, (list, tuple)):
        out = torch.zeros((len(plan), volume.shape[0], L, L), dtype=volume.dtype, device=volume.device)
        for i, p in enumerate(plan):
            out[i] = vol_forward(volume, p, filters[i] if filters is not None else None)
        return out
    if isinstance(plan, NufftPlanDiscretized):
        vp = plan._plan
        proj = _InterpFn.apply(volume, vp, filters, _lib.APPLY_NYQUIST, 1.0 / L)
        proj = proj.reshape(volume.shape[0], vp.n_images, vp.points_L, vp.points_L).transpose(0, 1)
        if volume.is_complex() and volume.dtype != proj.dtype:
            proj = proj.to(volume.dtype)
    elif isinstance(plan, NufftPlan) and plan._plan is not None and volume.is_cuda:
        # the exact plan: deapodise + pad + FFT + interpolation with the epilogue fused
        vol = volume if volume.ndim == 4 else volume.unsqueeze(0)
        vp = plan._plan
        proj = _ProjectFn.apply(vol, vp, filters, _lib.APPLY_NYQUIST, 1.0 / L)
        proj = proj.reshape(vol.shape[0], vp.n_images, vp.points_L, vp.points_L).transpose(0, 1)
        proj = proj.to(plan.complex_dtype)
    else:
        proj = nufft_forward(volume, plan)
        proj = proj.reshape((*volume.shape[:-3], -1, proj.shape[-2], proj.shape[-1])).transpose(0, 1)
        proj = _nyquist_zero(proj)
        if filters is not None:
            proj = proj * filters.unsqueeze(1)
        proj = proj / L
    if proj.shape[1] == 1:  # one volume: the reference squeezes axis 0 (a no-op unless one image)
        proj = proj.squeeze(0)
    return centered_ifft2(proj).real if not fourier_domain else proj


def im_backward(image: torch.Tensor, plan: BaseNufftPlan, filters: Optional[torch.Tensor] = None,
                fourier_domain: bool = False) -> torch.Tensor:
    """Backproject images to a volume, the adjoint of :func:`vol_forward`
    (reference ``projection_funcs.py:373-399``)."""
    L = image.shape[-1]
    im_fft = centered_fft2(image / L**2) if not fourier_domain else image
    if isinstance(plan, NufftPlanDiscretized):
        out = _SpreadFn.apply(im_fft.reshape(1, -1), plan._plan, filters, _lib.APPLY_NYQUIST, 1.0 / L)
        if im_fft.dtype == torch.complex128:
            out = out.to(torch.complex128)
        return out.real if not fourier_domain else out
    if isinstance(plan, NufftPlan) and plan._plan is not None and im_fft.is_cuda:
        # the exact adjoint with the prologue (CTF, Nyquist zeroing, 1/L) fused into the spreading
        back = _BackprojectFn.apply(im_fft.reshape(1, -1), plan._plan, filters, _lib.APPLY_NYQUIST, 1.0 / L)
        back = back.to(plan.complex_dtype)
        return back.real if not fourier_domain else back
    im_fft = im_fft.clone()
    if filters is not None:
        im_fft = im_fft * filters
    im_fft = _nyquist_zero(im_fft)
    back = nufft_adjoint(im_fft, plan)
    return back.real / L if not fourier_domain else back / L


def _set_pose(plan: BaseNufftPlan, poses: torch.Tensor) -> None:
    """Points (B, 3, L^2) as the reference passes them, or rotation matrices (B, 3, 3) whose
    points the kernels generate."""
    if poses.ndim == 3 and tuple(poses.shape[-2:]) == (3, 3):
        plan.setrot(poses)
    else:
        plan.setpts(poses)


def preprocess_image_batch(images: torch.Tensor, nufft_plan: BaseNufftPlan, filters: torch.Tensor,
                           pose: Tuple[torch.Tensor, torch.Tensor], mean_volume: torch.Tensor,
                           mask: Optional[torch.Tensor] = None, mask_threshold: Optional[float] = None,
                           softening_kernel_fourier: Optional[torch.Tensor] = None,
                           fourier_domain: bool = False) -> torch.Tensor:
    """Shift the images by their offsets, subtract the projected mean and apply the soft
    projected mask (reference ``projection_funcs.py:199-252``).  ``pose`` is (points or
    rotations, phase shift (B, L, L)); ``mean_volume`` / ``mask`` are in the domain the plan
    expects (the upsampled centered Fourier grid for :class:`NufftPlanDiscretized`, spatial for
    :class:`NufftPlan`).  The projections are one single-channel interpolation each (with the
    CTF in its epilogue for the mean); the rest is 2D FFTs and elementwise work."""
    pts_rot, phase_shift = pose
    _set_pose(nufft_plan, pts_rot)
    if not fourier_domain:
        images = centered_fft2(images)
    images = images * phase_shift
    mean_forward = vol_forward(mean_volume, nufft_plan, filters=filters, fourier_domain=True)
    if mean_forward.ndim == 4:
        mean_forward = mean_forward.squeeze(1)
    images = images - mean_forward
    if mask is not None:
        images = centered_ifft2(images).real
        mask_forward = vol_forward(mask, nufft_plan, filters=None, fourier_domain=False).detach()
        if mask_forward.ndim == 4:
            mask_forward = mask_forward.squeeze(1)
        mask_forward = mask_forward > mask_threshold
        soft_mask = centered_ifft2(centered_fft2(mask_forward) * softening_kernel_fourier).real
        images = images * soft_mask
        if fourier_domain:
            images = centered_fft2(images)
    elif not fourier_domain:
        images = centered_ifft2(images).real
    return images


def get_mask_threshold(mask: torch.Tensor, nufft_plan: BaseNufftPlan) -> float:
    """10th percentile of the projected mask values above 10^-1.5 (reference
    ``projection_funcs.py:255-269``), for the plan's current points."""
    projected = vol_forward(mask, nufft_plan)
    vals = projected.reshape(-1).detach().cpu().double()
    vals = vals[vals > 10 ** (-1.5)]
    import numpy as np

    return float(np.percentile(vals.numpy(), 10))
