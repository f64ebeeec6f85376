"""Per-image Wiener / latent-MAP coordinates (drop-in for ``cov3d.wiener_coords``).

``compute_latentMAP_batch`` runs the per-image Gram contractions in FP32 on the GPU and the
r x r Hermitian solve (Cholesky) in FP64, one thread per image (reference
``wiener_coords.py:168-203``).  ``latentMAP`` loops over the dataset in batches like
``wiener_coords.py:85-165``; ``wiener_coords`` (``wiener_coords.py:13-82``) gives the same
posterior mean through the same two kernels (see its docstring).
"""

import math
from typing import Any, Optional, Tuple, Union

import torch

from . import _lib
from .nufft_plan import NufftPlan, NufftPlanDiscretized
from .projection_funcs import _set_pose, centered_fft3, centered_ifft2, vol_forward


def compute_latentMAP_batch(images: torch.Tensor, eigen_forward: torch.Tensor, noise_var: float,
                            eigenvals_inv: Optional[torch.Tensor] = None) -> Tuple[torch.Tensor, torch.Tensor,
                                                                                    torch.Tensor]:
    """MAP latent coordinates z = m^-1 b with m = conj(Q) Q^T / noise_var + Linv and
    b = conj(Q) y / noise_var.  Returns (z (n, r, 1), m (n, r, r), b (n, r, 1)) in the inputs'
    dtype family.  Not differentiable (the covariance cost has its own adjoint)."""
    n = images.shape[0]
    r = eigen_forward.shape[1]
    dev = eigen_forward.device
    if not dev.type == "cuda":
        raise ValueError("compute_latentMAP_batch takes CUDA tensors (no CPU path)")
    Q = eigen_forward.detach().reshape(n, r, -1).to(torch.complex64)
    P = Q.shape[-1]
    y = images.detach().reshape(n, P).to(torch.complex64).contiguous()
    gram = torch.empty((n, r, r), dtype=torch.complex64, device=dev)
    h = torch.empty((n, r), dtype=torch.complex64, device=dev)
    yy = torch.empty((n,), dtype=torch.float32, device=dev)
    z = torch.empty((n, r), dtype=torch.complex64, device=dev)
    m = torch.empty((n, r, r), dtype=torch.complex64, device=dev)
    bad = torch.zeros((1,), dtype=torch.int32, device=dev)
    linv = None
    if eigenvals_inv is not None:
        li = eigenvals_inv.detach()
        if li.is_complex():
            li = li.real
        linv = li.to(device=dev, dtype=torch.float64).contiguous()
    st = _lib.stream_ptr(dev)
    s = Q.stride()
    _lib.call("cov3d_gram", st, n, P, r, _lib.ptr(Q), s[0], s[2], s[1], _lib.ptr(y), _lib.ptr(gram), _lib.ptr(h),
              _lib.ptr(yy))
    _lib.call("cov3d_cost_solve", st, n, r, 0, _lib.ptr(gram), _lib.ptr(h), float(noise_var), _lib.ptr(linv), 1.0,
              1.0, None, None, None, None, _lib.ptr(z), _lib.ptr(m), _lib.ptr(bad))
    if bool(bad.item()):
        raise FloatingPointError("cov3d: a per-image matrix m is not positive definite")
    b = h / noise_var
    if images.is_complex() or eigen_forward.is_complex():
        dt = torch.complex128 if torch.complex128 in (images.dtype, eigen_forward.dtype) else torch.complex64
        return z.to(dt).unsqueeze(-1), m.to(dt), b.to(dt).unsqueeze(-1)
    dt = torch.float64 if torch.float64 in (images.dtype, eigen_forward.dtype) else torch.float32
    return z.real.to(dt).unsqueeze(-1), m.real.to(dt), b.real.to(dt).unsqueeze(-1)


def wiener_coords(dataset, eigenvecs: torch.Tensor, eigenvals: torch.Tensor, batch_size: int = 1024,
                  start_ind: Optional[int] = None, end_ind: Optional[int] = None, return_eigen_forward: bool = False,
                  **nufft_plan_kwargs: Any):
    """Wiener-filtered latent coordinates (reference ``wiener_coords.py:13-82``).

    The reference takes, per image with projections A (r, P) and A^T = QR, the coordinates
    Lambda R^T (R Lambda R^T + noise_var I)^-1 Q^T y.  Since R^T (R Lambda R^T + s I)^-1 R^-T =
    (G Lambda + s I)^-1 with G = A A^T, this is Lambda (G Lambda + s I)^-1 A y, and with
    Lambda = S S (S the symmetric square root) it is S (S G S / s + I)^-1 S A y / s: the
    latent-MAP solve of the projections of the eigenvolumes scaled by S, with an identity prior,
    then multiplied by S.  So no per-image QR is needed and Lambda may be singular; the Gram
    contraction runs in FP32 and the r x r Cholesky solve in FP64 (``cov3d_gram`` +
    ``cov3d_cost_solve``).  Points come from ``dataset[i:j]`` = (images, pts_rot, filters, idx);
    images are spatial, like the reference's."""
    start_ind = 0 if start_ind is None else start_ind
    end_ind = len(dataset) if end_ind is None else end_ind
    L = eigenvecs.shape[-1]
    rank = eigenvecs.shape[0]
    dtype, device = eigenvecs.dtype, eigenvecs.device
    lam = eigenvals.to(device=device, dtype=torch.float64)
    if lam.ndim == 1:
        lam = torch.diag(lam)
    w, U = torch.linalg.eigh((lam + lam.T) / 2)
    S = (U * torch.sqrt(torch.clamp(w, min=0.0))) @ U.T  # symmetric square root of Lambda
    scaled = torch.einsum("ij,jxyz->ixyz", S.to(torch.float32), eigenvecs.to(torch.float32)).contiguous()
    plan = NufftPlan((L,) * 3, batch_size=rank, dtype=dtype, device=device, **nufft_plan_kwargs)
    count = end_ind - start_ind
    coords = torch.zeros((count, rank), device=device)
    fwd = torch.zeros((count, rank, L, L), dtype=dtype) if return_eigen_forward else None
    for i in range(0, count, batch_size):
        images, pts_rot, filters, _ = dataset[start_ind + i: min(start_ind + i + batch_size, end_ind)]
        images, pts_rot, filters = images.to(device), pts_rot.to(device), filters.to(device)
        n = images.shape[0]
        _set_pose(plan, pts_rot)
        q = vol_forward(scaled, plan, filters)
        if q.ndim == 3:
            q = q.unsqueeze(0)
        z, _, _ = compute_latentMAP_batch(images.reshape(n, -1), q.reshape(n, rank, -1), dataset.noise_var)
        coords[i: i + n] = (z.squeeze(-1).real.to(torch.float64) @ S.T).to(coords.dtype)
        if return_eigen_forward:
            fwd[i: i + n] = vol_forward(eigenvecs, plan, filters).reshape(n, rank, L, L).to("cpu", dtype)
    return (coords, fwd) if return_eigen_forward else coords


class _EigenProjector:
    """Projections of fixed eigenvolumes on an exact plan for many batches of poses, as
    ``vol_forward`` gives them (Nyquist zeroing, CTF, 1/L): the fine grid is transformed once
    (``cov3d_fine_grid``) and each batch only interpolates it (``cov3d_interp``), written
    point-major so the Gram contractions read it directly."""

    def __init__(self, plan: NufftPlan, vols: torch.Tensor):
        self.plan, self.vols, self.grid = plan, vols, None

    def __call__(self, filters: Optional[torch.Tensor], fourier_domain: bool = False) -> torch.Tensor:
        """(n, r, L, L) projections of the current batch, Fourier domain (point-major storage) or,
        like ``vol_forward``'s default, the real part of their centered inverse 2D FFT."""
        p = self.plan._plan
        if self.grid is None:
            self.grid = p.fine_grid(self.vols)
        L = self.vols.shape[-1]
        ctf = None if filters is None else filters.reshape(p.n_images, -1)
        out = p.interp_native(self.grid, ctf, _lib.APPLY_NYQUIST, 1.0 / L)
        q = out.view(p.n_images, L * L, -1).permute(0, 2, 1).reshape(p.n_images, -1, L, L)
        return q if fourier_domain else centered_ifft2(q).real


def latentMAP(dataset, eigenvecs: torch.Tensor, eigenvals: torch.Tensor, batch_size: int = 1024,
              start_ind: Optional[int] = None, end_ind: Optional[int] = None, return_coords_covar: bool = False,
              nufft_plan: type = NufftPlan, **nufft_plan_kwargs: Any):
    """Latent coordinates for every image of ``dataset`` (reference ``wiener_coords.py:85-165``).
    ``dataset[i:j]`` must return (images, pts_rot or rotations (B, 3, 3), filters, idx) and expose
    ``noise_var``."""
    start_ind = 0 if start_ind is None else start_ind
    end_ind = len(dataset) if end_ind is None else end_ind
    L = eigenvecs.shape[-1]
    rank = eigenvecs.shape[0]
    dtype, device = eigenvecs.dtype, eigenvecs.device
    if eigenvals.ndim == 1:
        eigenvals = torch.diag(eigenvals)
    eigenvals_inv = torch.inverse(eigenvals + 1e-6 * torch.eye(rank, device=device, dtype=dtype))
    if nufft_plan == NufftPlan:
        plan = NufftPlan((L,) * 3, batch_size=rank, dtype=dtype, device=device, **nufft_plan_kwargs)
        vols = eigenvecs
    else:
        kw = {"upsample_factor": 2, "mode": "bilinear"}
        kw.update(nufft_plan_kwargs)
        plan = NufftPlanDiscretized((L,) * 3, **kw)
        vols = centered_fft3(eigenvecs, padding_size=(L * kw["upsample_factor"],) * 3)
    count = end_ind - start_ind
    coords = torch.zeros((count, rank), device=device)
    covar_inv = torch.zeros((count, rank, rank), dtype=dtype) if return_coords_covar else None
    project = _EigenProjector(plan, vols) if nufft_plan == NufftPlan else None
    for i in range(0, count, batch_size):
        images, pts_rot, filters, _ = dataset[start_ind + i: min(start_ind + i + batch_size, end_ind)]
        images, pts_rot, filters = images.to(device), pts_rot.to(device), filters.to(device)
        _set_pose(plan, pts_rot)
        if project is not None:  # the eigenvolumes are transformed once, not per batch
            eig_fwd = project(filters)
        else:
            eig_fwd = vol_forward(vols, plan, filters)
            if eig_fwd.ndim == 3:
                eig_fwd = eig_fwd.unsqueeze(0)
        z, m, _ = compute_latentMAP_batch(images, eig_fwd, dataset.noise_var, eigenvals_inv)
        coords[i: i + batch_size] = z.squeeze(-1).real.to(coords.dtype)
        if return_coords_covar:
            covar_inv[i: i + batch_size] = m.real.to(dtype).cpu()
    return (coords, covar_inv) if return_coords_covar else coords
