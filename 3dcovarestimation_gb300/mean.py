"""Mean-volume reconstruction on GB300: drop-in for ``cov3d.mean`` (reference ``mean.py``).

``reconstruct_mean`` backprojects the phase-shifted, CTF-weighted images and the squared CTFs
with the nearest-neighbour plan (``cov3d_mean_accumulate``), floors the kernel
(``cov3d_regularize_lhs``), takes the Fourier-diagonal solve as the starting point and corrects
it for the zero padding with conjugate gradients run entirely on the device
(``cov3d_cg_solve``: FP64 inner products and residual norms, FP32 vectors, hand-written
pruned line DFTs for the operator on fine grids of 128 .. 512, cuFFT otherwise).

Preconditioners of the CG (``precond``): ``None`` is the reference's plain CG;
``"diagonal"`` divides by the kernel on the fine grid (the operator the reference uses for its
starting point); ``"circulant"`` divides by the symbol of the optimal circulant approximation
of the CG operator on the L^3 grid (``circulant_symbol``); a tensor (L, L, L) is used as that
symbol directly (the learned preconditioner supplies one).
"""

import ctypes
import logging
import math
from typing import Optional, Tuple, Union

import torch

from . import _lib
from .nufft_plan import _Plan
from .projection_funcs import centered_fft3, centered_ifft3

logger = logging.getLogger(__name__)

PRECOND_CODES = {None: 0, "none": 0, "diagonal": 1, "circulant": 2}


def get_grid_correction(L: int, upsampling_factor: int, nufft_disc: str) -> torch.Tensor:
    """sinc (nearest) or sinc^2 (bilinear) of pi k / (upsampling_factor L) per axis, outer
    product (reference ``mean.py:27-40``)."""
    assert nufft_disc in ("bilinear", "nearest"), "nufft_disc must be 'bilinear' or 'nearest'"
    pixel_pos = torch.arange(-(L // 2), (L - 1) // 2 + 1) / L
    pixel_pos = torch.pi * pixel_pos / upsampling_factor
    sinc_val = torch.sin(pixel_pos) / pixel_pos
    sinc_val[pixel_pos == 0] = 1
    sinc_val[sinc_val < 1e-6] = 1
    if nufft_disc == "bilinear":
        sinc_val = sinc_val**2
    return torch.einsum("i,j,k->ijk", sinc_val, sinc_val, sinc_val)


def complex_conjugate_gradient(A_mv, b, x0=None, rtol=1e-6, maxiter=None):
    """CG for a Hermitian positive-definite operator given as a callable (reference
    ``mean.py:43-93``: same iteration, stopping rule ||r|| < rtol ||b|| and default
    maxiter = 10 len(b)).  The inner products and norms are taken in FP64.  For the mean's
    padding operator use :func:`correct_upsampling_padding`, which runs the whole loop on the
    device without host round trips."""
    if not b.is_complex():
        raise ValueError("Input vector b must be a complex tensor.")
    if not b.is_cuda:
        raise ValueError("complex_conjugate_gradient takes CUDA tensors")
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    r = b - A_mv(x)
    p = r.clone()
    rs_old = torch.vdot(r.to(torch.complex128), r.to(torch.complex128)).real
    if maxiter is None:
        maxiter = len(b) * 10
    b_norm = torch.linalg.vector_norm(b.to(torch.complex128))
    num_iter = 0
    for num_iter in range(maxiter):
        Ap = A_mv(p)
        alpha = rs_old / torch.vdot(p.to(torch.complex128), Ap.to(torch.complex128))
        x += alpha.to(x.dtype) * p
        r -= alpha.to(r.dtype) * Ap
        rs_new = torch.vdot(r.to(torch.complex128), r.to(torch.complex128)).real
        if torch.sqrt(rs_new) < rtol * b_norm:
            break
        p = r + (rs_new / rs_old).to(r.real.dtype) * p
        rs_old = rs_new
    logger.debug(f"CG converged in {num_iter} iterations")
    return x


class _MeanSolver:
    """A plan used for the mean's grids, CG operator and transform workspaces."""

    _cache = {}

    @classmethod
    def get(cls, L, upsampling_factor, device, kernel=_lib.KERNEL_NEAREST):
        key = (int(L), int(upsampling_factor), str(device), kernel)
        plan = cls._cache.get(key)
        if plan is None:
            plan = _Plan(L, 2, 1e-6, kernel, upsampling_factor, compensated=True, device=device)
            cls._cache[key] = plan
        return plan


def _check_grid(t, n, name):
    if t.shape[-3:] != (n, n, n):
        raise ValueError(f"{name} must be ({n}, {n}, {n}); got {tuple(t.shape)}")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")


def regularize_lhs(lhs: torch.Tensor) -> torch.Tensor:
    """``max(|lhs|, 1e-3 * Fourier-shell mean of Re lhs)`` clamped at 1e-8 (reference
    ``mean.py:135-142``).  lhs is a centered (n, n, n) grid on the GPU; returns float32."""
    n = lhs.shape[-1]
    _check_grid(lhs, n, "lhs")
    plan = _MeanSolver.get(n, 1, lhs.device)
    src = lhs.to(torch.complex64).contiguous()
    out = torch.empty((n, n, n), dtype=torch.float32, device=lhs.device)
    with torch.cuda.device(lhs.device):
        _lib.call("cov3d_regularize_lhs", plan.bind(), _lib.ptr(src), _lib.ptr(out))
    return out


def circulant_symbol(reg_lhs: torch.Tensor, L: int) -> torch.Tensor:
    """Fourier symbol (L, L, L), centered, of T. Chan's optimal circulant approximation of the
    CG operator A(x) = crop_L(ifft3(reg_lhs * fft3(pad x))) (no counterpart in the reference)."""
    n = reg_lhs.shape[-1]
    _check_grid(reg_lhs, n, "reg_lhs")
    plan = _MeanSolver.get(L, n // L, reg_lhs.device)
    reg = reg_lhs.to(torch.float32).contiguous()
    out = torch.empty((L, L, L), dtype=torch.float32, device=reg.device)
    with torch.cuda.device(reg.device):
        _lib.call("cov3d_circulant_symbol", plan.bind(), _lib.ptr(reg), _lib.ptr(out))
    return out


class CGResult:
    """Outcome of a device CG solve: iterations (the reference's num_iter), relative residual,
    residual history (when requested) and whether the tolerance was reached."""

    def __init__(self, iters, relres, converged, history=None):
        self.iters, self.relres, self.converged, self.history = iters, relres, converged, history

    def __repr__(self):
        return f"CGResult(iters={self.iters}, relres={self.relres:.3e}, converged={self.converged})"


def cg_solve(reg_lhs: torch.Tensor, b: torch.Tensor, x0: torch.Tensor, L: int, rtol: float = 1e-6,
             maxiter: Optional[int] = None, precond: Union[None, str, torch.Tensor] = None,
             history: bool = False) -> Tuple[torch.Tensor, CGResult]:
    """Device CG on the padding operator (``cov3d_cg_solve``).  b and x0 are (L, L, L) or L^3
    complex; returns (x, CGResult).  Does not raise when maxiter is reached (the reference
    returns its last iterate too); ``CGResult.converged`` says whether it converged."""
    n = reg_lhs.shape[-1]
    _check_grid(reg_lhs, n, "reg_lhs")
    dev = reg_lhs.device
    plan = _MeanSolver.get(L, n // L, dev)
    reg = reg_lhs.to(torch.float32).contiguous()
    bb = b.reshape(-1).to(torch.complex64).contiguous()
    x = x0.reshape(-1).to(device=dev, dtype=torch.complex64).clone()
    if bb.numel() != L**3 or x.numel() != L**3:
        raise ValueError(f"b and x0 must hold L^3 = {L**3} values")
    symbol = None
    if isinstance(precond, torch.Tensor):
        symbol = precond.to(device=dev, dtype=torch.float32).contiguous()
        if symbol.numel() != L**3:
            raise ValueError("a preconditioner symbol must be (L, L, L)")
        code = 2
    else:
        if precond not in PRECOND_CODES:
            raise ValueError(f"precond must be None, 'diagonal', 'circulant' or a tensor; got {precond!r}")
        code = PRECOND_CODES[precond]
        if code == 2:
            symbol = circulant_symbol(reg, L)
    if maxiter is None:
        maxiter = 10 * L**3
    hist = torch.zeros(maxiter + 1, dtype=torch.float64, device=dev) if history else None
    iters, relres = ctypes.c_int(), ctypes.c_double()
    with torch.cuda.device(dev):
        st = plan._lib.cov3d_cg_solve(plan.bind(), _lib.ptr(reg), _lib.ptr(bb), _lib.ptr(x), float(rtol), int(maxiter),
                                      code, _lib.ptr(symbol), ctypes.byref(iters), ctypes.byref(relres), _lib.ptr(hist))
    converged = st == _lib.OK
    if st not in (_lib.OK, _lib.EMAXITER):
        _lib.check(st)
    if not converged:
        logger.warning(f"CG stopped at maxiter={maxiter} with relative residual {relres.value:.3e}")
    logger.debug(f"CG converged in {iters.value} iterations")
    h = hist[: iters.value + 2].cpu() if hist is not None else None
    return x, CGResult(iters.value, relres.value, converged, h)


def correct_upsampling_padding(lhs: torch.Tensor, rhs: torch.Tensor, cg_init: torch.Tensor, L: int,
                               upsampling_factor: int, rtol: float = 1e-6, maxiter: Optional[int] = None,
                               precond: Union[None, str, torch.Tensor] = None) -> torch.Tensor:
    """CG correction of the Fourier-diagonal solve for the zero padding (reference
    ``mean.py:96-132``): solves crop(ifft3(lhs * fft3(pad x))) = crop(ifft3(rhs)) from
    x0 = cg_init and returns the real part, (L, L, L)."""
    n = L * upsampling_factor
    _check_grid(rhs, n, "rhs")
    plan = _MeanSolver.get(L, upsampling_factor, rhs.device)
    src = rhs.to(torch.complex64).contiguous()
    b = torch.empty((L, L, L), dtype=torch.complex64, device=rhs.device)
    with torch.cuda.device(rhs.device):
        _lib.call("cov3d_mean_init", plan.bind(), _lib.ptr(src), None, _lib.ptr(b), None)
    x0 = torch.complex(cg_init.reshape(-1).to(torch.float32), torch.zeros_like(cg_init.reshape(-1), dtype=torch.float32))
    x, _ = cg_solve(lhs.real if lhs.is_complex() else lhs, b, x0, L, rtol=rtol, maxiter=maxiter, precond=precond)
    return x.reshape((L, L, L)).real


def _sphere_mask(L, device):
    g = torch.ceil(torch.arange(-L / 2, L / 2, dtype=torch.float64)) / (L / 2)
    z, y, x = torch.meshgrid(g, g, g, indexing="ij")
    return (torch.sqrt(x * x + y * y + z * z) <= 1).to(device)


class MeanBackprojector:
    """Accumulates the mean's rhs and lhs grids batch by batch on the device (the loop of
    reference ``mean.py:196-215``)."""

    def __init__(self, L: int, upsampling_factor: int = 2, device=None, nufft_disc: str = "nearest"):
        kernel = {"nearest": _lib.KERNEL_NEAREST, "bilinear": _lib.KERNEL_LINEAR}[nufft_disc]
        self.L, self.us, self.n = int(L), int(upsampling_factor), int(L) * int(upsampling_factor)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.plan = _Plan(L, 2, 1e-6, kernel, upsampling_factor, compensated=True, device=self.device)
        self.grids = torch.zeros((2, self.n, self.n, self.n), dtype=torch.complex64, device=self.device)

    def add(self, images: torch.Tensor, filters: Optional[torch.Tensor] = None, offsets: Optional[torch.Tensor] = None,
            contrasts: Optional[torch.Tensor] = None, pts_rot: Optional[torch.Tensor] = None,
            rotations: Optional[torch.Tensor] = None) -> None:
        """One batch: Fourier images (B, L, L), CTFs (B, L, L), offsets (B, 2) in pixels,
        contrasts (B,), and either the reference's points (B, 3, L^2) or rotations (B, 3, 3)."""
        dev = self.device
        B = images.shape[0]
        if (pts_rot is None) == (rotations is None):
            raise ValueError("give exactly one of pts_rot and rotations")
        if pts_rot is not None:
            self.plan.setpts(pts_rot.to(dev), wrap=False)
        else:
            self.plan.setrot(rotations.to(dev), self.L)
        y = images.to(device=dev, dtype=torch.complex64).reshape(B, -1).contiguous()
        f = filters.to(device=dev, dtype=torch.float32).reshape(B, -1).contiguous() if filters is not None else None
        o = offsets.to(device=dev, dtype=torch.float32).reshape(B, 2).contiguous() if offsets is not None else None
        c = contrasts.to(device=dev, dtype=torch.float32).reshape(B).contiguous() if contrasts is not None else None
        with torch.cuda.device(dev):
            _lib.call("cov3d_mean_accumulate", self.plan.bind(), _lib.ptr(y), _lib.ptr(f), _lib.ptr(o), _lib.ptr(c),
                      _lib.ptr(self.grids), 1)

    @property
    def rhs(self):
        return self.grids[0]

    @property
    def lhs(self):
        return self.grids[1]


def solve_mean(rhs: torch.Tensor, lhs: torch.Tensor, L: int, upsampling_factor: int = 2, mask=None,
               do_grid_correction: bool = True, rtol: float = 1e-6, maxiter: Optional[int] = None,
               precond: Union[None, str, torch.Tensor] = None, return_info: bool = False,
               reg_lhs: Optional[torch.Tensor] = None):
    """The solve part of ``reconstruct_mean`` (reference ``mean.py:215-259``): regularize_lhs (or
    the given regularised kernel ``reg_lhs``), Fourier-diagonal solve, CG padding correction,
    sphere mask, grid correction, mask."""
    dev = rhs.device
    reg = regularize_lhs(lhs) if reg_lhs is None else reg_lhs.to(device=dev, dtype=torch.float32).contiguous()
    plan = _MeanSolver.get(L, upsampling_factor, dev)
    src = rhs.to(torch.complex64).contiguous()
    b = torch.empty((L, L, L), dtype=torch.complex64, device=dev)
    x0 = torch.empty((L, L, L), dtype=torch.complex64, device=dev)
    with torch.cuda.device(dev):
        _lib.call("cov3d_mean_init", plan.bind(), _lib.ptr(src), _lib.ptr(reg), _lib.ptr(b), _lib.ptr(x0))
    info = None
    if upsampling_factor > 1:
        x, info = cg_solve(reg, b, x0, L, rtol=rtol, maxiter=maxiter, precond=precond)
        vol = x.reshape((L, L, L)).real
    else:
        vol = x0.real
    vol = centered_ifft3(centered_fft3(vol) * _sphere_mask(L, dev)).real
    if do_grid_correction:
        vol = vol / get_grid_correction(L, upsampling_factor, "nearest").to(dev)
    if mask is not None:
        vol = vol * mask.squeeze(0)
    return (vol, info) if return_info else vol


def reconstruct_mean(dataset, init_vol: Optional[torch.Tensor] = None, mask: Optional[torch.Tensor] = None,
                     upsampling_factor: int = 2, batch_size: int = 1024, idx: Optional[torch.Tensor] = None,
                     do_grid_correction: Optional[bool] = True, return_lhs_rhs: bool = False,
                     device=None, precond: Union[None, str, torch.Tensor] = None, rtol: float = 1e-6):
    """Reconstruct the mean volume (reference ``mean.py:145-259``).

    ``dataset`` is a torch DataLoader yielding ``(images, pts_rot, filters, idx)`` batches
    whose ``.dataset`` has ``offsets``, ``contrasts`` and ``resolution`` (the reference's
    CovarDataset contract), or such a dataset itself.  Images are taken in the Fourier domain.
    Returns the volume, or (volume, rhs, lhs) with ``return_lhs_rhs``."""
    if not isinstance(dataset, torch.utils.data.DataLoader):
        if idx is None:
            idx = torch.arange(len(dataset))
        loader = torch.utils.data.DataLoader(torch.utils.data.Subset(dataset, idx), batch_size=batch_size,
                                             shuffle=False)
        ds = dataset
    else:
        loader = dataset
        ds = dataset.dataset
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    L = ds.resolution
    acc = MeanBackprojector(L, upsampling_factor, device)
    for images, pts_rot, filters, batch_idx in loader:
        acc.add(images, filters, ds.offsets[batch_idx], ds.contrasts[batch_idx], pts_rot=pts_rot)
    reg_lhs = None
    if init_vol is not None:
        # regulariser from the initial volume (mean.py:220-233): noise_var over its radial PSD,
        # upsampled to the fine grid, / L, added to the kernel (which is real: the backprojection
        # of real |CTF|^2 at point pairs +-k); the reference's diagnostic plot is not made
        from .fsc_utils import rpsd, upsample_and_expand_fourier_shell

        r = rpsd(init_vol.squeeze(0).to(device))
        reg = ds.noise_var / upsample_and_expand_fourier_shell(r, L * upsampling_factor, 3) / L
        reg_lhs = acc.lhs.real + reg.reshape(acc.lhs.shape)
    vol = solve_mean(acc.rhs, acc.lhs, L, upsampling_factor, mask=mask, do_grid_correction=do_grid_correction,
                     rtol=rtol, precond=precond, reg_lhs=reg_lhs)
    if return_lhs_rhs:
        return vol, acc.rhs, acc.lhs
    return vol


def regularize_mean_from_halfsets(mean_half1: torch.Tensor, rhs1: torch.Tensor, lhs1: torch.Tensor,
                                  mean_half2: torch.Tensor, rhs2: torch.Tensor, lhs2: torch.Tensor,
                                  mask: Optional[torch.Tensor] = None, do_grid_correction: Optional[bool] = True,
                                  precond: Union[None, str, torch.Tensor] = None, rtol: float = 1e-6) -> torch.Tensor:
    """Mean from the two half-set backprojections with the FSC-based shell regulariser
    (reference ``mean.py:359-421``)."""
    from .fsc_utils import average_fourier_shell, upsample_and_expand_fourier_shell, vol_fsc

    L = mean_half1.shape[-1]
    us = lhs1.shape[-1] // L
    filter_gain = centered_fft3(centered_ifft3(lhs1 + lhs2, cropping_size=(L,) * 3)).abs() / 2
    averaged_filter_gain = average_fourier_shell(1 / filter_gain)
    fsc = torch.clamp(vol_fsc(mean_half1, mean_half2), 1e-3, 1 - 1e-3)
    reg = 1 / ((fsc / (1 - fsc)) * averaged_filter_gain)
    reg = upsample_and_expand_fourier_shell(reg.unsqueeze(0), rhs1.shape[-1], 3)
    return solve_mean(rhs1 + rhs2, lhs1 + lhs2 + reg, L, us, mask=mask, do_grid_correction=do_grid_correction,
                      rtol=rtol, precond=precond)


def reconstruct_mean_from_halfsets(dataset, idx: Optional[torch.Tensor] = None, **reconstruction_kwargs):
    """Means of the two halves of the dataset, then ``regularize_mean_from_halfsets``
    (reference ``mean.py:262-291``; halves are the first and second half of ``idx``)."""
    if idx is None:
        idx = torch.arange(len(dataset))
    kw = dict(reconstruction_kwargs)
    kw["return_lhs_rhs"] = True
    mask = kw.get("mask", None)
    m1, rhs1, lhs1 = reconstruct_mean(dataset, idx=idx[: len(idx) // 2], **kw)
    m2, rhs2, lhs2 = reconstruct_mean(dataset, idx=idx[len(idx) // 2:], **kw)
    return regularize_mean_from_halfsets(m1, rhs1, lhs1, m2, rhs2, lhs2, mask=mask,
                                         do_grid_correction=kw.get("do_grid_correction", True))


def reconstruct_mean_from_halfsets_DDP(dataset, ranks=None, **reconstruction_kwargs):
    """Half-set mean across data-parallel ranks (reference ``mean.py:294-356``): each rank
    backprojects the images of its shard (``dataset`` is this rank's DataLoader, e.g. with a
    DistributedSampler), the ranks of each half-set group sum their partial rhs / lhs grids,
    every rank receives both halves, and the regularised mean is solved on every rank.  With one
    rank this is :func:`reconstruct_mean_from_halfsets` on the sampler's indices."""
    import torch.distributed as dist

    from .distributed import reduce_halfset_backprojections, world

    if world() == 1 or (ranks is not None and len(ranks) == 1):
        return reconstruct_mean_from_halfsets(dataset.dataset, idx=torch.tensor(list(iter(dataset.sampler))),
                                              **reconstruction_kwargs)
    kw = dict(reconstruction_kwargs)
    kw["return_lhs_rhs"] = True
    mean, rhs, lhs = reconstruct_mean(dataset, **kw)
    half1, half2 = reduce_halfset_backprojections(rhs.contiguous(), lhs.contiguous(), mean.shape[-1], ranks)
    return regularize_mean_from_halfsets(*half1, *half2, mask=kw.get("mask", None),
                                         do_grid_correction=kw.get("do_grid_correction", True))
