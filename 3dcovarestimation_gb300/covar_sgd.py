"""Covariance-SGD costs, their hand-written adjoint, and the fused training step.

Drop-in cost functions (same signatures and values as ``cov3d.covar_sgd``,
``covar_sgd.py:1190-1432``) are built from two autograd pieces: the projection operator
(``vol_forward``, whose backward is the exact adjoint spreading kernel) and
:class:`ProjectedCost`, whose backward is the closed-form derivative of the per-image cost
with respect to the projections (per-image r x r Gram + FP64 Hermitian solve; no autograd
through ``linalg.solve`` / ``logdet``).

:class:`CovarTrainer` mirrors the reference trainer (``covar_sgd.py:48-409``) but each batch
is a single call of ``cov3d_covar_cost_grad``: pack + FFT + interpolation + Gram + solve +
adjoint + spreading + inverse FFT + unpack, writing the parameter gradients directly.
"""

import logging
import time
from typing import Any, Dict, List, Optional, Tuple

import torch

from . import _lib
from .covar import Covar
from .nufft_plan import NufftPlan, NufftPlanDiscretized, _Plan
from .projection_funcs import centered_fft2, centered_fft3, vol_forward

logger = logging.getLogger(__name__)

OBJECTIVE_ML, OBJECTIVE_LS = 0, 1


class ProjectedCost(torch.autograd.Function):
    """Per-image data term of the ML (objective 0) or LS (objective 1) cost from projections
    Q (B, r, P) and Fourier images y (B, P).  Returns (B,) costs; backward returns
    2 * dcost/dconj(Q) (torch's convention for complex inputs)."""

    @staticmethod
    def forward(ctx, Q, y, noise_var, objective, eigenvals_inv=None):
        B, r, P = Q.shape
        dev = Q.device
        Qc = Q.to(torch.complex64)
        yc = y.reshape(B, P).to(torch.complex64).contiguous()
        gram = torch.empty((B, r, r), dtype=torch.complex64, device=dev)
        h = torch.empty((B, r), dtype=torch.complex64, device=dev)
        yy = torch.empty((B,), dtype=torch.float32, device=dev)
        C = torch.empty((B, r, r), dtype=torch.complex64, device=dev)
        u = torch.empty((B, r), dtype=torch.complex64, device=dev)
        cost = torch.empty((B,), dtype=torch.float64, device=dev)
        bad = torch.zeros((1,), dtype=torch.int32, device=dev)
        linv = None if eigenvals_inv is None else eigenvals_inv.to(device=dev, dtype=torch.float64).contiguous()
        st = _lib.stream_ptr(dev)
        s = Qc.stride()
        _lib.call("cov3d_gram", st, B, P, r, _lib.ptr(Qc), s[0], s[2], s[1], _lib.ptr(yc), _lib.ptr(gram), _lib.ptr(h),
                  _lib.ptr(yy))
        _lib.call("cov3d_cost_solve", st, B, r, int(objective), _lib.ptr(gram), _lib.ptr(h), float(noise_var),
                  _lib.ptr(linv), 1.0, 1.0, _lib.ptr(C), _lib.ptr(u), _lib.ptr(cost), None, None, None, _lib.ptr(bad))
        if objective == OBJECTIVE_ML and bool(bad.item()):
            raise FloatingPointError("cov3d: a per-image matrix m is not positive definite")
        ctx.save_for_backward(Qc, yc, C, u)
        ctx.q_dtype = Q.dtype
        real = torch.float64 if Q.dtype in (torch.complex128, torch.float64) else torch.float32
        return cost.to(real)

    @staticmethod
    def backward(ctx, g):
        Qc, yc, C, u = ctx.saved_tensors
        B, r, P = Qc.shape
        w = (2.0 * g.to(torch.float32)).reshape(B, 1)
        Cw = (C * w.reshape(B, 1, 1)).contiguous()
        uw = (u * w).contiguous()
        W = torch.empty((B, r, P), dtype=torch.complex64, device=Qc.device)
        s = Qc.stride()
        _lib.call("cov3d_wpass", _lib.stream_ptr(Qc.device), B, P, r, _lib.ptr(Qc), s[0], s[2], s[1], _lib.ptr(yc),
                  _lib.ptr(Cw), _lib.ptr(uw), _lib.ptr(W), r * P, 1, P)
        return W.to(ctx.q_dtype) if ctx.q_dtype.is_complex else W.real.to(ctx.q_dtype), None, None, None, None


def _project(vols, nufft_plans, filters, fourier_domain):
    proj = vol_forward(vols, nufft_plans, filters, fourier_domain=fourier_domain)
    if proj.ndim == 3:  # a single image was squeezed by vol_forward
        proj = proj.unsqueeze(0)
    return proj


def _data_term(projected, images, noise_var, objective, apply_mean_const_term, mean_aggregate, L):
    B = images.shape[0]
    Q = projected.reshape(B, projected.shape[1], -1)
    Qc = Q if Q.is_complex() else Q.to(torch.complex64 if Q.dtype == torch.float32 else torch.complex128)
    y = images.reshape(B, -1)
    per = ProjectedCost.apply(Qc, y, noise_var, objective)
    ynorm2 = (y.abs() ** 2).sum(dim=1).to(per.dtype)
    if objective == OBJECTIVE_ML:  # ProjectedCost holds 0.5 * (-b^H z + logdet m)
        if apply_mean_const_term:
            per = per + 0.5 * ynorm2 / noise_var
    elif apply_mean_const_term:
        per = per + ynorm2**2 - (2 * noise_var * ynorm2 + (noise_var * L) ** 2)
    return per.mean() if mean_aggregate else per


def raw_cost_maximum_liklihood_fourier_domain(projected_eigenvecs, images, noise_var, apply_mean_const_term=False,
                                              mean_aggregate=True):
    """Reference ``covar_sgd.py:1381-1399``."""
    return _data_term(projected_eigenvecs, images, noise_var, OBJECTIVE_ML, apply_mean_const_term, mean_aggregate,
                      images.shape[-1])


def raw_cost_fourier_domain(projected_vols, images, noise_var, apply_mean_const_term=False, mean_aggregate=True):
    """Reference ``covar_sgd.py:1320-1347``."""
    return _data_term(projected_vols, images, noise_var, OBJECTIVE_LS, apply_mean_const_term, mean_aggregate,
                      images.shape[-1])


def cost_maximum_liklihood_fourier_domain(vols, images, nufft_plans, filters, noise_var, reg_scale=0,
                                          fourier_reg=None, apply_mean_const_term=False, mean_aggregate=True):
    """ML cost on Fourier-domain eigenvolumes (reference ``covar_sgd.py:1350-1378``)."""
    rank = vols.shape[0]
    proj = _project(vols, nufft_plans, filters, True)
    cost = raw_cost_maximum_liklihood_fourier_domain(proj, images, noise_var, apply_mean_const_term, mean_aggregate)
    if fourier_reg is not None and reg_scale != 0:
        vf = vols * torch.sqrt(fourier_reg / noise_var)
        cost = cost + reg_scale * torch.sum(torch.norm(vf.reshape((rank, -1)), dim=1) ** 2) / 2
    return cost


def cost_fourier_domain(vols, images, nufft_plans, filters, noise_var, reg_scale=0, fourier_reg=None,
                        apply_mean_const_term=False, mean_aggregate=True):
    """LS cost on Fourier-domain eigenvolumes (reference ``covar_sgd.py:1290-1317``).  Like the
    reference, the regulariser reshapes the volumes to (vols[0].shape[0], -1)."""
    rank = vols[0].shape[0]
    L = images.shape[-1]
    proj = _project(vols, nufft_plans, filters, True)
    cost = raw_cost_fourier_domain(proj, images, noise_var, apply_mean_const_term, mean_aggregate)
    if fourier_reg is not None and reg_scale != 0:
        vf = (vols * torch.sqrt(fourier_reg)).reshape((rank, -1))
        cost = cost + reg_scale * torch.sum(torch.abs(vf @ vf.conj().T) ** 2)
    return cost / (L**4)


def cost(vols, images, nufft_plans, filters, noise_var, reg_scale=0, fourier_reg=None, apply_mean_const_term=False,
         mean_aggregate=True):
    """Spatial-domain LS cost (reference ``covar_sgd.py:1190-1235``)."""
    rank = vols.shape[0]
    L = vols.shape[-1]
    proj = _project(vols, nufft_plans, filters, False)
    c = _data_term(proj, images, noise_var, OBJECTIVE_LS, apply_mean_const_term, mean_aggregate, L)
    if fourier_reg is not None and reg_scale != 0:
        vf = (centered_fft3(vols) * torch.sqrt(fourier_reg)).reshape((rank, -1))
        c = c + reg_scale * torch.sum(torch.abs(vf @ vf.conj().T) ** 2)
    return c


def cost_maximum_liklihood(vols, images, nufft_plans, filters, noise_var, reg_scale=0, fourier_reg=None,
                           apply_mean_const_term=False, mean_aggregate=True):
    """Spatial-domain ML cost (reference ``covar_sgd.py:1238-1286``)."""
    rank = vols.shape[0]
    proj = _project(vols, nufft_plans, filters, False)
    c = _data_term(proj, images, noise_var, OBJECTIVE_ML, apply_mean_const_term, mean_aggregate, images.shape[-1])
    if fourier_reg is not None and reg_scale != 0:
        vf = centered_fft3(vols) * torch.sqrt(fourier_reg / noise_var)
        c = c + reg_scale * torch.sum(torch.norm(vf.reshape((rank, -1)), dim=1) ** 2) / 2
    return c


# ----------------------------------------------------------------------------- fused step


class FusedCovarStep:
    """One plan + the fused cost/gradient call for a fixed (L, rank, kernel) configuration.

    ``nufft_disc`` is "nufft" (ES kernel, exact NUFFT), "bilinear" or "nearest" (grid_sample
    semantics).  Images are Fourier-domain (centered_fft2 of the spatial images) and
    ``noise_var`` is the Fourier-domain variance (spatial variance * L**2), exactly as the
    reference trainer holds them after ``dataset.to_fourier_domain()`` (``dataset.py:426-433``);
    by Parseval the resulting cost equals the reference's spatial-domain cost for "nufft".
    """

    def __init__(self, resolution, rank, nufft_disc="nufft", upsampling_factor=2, width=6, eps=1e-6,
                 compensated=True, device=None, bin_size=0, gram_precision="fp32"):
        kernel = {"nufft": _lib.KERNEL_ES, "bilinear": _lib.KERNEL_LINEAR, "nearest": _lib.KERNEL_NEAREST}[nufft_disc]
        if gram_precision not in ("fp32", "bf16"):
            raise ValueError("gram_precision must be 'fp32' or 'bf16'")
        self.gram_bf16 = gram_precision == "bf16"
        self.plan = _Plan(resolution, rank, eps, kernel, upsampling_factor,
                          width=width if kernel == _lib.KERNEL_ES else 0, compensated=compensated, bin_size=bin_size,
                          device=device)
        self.L, self.rank, self.nufft_disc = resolution, rank, nufft_disc
        self.device = self.plan.device
        self.d_cost = torch.zeros((1,), dtype=torch.float64, device=self.device)

    def set_rotations(self, rotmats):
        self.plan.setrot(rotmats, self.L)

    def set_points(self, pts):
        self.plan.setpts(pts, wrap=self.nufft_disc == "nufft")

    def __call__(self, vectors, log_sqrt, images, ctf, noise_var, reg_scale=0.0, fourier_reg=None, objective=0,
                 grad_vectors=None, grad_log_sqrt=None, per_image=None, sync_cost=False):
        """Cost (device scalar, float64) and gradients w.r.t. (vectors, log_sqrt)."""
        r = self.rank
        vectors = vectors.detach().to(torch.float32).contiguous()
        log_sqrt = log_sqrt.detach().to(torch.float32).contiguous()
        gv = grad_vectors if grad_vectors is not None else torch.empty_like(vectors)
        gl = grad_log_sqrt if grad_log_sqrt is not None else torch.empty_like(log_sqrt)
        for name, t in (("grad_vectors", gv), ("grad_log_sqrt", gl)):
            if t.dtype != torch.float32 or not t.is_contiguous() or not t.is_cuda:
                raise ValueError(f"{name} must be a contiguous float32 CUDA tensor")
        if per_image is not None and (per_image.dtype != torch.float64 or not per_image.is_contiguous()):
            raise ValueError("per_image must be a contiguous float64 tensor")
        imgs = images.detach().to(torch.complex64).contiguous()
        ctf_t = None if ctf is None else ctf.detach().to(torch.float32).contiguous()
        fr = None if fourier_reg is None or reg_scale == 0 else fourier_reg.to(torch.float32).contiguous()
        args = _lib.CostArgs(objective=objective, rank=r, d_vectors=vectors.data_ptr(), d_log_sqrt=log_sqrt.data_ptr(),
                             d_images=imgs.data_ptr(), d_ctf=ctf_t.data_ptr() if ctf_t is not None else None,
                             noise_var=float(noise_var), reg_scale=float(reg_scale),
                             d_fourier_reg=fr.data_ptr() if fr is not None else None,
                             use_grid_correction=0 if self.nufft_disc == "nufft_nogc" else 1,
                             d_cost=self.d_cost.data_ptr(), gram_bf16=1 if self.gram_bf16 else 0)
        host_cost = _lib.c_double() if sync_cost else None
        with torch.cuda.device(self.device):
            _lib.call("cov3d_covar_cost_grad", self.plan.bind(), _lib.ctypes.byref(args),
                      _lib.ctypes.byref(host_cost) if host_cost is not None else None, _lib.ptr(gv), _lib.ptr(gl),
                      _lib.ptr(per_image))
        return (host_cost.value if host_cost is not None else self.d_cost), gv, gl


def compute_updated_fourier_reg(eigenvecs1, eigenvecs2, filter_gain, current_fourier_reg, L,
                                optimize_in_fourier_domain, mask=None):
    """Half-set Fourier regulariser from the covariance FSC of the two half-set estimates and
    the dataset's shell-pair gain (reference ``covar_sgd.py:1155-1187``): returns
    (regulariser (L, L, L), covariance FSC (S, S))."""
    from .fsc_utils import covar_fsc, expand_fourier_shell

    correction = 1 / filter_gain
    correction[:, L // 2:] = correction[L // 2, L // 2]
    correction[L // 2:, :] = correction[L // 2, L // 2]
    if mask is not None:
        mask = mask.clone().to(eigenvecs1.device)
        eigenvecs1 = eigenvecs1 * mask
        eigenvecs2 = eigenvecs2 * mask
    fsc = covar_fsc(eigenvecs1, eigenvecs2)
    eps = 1e-6
    fsc = torch.clamp(fsc, eps, 1 - eps)
    reg = 1 / ((fsc / (1 - fsc)) * correction)
    reg[reg < 0] = 0
    reg = expand_fourier_shell(reg.diag().sqrt().unsqueeze(0), L, 3)
    if not optimize_in_fourier_domain:
        reg = reg / L**2
    return reg, fsc


def gram_bf16(Q, y, plan=None):
    """Per-image gram (n, r, r), h (n, r), |y|^2 (n) of projections Q (n, r, P) and images y
    (n, P) with BF16 inputs and FP32 accumulation on the tensor cores (``cov3d_gram_bf16``).
    ``plan`` (a ``_Plan``) provides the BF16 workspace; one is made when not given."""
    if not Q.is_cuda:
        raise ValueError("gram_bf16 takes CUDA tensors")
    n, r, P = Q.shape
    dev = Q.device
    Qc = Q.to(torch.complex64)
    yc = y.to(torch.complex64).reshape(n, P).contiguous()
    if plan is None:
        plan = _Plan(8, 1, 1e-6, _lib.KERNEL_NEAREST, 1, device=dev)
    gram = torch.empty((n, r, r), dtype=torch.complex64, device=dev)
    h = torch.empty((n, r), dtype=torch.complex64, device=dev)
    yy = torch.empty((n,), dtype=torch.float32, device=dev)
    s = Qc.stride()
    with torch.cuda.device(dev):
        _lib.call("cov3d_gram_bf16", plan.bind(), n, P, r, _lib.ptr(Qc), s[0], s[2], s[1], _lib.ptr(yc), _lib.ptr(gram),
                  _lib.ptr(h), _lib.ptr(yy))
    return gram, h, yy


class CovarTrainer:
    """Covariance SGD trainer (reference ``covar_sgd.py:48-409``) on GPU-resident data.

    ``train_data`` is an iterable of batches ``(images, poses, filters)`` already on the GPU:
    images in the Fourier domain, ``poses`` either rotation matrices (B, 3, 3) (points generated
    in the kernels) or reference-style points (B, 3, L**2)."""

    def __init__(self, covar: Covar, train_data, device, noise_var: float, dataset_size: int,
                 save_path: Optional[str] = None) -> None:
        self.device = torch.device(device)
        self.train_data = train_data
        self.covar = covar.to(self.device)
        self.noise_var = noise_var
        self.dataset_size = dataset_size
        self.save_path = save_path
        self.num_reduced_lr_before_stop = 4
        self.scheduler_patiece = 0
        self.fourier_reg = None
        self.training_log = {"epoch_ind": [], "lr_history": [], "cost_val": [], "epoch_run_time": []}

    def compute_fourier_reg_term(self, eigenvecs: torch.Tensor) -> None:
        """Fourier regulariser from an estimate of the eigenvectors: noise_var over their radial
        PSD, upsampled to the fine grid (reference ``covar_sgd.py:420-430``)."""
        from .fsc_utils import rpsd, upsample_and_expand_fourier_shell

        us = self.covar.upsampling_factor
        eigen_rpsd = rpsd(*eigenvecs) * (us**3)
        self.fourier_reg = self.noise_var / upsample_and_expand_fourier_shell(eigen_rpsd, self.covar.resolution * us, 3)

    def update_fourier_reg_halfsets(self, fourier_reg: torch.Tensor) -> None:
        """Install a regulariser computed from the half-sets, resampled to the fine grid
        (reference ``covar_sgd.py:432-447``; this trainer optimises in the Fourier domain)."""
        from .fsc_utils import average_fourier_shell, upsample_and_expand_fourier_shell

        fourier_reg = fourier_reg.to(self.device)
        us = self.covar.upsampling_factor
        radial = average_fourier_shell(fourier_reg) / (us**3)
        self.fourier_reg = upsample_and_expand_fourier_shell(radial, self.covar.resolution * us, 3)

    def setup_training(self, lr: Optional[float] = None, momentum: float = 0.9, optim_type: str = "Adam",
                       reg: float = 1, nufft_disc: str = "nufft", orthogonal_projection: bool = False,
                       objective_func: str = "ml", batch_size: int = 1024, width: int = 6, compensated: bool = True):
        self.use_orthogonal_projection = orthogonal_projection
        if lr is None:
            lr = 1e-1 if optim_type == "Adam" else 1e-2
        self.batch_size = batch_size
        self.lr = lr * batch_size
        self.optim_type, self.momentum = optim_type, momentum
        self.objective = OBJECTIVE_ML if objective_func == "ml" else OBJECTIVE_LS
        self.step_fn = FusedCovarStep(self.covar.resolution, self.covar.rank, nufft_disc,
                                      self.covar.upsampling_factor, width=width, compensated=compensated,
                                      device=self.device)
        self.reg_scale = reg / self.dataset_size
        self.restart_optimizer()
        self.epoch_index = 0

    def restart_optimizer(self) -> None:
        groups = self.covar.grad_lr_factor()
        for g in groups:
            g["lr"] *= self.lr
        if self.optim_type == "SGD":
            self.optimizer = torch.optim.SGD(groups, momentum=self.momentum)
        else:
            self.optimizer = torch.optim.Adam(groups)
        self.scheduler = torch.optim.lr_scheduler.ReduceLROnPlateau(self.optimizer, patience=self.scheduler_patiece)

    def run_batch(self, images, poses, filters):
        """One SGD step (reference ``covar_sgd.py:199-229``); returns the cost as a device tensor."""
        if poses.ndim == 3 and poses.shape[-1] == 3 and poses.shape[-2] == 3:
            self.step_fn.set_rotations(poses)
        else:
            self.step_fn.set_points(poses)
        cv = self.covar
        if cv.vectors.grad is None:
            cv.vectors.grad = torch.empty_like(cv.vectors)
            cv.log_sqrt_eigenvals.grad = torch.empty_like(cv.log_sqrt_eigenvals)
        c, _, _ = self.step_fn(cv.vectors.detach(), cv.log_sqrt_eigenvals.detach(), images, filters, self.noise_var,
                               self.reg_scale, self.fourier_reg, self.objective, grad_vectors=cv.vectors.grad,
                               grad_log_sqrt=cv.log_sqrt_eigenvals.grad)
        self.optimizer.step()
        if self.use_orthogonal_projection:
            cv.orthogonal_projection()
        return c

    def run_epoch(self, epoch: int) -> None:
        self.cost_in_epoch = torch.zeros((), dtype=torch.float64, device=self.device)
        for images, poses, filters in self.train_data:
            c = self.run_batch(images, poses, filters)
            self.cost_in_epoch += c.reshape(()) * images.shape[0]

    def train_epochs(self, max_epochs: int, restart_optimizer: bool = False) -> None:
        if restart_optimizer:
            self.restart_optimizer()
        for _ in range(max_epochs):
            t0 = time.time()
            self.run_epoch(self.epoch_index)
            self.training_log["epoch_run_time"].append(time.time() - t0)
            self.training_log["cost_val"].append(float(self.cost_in_epoch))
            self.scheduler.step(self.cost_in_epoch)
            self.epoch_index += 1
            if self.scheduler.get_last_lr()[0] <= self.lr * (self.scheduler.factor**self.num_reduced_lr_before_stop):
                break
