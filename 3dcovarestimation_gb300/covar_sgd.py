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
    ``max_batch`` sizes every workspace at construction (later steps of up to that many images
    allocate nothing); ``ls_regulariser`` also sizes the least-squares Fourier regulariser's.
    """

    def __init__(self, resolution, rank, nufft_disc="nufft", upsampling_factor=2, width=6, eps=1e-6,
                 compensated=True, device=None, bin_size=0, gram_precision="fp32", max_batch=None,
                 ls_regulariser=False):
        kernel = {"nufft": _lib.KERNEL_ES, "bilinear": _lib.KERNEL_LINEAR, "nearest": _lib.KERNEL_NEAREST}[nufft_disc]
        if gram_precision not in ("fp32", "bf16"):
            raise ValueError("gram_precision must be 'fp32' or 'bf16'")
        self.gram_bf16 = gram_precision == "bf16"
        self.plan = _Plan(resolution, rank, eps, kernel, upsampling_factor,
                          width=width if kernel == _lib.KERNEL_ES else 0, compensated=compensated, bin_size=bin_size,
                          device=device)
        self.L, self.rank, self.nufft_disc = resolution, rank, nufft_disc
        self.device = self.plan.device
        if max_batch:  # every workspace sized now: steps of up to max_batch images allocate nothing
            self.plan.reserve(max_batch, resolution, rank, points=True, gram_bf16=self.gram_bf16,
                              ls_reg=ls_regulariser)
        self.d_cost = torch.zeros((1,), dtype=torch.float64, device=self.device)

    def set_rotations(self, rotmats):
        self.plan.setrot(rotmats, self.L)

    def set_points(self, pts):
        self.plan.setpts(pts, wrap=self.nufft_disc == "nufft")

    def __call__(self, vectors, log_sqrt, images, ctf, noise_var, reg_scale=0.0, fourier_reg=None, objective=0,
                 grad_vectors=None, grad_log_sqrt=None, per_image=None, sync_cost=False, ctf_params=None):
        """Cost (device scalar, float64) and gradients w.r.t. (vectors, log_sqrt).  ``ctf`` is the
        (B, L^2) CTF array, or None with ``ctf_params`` (B, 8): the CTF is then computed in the
        kernels from each image's parameters (see ``synthetic.ctf_params``)."""
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
        if ctf_params is not None:
            if ctf_t is not None:
                raise ValueError("give ctf or ctf_params, not both")
            ctf_t = ctf_params.detach().to(torch.float32).contiguous()
            if ctf_t.shape != (self.plan.n_images, _lib.CTF_NPARAMS):
                raise ValueError(f"ctf_params must be ({self.plan.n_images}, {_lib.CTF_NPARAMS})")
        fr = None if fourier_reg is None or reg_scale == 0 else fourier_reg.to(torch.float32).contiguous()
        n3 = (self.L * self.plan.n // self.L) ** 3
        per_channel = 0
        if fr is not None:
            # one regulariser for every eigenvolume (n^3), or one each (r, n^3) as
            # CovarTrainer.compute_fourier_reg_term builds it (covar_sgd.py:420-430)
            if fr.numel() == r * n3 and r > 1:
                per_channel = 1
            elif fr.numel() != n3:
                raise ValueError(f"fourier_reg must hold n^3 or rank * n^3 values (n = {self.plan.n}); "
                                 f"got shape {tuple(fr.shape)}")
        args = _lib.CostArgs(objective=objective, rank=r, d_vectors=vectors.data_ptr(), d_log_sqrt=log_sqrt.data_ptr(),
                             d_images=imgs.data_ptr(), d_ctf=ctf_t.data_ptr() if ctf_t is not None else None,
                             noise_var=float(noise_var), reg_scale=float(reg_scale),
                             d_fourier_reg=fr.data_ptr() if fr is not None else None,
                             use_grid_correction=0 if self.nufft_disc == "nufft_nogc" else 1,
                             d_cost=self.d_cost.data_ptr(), gram_bf16=1 if self.gram_bf16 else 0,
                             ctf_params=1 if ctf_params is not None else 0, fourier_reg_per_channel=per_channel)
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


def _loader_batch_size(train_data) -> Optional[int]:
    """Batch size of a DataLoader (its ``batch_size`` or its sampler's, as the reference's
    ``get_dataloader_batch_size``) or of a :class:`ResidentLoader`."""
    bs = getattr(train_data, "batch_size", None)
    if bs is None:
        for attr in ("batch_sampler", "sampler"):
            bs = getattr(getattr(train_data, attr, None), "batch_size", None)
            if bs is not None:
                break
    return bs


class CovarTrainer:
    """Covariance SGD trainer (reference ``covar_sgd.py:48-545``); every batch is one call of
    the fused cost/gradient step (:class:`FusedCovarStep`) followed by the optimizer step.

    ``train_data`` is what the reference takes -- a DataLoader whose batches are ``(images,
    pts_rot, filters, idx)`` over a dataset exposing ``noise_var``, ``mask`` and the
    ``to_fourier_domain`` / ``to_spatial_domain`` switches -- or a
    :class:`~.dataset.ResidentLoader` over a device-resident dataset, whose batches carry
    rotation matrices (B, 3, 3) instead of points (generated in the kernels).  ``noise_var``
    and ``dataset_size`` may be given for any other iterable of batches."""

    def __init__(self, covar: Covar, train_data, device, save_path: Optional[str] = None, gt_data=None,
                 training_log_freq: int = 50, *, noise_var: Optional[float] = None,
                 dataset_size: Optional[int] = None) -> None:
        self.device = torch.device(device)
        self.train_data = train_data
        self._covar = covar.to(self.device)
        self.batch_size = _loader_batch_size(train_data)
        self.save_path = save_path
        self.gt_data = gt_data
        self.training_log_freq = training_log_freq
        self._noise_var = noise_var
        self._dataset_size = dataset_size
        self.num_reduced_lr_before_stop = 4
        self.scheduler_patiece = 0
        self.fourier_reg = None
        self.logTraining = True
        self.training_log = {"epoch_ind": [], "lr_history": [], "cost_val": [], "epoch_run_time": []}
        self.step_fn = None

    @property
    def dataset(self):
        return getattr(self.train_data, "dataset", None)

    @property
    def covar(self) -> Covar:
        return self._covar

    @property
    def noise_var(self) -> float:
        return self._noise_var if self._noise_var is not None else self.dataset.noise_var

    @property
    def vectorsGT(self):
        return getattr(self.gt_data, "eigenvecs", None) if self.gt_data is not None else None

    @property
    def filter_gain(self) -> torch.Tensor:
        """Shell-pair covariance gain of the dataset (``dataset.get_total_covar_gain``)."""
        from .dataset import get_total_covar_gain

        return get_total_covar_gain(self.dataset, device=self.device)

    def to(self, *args: Any, **kwargs: Any) -> "CovarTrainer":
        self._covar = self._covar.to(*args, **kwargs)
        if self.fourier_reg is not None:
            self.fourier_reg = self.fourier_reg.to(*args, **kwargs)
        return self

    def compute_fourier_reg_term(self, eigenvecs: torch.Tensor) -> None:
        """Fourier regulariser from an estimate of the eigenvectors: noise_var over their radial
        PSD, upsampled to the fine grid (reference ``covar_sgd.py:420-430``)."""
        from .fsc_utils import rpsd, upsample_and_expand_fourier_shell

        us = self.covar.upsampling_factor
        eigen_rpsd = rpsd(*eigenvecs) * (us**3)
        self.fourier_reg = self.noise_var / upsample_and_expand_fourier_shell(eigen_rpsd, self.covar.resolution * us, 3)

    def update_fourier_reg_halfsets(self, fourier_reg: torch.Tensor) -> None:
        """Install a regulariser computed from the half-sets, resampled to the fine grid when the
        optimisation runs in the Fourier domain (reference ``covar_sgd.py:432-447``)."""
        from .fsc_utils import average_fourier_shell, upsample_and_expand_fourier_shell

        fourier_reg = fourier_reg.to(self.device)
        if getattr(self, "optimize_in_fourier_domain", True):
            us = self.covar.upsampling_factor
            radial = average_fourier_shell(fourier_reg) / (us**3)
            fourier_reg = upsample_and_expand_fourier_shell(radial, self.covar.resolution * us, 3)
        self.fourier_reg = fourier_reg

    def setup_training(self, lr: Optional[float] = None, momentum: float = 0.9, optim_type: str = "Adam",
                       reg: float = 1, nufft_disc: str = "bilinear", orthogonal_projection: bool = False,
                       objective_func: str = "ml", width: int = 6, compensated: bool = True,
                       gram_precision: str = "fp32") -> None:
        """Reference ``covar_sgd.py:302-358``: lr x batch size, Adam or SGD, the plan of
        ``nufft_disc`` ("bilinear" / "nearest": discretized plans, Fourier-domain data; "nufft":
        the ES kernel), reg_scale = reg / len(dataset)."""
        self.use_orthogonal_projection = orthogonal_projection
        if lr is None:
            lr = 1e-1 if optim_type == "Adam" else 1e-2
        if self.batch_size is None:
            raise ValueError("the batch size of train_data is unknown")
        self.lr = lr * self.batch_size
        self.optim_type, self.momentum = optim_type, momentum
        self.restart_optimizer()
        self.optimize_in_fourier_domain = nufft_disc != "nufft"
        self.objective_func = objective_func
        self.objective = OBJECTIVE_ML if objective_func == "ml" else OBJECTIVE_LS
        self.nufft_disc = nufft_disc
        ds = self.dataset
        if ds is not None and hasattr(ds, "to_fourier_domain"):
            ds.to_fourier_domain() if self.optimize_in_fourier_domain else ds.to_spatial_domain()
        self.step_fn = FusedCovarStep(self.covar.resolution, self.covar.rank, nufft_disc, self.covar.upsampling_factor,
                                      width=width, compensated=compensated, device=self.device,
                                      gram_precision=gram_precision, max_batch=self.batch_size,
                                      ls_regulariser=self.objective == OBJECTIVE_LS and reg != 0)
        if nufft_disc == "nufft":
            self.covar.grid_correction = self.step_fn.plan.grid_correction().to(self.device)
        else:
            self.covar.init_grid_correction(nufft_disc)
        n = self._dataset_size if self._dataset_size is not None else len(ds)
        self.reg_scale = reg / n
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

    def prepare_batch(self, batch) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        images, poses, filters = batch[0], batch[1], batch[2]
        return images.to(self.device), poses.to(self.device), filters.to(self.device)

    def run_batch(self, images: torch.Tensor, pts_rot: torch.Tensor, filters: torch.Tensor) -> torch.Tensor:
        """One SGD step (reference ``covar_sgd.py:199-229``); returns the cost (device scalar).
        ``pts_rot`` is (B, 3, L^2) points or (B, 3, 3) rotations.  With ``nufft_disc="nufft"`` the
        data are spatial (as the reference's) and enter the Fourier-domain step through a
        centered 2D FFT with noise_var * L^2, which leaves the cost unchanged (Parseval)."""
        L = self.covar.resolution
        B = images.shape[0]
        if pts_rot.ndim == 3 and tuple(pts_rot.shape[-2:]) == (3, 3):
            self.step_fn.set_rotations(pts_rot)
        else:
            self.step_fn.set_points(pts_rot)
        noise_var = self.noise_var
        if not self.optimize_in_fourier_domain and not images.is_complex():
            images = centered_fft2(images.reshape(B, L, L))
            noise_var = noise_var * L**2
        cv = self.covar
        if cv.vectors.grad is None:
            cv.vectors.grad = torch.empty_like(cv.vectors)
            cv.log_sqrt_eigenvals.grad = torch.empty_like(cv.log_sqrt_eigenvals)
        c, _, _ = self.step_fn(cv.vectors.detach(), cv.log_sqrt_eigenvals.detach(), images.reshape(B, -1),
                               filters.reshape(B, -1), noise_var, self.reg_scale, self.fourier_reg, self.objective,
                               grad_vectors=cv.vectors.grad, grad_log_sqrt=cv.log_sqrt_eigenvals.grad)
        self.optimizer.step()
        if self.use_orthogonal_projection:
            cv.orthogonal_projection()
        return c.reshape(())

    def run_epoch(self, epoch: int) -> None:
        """Reference ``covar_sgd.py:246-281``: the summed cost of the epoch (cost x batch size,
        as the reference accumulates it) stays on the device."""
        self.cost_in_epoch = torch.zeros((), dtype=torch.float64, device=self.device)
        for batch in self.train_data:
            images, poses, filters = self.prepare_batch(batch)
            c = self.run_batch(images, poses, filters)
            self.cost_in_epoch += c * self.batch_size

    def train_epochs(self, max_epochs: int, restart_optimizer: bool = False) -> None:
        """Reference ``covar_sgd.py:375-409``: ReduceLROnPlateau on the epoch cost, stop after
        ``num_reduced_lr_before_stop`` reductions."""
        if restart_optimizer:
            self.restart_optimizer()
        for _ in range(max_epochs):
            t0 = time.time()
            self.run_epoch(self.epoch_index)
            dt = time.time() - t0
            cost = float(self.cost_in_epoch)
            self.scheduler.step(cost)
            ds = self.dataset
            if ds is not None and getattr(ds, "mask", None) is not None:
                with torch.no_grad():
                    m = ds.mask.to(self.device) > 0.3
                    self.covar.vectors.data.copy_(self.covar.vectors.data * m)
            self.training_log["epoch_ind"].append(self.epoch_index)
            self.training_log["lr_history"].append(self.scheduler.get_last_lr()[0])
            self.training_log["cost_val"].append(cost)
            self.training_log["epoch_run_time"].append(dt)
            if self.save_path is not None:
                self.save_result()
            self.epoch_index += 1
            if self.scheduler.get_last_lr()[0] <= self.lr * (self.scheduler.factor**self.num_reduced_lr_before_stop):
                logger.debug("learning rate reduced %d times; stopping", self.num_reduced_lr_before_stop)
                break

    def train(self, max_epochs: int, **training_kwargs: Any) -> None:
        self.setup_training(**training_kwargs)
        self.train_epochs(max_epochs)
        self.complete_training()

    def complete_training(self) -> None:
        ds = self.dataset
        if getattr(self, "optimize_in_fourier_domain", False) and ds is not None and hasattr(ds, "to_spatial_domain"):
            ds.to_spatial_domain()

    def results_dict(self) -> Dict[str, Any]:
        """The checkpoint the reference saves as ``training_results.bin`` (``covar_sgd.py:524-545``):
        the Covar state_dict, ``vectorsGT``, ``fourier_reg`` and the training log."""
        ckp = self.covar.state_dict()
        ckp["vectorsGT"] = self.vectorsGT
        ckp["fourier_reg"] = self.fourier_reg
        ckp.update(self.training_log)
        return ckp

    def save_result(self) -> None:
        import os

        d = os.path.split(self.save_path)[0]
        if d:
            os.makedirs(d, exist_ok=True)
        torch.save(self.results_dict(), self.save_path)


def update_fourier_reg(trainer1: CovarTrainer, trainer2: CovarTrainer) -> None:
    """Half-set regulariser update (reference ``covar_sgd.py:1121-1152``): the covariance FSC of
    the two half-set estimates and the averaged shell-pair gain give the new regulariser of
    both trainers."""
    L = trainer1.covar.resolution
    filter_gain = (trainer1.filter_gain + trainer2.filter_gain) / 2
    e1, l1 = trainer1.covar.eigenvecs
    e1 = e1 * (l1**0.5).reshape(-1, 1, 1, 1)
    e2, l2 = trainer2.covar.eigenvecs
    e2 = e2 * (l2**0.5).reshape(-1, 1, 1, 1)
    mask = getattr(trainer1.dataset, "mask", None)
    reg, fsc = compute_updated_fourier_reg(e1, e2, filter_gain, trainer1.fourier_reg, L,
                                           trainer1.optimize_in_fourier_domain, mask=mask)
    trainer1.update_fourier_reg_halfsets(reg)
    trainer2.update_fourier_reg_halfsets(reg)
    trainer1.training_log["covariance_fsc_halfset"] = fsc


def trainCovar(covar_model: Covar, dataset, batch_size: int, savepath: Optional[str] = None, gt_data=None,
               **kwargs: Any) -> CovarTrainer:
    """Training schedule of the reference (``covar_sgd.py:1479-1612``) on a device-resident
    dataset (:class:`~.dataset.ResidentDataset`, or anything with its ``half_split`` /
    ``get_total_covar_gain`` / domain switches).  Without half-sets: ``num_reg_update_iters``
    rounds of training, each followed by the regulariser from the current eigenvectors and an
    orthogonal projection, then a final run.  With half-sets (``use_halfsets``, the default of
    the command line): a second model initialised at random vectors trains on the other half;
    after each round both regularisers are updated from the half-sets' covariance FSC
    (:func:`update_fourier_reg`); then the first model trains on the whole dataset.  Returns
    the trainer of the final run."""
    import copy

    from .dataset import ResidentLoader

    use_halfsets = kwargs.pop("use_halfsets", True)
    num_reg_update_iters = kwargs.pop("num_reg_update_iters", 1) or 1
    num_epochs = kwargs.pop("max_epochs", 20)
    device = covar_model.device

    def loader(ds):
        return ResidentLoader(ds, batch_size)

    if not use_halfsets:
        trainer = CovarTrainer(covar_model, loader(dataset), device, savepath, gt_data=gt_data)
        trainer.setup_training(**kwargs)
        for _ in range(num_reg_update_iters):
            trainer.train_epochs(num_epochs, restart_optimizer=True)
            e, lam = trainer.covar.eigenvecs
            trainer.compute_fourier_reg_term(e * (lam**0.5).reshape(-1, 1, 1, 1))
            trainer.covar.orthogonal_projection()
        trainer.train_epochs(num_epochs, restart_optimizer=True)
        trainer.complete_training()
        return trainer

    covar_copy = copy.deepcopy(covar_model)
    with torch.no_grad():
        covar_copy.set_vectors(covar_copy.init_random_vectors(covar_model.rank).to(covar_copy.device))
    half1, half2, _ = dataset.half_split()
    trainer1 = CovarTrainer(covar_model, loader(half1), device, savepath, gt_data=gt_data)
    trainer2 = CovarTrainer(covar_copy, loader(half2), device, None, gt_data=gt_data)
    trainer1.setup_training(**kwargs)
    trainer2.setup_training(**kwargs)
    for _ in range(num_reg_update_iters):
        trainer1.train_epochs(num_epochs, restart_optimizer=True)
        trainer2.train_epochs(num_epochs, restart_optimizer=True)
        update_fourier_reg(trainer1, trainer2)
    trainer2.complete_training()
    del trainer2
    trainer1.train_data = loader(dataset)
    trainer1.train(max_epochs=num_epochs, **kwargs)
    return trainer1
