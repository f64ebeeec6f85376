"""NUFFT plans on GB300: drop-in replacements for ``cov3d.nufft_plan``.

Same class names, constructor arguments, attributes and call semantics as the reference
(``nufft_plan.py:40-518``); the work runs in the hand-written sm_103a kernels of
``libcov3d_gb300.so`` (interpolation / spreading over bin-sorted points, deapodisation and
padding around cuFFT).  Every operator takes CUDA tensors and fails loudly otherwise: there is
no CPU path.

* :class:`NufftPlanDiscretized` -- ``grid_sample`` semantics (trilinear "bilinear" or
  "nearest", zero padding, align_corners) on a centered Fourier grid given by the caller
  (reference ``nufft_plan.py:67-242``).
* :class:`NufftPlan` -- exact NUFFT with the exponential-of-semicircle kernel on a
  ``upsample``x fine grid, the semantics of the reference's cuFINUFFT plan
  (``nufft_plan.py:245-392``): type 2 ``c_j = sum_k f_k exp(-i k.x_j)`` and its adjoint.
"""

import inspect
import logging
import math
from abc import ABC
from dataclasses import dataclass
from enum import Enum
from typing import Any, Tuple, Union

import torch

from . import _lib

logger = logging.getLogger(__name__)

_MODE_KERNEL = {"bilinear": _lib.KERNEL_LINEAR, "nearest": _lib.KERNEL_NEAREST}


def get_half_fourier_grid(points: torch.Tensor, dim: Tuple[int, int]) -> torch.Tensor:
    """Keep the non-negative half of the first grid dimension (and drop the unmatched most
    negative frequency of the second one when L is even) (reference ``nufft_plan.py:18-37``)."""
    L = points.shape[dim[0]]
    index = [slice(None)] * points.ndim
    index[dim[0]] = slice(L // 2, L)
    if L % 2 == 0:
        index[dim[1]] = slice(1, L)
    return points[tuple(index)]


class _Plan:
    """Owner of one C plan (``cov3d_plan``)."""

    def __init__(self, L, n_trans, eps, kernel, upsample, width=0, beta=0.0, compensated=True, bin_size=0,
                 device=None):
        lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        opts = _lib.Opts(kernel=kernel, upsample=upsample, width=width or 0, beta=beta or 0.0,
                         compensated=1 if compensated else 0, bin_size=bin_size or 0, stream=None)
        handle = _lib.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(lib.cov3d_plan_create(int(L), int(n_trans), float(eps), _lib.ctypes.byref(opts),
                                             _lib.ctypes.byref(handle)))
        self.handle = handle
        self._lib = lib
        n, w, b = _lib.c_int(), _lib.c_int(), _lib.c_double()
        _lib.check(lib.cov3d_plan_info(handle, _lib.ctypes.byref(n), _lib.ctypes.byref(w), _lib.ctypes.byref(b)))
        self.L, self.n, self.width, self.beta, self.kernel = int(L), n.value, w.value, b.value, kernel
        self.n_trans = int(n_trans)
        self.n_images = 0
        self.points_L = 0

    def bind(self):
        """Route subsequent launches to the current torch stream of the plan's device."""
        _lib.check(self._lib.cov3d_plan_set_stream(self.handle, _lib.stream_ptr(self.device)))
        return self.handle

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._lib.cov3d_plan_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self.handle = None

    # -- points --
    def setpts(self, points, wrap):
        if points.ndim != 3 or points.shape[1] != 3:
            raise ValueError(f"points must have shape (N, 3, L**2); got {tuple(points.shape)}")
        P = points.shape[-1]
        pL = int(round(math.sqrt(P)))
        if pL * pL != P:
            raise ValueError("the number of points per image must be a square")
        pts = points.detach().to(device=self.device, dtype=torch.float32).contiguous()
        with torch.cuda.device(self.device):
            h = self.bind()
            _lib.call("cov3d_setpts", h, _lib.ptr(pts), pts.shape[0], pL, 3 * P, P, 1 if wrap else 0)
        self.n_images, self.points_L = pts.shape[0], pL

    def setrot(self, rotmats, points_L):
        rot = rotmats.detach().to(device=self.device, dtype=torch.float32).reshape(-1, 9).contiguous()
        with torch.cuda.device(self.device):
            h = self.bind()
            _lib.call("cov3d_setrot", h, _lib.ptr(rot), rot.shape[0], int(points_L))
        self.n_images, self.points_L = rot.shape[0], int(points_L)

    def reserve(self, max_images, points_L, nchan, points=False, gram_bf16=False, ls_reg=False):
        """Size the plan's workspaces at set-up (``cov3d_plan_reserve``) so that later calls on
        up to ``max_images`` images allocate nothing (``ls_reg``: also the least-squares
        Fourier regulariser's workspace and cuBLAS handle)."""
        flags = ((_lib.RESERVE_POINTS if points else 0) | (_lib.RESERVE_GRAM_BF16 if gram_bf16 else 0) |
                 (_lib.RESERVE_LS_REG if ls_reg else 0))
        with torch.cuda.device(self.device):
            _lib.call("cov3d_plan_reserve", self.bind(), int(max_images), int(points_L), int(nchan), flags)

    def timing(self, enable=True):
        """Enable CUDA-event timing of the plan's phases (sort, pack, FFTs, interp, gram, ...)."""
        _lib.call("cov3d_plan_timing", self.handle, 1 if enable else 0)

    def timing_read(self):
        """{phase: (milliseconds, count)} recorded since timing was enabled or last read."""
        ms = (_lib.c_double * _lib.NUM_PHASES)()
        cnt = (_lib.c_int * _lib.NUM_PHASES)()
        with torch.cuda.device(self.device):
            _lib.call("cov3d_plan_timing_read", self.handle, ms, cnt, _lib.NUM_PHASES)
        return {name: (ms[i], cnt[i]) for i, name in enumerate(_lib.phase_names())}

    @property
    def n_points(self):
        return self.n_images * self.points_L**2

    # -- operators on a caller-provided centered grid (C, n, n, n) --
    def interp(self, grid, ctf=None, flags=0, scale=1.0):
        C = grid.shape[0]
        grid = grid.to(torch.complex64).contiguous()
        out = torch.empty((C, self.n_points), dtype=torch.complex64, device=self.device)
        n3 = self.n**3
        layout = _lib.GridLayout(order=_lib.GRID_CENTERED, cell_stride=1, chan_stride=n3)
        ctf_t = None if ctf is None else ctf.detach().to(device=self.device, dtype=torch.float32).contiguous()
        with torch.cuda.device(self.device):
            _lib.call("cov3d_interp", self.bind(), _lib.ptr(grid), _lib.ctypes.byref(layout), C, _lib.ptr(out), 1,
                      self.n_points, _lib.ptr(ctf_t), flags | (_lib.APPLY_CTF if ctf_t is not None else 0),
                      float(scale))
        return out

    def spread(self, values, ctf=None, flags=0, scale=1.0):
        """values (C, n_points) complex -> centered grid (C, n, n, n)."""
        C = values.shape[0]
        vals = values.to(torch.complex64).contiguous()
        out = torch.empty((C, self.n, self.n, self.n), dtype=torch.complex64, device=self.device)
        layout = _lib.GridLayout(order=_lib.GRID_CENTERED, cell_stride=1, chan_stride=self.n**3)
        ctf_t = None if ctf is None else ctf.detach().to(device=self.device, dtype=torch.float32).contiguous()
        with torch.cuda.device(self.device):
            _lib.call("cov3d_spread", self.bind(), _lib.ptr(vals), 1, self.n_points, C, _lib.ptr(ctf_t),
                      flags | (_lib.APPLY_CTF if ctf_t is not None else 0), float(scale), _lib.ptr(out),
                      _lib.ctypes.byref(layout), 0)
        return out

    def spread_unaggregated(self, values, ctf=None, flags=0, scale=1.0):
        vals = values.to(torch.complex64).reshape(-1).contiguous()
        out = torch.empty((self.n_images, self.n, self.n, self.n), dtype=torch.complex64, device=self.device)
        ctf_t = None if ctf is None else ctf.detach().to(device=self.device, dtype=torch.float32).contiguous()
        with torch.cuda.device(self.device):
            _lib.call("cov3d_spread_unaggregated", self.bind(), _lib.ptr(vals), 1, _lib.ptr(ctf_t),
                      flags | (_lib.APPLY_CTF if ctf_t is not None else 0), float(scale), _lib.ptr(out))
        return out

    # -- exact NUFFT on spatial volumes --
    def type2(self, vol):
        C = vol.shape[0]
        out = torch.empty((C, self.n_points), dtype=torch.complex64, device=self.device)
        with torch.cuda.device(self.device):
            if vol.is_complex():
                v = vol.to(torch.complex64).contiguous()
                _lib.call("cov3d_execute_type2", self.bind(), None, _lib.ptr(v), C, _lib.ptr(out))
            else:
                v = vol.to(torch.float32).contiguous()
                _lib.call("cov3d_execute_type2", self.bind(), _lib.ptr(v), None, C, _lib.ptr(out))
        return out

    def type1(self, values):
        C = values.shape[0]
        vals = values.to(torch.complex64).contiguous()
        out = torch.empty((C, self.L, self.L, self.L), dtype=torch.complex64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.call("cov3d_execute_type1", self.bind(), _lib.ptr(vals), C, _lib.ptr(out))
        return out

    def project(self, vol, ctf=None, flags=0, scale=1.0):
        """Type 2 with vol_forward's epilogue fused (cov3d_project): (C, L, L, L) -> (C, n_points)."""
        C = vol.shape[0]
        out = torch.empty((C, self.n_points), dtype=torch.complex64, device=self.device)
        ctf_t = None if ctf is None else ctf.detach().to(device=self.device, dtype=torch.float32).contiguous()
        fl = flags | (_lib.APPLY_CTF if ctf_t is not None else 0)
        with torch.cuda.device(self.device):
            if vol.is_complex():
                v = vol.to(torch.complex64).contiguous()
                _lib.call("cov3d_project", self.bind(), None, _lib.ptr(v), C, _lib.ptr(out), 1, self.n_points,
                          _lib.ptr(ctf_t), fl, float(scale))
            else:
                v = vol.to(torch.float32).contiguous()
                _lib.call("cov3d_project", self.bind(), _lib.ptr(v), None, C, _lib.ptr(out), 1, self.n_points,
                          _lib.ptr(ctf_t), fl, float(scale))
        return out

    def fine_grid(self, vol):
        """Deapodised, zero-padded FFT of (C, L, L, L) volumes (cov3d_fine_grid): (C, n, n, n)
        complex64 in FFT-native order, for :meth:`interp_native` over many batches of points."""
        C = vol.shape[0]
        grid = torch.empty((C, self.n, self.n, self.n), dtype=torch.complex64, device=self.device)
        with torch.cuda.device(self.device):
            if vol.is_complex():
                v = vol.to(torch.complex64).contiguous()
                _lib.call("cov3d_fine_grid", self.bind(), None, _lib.ptr(v), C, _lib.ptr(grid))
            else:
                v = vol.to(torch.float32).contiguous()
                _lib.call("cov3d_fine_grid", self.bind(), _lib.ptr(v), None, C, _lib.ptr(grid))
        return grid

    def interp_native(self, grid, ctf=None, flags=0, scale=1.0):
        """Interpolation of a :meth:`fine_grid` result with the projection epilogue, written
        point-major: returns (n_points, C) complex64."""
        C = grid.shape[0]
        out = torch.empty((self.n_points, C), dtype=torch.complex64, device=self.device)
        layout = _lib.GridLayout(order=_lib.GRID_FFT_NATIVE, cell_stride=1, chan_stride=self.n**3)
        ctf_t = None if ctf is None else ctf.detach().to(device=self.device, dtype=torch.float32).contiguous()
        with torch.cuda.device(self.device):
            _lib.call("cov3d_interp", self.bind(), _lib.ptr(grid), _lib.ctypes.byref(layout), C, _lib.ptr(out), C, 1,
                      _lib.ptr(ctf_t), flags | (_lib.APPLY_CTF if ctf_t is not None else 0), float(scale))
        return out

    def backproject(self, values, ctf=None, flags=0, scale=1.0):
        """Type 1 with im_backward's prologue fused (cov3d_backproject): (C, n_points) -> (C, L, L, L)."""
        C = values.shape[0]
        vals = values.to(torch.complex64).contiguous()
        out = torch.empty((C, self.L, self.L, self.L), dtype=torch.complex64, device=self.device)
        ctf_t = None if ctf is None else ctf.detach().to(device=self.device, dtype=torch.float32).contiguous()
        fl = flags | (_lib.APPLY_CTF if ctf_t is not None else 0)
        with torch.cuda.device(self.device):
            _lib.call("cov3d_backproject", self.bind(), _lib.ptr(vals), 1, self.n_points, C, _lib.ptr(ctf_t), fl,
                      float(scale), _lib.ptr(out))
        return out

    def grid_correction(self):
        out = torch.empty((self.L,) * 3, dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.call("cov3d_grid_correction", self.bind(), _lib.ptr(out))
        return out


def _require_cuda(t, what):
    if not t.is_cuda:
        raise ValueError(f"{what} must be a CUDA tensor: the GB300 plans have no CPU path")


class _InterpFn(torch.autograd.Function):
    """Interpolation of a centered grid; backward is the exact adjoint (spreading)."""

    @staticmethod
    def forward(ctx, grid, plan, ctf, flags, scale):
        ctx.plan, ctx.ctf, ctx.flags, ctx.scale = plan, ctf, flags, scale
        ctx.grid_dtype = grid.dtype
        return plan.interp(grid, ctf, flags, scale)

    @staticmethod
    def backward(ctx, g):
        grad = ctx.plan.spread(g, ctx.ctf, ctx.flags, ctx.scale) if ctx.needs_input_grad[0] else None
        if grad is not None and not ctx.grid_dtype.is_complex:
            grad = grad.real
        return grad, None, None, None, None


class _SpreadFn(torch.autograd.Function):
    """Spreading into a centered grid; backward is interpolation."""

    @staticmethod
    def forward(ctx, values, plan, ctf, flags, scale):
        ctx.plan, ctx.ctf, ctx.flags, ctx.scale = plan, ctf, flags, scale
        return plan.spread(values, ctf, flags, scale)

    @staticmethod
    def backward(ctx, g):
        return ctx.plan.interp(g, ctx.ctf, ctx.flags, ctx.scale), None, None, None, None


class _ProjectFn(torch.autograd.Function):
    """Exact projection with its epilogue (Nyquist zeroing, CTF, scale) in one launch sequence;
    backward is the exact adjoint with the same prologue."""

    @staticmethod
    def forward(ctx, vol, plan, ctf, flags, scale):
        ctx.plan, ctx.ctf, ctx.flags, ctx.scale = plan, ctf, flags, scale
        ctx.complex_input = vol.is_complex()
        return plan.project(vol, ctf, flags, scale)

    @staticmethod
    def backward(ctx, g):
        if not ctx.needs_input_grad[0]:
            return None, None, None, None, None
        grad = ctx.plan.backproject(g, ctx.ctf, ctx.flags, ctx.scale)
        return (grad if ctx.complex_input else grad.real), None, None, None, None


class _BackprojectFn(torch.autograd.Function):
    """Exact adjoint with im_backward's prologue; backward is the projection."""

    @staticmethod
    def forward(ctx, values, plan, ctf, flags, scale):
        ctx.plan, ctx.ctf, ctx.flags, ctx.scale = plan, ctf, flags, scale
        ctx.complex_input = values.is_complex()
        return plan.backproject(values, ctf, flags, scale)

    @staticmethod
    def backward(ctx, g):
        if not ctx.needs_input_grad[0]:
            return None, None, None, None, None
        grad = ctx.plan.project(g, ctx.ctf, ctx.flags, ctx.scale)
        return (grad if ctx.complex_input else grad.real), None, None, None, None


class BaseNufftPlan(ABC):
    """Interface of the NUFFT plans (reference ``nufft_plan.py:40-64``)."""

    def setpts(self, points: torch.Tensor) -> None:
        raise NotImplementedError

    def execute_forward(self, volume: torch.Tensor) -> torch.Tensor:
        raise NotImplementedError


class NufftPlanDiscretized(BaseNufftPlan):
    """grid_sample-semantics plan (reference ``nufft_plan.py:67-242``).

    ``execute_forward`` expects the volume already in the (upsampled, centered) Fourier domain,
    as ``NufftSpec.input_in_fourier`` says.  Extra keyword ``compensated`` selects TwoSum
    compensated spreading (default True)."""

    def __init__(self, sz: Tuple[int, ...], upsample_factor: int = 1, mode: str = "bilinear",
                 use_half_grid: bool = False, compensated: bool = True) -> None:
        assert not use_half_grid, "half_grid not supported with NufftPlanDiscretized"
        if mode not in _MODE_KERNEL:
            raise ValueError(f"mode must be 'bilinear' or 'nearest'; got {mode!r}")
        self.sz = sz
        self.upsample_factor = upsample_factor
        self.mode = mode
        self.use_half_grid = use_half_grid
        self.compensated = compensated
        self._plan = None

    def _ensure_plan(self, device):
        if self._plan is None or self._plan.device != device:
            self._plan = _Plan(self.sz[0], 1, 1e-6, _MODE_KERNEL[self.mode], self.upsample_factor,
                               compensated=self.compensated, device=device)
        return self._plan

    def setpts(self, points: torch.Tensor) -> None:
        """Points of shape (N, 3, L**2), used as given (no wrapping), like ``nufft_plan.py:94-118``."""
        _require_cuda(points, "points")
        plan = self._ensure_plan(points.device)
        plan.setpts(points, wrap=False)
        self.points = points
        self.points_L = plan.points_L
        self.batch_points = plan.n_images

    def setrot(self, rotmats: torch.Tensor, points_L: int = None) -> None:
        """Points from rotation matrices (N, 3, 3), generated on the fly by the kernels
        (same values as ``PoseModule.forward``, ``poses.py:237-269``)."""
        _require_cuda(rotmats, "rotmats")
        plan = self._ensure_plan(rotmats.device)
        plan.setrot(rotmats, points_L or self.sz[0])
        self.points = None
        self.points_L = plan.points_L
        self.batch_points = plan.n_images

    def execute_forward(self, volume: Union[torch.Tensor, Tuple[torch.Tensor, torch.Tensor]]) -> torch.Tensor:
        """(C, n, n, n) complex centered Fourier grid (or a (real, imag) pair) -> (C, N, L, L)."""
        if isinstance(volume, tuple):
            volume = torch.complex(volume[0], volume[1])
        _require_cuda(volume, "volume")
        plan = self._plan
        out = _InterpFn.apply(volume, plan, None, 0, 1.0)
        out = out.reshape(volume.shape[0], plan.n_images, plan.points_L, plan.points_L)
        return out.to(volume.dtype) if volume.dtype != torch.complex64 and volume.is_complex() else out

    def execute_adjoint(self, signal: torch.Tensor) -> torch.Tensor:
        """(N, L, L) complex -> (1, n, n, n): adjoint summed over images (``nufft_plan.py:171-200``)."""
        _require_cuda(signal, "signal")
        plan = self._plan
        out = _SpreadFn.apply(signal.reshape(1, -1), plan, None, 0, 1.0)
        return out.to(signal.dtype) if signal.dtype == torch.complex128 else out

    def execute_adjoint_unaggregated(self, signal: torch.Tensor) -> torch.Tensor:
        """(N, L, L) complex -> (N, n, n, n): per-image adjoint (``nufft_plan.py:202-242``)."""
        _require_cuda(signal, "signal")
        out = self._plan.spread_unaggregated(signal.reshape(-1))
        return out.to(signal.dtype) if signal.dtype == torch.complex128 else out


class NufftPlan(BaseNufftPlan):
    """Exact NUFFT plan (reference ``nufft_plan.py:245-392``, cuFINUFFT semantics).

    Keyword arguments beyond the reference's: ``upsample`` (sigma, default 2), ``width`` (ES
    width; default from ``eps``), ``beta``, ``compensated``, ``bin_size``.  cuFINUFFT-specific
    keywords (``gpu_method``, ``gpu_sort``, ...) are accepted and ignored.  Computation is
    float32; a float64 plan returns float64/complex128 tensors holding float32-accurate values.
    """

    def __init__(self, sz: Tuple[int, ...], batch_size: int = 1, eps: float = 1e-6,
                 dtype: torch.dtype = torch.float32, device: torch.device = torch.device("cpu"), **kwargs: Any) -> None:
        self.sz = sz
        self.batch_size = batch_size
        self.device = torch.device(device)
        if dtype in (torch.float64, torch.complex128):
            self.dtype, self.complex_dtype = torch.float64, torch.complex128
            logger.warning("NufftPlan(dtype=float64): computed in float32 on the GPU")
        else:
            self.dtype, self.complex_dtype = torch.float32, torch.complex64
        self.eps = max(eps, 1.1920928955078125e-07 * 10)
        self._kw = dict(upsample=int(kwargs.get("upsample", 2)), width=int(kwargs.get("width", 0) or 0),
                        beta=float(kwargs.get("beta", 0.0) or 0.0), compensated=bool(kwargs.get("compensated", True)),
                        bin_size=int(kwargs.get("bin_size", 0) or 0))
        self._plan = None
        if self.device.type == "cuda":
            self._ensure_plan(self.device)

    def _ensure_plan(self, device):
        if self._plan is None or self._plan.device != device:
            self._plan = _Plan(self.sz[0], self.batch_size, self.eps, _lib.KERNEL_ES, self._kw["upsample"],
                               width=self._kw["width"], beta=self._kw["beta"], compensated=self._kw["compensated"],
                               bin_size=self._kw["bin_size"], device=device)
        return self._plan

    def setpts(self, points: torch.Tensor) -> None:
        """Points (N, 3, L**2), wrapped to [-pi, pi) (``nufft_plan.py:318-336``)."""
        _require_cuda(points, "points")
        plan = self._ensure_plan(points.device)
        plan.setpts(points, wrap=True)
        self.points_N = plan.n_images
        self.points_L = plan.points_L
        self.points = points

    def setrot(self, rotmats: torch.Tensor, points_L: int = None) -> None:
        """Points from rotation matrices (N, 3, 3), generated on the fly."""
        _require_cuda(rotmats, "rotmats")
        plan = self._ensure_plan(rotmats.device)
        plan.setrot(rotmats, points_L or self.sz[0])
        self.points_N = plan.n_images
        self.points_L = plan.points_L
        self.points = None

    @property
    def grid_correction(self) -> torch.Tensor:
        """ES deapodisation factors on the L^3 voxel grid."""
        return self._plan.grid_correction()

    def execute_forward(self, signal: torch.Tensor) -> torch.Tensor:
        """(B, L, L, L) spatial volumes, B <= batch_size -> (B, N, L, L) complex."""
        _require_cuda(signal, "signal")
        if signal.ndim == 3:
            signal = signal.unsqueeze(0)
        out = self._plan.type2(signal)
        return out.reshape(signal.shape[0], self.points_N, self.points_L, self.points_L).to(self.complex_dtype)

    def execute_adjoint(self, signal: torch.Tensor) -> torch.Tensor:
        """(B, ...) with N*L*L samples per row -> (B, L, L, L) complex."""
        _require_cuda(signal, "signal")
        B = signal.shape[0] if signal.numel() != self._plan.n_points else 1
        out = self._plan.type1(signal.reshape(B, -1))
        return out.to(self.complex_dtype)


class NufftType(Enum):
    DISCRETIZED = NufftPlanDiscretized
    FINUFFT = NufftPlan


@dataclass
class NufftSpec:
    """Plan specification (reference ``nufft_plan.py:399-422``)."""

    nufft_type: NufftType
    sz: Tuple[int, int, int]
    upsample_factor: int = None
    mode: str = None
    batch_size: int = None
    eps: float = None
    dtype: torch.dtype = None
    device: str = None

    def get_nufft_kwargs(self) -> dict:
        params = inspect.signature(self.nufft_type.__init__).parameters.keys()
        return {k: v for k, v in self.__dict__.items() if k in params and v is not None}

    @property
    def input_in_fourier(self) -> bool:
        return self.nufft_type == NufftPlanDiscretized


class TorchNufftForward(torch.autograd.Function):
    """Autograd wrapper of ``NufftPlan.execute_forward`` (reference ``nufft_plan.py:425-465``).
    The gradient with respect to the points is not provided (pose refinement is not part of
    this library)."""

    @staticmethod
    def forward(ctx: Any, signal: torch.Tensor, points: torch.Tensor, nufft_plan: Any, reset_pts: bool = False):
        if reset_pts:
            nufft_plan.setpts(points)
        ctx.signal_shape = signal.shape
        ctx.nufft_plan = nufft_plan
        ctx.complex_input = signal.is_complex()
        return nufft_plan.execute_forward(signal)

    @staticmethod
    def backward(ctx, grad_output):
        grad = None
        if ctx.needs_input_grad[0]:
            grad = ctx.nufft_plan.execute_adjoint(grad_output).reshape(ctx.signal_shape)
            if not ctx.complex_input:
                grad = grad.real
        return grad, None, None, None


class TorchNufftAdjoint(torch.autograd.Function):
    """Autograd wrapper of ``NufftPlan.execute_adjoint`` (reference ``nufft_plan.py:468-484``)."""

    @staticmethod
    def forward(ctx: Any, signal: torch.Tensor, nufft_plan: Any) -> torch.Tensor:
        ctx.signal_shape = signal.shape
        ctx.nufft_plan = nufft_plan
        ctx.complex_input = signal.is_complex()
        return nufft_plan.execute_adjoint(signal)

    @staticmethod
    def backward(ctx, grad_output):
        grad = ctx.nufft_plan.execute_forward(grad_output).reshape(ctx.signal_shape)
        if not ctx.complex_input:
            grad = grad.real
        return grad, None


def nufft_forward(signal: torch.Tensor, nufft_plan: BaseNufftPlan) -> torch.Tensor:
    """Forward NUFFT with autograd (reference ``nufft_plan.py:487-501``)."""
    if isinstance(nufft_plan, NufftPlan):
        return TorchNufftForward.apply(signal, nufft_plan.points, nufft_plan)
    return nufft_plan.execute_forward(signal)


def nufft_adjoint(signal: torch.Tensor, nufft_plan: BaseNufftPlan) -> torch.Tensor:
    """Adjoint NUFFT with autograd (reference ``nufft_plan.py:504-518``)."""
    if isinstance(nufft_plan, NufftPlan):
        return TorchNufftAdjoint.apply(signal, nufft_plan)
    return nufft_plan.execute_adjoint(signal)
