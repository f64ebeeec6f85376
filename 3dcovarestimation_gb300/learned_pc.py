"""Learned CG preconditioner for the mean solve (no counterpart in the reference).

The padding CG of the mean (``mean.py``, ``cov3d_cg_solve``) converges slowly when the poses
sample Fourier space anisotropically.  Two Fourier-diagonal preconditioners on the L^3 grid
come from the kernel directly: the symbol of T. Chan's optimal circulant approximation of the
CG operator, and that of its inverse-symbol counterpart.  A 3-level 3D U-Net with 16 base
channels reads both (log, on a 32^3 grid, with the block-averaged log kernel and the
frequency radius) and predicts a smooth
log-correction delta; the preconditioner symbol is

    s = chan(A) * exp(trilinear_upsample(delta))     (delta = 0: the plain circulant PC)

Every layer of the network runs in the hand-written kernels of ``csrc/unet.cu`` through the C
ABI, forward and backward (``Conv3dFn`` and friends are torch.autograd.Functions over them),
so the network is trained on the GPU by this library.  Training (``train``) generates mean
problems with the method itself (clustered poses, CTFs, backprojection, the kernel, a solution
by diagonal-preconditioned CG) and minimises the energy-norm error left after K unrolled
preconditioned CG steps.  The plain diagonal-preconditioned CG stays the fallback, and the
residual of every solve is checked by the CG itself.
"""

import ctypes
import math
import os
from typing import Dict, List, Optional, Tuple

import torch

from . import _lib

_HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS_PATH = os.path.join(_HERE, "learned_pc_weights.npz")


def _stream(t):
    return _lib.stream_ptr(t.device)


def _f32(t):
    if not t.is_cuda:
        raise ValueError("learned-preconditioner layers take CUDA tensors")
    return t.detach().to(torch.float32).contiguous()


class Conv3dFn(torch.autograd.Function):
    """y = conv3d(x, w) + b (ReLU when relu), kernel 1 or 3, zero padding."""

    @staticmethod
    def forward(ctx, x, w, b, relu):
        x, w, b = _f32(x), _f32(w), _f32(b)
        N, Cin, D, H, W = x.shape
        Cout, k = w.shape[0], w.shape[-1]
        y = torch.empty((N, Cout, D, H, W), dtype=torch.float32, device=x.device)
        _lib.call("cov3d_conv3d_forward", _stream(x), _lib.ptr(x), N, Cin, D, H, W, _lib.ptr(w), _lib.ptr(b), Cout, k,
                  1 if relu else 0, _lib.ptr(y))
        ctx.save_for_backward(x, w, y)
        ctx.relu = relu
        return y

    @staticmethod
    def backward(ctx, gy):
        x, w, y = ctx.saved_tensors
        N, Cin, D, H, W = x.shape
        Cout, k = w.shape[0], w.shape[-1]
        g = _f32(gy)
        if ctx.relu:
            gm = torch.empty_like(g)
            _lib.call("cov3d_relu_backward", _stream(g), _lib.ptr(y), _lib.ptr(g), g.numel(), _lib.ptr(gm))
            g = gm
        gx = torch.empty_like(x)
        scratch = torch.empty_like(w)
        _lib.call("cov3d_conv3d_backward_data", _stream(g), _lib.ptr(g), N, Cout, D, H, W, _lib.ptr(w), Cin, k,
                  _lib.ptr(scratch), _lib.ptr(gx))
        gw = torch.empty_like(w)
        gb = torch.empty((Cout,), dtype=torch.float32, device=x.device)
        _lib.call("cov3d_conv3d_backward_weight", _stream(g), _lib.ptr(x), _lib.ptr(g), N, Cin, Cout, D, H, W, k,
                  _lib.ptr(gw), _lib.ptr(gb))
        return gx, gw, gb, None


class AvgPool2Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        x = _f32(x)
        N, C, D, H, W = x.shape
        y = torch.empty((N, C, D // 2, H // 2, W // 2), dtype=torch.float32, device=x.device)
        _lib.call("cov3d_avgpool2", _stream(x), _lib.ptr(x), N * C, D, H, W, 0, _lib.ptr(y))
        ctx.shape = x.shape
        return y

    @staticmethod
    def backward(ctx, gy):
        g = _f32(gy)
        N, C, D, H, W = ctx.shape
        gx = torch.empty(ctx.shape, dtype=torch.float32, device=g.device)
        _lib.call("cov3d_avgpool2", _stream(g), _lib.ptr(g), N * C, D, H, W, 1, _lib.ptr(gx))
        return gx


class Upsample2Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        x = _f32(x)
        N, C, d, h, w = x.shape
        y = torch.empty((N, C, 2 * d, 2 * h, 2 * w), dtype=torch.float32, device=x.device)
        _lib.call("cov3d_upsample2", _stream(x), _lib.ptr(x), N * C, d, h, w, 0, _lib.ptr(y))
        ctx.shape = x.shape
        return y

    @staticmethod
    def backward(ctx, gy):
        g = _f32(gy)
        N, C, d, h, w = ctx.shape
        gx = torch.empty(ctx.shape, dtype=torch.float32, device=g.device)
        _lib.call("cov3d_upsample2", _stream(g), _lib.ptr(g), N * C, d, h, w, 1, _lib.ptr(gx))
        return gx


class TrilinearFn(torch.autograd.Function):
    """(N, C, d, d, d) -> (N, C, D, D, D), align_corners = False."""

    @staticmethod
    def forward(ctx, x, D):
        x = _f32(x)
        N, C, d = x.shape[0], x.shape[1], x.shape[-1]
        y = torch.empty((N, C, D, D, D), dtype=torch.float32, device=x.device)
        _lib.call("cov3d_resample3d", _stream(x), _lib.ptr(x), N * C, d, D, 0, _lib.ptr(y))
        ctx.d = d
        return y

    @staticmethod
    def backward(ctx, gy):
        g = _f32(gy)
        N, C, D = g.shape[0], g.shape[1], g.shape[-1]
        gx = torch.empty((N, C, ctx.d, ctx.d, ctx.d), dtype=torch.float32, device=g.device)
        _lib.call("cov3d_resample3d", _stream(g), _lib.ptr(g), N * C, ctx.d, D, 1, _lib.ptr(gx))
        return gx, None


def block_mean(x, d):
    """(N, C, D, D, D) -> (N, C, d, d, d), mean over (D/d)^3 blocks (no gradient)."""
    x = _f32(x)
    N, C, D = x.shape[0], x.shape[1], x.shape[-1]
    y = torch.empty((N, C, d, d, d), dtype=torch.float32, device=x.device)
    _lib.call("cov3d_resample3d", _stream(x), _lib.ptr(x), N * C, d, D, 2, _lib.ptr(y))
    return y


def architecture(cin: int, c: int) -> List[Tuple[str, int, int, int, bool]]:
    """(name, input channels, output channels, kernel size, ReLU) of every convolution: two
    3x3x3 convolutions per level on 3 levels, 2x average pooling down, 2x nearest upsampling
    up with skip connections concatenated after the upsampled channels, a 1x1x1 head."""
    return [("enc0a", cin, c, 3, True), ("enc0b", c, c, 3, True),
            ("enc1a", c, 2 * c, 3, True), ("enc1b", 2 * c, 2 * c, 3, True),
            ("mida", 2 * c, 4 * c, 3, True), ("midb", 4 * c, 4 * c, 3, True),
            ("dec1a", 6 * c, 2 * c, 3, True), ("dec1b", 2 * c, 2 * c, 3, True),
            ("dec0a", 3 * c, c, 3, True), ("dec0b", c, c, 3, True),
            ("head", c, 1, 1, False)]


class UNet3D:
    """The network: parameters are plain CUDA tensors (name -> (w, b))."""

    def __init__(self, cin: int = 4, c: int = 16, device=None, seed: int = 0):
        self.cin, self.c = cin, c
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.params: Dict[str, Tuple[torch.Tensor, torch.Tensor]] = {}
        for name, ci, co, k, _ in architecture(cin, c):
            std = math.sqrt(2.0 / (ci * k**3))
            w = torch.randn((co, ci, k, k, k), generator=g) * std
            if name == "head":
                w.zero_()  # the untrained network predicts no correction
            self.params[name] = (w.to(dev).requires_grad_(), torch.zeros(co, device=dev).requires_grad_())

    def parameters(self):
        return [t for wb in self.params.values() for t in wb]

    def __call__(self, x: torch.Tensor) -> torch.Tensor:
        relu = {name: r for name, _, _, _, r in architecture(self.cin, self.c)}

        def conv(name, inp):
            w, b = self.params[name]
            return Conv3dFn.apply(inp, w, b, relu[name])

        e0 = conv("enc0b", conv("enc0a", x))
        e1 = conv("enc1b", conv("enc1a", AvgPool2Fn.apply(e0)))
        m = conv("midb", conv("mida", AvgPool2Fn.apply(e1)))
        d1 = conv("dec1b", conv("dec1a", torch.cat([Upsample2Fn.apply(m), e1], dim=1)))
        d0 = conv("dec0b", conv("dec0a", torch.cat([Upsample2Fn.apply(d1), e0], dim=1)))
        return conv("head", d0)

    def state_dict(self):
        out = {}
        for name, (w, b) in self.params.items():
            out[name + ".w"] = w.detach().cpu().numpy()
            out[name + ".b"] = b.detach().cpu().numpy()
        return out

    def load_state_dict(self, sd):
        for name, (w, b) in self.params.items():
            with torch.no_grad():
                w.copy_(torch.as_tensor(sd[name + ".w"]))
                b.copy_(torch.as_tensor(sd[name + ".b"]))


# ----------------------------------------------------------------------------- features / symbol


def feature_grid(L: int) -> int:
    """Resolution of the network's grid: 32 when L is a multiple of 32, else L (a multiple of 4)."""
    if L % 32 == 0:
        return 32
    if L % 4 != 0:
        raise ValueError("the learned preconditioner needs L divisible by 4")
    return L


def features(reg_lhs: torch.Tensor, L: int):
    """Network input (1, 4, G, G, G) and the base log-symbol (L, L, L): log chan(A), the log of
    1 / chan of the inverse symbol, the block mean of log reg_lhs over the fine grid (all three
    shifted by the mean of the first) and the radius |k| / (G/2)."""
    from .mean import circulant_symbol

    reg = reg_lhs.to(torch.float32).contiguous()
    n = reg.shape[-1]
    log_a = torch.log(circulant_symbol(reg, L))
    log_i = -torch.log(torch.clamp(circulant_symbol((1.0 / reg).contiguous(), L), min=1e-30))
    mu = log_a.mean()
    G = feature_grid(L)
    f = torch.stack([log_a - mu, log_i - mu])[None]
    f = block_mean(f, G) if G != L else f.contiguous()
    fine = block_mean((torch.log(reg) - mu)[None, None], G)
    k = torch.ceil(torch.arange(-G / 2, G / 2, device=reg.device, dtype=torch.float32)) / (G / 2)
    z, y, x = torch.meshgrid(k, k, k, indexing="ij")
    rad = torch.sqrt(x * x + y * y + z * z)[None, None]
    return torch.cat([f, fine, rad], dim=1).contiguous(), log_a


def learned_symbol(net: UNet3D, reg_lhs: torch.Tensor, L: int, with_grad: bool = False) -> torch.Tensor:
    """Preconditioner symbol s (L, L, L) for ``cg_solve(precond=s)``."""
    feats, log_a = features(reg_lhs, L)
    with torch.set_grad_enabled(with_grad):
        return symbol_from_features(net, feats, log_a, L)


class LearnedPreconditioner:
    """Loads the trained network and turns a regularised kernel into a CG preconditioner."""

    def __init__(self, path: str = WEIGHTS_PATH, device=None):
        import numpy as np

        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        sd = dict(np.load(path))
        c = int(sd["enc0a.w"].shape[0])
        cin = int(sd["enc0a.w"].shape[1])
        self.net = UNet3D(cin, c, dev)
        self.net.load_state_dict(sd)

    def symbol(self, reg_lhs: torch.Tensor, L: int) -> torch.Tensor:
        return learned_symbol(self.net, reg_lhs, L).detach()


# ----------------------------------------------------------------------------- training


class MeanProblem:
    """One mean solve generated by the method: regularised kernel, right-hand side, starting
    point, a reference solution (diagonal-preconditioned CG) and the network's features."""

    def __init__(self, reg, b, x0, xs, L):
        self.reg, self.b, self.x0, self.xs, self.L = reg, b, x0, xs, L
        self.feats, self.log_a = features(reg, L)


class ProblemGenerator:
    """Seeded mean problems: a Gaussian-blob volume, poses from a mixture of von Mises-Fisher
    clusters (random count and concentration), random-defocus CTFs, white noise at SNR 0.05,
    backprojected with the nearest plan at upsampling 2."""

    def __init__(self, L: int, n_images: int, device=None, batch: int = 1024, width: int = 6):
        from .mean import MeanBackprojector
        from .nufft_plan import NufftPlan

        self.L, self.n_images, self.batch = L, n_images, batch
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.fwd = NufftPlan((L,) * 3, batch_size=1, device=self.device, width=width)
        self.acc = MeanBackprojector(L, 2, self.device)

    def __call__(self, seed: int, solve_rtol: float = 1e-6) -> MeanProblem:
        from . import synthetic as syn
        from .mean import _MeanSolver, cg_solve, regularize_lhs
        from .projection_funcs import vol_forward

        L, dev = self.L, self.device
        g = torch.Generator(device=dev).manual_seed(int(seed))
        clusters = int(torch.randint(3, 13, (1,), generator=g, device=dev))
        kappa = float(torch.rand((1,), generator=g, device=dev)) * 10.0 + 2.0
        vol = syn.gaussian_blob_volumes(1, L, generator=g, device=dev)
        rot = syn.vmf_cluster_rotations(self.n_images, clusters, kappa, generator=g, device=dev)
        self.acc.grids.zero_()
        noise_sd = None
        for i in range(0, self.n_images, self.batch):
            rb = rot[i:i + self.batch]
            defocus = torch.rand((rb.shape[0],), generator=g, device=dev) * 2.0 + 1.0
            ctf = syn.ctf_images(defocus, L, 1.5, device=dev)
            self.fwd.setrot(rb)
            img = vol_forward(vol, self.fwd, ctf, fourier_domain=True)[:, 0]
            if noise_sd is None:
                noise_sd = (float((img.abs() ** 2).mean()) / 0.05) ** 0.5
            img = img + torch.randn(img.shape, generator=g, device=dev, dtype=torch.complex64) * noise_sd
            self.acc.add(img, ctf, rotations=rb)
        reg = regularize_lhs(self.acc.lhs)
        plan = _MeanSolver.get(L, 2, dev)
        b = torch.empty((L,) * 3, dtype=torch.complex64, device=dev)
        x0 = torch.empty_like(b)
        _lib.call("cov3d_mean_init", plan.bind(), _lib.ptr(self.acc.rhs.contiguous()), _lib.ptr(reg), _lib.ptr(b),
                  _lib.ptr(x0))
        xs, _ = cg_solve(reg, b, x0, L, rtol=solve_rtol, maxiter=20000, precond="diagonal")
        return MeanProblem(reg, b, x0, xs.reshape((L,) * 3), L)


def symbol_from_features(net: UNet3D, feats: torch.Tensor, log_a: torch.Tensor, L: int) -> torch.Tensor:
    delta = net(feats)
    if delta.shape[-1] != L:
        delta = TrilinearFn.apply(delta, L)
    return torch.exp(log_a + delta[0, 0])


def pcg_energy_loss(prob: MeanProblem, s: torch.Tensor, K: int) -> torch.Tensor:
    """log of ||x_K - x*||_A^2 / ||x_0 - x*||_A^2 after K preconditioned CG steps with the
    symbol s (differentiable in s; complex128, torch's cuFFT)."""
    from .projection_funcs import centered_fft3, centered_ifft3

    L = prob.L
    n = prob.reg.shape[-1]
    reg = prob.reg.to(torch.float64)
    s = s.to(torch.float64)

    def A(v):
        return centered_ifft3(reg * centered_fft3(v, padding_size=(n,) * 3), cropping_size=(L,) * 3)

    def M(v):
        return centered_ifft3(centered_fft3(v) / s)

    def dot(a, c):
        return torch.vdot(a.reshape(-1), c.reshape(-1))

    xs = prob.xs.to(torch.complex128)
    x = prob.x0.to(torch.complex128)
    r = prob.b.to(torch.complex128) - A(x)
    z = M(r)
    p = z
    rz = dot(r, z).real
    for _ in range(K):
        Ap = A(p)
        alpha = rz / dot(p, Ap)
        x = x + alpha * p
        r = r - alpha * Ap
        z = M(r)
        rz_new = dot(r, z).real
        p = z + (rz_new / rz) * p
        rz = rz_new
    e, e0 = x - xs, prob.x0.to(torch.complex128) - xs
    return torch.log(dot(e, A(e)).real / dot(e0, A(e0)).real)


def train(net: UNet3D, problems: List[MeanProblem], epochs: int = 4, lr: float = 1e-3, K: int = 30,
          log=None) -> List[float]:
    """Adam on the unrolled-PCG energy loss; every layer's forward and backward runs in the
    library's kernels.  Returns the mean loss of every epoch."""
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    history = []
    g = torch.Generator().manual_seed(0)
    for ep in range(epochs):
        total = 0.0
        for i in torch.randperm(len(problems), generator=g).tolist():
            prob = problems[i]
            s = symbol_from_features(net, prob.feats, prob.log_a, prob.L)
            loss = pcg_energy_loss(prob, s, K)
            opt.zero_grad()
            loss.backward()
            opt.step()
            total += float(loss.detach())
        history.append(total / len(problems))
        if log:
            log(f"epoch {ep}: mean loss {history[-1]:.4f}")
    return history


def evaluate(net: Optional[UNet3D], problems: List[MeanProblem], rtol: float = 1e-5, maxiter: int = 20000):
    """CG iterations to rtol per problem: diagonal PC, circulant PC (the untrained network's
    symbol) and, with a network, the learned symbol."""
    from .mean import cg_solve

    rows = []
    for prob in problems:
        row = {}
        for name, pc in (("diagonal", "diagonal"), ("circulant", torch.exp(prob.log_a))):
            _, info = cg_solve(prob.reg, prob.b, prob.x0, prob.L, rtol=rtol, maxiter=maxiter, precond=pc)
            row[name] = info.iters if info.converged else None
        if net is not None:
            with torch.no_grad():
                s = symbol_from_features(net, prob.feats, prob.log_a, prob.L)
            _, info = cg_solve(prob.reg, prob.b, prob.x0, prob.L, rtol=rtol, maxiter=maxiter, precond=s)
            row["learned"] = info.iters if info.converged else None
        rows.append(row)
    return rows


def save(net: UNet3D, path: str = WEIGHTS_PATH):
    import numpy as np

    np.savez(path, **net.state_dict())


def main(argv=None):
    """Train the preconditioner network on the GPU and save its weights (the committed weights
    were made with the defaults: L=128, 48 problems of 100,000 images, 8 epochs, K=60)."""
    import argparse

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--L", type=int, default=128)
    ap.add_argument("--images", type=int, default=100000)
    ap.add_argument("--problems", type=int, default=48)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--K", type=int, default=60)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--out", default=WEIGHTS_PATH)
    a = ap.parse_args(argv)
    dev = torch.device("cuda", torch.cuda.current_device())
    gen = ProblemGenerator(a.L, a.images, dev)
    problems = [gen(a.seed + i, solve_rtol=1e-5) for i in range(a.problems)]
    net = UNet3D(4, 16, dev)
    train(net, problems, epochs=a.epochs, lr=a.lr, K=a.K, log=print)
    save(net, a.out)
    print(f"saved {a.out}")


if __name__ == "__main__":
    main()
