"""CPU port of the covariance-SGD step with the ES kernel (test infrastructure and the timed
CPU baseline of ``bench.py``): the same algorithm as the GPU step -- deapodise + pad + centered
FFT3, ES interpolation at the rotated central slices, projection epilogue, per-image ML Gram +
solve, closed-form adjoint, ES spreading, inverse FFT3, crop -- built from
``nufft_oracle`` (numpy) and the C loops of ``es_oracle.c`` (OpenMP).  Follows the reference's
``Covar.get_vectors_fourier_domain`` (covar.py:440-446), ``vol_forward`` (projection_funcs.py:
321-370), ``raw_cost_maximum_liklihood_fourier_domain`` (covar_sgd.py:1381-1399) and its
autograd backward.
"""

import ctypes
import os
import time

import numpy as np

from . import build_c
from . import nufft_oracle as O

try:
    import scipy.fft as _sfft
except ImportError:  # pragma: no cover
    _sfft = None

_libs = {}


def _lib(real):
    if real not in _libs:
        path = build_c.lib_path(real)
        if not os.path.exists(path):
            build_c.build()
        lib = ctypes.CDLL(path)
        ptr = ctypes.c_void_p
        for name in ("oracle_es_interp", "oracle_es_spread"):
            fn = getattr(lib, name)
            fn.restype = None
            fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ptr, ctypes.c_int64, ptr, ptr,
                           ctypes.c_int]
        _libs[real] = lib
    return _libs[real]


def _np_real(real):
    return np.float64 if real == "double" else np.float32


def c_interp(grid_cl, t, width, beta, real="double", threads=None):
    """grid_cl: (n, n, n, C) complex centered channels-last; t: (M, 3) fractional indices.
    Returns (M, C) complex."""
    rt = _np_real(real)
    ct = np.complex128 if real == "double" else np.complex64
    n, C = grid_cl.shape[0], grid_cl.shape[-1]
    g = np.ascontiguousarray(grid_cl, dtype=ct)
    tt = np.ascontiguousarray(t, dtype=rt)
    out = np.zeros((len(tt), C), dtype=ct)
    _lib(real).oracle_es_interp(n, width, beta, C, g.ctypes.data, len(tt), tt.ctypes.data, out.ctypes.data,
                                threads or os.cpu_count())
    return out


def c_spread(vals, t, n, width, beta, real="double", threads=None):
    """vals: (M, C) complex; returns the (n, n, n, C) centered channels-last grid."""
    rt = _np_real(real)
    ct = np.complex128 if real == "double" else np.complex64
    v = np.ascontiguousarray(vals, dtype=ct)
    tt = np.ascontiguousarray(t, dtype=rt)
    C = v.shape[1]
    grid = np.zeros((n, n, n, C), dtype=ct)
    _lib(real).oracle_es_spread(n, width, beta, C, grid.ctypes.data, len(tt), tt.ctypes.data, v.ctypes.data,
                                threads or os.cpu_count())
    return grid


def _fftn(x, axes, inverse=False, workers=None):
    if _sfft is not None:
        f = _sfft.ifftn if inverse else _sfft.fftn
        return f(x, axes=axes, workers=workers or os.cpu_count())
    return (np.fft.ifftn if inverse else np.fft.fftn)(x, axes=axes)


class CpuCovarStep:
    """ES-kernel ML cost + gradient for (r, L, L, L) Covar parameters on the CPU."""

    def __init__(self, L, r, width=6, upsample=2, real="float", threads=None):
        self.L, self.r, self.w, self.n = L, r, width, upsample * L
        self.beta = O.es_beta(width, upsample)
        self.gc = O.grid_correction_es(L, self.n, width, self.beta)
        self.real = real
        self.ct = np.complex128 if real == "double" else np.complex64
        self.threads = threads or os.cpu_count()

    def forward_grid(self, vectors, log_sqrt):
        V = vectors * np.exp(log_sqrt)[:, None, None, None]
        x = O.pad_center((V / self.gc).astype(self.ct), self.n, (-3, -2, -1))
        ax = (-3, -2, -1)
        G = np.fft.fftshift(_fftn(np.fft.ifftshift(x, axes=ax), ax, workers=self.threads), axes=ax)
        return V, np.ascontiguousarray(np.moveaxis(G, 0, -1)).astype(self.ct)

    def per_image(self, grid_cl, rotmats, images, ctf, noise_var, B_total):
        """Projection, cost and spread for a block of images; returns (cost_sum, fine-grid gradient)."""
        L, r = self.L, self.r
        B = len(rotmats)
        pts = O.rotated_points(rotmats, L)
        t = O.es_index(pts, self.n)
        samples = c_interp(grid_cl, t, self.w, self.beta, self.real, self.threads)  # (B*P, r)
        mask = O.nyquist_mask(L).reshape(-1)
        scale = (ctf.reshape(B, -1) * mask[None]) / L
        Q = samples.reshape(B, L * L, r).transpose(0, 2, 1) * scale[:, None, :]
        per, W = O.ml_cost_and_w(Q, images.reshape(B, -1), noise_var)
        W = W / B_total * scale[:, None, :]
        vals = W.transpose(0, 2, 1).reshape(-1, r)
        return per.sum(), c_spread(vals, t, self.n, self.w, self.beta, self.real, self.threads)

    def backward_grid(self, ggrid_cl, V):
        ax = (-3, -2, -1)
        gg = np.moveaxis(ggrid_cl, -1, 0)
        back = np.fft.fftshift(_fftn(np.fft.ifftshift(gg, axes=ax), ax, inverse=True, workers=self.threads), axes=ax)
        gV = 2.0 * np.real(O.crop_center(back, self.L, ax) * self.n**3) / self.gc
        return gV

    def step(self, vectors, log_sqrt, rotmats, images, ctf, noise_var):
        V, G = self.forward_grid(vectors, log_sqrt)
        csum, gg = self.per_image(G, rotmats, images, ctf, noise_var, len(rotmats))
        gV = self.backward_grid(gg, V)
        scale = np.exp(log_sqrt)
        return csum / len(rotmats), gV * scale[:, None, None, None], np.sum(gV * V, axis=(1, 2, 3))


def time_baseline(L, r, batch, sample_images, width=6, real="float", seed=0, threads=None):
    """Images/s of the CPU port for one SGD step of ``batch`` images, measured on a bounded
    sample: the per-step part (FFTs, pad, crop) is timed once and the per-image part (points,
    interpolation, Gram/solve, adjoint, spreading) on ``sample_images`` images, then
    throughput = batch / (t_step + batch * t_image).  Returns (images_per_s, detail dict)."""
    rng = np.random.default_rng(seed)
    step = CpuCovarStep(L, r, width, real=real, threads=threads)
    vec = rng.standard_normal((r, L, L, L)).astype(np.float32)
    vec /= np.linalg.norm(vec.reshape(r, -1), axis=1)[:, None, None, None]
    ls = np.zeros(r, np.float32)
    q = rng.standard_normal((sample_images, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    rv = 2 * np.arccos(np.clip(q[:, :1], -1, 1)) * q[:, 1:] / np.maximum(np.linalg.norm(q[:, 1:], axis=1,
                                                                                        keepdims=True), 1e-12)
    R = O.rotvec_to_rotmat(rv)
    imgs = (rng.standard_normal((sample_images, L, L)) + 1j * rng.standard_normal((sample_images, L, L))) * L
    ctf = rng.uniform(0.2, 1.0, (sample_images, L, L))
    t0 = time.perf_counter()
    V, G = step.forward_grid(vec, ls)
    t1 = time.perf_counter()
    _, gg = step.per_image(G, R, imgs, ctf, float(L * L), batch)
    t2 = time.perf_counter()
    step.backward_grid(gg, V)
    t3 = time.perf_counter()
    t_step = (t1 - t0) + (t3 - t2)
    t_image = (t2 - t1) / sample_images
    ips = batch / (t_step + batch * t_image)
    return ips, {"t_step_s": t_step, "t_image_s": t_image, "sample_images": sample_images,
                 "threads": step.threads, "real": real}


def _centered_fft3_f64(x, n, threads):
    """centered_fft3 of x (L, L, L) zero-padded to n (``projection_funcs.py:148-165``), float64."""
    ax = (0, 1, 2)
    p = O.pad_center(np.asarray(x, np.complex128), n, ax)
    return np.fft.fftshift(_fftn(np.fft.ifftshift(p, axes=ax), ax, workers=threads), axes=ax)


def _adjoint_fft3_f64(g, L, threads):
    """Adjoint of :func:`_centered_fft3_f64`: n^3 * centered_ifft3 then crop to L."""
    ax = (0, 1, 2)
    n = g.shape[0]
    back = np.fft.fftshift(_fftn(np.fft.ifftshift(g, axes=ax), ax, inverse=True, workers=threads), axes=ax)
    return O.crop_center(back, L, ax) * float(n) ** 3


def covar_cost_grad_es(vectors, log_sqrt, rotmats, images, ctf, noise_var, width=6, upsample=2, reg_scale=0.0,
                       fourier_reg=None, threads=None, cost_only=False):
    """Float64 ES-kernel ML covariance cost and its gradient w.r.t. (vectors, log_sqrt), the
    same mathematics as ``nufft_oracle.covar_cost_grad(kind="es", objective="ml")`` (restating
    ``Covar.get_vectors_fourier_domain``, covar.py:440-449, and
    ``cost_maximum_liklihood_fourier_domain``, covar_sgd.py:1350-1378), organised one channel
    at a time so that fine grids of 256^3 and 512^3 fit: per channel a centered FFT, the C
    interpolation, and in the backward the C spreading, the regulariser and the inverse FFT.
    Returns (cost, g_vectors (r, L, L, L), g_logsqrt (r,)) or the cost alone."""
    threads = threads or os.cpu_count()
    vectors = np.asarray(vectors, np.float64)
    r, L = vectors.shape[0], vectors.shape[-1]
    n = upsample * L
    B = len(rotmats)
    P = L * L
    beta = O.es_beta(width, upsample)
    gc = O.grid_correction_es(L, n, width, beta)
    scale = np.exp(np.asarray(log_sqrt, np.float64))
    V = vectors * scale[:, None, None, None]
    t = O.es_index(O.rotated_points(np.asarray(rotmats, np.float64), L), n)
    fr = None if fourier_reg is None or reg_scale == 0 else np.asarray(fourier_reg, np.float64)
    Q = np.empty((B * P, r), np.complex128)
    reg = 0.0
    for ch in range(r):
        G = _centered_fft3_f64(V[ch] / gc, n, threads)
        Q[:, ch] = c_interp(G[..., None], t, width, beta, "double", threads)[:, 0]
        if fr is not None:
            reg += float(np.sum(np.abs(G) ** 2 * fr))
        del G
    sp = (np.asarray(ctf, np.float64).reshape(B, P) * O.nyquist_mask(L).reshape(1, P)) / L
    Qb = Q.reshape(B, P, r).transpose(0, 2, 1) * sp[:, None, :]
    y = np.asarray(images, np.complex128).reshape(B, P)
    per, W = O.ml_cost_and_w(Qb, y, noise_var)
    cost = float(np.mean(per)) + reg_scale * reg / noise_var / 2.0
    if cost_only:
        return cost
    vals = (W / B * sp[:, None, :]).transpose(0, 2, 1).reshape(-1, r)
    gV = np.empty_like(V)
    for ch in range(r):
        gg = c_spread(np.ascontiguousarray(vals[:, ch:ch + 1]), t, n, width, beta, "double", threads)[..., 0]
        if fr is not None:
            gg += (reg_scale / noise_var / 2.0) * fr * _centered_fft3_f64(V[ch] / gc, n, threads)
        gV[ch] = 2.0 * np.real(_adjoint_fft3_f64(gg, L, threads)) / gc
        del gg
    return cost, gV * scale[:, None, None, None], np.sum(gV * V, axis=(1, 2, 3))
