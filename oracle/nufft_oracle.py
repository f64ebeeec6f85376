"""Float64 numpy restatement of the COV3D hot path (test infrastructure only; see package doc).

Conventions shared with the reference:

* volumes are indexed ``[axis0, axis1, axis2]`` (C order, axis 2 fastest); point row ``d``
  of a ``(N, 3, L*L)`` point array pairs with volume axis ``d`` (``nufft_plan.py:326,335``;
  the discretized plan flips rows to grid_sample's xyz, ``nufft_plan.py:105-107``);
* Fourier grids are *centered*: index ``m`` of an ``n``-point axis holds frequency
  ``2*pi*(m - n//2)/n`` (``projection_funcs.py:148-165``), so a frequency ``omega`` sits at
  fractional index ``t = omega*n/(2*pi) + n//2``.
"""

import math

import numpy as np

# ----------------------------------------------------------------------------- poses


def grid_1d(n):
    """Normalised 1-D grid ``ceil(arange(-n/2, n/2)) / (n/2)`` (ASPIRE ``grid_2d``/``grid_3d``
    definition, used by ``poses.py:197-215`` and ``fsc_utils.py:43-47``)."""
    return np.ceil(np.arange(-n / 2, n / 2)) / (n / 2)


def rotvec_to_rotmat(rotvecs):
    """Rodrigues' formula with the reference's ``1e-6`` guard (``poses.py:44-67``)."""
    rotvecs = np.asarray(rotvecs, dtype=np.float64)
    theta = np.linalg.norm(rotvecs, axis=-1, keepdims=True)
    k = rotvecs / (theta + 1e-6)
    K = np.zeros((len(rotvecs), 3, 3))
    K[:, 0, 1] = -k[:, 2]
    K[:, 0, 2] = k[:, 1]
    K[:, 1, 0] = k[:, 2]
    K[:, 1, 2] = -k[:, 0]
    K[:, 2, 0] = -k[:, 1]
    K[:, 2, 1] = k[:, 0]
    th = theta[:, :, None]
    return np.eye(3)[None] + np.sin(th) * K + (1 - np.cos(th)) * (K @ K)


def image_plane(L):
    """``pi * [x, y, 0]`` over the L*L pixels, row-major (y slow, x fast) (``poses.py:197-213``).
    The reference builds this grid in float32 (ASPIRE's default grid dtype), so the values
    are rounded to float32 before use."""
    g = grid_1d(L).astype(np.float32)
    y, x = np.meshgrid(g, g, indexing="ij")
    plane = np.stack([x.ravel(), y.ravel(), np.zeros(L * L, np.float32)])
    return (np.float32(np.pi) * plane).astype(np.float64)


def wrap_pi(p):
    """Wrap to ``[-pi, pi)`` (``poses.py:259-261``, ``nufft_plan.py:327``)."""
    return np.remainder(p + np.pi, 2 * np.pi) - np.pi


def rotated_points(rotmats, L, wrap=True):
    """Rotated central-slice points ``flip_axis0(R @ pi[x, y, 0])`` of shape (N, 3, L*L)
    (``poses.py:254-261``; ``dataset.py:146-164``)."""
    pts = np.flip(np.einsum("nij,jp->nip", np.asarray(rotmats, np.float64), image_plane(L)), axis=1)
    return wrap_pi(pts) if wrap else pts


def phase_shift(offsets, L):
    """``exp(i (gx*ox + gy*oy))`` with ``g = ceil(arange(-L/2, L/2)) * 2*pi/L`` (``poses.py:70-125``)."""
    g = np.ceil(np.arange(-L / 2, L / 2)) * 2 * np.pi / L
    gx, gy = np.meshgrid(g, g, indexing="xy")
    o = np.asarray(offsets, np.float64)
    return np.exp(1j * (gx[None] * o[:, 0, None, None] + gy[None] * o[:, 1, None, None]))


# ----------------------------------------------------------------------------- centered FFTs


def pad_center(x, n, axes):
    """Zero-pad to ``n`` keeping the centre (``projection_funcs.py:11-38``)."""
    out_shape = list(x.shape)
    sl = [slice(None)] * x.ndim
    for a in axes:
        L = x.shape[a]
        start = n // 2 - L // 2
        out_shape[a] = n
        sl[a] = slice(start, start + L)
    out = np.zeros(out_shape, dtype=np.result_type(x, np.complex128))
    out[tuple(sl)] = x
    return out


def crop_center(x, L, axes):
    """Centered crop (``projection_funcs.py:41-64``)."""
    sl = [slice(None)] * x.ndim
    for a in axes:
        n = x.shape[a]
        start = n // 2 - L // 2
        sl[a] = slice(start, start + L)
    return x[tuple(sl)]


def centered_fftn(x, axes, pad_to=None):
    """``fftshift(fft(ifftshift(pad(x))))`` (``projection_funcs.py:148-165``)."""
    if pad_to is not None:
        x = pad_center(x, pad_to, axes)
    return np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(x, axes=axes), axes=axes), axes=axes)


def centered_ifftn(x, axes, crop_to=None):
    y = np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(x, axes=axes), axes=axes), axes=axes)
    return crop_center(y, crop_to, axes) if crop_to is not None else y


def centered_fft3(x, pad_to=None):
    return centered_fftn(x, (-3, -2, -1), pad_to)


def centered_ifft3(x, crop_to=None):
    return centered_ifftn(x, (-3, -2, -1), crop_to)


def centered_fft2(x):
    return centered_fftn(x, (-2, -1))


def centered_ifft2(x):
    return centered_ifftn(x, (-2, -1))


# ----------------------------------------------------------------------------- discretized plan


def grid_sample_index(pts, n):
    """Fractional grid index per point, as ``NufftPlanDiscretized.setpts`` scales the points
    (``nufft_plan.py:109-116``) and grid_sample unnormalises them with ``align_corners=True``
    (``((g + 1) / 2) * (n - 1)``).  Returns (N*P, 3) indices for volume axes 0, 1, 2."""
    pts = np.asarray(pts, np.float64)
    g = pts * (n / (n - 1)) / np.pi
    if n % 2 == 0:
        g = g + 1 / (n - 1)
    t = ((g + 1) / 2) * (n - 1)
    return t.transpose(0, 2, 1).reshape(-1, 3)


def _linear_taps(t, n):
    """Per-axis trilinear taps (index, weight, valid) for grid_sample zeros padding."""
    i0 = np.floor(t).astype(np.int64)
    f = t - i0
    idx = np.stack([i0, i0 + 1], axis=-1)
    wts = np.stack([1 - f, f], axis=-1)
    return idx, wts


def _nearest_taps(t, n):
    idx = np.rint(t).astype(np.int64)[..., None]
    return idx, np.ones_like(idx, dtype=np.float64)


def _taps(t, n, mode):
    return _linear_taps(t, n) if mode == "bilinear" else _nearest_taps(t, n)


def interp_discretized(grid, pts, mode="bilinear"):
    """``NufftPlanDiscretized.execute_forward`` (``nufft_plan.py:120-169``): grid_sample of a
    centered complex grid (C, n, n, n) at (N, 3, P) points, zeros padding, align_corners.
    Returns (C, N, P) complex."""
    grid = np.asarray(grid)
    C, n = grid.shape[0], grid.shape[-1]
    N, _, P = pts.shape
    t = grid_sample_index(pts, n)
    idx, wts = _taps(t, n, mode)
    out = np.zeros((C, N * P), dtype=np.complex128)
    W = idx.shape[-1]
    for a in range(W):
        for b in range(W):
            for c in range(W):
                i0, i1, i2 = idx[:, 0, a], idx[:, 1, b], idx[:, 2, c]
                ok = (i0 >= 0) & (i0 < n) & (i1 >= 0) & (i1 < n) & (i2 >= 0) & (i2 < n)
                wt = wts[:, 0, a] * wts[:, 1, b] * wts[:, 2, c] * ok
                vals = grid[:, np.clip(i0, 0, n - 1), np.clip(i1, 0, n - 1), np.clip(i2, 0, n - 1)]
                out += wt[None] * vals
    return out.reshape(C, N, P)


def spread_discretized(sig, pts, n, mode="bilinear", aggregate=True):
    """Exact adjoint of :func:`interp_discretized` (``nufft_plan.py:171-242``; the reference
    obtains it from autograd through grid_sample).  ``sig`` is (C, N, P) or (N, P).
    Returns (C, n, n, n), or (N, C, n, n, n) when ``aggregate`` is False."""
    sig = np.asarray(sig, np.complex128)
    if sig.ndim == 2:
        sig = sig[None]
    C, N, P = sig.shape
    t = grid_sample_index(pts, n)
    idx, wts = _taps(t, n, mode)
    W = idx.shape[-1]
    flat = sig.reshape(C, N * P)
    img = np.repeat(np.arange(N), P)
    out = np.zeros((N if not aggregate else 1, C, n, n, n), dtype=np.complex128)
    for a in range(W):
        for b in range(W):
            for c in range(W):
                i0, i1, i2 = idx[:, 0, a], idx[:, 1, b], idx[:, 2, c]
                ok = (i0 >= 0) & (i0 < n) & (i1 >= 0) & (i1 < n) & (i2 >= 0) & (i2 < n)
                wt = wts[:, 0, a] * wts[:, 1, b] * wts[:, 2, c]
                sel = np.nonzero(ok)[0]
                for ch in range(C):
                    target = out[:, ch]
                    np.add.at(target, (img[sel] if not aggregate else 0, i0[sel], i1[sel], i2[sel]),
                              wt[sel] * flat[ch, sel])
    return out[0] if aggregate else out


def grid_correction_discretized(L, upsample, mode):
    """sinc (nearest) or sinc^2 (bilinear) deapodisation (``covar.py:45-65``, ``mean.py:27-40``)."""
    pos = np.arange(-(L // 2), (L - 1) // 2 + 1) / L
    pos = np.pi * pos / upsample
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.sin(pos) / pos
    s[pos == 0] = 1
    s[s < 1e-6] = 1
    if mode == "bilinear":
        s = s**2
    return np.einsum("i,j,k->ijk", s, s, s)


# ----------------------------------------------------------------------------- ES kernel NUFFT


def es_beta(width, upsample=2.0):
    """ES shape parameter ``beta = gamma * pi * (1 - 1/(2 sigma)) * w`` with gamma = 0.97
    (Barnett, Magland & af Klinteberg, SIAM J. Sci. Comput. 2019, Sec. 4)."""
    return 0.97 * np.pi * (1.0 - 1.0 / (2.0 * upsample)) * width


def es_kernel(x, width, beta):
    """``exp(beta * (sqrt(1 - (2x/w)^2) - 1))`` on ``|x| < w/2``, else 0."""
    u = 2.0 * np.asarray(x, np.float64) / width
    inside = np.abs(u) < 1
    out = np.zeros_like(u)
    out[inside] = np.exp(beta * (np.sqrt(1.0 - u[inside] ** 2) - 1.0))
    return out


def es_fourier(alpha, width, beta, nodes=200):
    """``psi_hat(alpha) = int psi(x) exp(-i alpha x) dx`` by Gauss-Legendre quadrature."""
    xq, wq = np.polynomial.legendre.leggauss(nodes)
    half = width / 2.0
    x = (xq + 1) * half / 2.0
    wts = wq * half / 2.0
    alpha = np.asarray(alpha, np.float64)
    return 2.0 * np.sum(wts * es_kernel(x, width, beta) * np.cos(alpha[..., None] * x), axis=-1)


def grid_correction_es(L, n, width, beta):
    """Deapodisation ``psi_hat(2 pi k0/n) psi_hat(2 pi k1/n) psi_hat(2 pi k2/n)`` for voxel
    offsets ``k = j - L//2``; replaces the sinc^2 of ``covar.py:45-65`` for the ES kernel."""
    k = np.arange(L) - L // 2
    h = es_fourier(2 * np.pi * k / n, width, beta)
    return np.einsum("i,j,k->ijk", h, h, h)


def es_index(pts, n):
    """Fractional centered-grid index ``omega*n/(2 pi) + n//2`` of wrapped points, (N*P, 3)."""
    p = wrap_pi(np.asarray(pts, np.float64))
    t = p * n / (2 * np.pi) + n // 2
    return t.transpose(0, 2, 1).reshape(-1, 3)


def _es_taps(t, width, beta):
    base = np.ceil(t - width / 2.0).astype(np.int64)
    offs = np.arange(width)
    idx = base[..., None] + offs
    wts = es_kernel(t[..., None] - idx, width, beta)
    return idx, wts


def es_interp(grid, pts, width, beta):
    """ES-kernel interpolation of a centered fine grid (C, n, n, n) with periodic wrap.
    Returns (C, N*P)."""
    C, n = grid.shape[0], grid.shape[-1]
    t = es_index(pts, n)
    idx, wts = _es_taps(t, width, beta)
    out = np.zeros((C, len(t)), np.complex128)
    for a in range(width):
        for b in range(width):
            wab = wts[:, 0, a] * wts[:, 1, b]
            i0 = np.mod(idx[:, 0, a], n)
            i1 = np.mod(idx[:, 1, b], n)
            for c in range(width):
                out += (wab * wts[:, 2, c])[None] * grid[:, i0, i1, np.mod(idx[:, 2, c], n)]
    return out


def es_spread(sig, pts, n, width, beta):
    """Exact adjoint of :func:`es_interp`: (C, N*P) -> (C, n, n, n)."""
    sig = np.asarray(sig, np.complex128)
    C = sig.shape[0]
    t = es_index(pts, n)
    idx, wts = _es_taps(t, width, beta)
    out = np.zeros((C, n, n, n), np.complex128)
    for a in range(width):
        for b in range(width):
            for c in range(width):
                wt = wts[:, 0, a] * wts[:, 1, b] * wts[:, 2, c]
                key = (np.mod(idx[:, 0, a], n), np.mod(idx[:, 1, b], n), np.mod(idx[:, 2, c], n))
                for ch in range(C):
                    np.add.at(out[ch], key, wt * sig[ch])
    return out


def es_type2(vol, pts, upsample=2, width=7, beta=None):
    """Type-2 NUFFT of spatial volumes (C, L, L, L) at (N, 3, P) points by the ES algorithm:
    deapodise, zero-pad to n = upsample*L, centered FFT, ES interpolation.  Same semantics as
    ``NufftPlan.execute_forward`` (``nufft_plan.py:338-364``).  Returns (C, N, P)."""
    vol = np.asarray(vol)
    C, L = vol.shape[0], vol.shape[-1]
    n = int(round(upsample * L))
    beta = es_beta(width, upsample) if beta is None else beta
    gc = grid_correction_es(L, n, width, beta)
    grid = centered_fft3(vol / gc, pad_to=n)
    return es_interp(grid, pts, width, beta).reshape(C, pts.shape[0], pts.shape[2])


def es_type1(sig, pts, L, upsample=2, width=7, beta=None):
    """Type-1 (adjoint) NUFFT: (C, N, P) -> (C, L, L, L); exact adjoint of :func:`es_type2`
    (``NufftPlan.execute_adjoint``, ``nufft_plan.py:366-392``)."""
    sig = np.asarray(sig, np.complex128)
    C = sig.shape[0]
    n = int(round(upsample * L))
    beta = es_beta(width, upsample) if beta is None else beta
    gc = grid_correction_es(L, n, width, beta)
    fine = es_spread(sig.reshape(C, -1), pts, n, width, beta)
    # adjoint of centered_fft3 with padding = n^3 * centered_ifft3 followed by crop
    return centered_ifft3(fine, crop_to=L) * n**3 / gc


def nudft_type2(vol, pts):
    """Exact direct sum ``F(w) = sum_k V[k] exp(-i w.k)``, k = j - L//2 per axis, pairing
    point row d with volume axis d (``nufft_plan.py:326,335``).  (C, L, L, L) -> (C, N, P)."""
    vol = np.asarray(vol, np.complex128)
    C, L = vol.shape[0], vol.shape[-1]
    N, _, P = pts.shape
    k = np.arange(L) - L // 2
    p = np.asarray(pts, np.float64).transpose(0, 2, 1).reshape(-1, 3)
    e0 = np.exp(-1j * p[:, 0, None] * k[None])
    e1 = np.exp(-1j * p[:, 1, None] * k[None])
    e2 = np.exp(-1j * p[:, 2, None] * k[None])
    out = np.einsum("cabd,ma,mb,md->cm", vol, e0, e1, e2, optimize=True)
    return out.reshape(C, N, P)


def nudft_type1(sig, pts, L):
    """Adjoint of :func:`nudft_type2`: (C, N, P) -> (C, L, L, L)."""
    sig = np.asarray(sig, np.complex128)
    C = sig.shape[0]
    k = np.arange(L) - L // 2
    p = np.asarray(pts, np.float64).transpose(0, 2, 1).reshape(-1, 3)
    e0 = np.exp(1j * p[:, 0, None] * k[None])
    e1 = np.exp(1j * p[:, 1, None] * k[None])
    e2 = np.exp(1j * p[:, 2, None] * k[None])
    return np.einsum("cm,ma,mb,md->cabd", sig.reshape(C, -1), e0, e1, e2, optimize=True)


# ----------------------------------------------------------------------------- projection ops


def nyquist_mask(L):
    """1 everywhere except row 0 and column 0 when L is even (``projection_funcs.py:355-358``)."""
    m = np.ones((L, L))
    if L % 2 == 0:
        m[0, :] = 0
        m[:, 0] = 0
    return m


def vol_forward_fourier(samples, filters, L):
    """Epilogue of ``vol_forward(..., fourier_domain=True)`` (``projection_funcs.py:346-370``):
    (C, N, P) plan output -> (N, C, L, L): Nyquist zeroing, x CTF, / L."""
    C, N, _ = samples.shape
    out = samples.reshape(C, N, L, L).transpose(1, 0, 2, 3) * nyquist_mask(L)
    if filters is not None:
        out = out * np.asarray(filters)[:, None]
    return out / L


def im_backward_fourier_prologue(images, filters, L):
    """Prologue of ``im_backward(..., fourier_domain=True)`` (``projection_funcs.py:373-399``):
    x CTF, Nyquist zeroing.  The plan adjoint follows, then / L."""
    out = np.asarray(images, np.complex128)
    if filters is not None:
        out = out * filters
    return out * nyquist_mask(L)


# ----------------------------------------------------------------------------- costs


def latent_map_batch(images, eigen_forward, noise_var, eigenvals_inv=None):
    """``compute_latentMAP_batch`` (``wiener_coords.py:168-203``): m = conj(Q) Q^T / s2 + Linv,
    b = conj(Q) y / s2, z = m^-1 b (trace-normalised solve).  Returns (z, m, b)."""
    y = np.asarray(images).reshape(len(images), -1, 1).astype(np.complex128)
    Q = np.asarray(eigen_forward).reshape(y.shape[0], -1, y.shape[1]).astype(np.complex128)
    r = Q.shape[1]
    Linv = np.eye(r) if eigenvals_inv is None else np.asarray(eigenvals_inv)
    m = np.conj(Q) @ Q.transpose(0, 2, 1) / noise_var + Linv
    b = np.conj(Q) @ y / noise_var
    t = np.abs(np.diagonal(m, axis1=1, axis2=2)).sum(1) / r
    z = np.linalg.solve(m / t[:, None, None], b) / t[:, None, None]
    return z, m, b


def ml_cost_and_w(Q, y, noise_var, eigenvals_inv=None):
    """Per-image ML data term of ``raw_cost_maximum_liklihood_fourier_domain``
    (``covar_sgd.py:1381-1399``): ``0.5 * (-b^H z + logdet m)``, and its conjugate-Wirtinger
    derivative ``W = d cost / d conj(Q)`` = ``(conj(m^-1) Q - conj(z) (y - Q^T z)^T) / (2 s2)``.
    Q: (B, r, P) complex, y: (B, P).  Returns (cost (B,), W (B, r, P))."""
    Q = np.asarray(Q, np.complex128)
    y = np.asarray(y, np.complex128).reshape(Q.shape[0], -1)
    z, m, b = latent_map_batch(y, Q, noise_var, eigenvals_inv)
    z = z[..., 0]
    b = b[..., 0]
    sign, logabs = np.linalg.slogdet(m)
    cost = 0.5 * (-np.real(np.sum(np.conj(b) * z, axis=1)) + logabs)
    minv = np.linalg.inv(m)
    resid = y - np.einsum("bi,bip->bp", z, Q)
    W = (np.einsum("bij,bjp->bip", np.conj(minv), Q) - np.conj(z)[:, :, None] * resid[:, None, :]) / (2 * noise_var)
    return cost, W


def ls_cost_and_w(Q, y, noise_var):
    """Per-image LS data term of ``raw_cost_fourier_domain`` (``covar_sgd.py:1320-1347``):
    ``-2 sum |Q conj(y)|^2 + ||Q Q^H||_F^2 + 2 s2 tr(Q Q^H)`` and its conjugate-Wirtinger
    derivative ``2 (Q Q^H) Q + 2 s2 Q - 2 t y^T`` with ``t = Q conj(y)``."""
    Q = np.asarray(Q, np.complex128)
    y = np.asarray(y, np.complex128).reshape(Q.shape[0], -1)
    t = np.einsum("bip,bp->bi", Q, np.conj(y))
    M = np.einsum("bip,bjp->bij", Q, np.conj(Q))
    cost = -2 * np.sum(np.abs(t) ** 2, 1) + np.sum(np.abs(M) ** 2, (1, 2)) + 2 * noise_var * np.real(
        np.trace(M, axis1=1, axis2=2))
    W = 2 * np.einsum("bij,bjp->bip", M, Q) + 2 * noise_var * Q - 2 * t[:, :, None] * y[:, None, :]
    return cost, W


def covar_cost_grad(vectors, log_sqrt, images, pts, filters, noise_var, upsample=2, kind="bilinear",
                    objective="ml", reg_scale=0.0, fourier_reg=None, width=6, beta=None):
    """Covariance-SGD batch cost and its exact gradient w.r.t. the ``Covar`` parameters
    (``vectors`` (r, L, L, L), ``log_sqrt_eigenvals`` (r,)), restating
    ``Covar.get_vectors_fourier_domain`` (``covar.py:440-449``) followed by
    ``cost_maximum_liklihood_fourier_domain`` / ``cost_fourier_domain``
    (``covar_sgd.py:1290-1378``) in float64.  ``kind`` is "bilinear", "nearest" (grid_sample
    plans) or "es" (ES-kernel plan with periodic wrap).  Returns (cost, g_vectors, g_logsqrt)."""
    vectors = np.asarray(vectors, np.float64)
    r, L = vectors.shape[0], vectors.shape[-1]
    n = L * upsample
    B = images.shape[0]
    scale = np.exp(np.asarray(log_sqrt, np.float64))
    V = vectors * scale[:, None, None, None]
    if kind == "es":
        beta = es_beta(width, upsample) if beta is None else beta
        gc = grid_correction_es(L, n, width, beta)
        grid = centered_fft3(V / gc, pad_to=n)
        samples = es_interp(grid, pts, width, beta).reshape(r, B, -1)
    else:
        gc = grid_correction_discretized(L, upsample, kind)
        grid = centered_fft3(V / gc, pad_to=n)
        samples = interp_discretized(grid, pts, kind)
    Q = vol_forward_fourier(samples, filters, L).reshape(B, r, L * L)
    y = np.asarray(images, np.complex128).reshape(B, L * L)
    if objective == "ml":
        per, W = ml_cost_and_w(Q, y, noise_var)
        cost = np.mean(per)
        W = W / B
        greg_scale = reg_scale / noise_var / 2.0
    else:
        per, W = ls_cost_and_w(Q, y, noise_var)
        cost = np.mean(per) / L**4
        W = W / B / L**4
        greg_scale = None
    # adjoint of the epilogue: x CTF x Nyquist mask / L, back to (r, B*P)
    Wp = W.reshape(B, r, L, L) * nyquist_mask(L)
    if filters is not None:
        Wp = Wp * np.asarray(filters)[:, None]
    Wp = (Wp / L).transpose(1, 0, 2, 3).reshape(r, -1)
    if kind == "es":
        ggrid = es_spread(Wp, pts, n, width, beta)
    else:
        ggrid = spread_discretized(Wp.reshape(r, B, -1), pts, n, kind)
    if fourier_reg is not None and reg_scale != 0:
        fr = np.asarray(fourier_reg, np.float64)
        if objective == "ml":
            cost += reg_scale * np.sum(np.abs(grid) ** 2 * fr) / noise_var / 2.0
            ggrid = ggrid + greg_scale * fr * grid
        else:
            # the reference reads ``rank = vols[0].shape[0]`` (covar_sgd.py:1302), which is the
            # grid size n, so its Gram matrix is of the (n, r*n*n) reshape; kept for parity
            G = (grid * np.sqrt(fr)).reshape(n, -1)
            Mr = G @ np.conj(G).T
            cost += reg_scale * np.sum(np.abs(Mr) ** 2) / L**4
            ggrid = ggrid + (reg_scale / L**4) * 2 * (Mr @ G).reshape(grid.shape) * np.sqrt(fr)
    # adjoint of centered_fft3 with padding: n^3 * centered_ifft3 then crop; then / gc
    gV = 2.0 * np.real(centered_ifft3(ggrid, crop_to=L) * n**3) / gc
    g_vectors = gV * scale[:, None, None, None]
    g_logsqrt = np.sum(gV * V, axis=(1, 2, 3))
    return cost, g_vectors, g_logsqrt


# ----------------------------------------------------------------------------- mean / CG


def shell_index(L, dim):
    """Radial shell of every centered index (``fsc_utils.py:43-91``): shell i holds radii in
    (i - 0.5, i + 0.5), the last shell (i - 0.5, i + 1)."""
    g = np.ceil(np.arange(-L / 2, L / 2))
    grids = np.meshgrid(*([g] * dim), indexing="ij")
    rad = np.sqrt(sum(x * x for x in grids))
    nshell = int(np.ceil(rad.max()))
    idx = np.full(rad.shape, -1, np.int64)
    for i in range(nshell):
        lo = i - 0.5
        hi = i + 0.5 if i < nshell - 1 else i + 1
        idx[(rad > lo) & (rad < hi)] = i
    return idx, nshell


def average_fourier_shell(x):
    """Shell average (``fsc_utils.py:116-135``)."""
    idx, ns = shell_index(x.shape[-1], x.ndim)
    out = np.zeros(ns, dtype=x.dtype)
    for i in range(ns):
        sel = idx == i
        out[i] = x[sel].sum() / sel.sum()
    return out


def expand_fourier_shell(shells, L, dim):
    """Shell expansion (``fsc_utils.py:165-184``)."""
    idx, ns = shell_index(L, dim)
    out = np.zeros((L,) * dim)
    for i in range(len(shells)):
        out[idx == i] = shells[i]
    return out


def regularize_lhs(lhs):
    """``max(|lhs|, 1e-3 * shell mean of Re lhs)`` clamped at 1e-8 (``mean.py:135-142``)."""
    reg = average_fourier_shell(np.real(lhs)) * 1e-3
    reg = expand_fourier_shell(reg, lhs.shape[-1], 3)
    return np.maximum(np.maximum(np.abs(lhs), reg), 1e-8)


def padding_operator(reg_lhs, L):
    """``A(x) = crop(ifft3(reg_lhs * fft3(pad(x))))`` (``mean.py:118-123``)."""
    n = reg_lhs.shape[-1]

    def A(x):
        X = centered_fft3(x.reshape(L, L, L), pad_to=n)
        return centered_ifft3(reg_lhs * X, crop_to=L).reshape(-1)

    return A


def conjugate_gradient(A, b, x0=None, rtol=1e-6, maxiter=None, precond=None):
    """``complex_conjugate_gradient`` (``mean.py:43-93``); with ``precond`` given, the
    standard preconditioned variant (z = M r).  Returns (x, iterations, residual history)."""
    x = np.zeros_like(b) if x0 is None else x0.astype(np.complex128).copy()
    r = b - A(x)
    z = precond(r) if precond is not None else r
    p = z.copy()
    rz = np.real(np.vdot(r, z))
    maxiter = len(b) * 10 if maxiter is None else maxiter
    bn = np.linalg.norm(b)
    hist = [np.linalg.norm(r) / bn]
    it = 0
    for it in range(maxiter):
        Ap = A(p)
        alpha = rz / np.vdot(p, Ap)
        x = x + alpha * p
        r = r - alpha * Ap
        hist.append(np.linalg.norm(r) / bn)
        if np.linalg.norm(r) < rtol * bn:
            break
        z = precond(r) if precond is not None else r
        rz_new = np.real(np.vdot(r, z))
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, it, np.array(hist)


def sphere_mask(L):
    """``grid_3d(L, normalized=True)["r"] <= 1`` (``mean.py:248-250``)."""
    g = grid_1d(L)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    return np.sqrt(x * x + y * y + z * z) <= 1


def phase_shift_grid(L):
    """``get_phase_shift_grid`` (``poses.py:70-89``): (gx, gy) with gx[i, j] = g[j], gy[i, j] = g[i],
    g = ceil(k - L/2) 2 pi / L."""
    g = np.ceil(np.arange(-L / 2, L / 2)) * 2 * np.pi / L
    gx, gy = np.meshgrid(g, g, indexing="xy")
    return gx, gy


def mean_backprojection(images, pts, filters, offsets, contrasts, L, upsample=2):
    """Loop body of ``reconstruct_mean`` (``mean.py:196-215``) over all images at once with the
    nearest plan: rhs = sum im_backward(y * phase(-offset), c ctf), lhs = sum im_backward(c ctf,
    c ctf) / L.  Returns (rhs, lhs), centered (n, n, n) complex."""
    n = L * upsample
    N = images.shape[0]
    images = np.asarray(images, np.complex128).reshape(N, L, L)
    gx, gy = phase_shift_grid(L)
    off = -np.asarray(offsets, np.float64)
    ph = np.exp(1j * (gx[None] * off[:, 0, None, None] + gy[None] * off[:, 1, None, None]))
    f = np.asarray(filters, np.float64).reshape(N, L, L) * np.asarray(contrasts, np.float64)[:, None, None]
    y = im_backward_fourier_prologue(images * ph, f, L).reshape(N, L * L)
    k = im_backward_fourier_prologue(f.astype(np.complex128), f, L).reshape(N, L * L)
    rhs = spread_discretized(y, pts, n, mode="nearest")[0] / L
    lhs = spread_discretized(k, pts, n, mode="nearest")[0] / L / L
    return rhs, lhs


def reconstruct_mean(images, pts, filters, offsets, contrasts, L, upsample=2, rtol=1e-6, grid_correction=True,
                     precond=None):
    """``reconstruct_mean`` (``mean.py:145-259``) without init_vol / mask: backprojection,
    ``regularize_lhs``, the Fourier-diagonal solve, ``correct_upsampling_padding``, the
    sphere mask and the nearest grid correction.  Returns (volume, rhs, lhs, iterations)."""
    rhs, lhs = mean_backprojection(images, pts, filters, offsets, contrasts, L, upsample)
    reg = regularize_lhs(lhs)
    vol = np.real(centered_ifft3(rhs / reg, crop_to=L))
    it = -1
    if upsample > 1:
        b = centered_ifft3(rhs, crop_to=L).reshape(-1)
        x, it, _ = conjugate_gradient(padding_operator(reg, L), b, x0=vol.reshape(-1).astype(np.complex128),
                                      rtol=rtol, precond=precond)
        vol = x.reshape((L,) * 3).real
    vol = np.real(centered_ifft3(centered_fft3(vol) * sphere_mask(L)))
    if grid_correction:
        vol = vol / grid_correction_discretized(L, upsample, "nearest")
    return vol, rhs, lhs, it


def circulant_symbol(reg_lhs, L):
    """Fourier symbol (centered, L^3) of T. Chan's optimal circulant approximation of
    ``padding_operator(reg_lhs, L)``: its convolution kernel t = ifft_n(reg_lhs) folded per axis
    as c[tau] = ((L - tau) t[tau] + tau t[tau - L]) / L, then fft_L."""
    n = reg_lhs.shape[-1]
    t = np.fft.ifftn(np.fft.ifftshift(reg_lhs))
    tau = np.arange(L)
    opts = [(tau, (L - tau) / L), ((tau - L) % n, tau / L)]
    c = np.zeros((L, L, L), np.complex128)
    for i0, w0 in opts:
        for i1, w1 in opts:
            for i2, w2 in opts:
                c += t[np.ix_(i0, i1, i2)] * w0[:, None, None] * w1[None, :, None] * w2[None, None, :]
    return np.fft.fftshift(np.real(np.fft.fftn(c)))


def circulant_preconditioner(symbol):
    """M r = ifft_L(fft_L(r) / symbol) with a centered symbol (L^3)."""
    L = symbol.shape[-1]
    native = np.fft.ifftshift(symbol)

    def M(r):
        return np.fft.ifftn(np.fft.fftn(r.reshape(L, L, L)) / native).reshape(-1)

    return M


def fine_diagonal_preconditioner(reg_lhs, L):
    """M r = crop(ifft3(fft3(pad r) / reg_lhs)): the Fourier-diagonal solve on the fine grid."""
    n = reg_lhs.shape[-1]

    def M(r):
        return centered_ifft3(centered_fft3(r.reshape(L, L, L), pad_to=n) / reg_lhs, crop_to=L).reshape(-1)

    return M


# ----------------------------------------------------------------------------- half-set regularisation


def shell_average_batch(x):
    """``average_fourier_shell`` over the last three axes of (..., L, L, L) (fsc_utils.py:116-135,
    199-208): shape (..., S)."""
    L = x.shape[-1]
    idx, ns = shell_index(L, 3)
    flat = x.reshape(x.shape[:-3] + (-1,))
    out = np.zeros(x.shape[:-3] + (ns,), dtype=x.dtype)
    for i in range(ns):
        sel = (idx == i).reshape(-1)
        out[..., i] = flat[..., sel].sum(-1) / sel.sum()
    return out


def shell_sizes(L):
    idx, ns = shell_index(L, 3)
    return np.array([(idx == i).sum() for i in range(ns)], np.float64)


def expand_shells(shells, L):
    """``expand_fourier_shell`` (fsc_utils.py:166-184, 223-234) of (..., S) to (..., L, L, L)."""
    idx, ns = shell_index(L, 3)
    shells = np.asarray(shells)
    out = np.zeros(shells.shape[:-1] + (L, L, L), dtype=shells.dtype)
    for i in range(min(ns, shells.shape[-1])):
        out[..., idx == i] = shells[..., i:i + 1]
    return out


def upsample_expand_shells(shells, L):
    """``upsample_and_expand_fourier_shell`` (fsc_utils.py:237-255): linear resampling of the
    shell profile (align_corners=False) to the shell count of an L^3 grid, then expansion."""
    from .unet_oracle import _lin_matrix

    shells = np.atleast_2d(np.asarray(shells, np.float64))
    ns = shell_index(L, 3)[1]
    up = shells @ _lin_matrix(shells.shape[-1], ns).T
    up = up[0] if up.shape[0] == 1 else up
    return expand_shells(up, L)


def rpsd_batch(signals):
    """``rpsd`` (fsc_utils.py:137-147, 211-220): shell averages of |centered_fft3|^2."""
    return shell_average_batch(np.abs(centered_fft3(np.asarray(signals))) ** 2)


def vol_fsc(a, b):
    """``vol_fsc`` (fsc_utils.py:272-291)."""
    fa, fb = centered_fft3(a), centered_fft3(b)
    c, p1, p2 = shell_average_batch(np.stack([np.real(fa * np.conj(fb)), np.abs(fa) ** 2, np.abs(fb) ** 2]))
    return c / np.sqrt(p1 * p2)


def covar_correlate(f1, f2):
    """``covar_correlate`` (fsc_utils.py:312-340): sum_i s_i^T conj(s_i) with s_i the shell
    averages of f1[i] * conj(f2) (r x S)."""
    ns = shell_index(f1.shape[-1], 3)[1]
    out = np.zeros((ns, ns), np.complex128)
    for i in range(f1.shape[0]):
        s = shell_average_batch(f1[i][None] * np.conj(f2))
        out += s.T @ np.conj(s)
    return out


def covar_rpsd(e):
    f = centered_fft3(np.asarray(e))
    sz = shell_sizes(e.shape[-1])
    return np.real(covar_correlate(f, f)) * np.outer(sz, sz)


def covar_fsc(e1, e2):
    """``covar_fsc`` (fsc_utils.py:343-367)."""
    f1, f2 = centered_fft3(np.asarray(e1)), centered_fft3(np.asarray(e2))
    c = np.real(covar_correlate(f1, f2))
    r1, r2 = np.real(covar_correlate(f1, f1)), np.real(covar_correlate(f2, f2))
    return c / np.sqrt(r1 * r2)


def total_gain(pts, filters, L):
    """``CovarDataset.get_total_gain`` (dataset.py:322-356): |sum im_backward(ctf, ctf)| / L with
    the nearest plan at upsampling 1 (the magnitude per batch of 16 images, as the reference)."""
    f = np.asarray(filters, np.float64)
    out = np.zeros((L, L, L))
    for lo in range(0, len(f), 16):
        sl = slice(lo, lo + 16)
        sig = im_backward_fourier_prologue(f[sl].astype(np.complex128), f[sl], L).reshape(len(f[sl]), -1)
        out += np.abs(spread_discretized(sig, pts[sl], L, mode="nearest")[0] / L)
    return out / L


def total_covar_gain(pts, filters, L):
    """``CovarDataset.get_total_covar_gain`` (dataset.py:358-421): sum over images of the outer
    product of the shell averages of |per-image adjoint of ctf^2| / L^2."""
    f = np.asarray(filters, np.float64).copy()
    if L % 2 == 0:
        f[:, 0, :] = 0
        f[:, :, 0] = 0
    g = np.abs(spread_discretized((f**2).reshape(len(f), -1).astype(np.complex128), pts, L, mode="nearest",
                                  aggregate=False)[:, 0]) / L**2
    s = shell_average_batch(g)
    return s.T @ s


def updated_fourier_reg(e1, e2, filter_gain, L, fourier_domain=True):
    """``compute_updated_fourier_reg`` (covar_sgd.py:1155-1187) without a mask."""
    with np.errstate(divide="ignore"):
        corr = 1.0 / np.asarray(filter_gain, np.float64)
    corr[:, L // 2:] = corr[L // 2, L // 2]
    corr[L // 2:, :] = corr[L // 2, L // 2]
    fsc = np.clip(covar_fsc(e1, e2), 1e-6, 1 - 1e-6)
    reg = 1.0 / ((fsc / (1 - fsc)) * corr)
    reg[reg < 0] = 0
    out = expand_shells(np.sqrt(np.diag(reg))[None], L)[0]
    return (out if fourier_domain else out / L**2), fsc


def fourier_reg_term(e, upsample, L, noise_var):
    """``CovarTrainer.compute_fourier_reg_term`` (covar_sgd.py:420-430)."""
    rp = rpsd_batch(e) * upsample**3
    return noise_var / upsample_expand_shells(rp, L * upsample)


def fourier_reg_halfsets(reg, upsample, L):
    """``CovarTrainer.update_fourier_reg_halfsets`` (covar_sgd.py:432-447), Fourier domain."""
    radial = shell_average_batch(np.asarray(reg)) / upsample**3
    return upsample_expand_shells(radial, L * upsample)


def regularize_mean_from_halfsets(m1, rhs1, lhs1, m2, rhs2, lhs2, rtol=1e-6):
    """``regularize_mean_from_halfsets`` (mean.py:359-421) without a mask.  Returns (volume,
    iterations)."""
    L = m1.shape[-1]
    n = lhs1.shape[-1]
    us = n // L
    gain = np.abs(centered_fft3(centered_ifft3(lhs1 + lhs2, crop_to=L))) / 2
    avg_gain = shell_average_batch(1.0 / gain)
    fsc = np.clip(vol_fsc(m1, m2), 1e-3, 1 - 1e-3)
    reg = 1.0 / ((fsc / (1 - fsc)) * avg_gain)
    reg = upsample_expand_shells(reg[None], n)
    reg_lhs = regularize_lhs(lhs1 + lhs2 + reg)
    rhs = rhs1 + rhs2
    vol = np.real(centered_ifft3(rhs / reg_lhs, crop_to=L))
    it = -1
    if us > 1:
        b = centered_ifft3(rhs, crop_to=L).reshape(-1)
        x, it, _ = conjugate_gradient(padding_operator(reg_lhs, L), b, x0=vol.reshape(-1).astype(np.complex128),
                                      rtol=rtol)
        vol = x.reshape((L,) * 3).real
    vol = np.real(centered_ifft3(centered_fft3(vol) * sphere_mask(L)))
    return vol / grid_correction_discretized(L, us, "nearest"), it


# ----------------------------------------------------------------------------- CTF from parameters


def ctf_from_params(params, L):
    """(N, 8) CTF parameters -> (N, L, L) float64 CTF images: the weak-phase CTF
    ``sqrt(1 - w^2) sin(gamma) - w cos(gamma)``, ``gamma = 2 pi (-df lam s^2 / 2 + Cs lam^3 s^4 / 4) -
    phase``, ``df = (dfu + dfv + (dfu - dfv) cos(2 (atan2(fy, fx) - dfang))) / 2``,
    ``lam = 12.2639 / sqrt(V + 0.97845e-6 V^2)``, as cryoDRGN's ``compute_ctf`` defines it for the
    reference's ``ImageSource.get_ctf`` (``source.py:157-172``), on the frequency lattice of
    ``get_phase_shift_grid`` (``poses.py:70-89``; first coordinate along image rows) divided by
    the pixel size.  Columns: pixel size (A), dfu, dfv (A), dfang (deg), voltage (kV), Cs (mm),
    amplitude contrast, phase shift (deg).  cryoDRGN is not installed here, so this restatement
    of its published formula is the CTF's only pin (parity unpinned against cryoDRGN itself)."""
    p = np.asarray(params, np.float64).reshape(-1, 8)
    apix, dfu, dfv, dfang, volt, cs, w, ps = [p[:, i, None, None] for i in range(8)]
    k = np.ceil(np.arange(-L / 2, L / 2))
    fx = k[None, :, None] / (L * apix)
    fy = k[None, None, :] / (L * apix)
    volt = volt * 1e3
    cs = cs * 1e7
    lam = 12.2639 / np.sqrt(volt + 0.97845e-6 * volt**2)
    ang = np.arctan2(fy, fx)
    s2 = fx**2 + fy**2
    df = 0.5 * (dfu + dfv + (dfu - dfv) * np.cos(2 * (ang - dfang * np.pi / 180)))
    gamma = 2 * np.pi * (-0.5 * df * lam * s2 + 0.25 * cs * lam**3 * s2**2) - ps * np.pi / 180
    return np.sqrt(1 - w**2) * np.sin(gamma) - w * np.cos(gamma)
