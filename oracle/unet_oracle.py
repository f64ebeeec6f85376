"""Float64 numpy restatement of the learned-preconditioner network (test infrastructure: only
the tests import it, as the checker of the CUDA kernels in ``csrc/unet.cu``).

The network has no counterpart in the reference; it follows the architecture stated in
``3dcovarestimation_gb300/learned_pc.py``: a 3-level 3D U-Net (convolutions 3x3x3 with ReLU,
2x average pooling, 2x nearest upsampling, skip connections by channel concatenation, a 1x1x1
head).  Layout (N, C, D, H, W); weights (Cout, Cin, k, k, k).  The backward pass is written
out by hand (no autodiff) and is itself checked against finite differences in the CPU tests.
"""

import numpy as np


def _shifts(k):
    r = k // 2
    return [(a - r, b - r, c - r) for a in range(k) for b in range(k) for c in range(k)]


def _shifted(xp, r, s, shape):
    D, H, W = shape
    dz, dy, dx = s
    return xp[..., r + dz:r + dz + D, r + dy:r + dy + H, r + dx:r + dx + W]


def conv3d(x, w, b=None, relu=False):
    """y[n, o] = b[o] + sum_c sum_t w[o, c, t] x[n, c, v + off(t)], zero padding k // 2."""
    k = w.shape[-1]
    r = k // 2
    xp = np.pad(x, [(0, 0), (0, 0)] + [(r, r)] * 3)
    wf = w.reshape(w.shape[0], w.shape[1], -1)
    y = np.zeros((x.shape[0], w.shape[0]) + x.shape[2:])
    for t, s in enumerate(_shifts(k)):
        y += np.einsum("oc,ncdhw->nodhw", wf[:, :, t], _shifted(xp, r, s, x.shape[2:]))
    if b is not None:
        y += b[None, :, None, None, None]
    return np.maximum(y, 0.0) if relu else y


def conv3d_backward_data(gy, w):
    k = w.shape[-1]
    wt = np.flip(w, axis=(2, 3, 4)).transpose(1, 0, 2, 3, 4)
    return conv3d(gy, np.ascontiguousarray(wt))


def conv3d_backward_weight(x, gy, k):
    r = k // 2
    xp = np.pad(x, [(0, 0), (0, 0)] + [(r, r)] * 3)
    gw = np.zeros((gy.shape[1], x.shape[1], k * k * k))
    for t, s in enumerate(_shifts(k)):
        gw[:, :, t] = np.einsum("nodhw,ncdhw->oc", gy, _shifted(xp, r, s, x.shape[2:]))
    return gw.reshape(gy.shape[1], x.shape[1], k, k, k), gy.sum(axis=(0, 2, 3, 4))


def avgpool2(x):
    s = x.shape
    return x.reshape(s[:2] + (s[2] // 2, 2, s[3] // 2, 2, s[4] // 2, 2)).mean(axis=(3, 5, 7))


def avgpool2_adjoint(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 2), 2, 3), 2, 4) / 8.0


def upsample2(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 2), 2, 3), 2, 4)


def upsample2_adjoint(g):
    s = g.shape
    return g.reshape(s[:2] + (s[2] // 2, 2, s[3] // 2, 2, s[4] // 2, 2)).sum(axis=(3, 5, 7))


def _lin_matrix(d, D):
    """(D, d) matrix of 1-D linear interpolation with align_corners = False (edge-clamped)."""
    M = np.zeros((D, d))
    for i in range(D):
        s = max((i + 0.5) * d / D - 0.5, 0.0)
        i0 = min(int(np.floor(s)), d - 1)
        i1 = min(i0 + 1, d - 1)
        f = s - i0
        M[i, i0] += 1 - f
        M[i, i1] += f
    return M


def trilinear(x, D):
    """(..., d, d, d) -> (..., D, D, D)."""
    M = _lin_matrix(x.shape[-1], D)
    return np.einsum("ia,jb,kc,...abc->...ijk", M, M, M, x)


def trilinear_adjoint(g, d):
    M = _lin_matrix(d, g.shape[-1])
    return np.einsum("ia,jb,kc,...ijk->...abc", M, M, M, g)


def block_mean(x, d):
    D = x.shape[-1]
    k = D // d
    s = x.shape[:-3]
    return x.reshape(s + (d, k, d, k, d, k)).mean(axis=(-5, -3, -1))


def architecture(cin, c):
    """(name, input channels, output channels, kernel size, relu) of every convolution."""
    return [("enc0a", cin, c, 3, True), ("enc0b", c, c, 3, True),
            ("enc1a", c, 2 * c, 3, True), ("enc1b", 2 * c, 2 * c, 3, True),
            ("mida", 2 * c, 4 * c, 3, True), ("midb", 4 * c, 4 * c, 3, True),
            ("dec1a", 6 * c, 2 * c, 3, True), ("dec1b", 2 * c, 2 * c, 3, True),
            ("dec0a", 3 * c, c, 3, True), ("dec0b", c, c, 3, True),
            ("head", c, 1, 1, False)]


def unet_forward(params, x):
    """params: name -> (w, b).  Returns (out (N, 1, D, D, D), cache)."""
    a = {}

    def conv(name, inp):
        w, b = params[name]
        a[name + ":in"] = inp
        out = conv3d(inp, w, b, relu=name != "head")
        a[name] = out
        return out

    e0 = conv("enc0b", conv("enc0a", x))
    e1 = conv("enc1b", conv("enc1a", avgpool2(e0)))
    m = conv("midb", conv("mida", avgpool2(e1)))
    d1 = conv("dec1b", conv("dec1a", np.concatenate([upsample2(m), e1], axis=1)))
    d0 = conv("dec0b", conv("dec0a", np.concatenate([upsample2(d1), e0], axis=1)))
    return conv("head", d0), a


def unet_backward(params, cache, gout):
    """Gradients of sum(gout * out) with respect to every (w, b) and to the input."""
    grads = {}

    def back(name, g):
        w, _ = params[name]
        if name != "head":
            g = g * (cache[name] > 0)
        x = cache[name + ":in"]
        grads[name] = conv3d_backward_weight(x, g, w.shape[-1])
        return conv3d_backward_data(g, w)

    c = params["enc0b"][0].shape[0]
    g = back("dec0a", back("dec0b", back("head", gout)))
    g_up_d1, g_e0 = g[:, :2 * c], g[:, 2 * c:]
    g = back("dec1a", back("dec1b", upsample2_adjoint(g_up_d1)))
    g_up_m, g_e1 = g[:, :4 * c], g[:, 4 * c:]
    g = back("mida", back("midb", upsample2_adjoint(g_up_m)))
    g = back("enc1a", back("enc1b", avgpool2_adjoint(g) + g_e1))
    gx = back("enc0a", back("enc0b", avgpool2_adjoint(g) + g_e0))
    return grads, gx


def init_params(cin, c, rng, zero_head=True):
    """He-initialised weights, zero biases; the head starts at zero so the untrained network
    outputs a zero correction."""
    params = {}
    for name, ci, co, k, _ in architecture(cin, c):
        std = np.sqrt(2.0 / (ci * k**3))
        w = rng.standard_normal((co, ci, k, k, k)) * std
        if name == "head" and zero_head:
            w = np.zeros_like(w)
        params[name] = (w, np.zeros(co))
    return params
