"""CPU pinning of the learned-preconditioner network oracle: adjointness of every resampling
operator and a finite-difference check of the hand-written U-Net backward pass."""
import numpy as np

from oracle import unet_oracle as U


def test_resampling_adjoints():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((2, 3, 8, 8, 8))
    g = rng.standard_normal((2, 3, 4, 4, 4))
    assert np.isclose(np.vdot(U.avgpool2(x), g), np.vdot(x, U.avgpool2_adjoint(g)))
    assert np.isclose(np.vdot(U.upsample2(g), x), np.vdot(g, U.upsample2_adjoint(x)))
    y = rng.standard_normal((2, 3, 12, 12, 12))
    assert np.isclose(np.vdot(U.trilinear(g, 12), y), np.vdot(g, U.trilinear_adjoint(y, 4)))
    assert np.allclose(U.trilinear(np.ones((1, 4, 4, 4)), 12), 1.0)
    assert np.allclose(U.block_mean(np.ones((1, 12, 12, 12)), 4), 1.0)


def test_conv_gradients_by_finite_differences():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 3, 5, 5, 5))
    w = rng.standard_normal((4, 3, 3, 3, 3))
    b = rng.standard_normal(4)
    gy = rng.standard_normal((2, 4, 5, 5, 5))
    gw, gb = U.conv3d_backward_weight(x, gy, 3)
    gx = U.conv3d_backward_data(gy, w)
    f = lambda x_, w_, b_: np.vdot(gy, U.conv3d(x_, w_, b_))
    e = 1e-6
    dx = rng.standard_normal(x.shape)
    dw = rng.standard_normal(w.shape)
    assert np.isclose((f(x + e * dx, w, b) - f(x - e * dx, w, b)) / (2 * e), np.vdot(gx, dx), rtol=1e-7)
    assert np.isclose((f(x, w + e * dw, b) - f(x, w - e * dw, b)) / (2 * e), np.vdot(gw, dw), rtol=1e-7)
    assert np.isclose((f(x, w, b + e) - f(x, w, b - e)) / (2 * e), gb.sum(), rtol=1e-7)


def test_unet_backward_by_finite_differences():
    rng = np.random.default_rng(2)
    params = U.init_params(3, 2, rng, zero_head=False)
    params = {k: (w, b + 0.05 * rng.standard_normal(b.shape)) for k, (w, b) in params.items()}
    x = rng.standard_normal((1, 3, 8, 8, 8))
    gout = rng.standard_normal((1, 1, 8, 8, 8))
    out, cache = U.unet_forward(params, x)
    grads, gx = U.unet_backward(params, cache, gout)
    e = 1e-6
    for name in ("enc0a", "mida", "dec1a", "dec0b", "head"):
        w, b = params[name]
        dw = rng.standard_normal(w.shape)
        plus = dict(params, **{name: (w + e * dw, b)})
        minus = dict(params, **{name: (w - e * dw, b)})
        fd = (np.vdot(gout, U.unet_forward(plus, x)[0]) - np.vdot(gout, U.unet_forward(minus, x)[0])) / (2 * e)
        assert np.isclose(fd, np.vdot(grads[name][0], dw), rtol=1e-5, atol=1e-9), name
    dx = rng.standard_normal(x.shape)
    fd = (np.vdot(gout, U.unet_forward(params, x + e * dx)[0]) - np.vdot(gout, U.unet_forward(params, x - e * dx)[0]))
    assert np.isclose(fd / (2 * e), np.vdot(gx, dx), rtol=1e-5)
