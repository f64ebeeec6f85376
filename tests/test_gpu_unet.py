"""GPU kernels of the learned CG preconditioner (csrc/unet.cu, through the C ABI) against the
float64 oracle: every layer forward and adjoint, and the whole U-Net's parameter gradients."""
import numpy as np
import pytest
import torch

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu

TOL_FWD = 1e-5   # float32 sums of at most a few thousand terms against float64
TOL_GRAD = 1e-4  # the weight gradients sum over every voxel of the batch


def rel(a, b):
    a = a.detach().double().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def T(x, dev):
    return torch.as_tensor(np.asarray(x, np.float32)).to(dev)


@pytest.fixture(scope="module")
def lp(pkg):
    return pkg.learned_pc


@pytest.mark.parametrize("k,relu", [(3, True), (3, False), (1, False)])
def test_conv3d_forward_and_gradients(pkg, lp, dev, k, relu):
    rng = np.random.default_rng(k + relu)
    x = rng.standard_normal((2, 5, 6, 5, 7))
    w = rng.standard_normal((11, 5, k, k, k)) / np.sqrt(5 * k**3)
    b = rng.standard_normal(11)
    gy = rng.standard_normal((2, 11, 6, 5, 7))
    xt, wt, bt = (T(v, dev).requires_grad_() for v in (x, w, b))
    y = lp.Conv3dFn.apply(xt, wt, bt, relu)
    yo = U.conv3d(x, w, b, relu)
    assert rel(y, yo) < TOL_FWD
    y.backward(T(gy, dev))
    g = gy * (yo > 0) if relu else gy
    gw, gb = U.conv3d_backward_weight(x, g, k)
    assert rel(xt.grad, U.conv3d_backward_data(g, w)) < TOL_FWD
    assert rel(wt.grad, gw) < TOL_GRAD
    assert rel(bt.grad, gb) < TOL_GRAD


def test_resampling_layers(pkg, lp, dev):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2, 3, 8, 6, 4))
    xt = T(x, dev).requires_grad_()
    y = lp.AvgPool2Fn.apply(xt)
    assert rel(y, U.avgpool2(x)) < TOL_FWD
    g = rng.standard_normal(y.shape)
    y.backward(T(g, dev))
    assert rel(xt.grad, U.avgpool2_adjoint(g)) < TOL_FWD
    xt = T(x, dev).requires_grad_()
    y = lp.Upsample2Fn.apply(xt)
    assert rel(y, U.upsample2(x)) < TOL_FWD
    g = rng.standard_normal(y.shape)
    y.backward(T(g, dev))
    assert rel(xt.grad, U.upsample2_adjoint(g)) < TOL_FWD
    c = rng.standard_normal((1, 2, 8, 8, 8))
    ct = T(c, dev).requires_grad_()
    y = lp.TrilinearFn.apply(ct, 24)
    assert rel(y, U.trilinear(c, 24)) < TOL_FWD
    g = rng.standard_normal(y.shape)
    y.backward(T(g, dev))
    assert rel(ct.grad, U.trilinear_adjoint(g, 8)) < TOL_FWD
    big = rng.standard_normal((1, 2, 24, 24, 24))
    assert rel(lp.block_mean(T(big, dev), 8), U.block_mean(big, 8)) < TOL_FWD


def test_unet_gradients_match_oracle(pkg, lp, dev):
    rng = np.random.default_rng(4)
    net = lp.UNet3D(3, 4, dev, seed=1)
    params = U.init_params(3, 4, rng, zero_head=False)
    params = {k: (w, b + 0.05 * rng.standard_normal(b.shape)) for k, (w, b) in params.items()}
    for name, (w, b) in params.items():
        with torch.no_grad():
            net.params[name][0].copy_(T(w, dev))
            net.params[name][1].copy_(T(b, dev))
    x = rng.standard_normal((1, 3, 16, 16, 16))
    gout = rng.standard_normal((1, 1, 16, 16, 16))
    out = net(T(x, dev))
    ref, cache = U.unet_forward(params, x)
    assert rel(out, ref) < TOL_FWD
    out.backward(T(gout, dev))
    grads, _ = U.unet_backward(params, cache, gout)
    for name, (gw, gb) in grads.items():
        assert rel(net.params[name][0].grad, gw) < TOL_GRAD, name
        assert rel(net.params[name][1].grad, gb) < TOL_GRAD, name
