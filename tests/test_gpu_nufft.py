"""GPU parity of the NUFFT / projection kernels (through the C ABI) against the reference's
outputs (golden fixtures) and the float64 oracle."""
import glob
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, load_golden
from oracle import nufft_oracle as O

pytestmark = pytest.mark.gpu

# float32 kernels against float64 truths
TOL_FP32 = 1e-5


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def T(x, dev, dtype=None):
    t = torch.as_tensor(np.asarray(x))
    return t.to(device=dev, dtype=dtype) if dtype is not None else t.to(dev)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "disc_*.npz"))))
def test_discretized_plan_matches_reference(pkg, dev, path):
    d = np.load(path)
    mode = "bilinear" if "bilinear" in path else "nearest"
    L, us = int(d["L"]), int(d["us"])
    plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=us, mode=mode)
    plan.setpts(T(d["pts"], dev, torch.float32))
    vol = T(d["vol"], dev)
    sig = T(d["sig"], dev)
    filt = T(d["filters"], dev)
    assert rel(plan.execute_forward(vol), d["fwd"]) < TOL_FP32
    assert rel(plan.execute_adjoint(sig), d["adj"]) < TOL_FP32
    assert rel(pkg.vol_forward(vol, plan, filt, fourier_domain=True), d["vol_forward"]) < TOL_FP32
    assert rel(pkg.im_backward(sig, plan, filt, fourier_domain=True), d["im_backward"]) < TOL_FP32
    if "adj_unagg" in d:
        assert rel(plan.execute_adjoint_unaggregated(sig), d["adj_unagg"]) < TOL_FP32


@pytest.mark.parametrize("mode", ["bilinear", "nearest"])
@pytest.mark.parametrize("C", [1, 3, 5, 7, 10, 16, 33, 40])
def test_discretized_channel_passes_match_oracle(pkg, dev, mode, C):
    """Interpolation and spreading with every channel-pass shape of the narrow windows
    (several points per warp, tiles of 3, 4, 5, 8 and 16 channel pairs, two passes) against
    the float64 grid_sample restatement; 40 images so block point counts are ragged."""
    L, us, N = 12, 2, 40
    n = L * us
    rng = np.random.default_rng(100 + C)
    q, _ = np.linalg.qr(rng.standard_normal((N, 3, 3)))
    pts = np.ascontiguousarray(O.rotated_points(q, L, wrap=False))
    grid = (rng.standard_normal((C, n, n, n)) + 1j * rng.standard_normal((C, n, n, n))).astype(np.complex64)
    sig = (rng.standard_normal((C, N, L * L)) + 1j * rng.standard_normal((C, N, L * L))).astype(np.complex64)
    plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=us, mode=mode)
    plan.setpts(T(pts, dev, torch.float32))
    got = plan._plan.interp(T(grid, dev))
    assert rel(got.reshape(C, N, -1), O.interp_discretized(grid, pts, mode)) < TOL_FP32
    back = plan._plan.spread(T(sig.reshape(C, -1), dev))
    assert rel(back, O.spread_discretized(sig, pts, n, mode)) < TOL_FP32


@pytest.mark.parametrize("width,tol", [(6, 5e-5), (7, 5e-6)])
@pytest.mark.parametrize("L", [10, 15, 16])
def test_es_nufft_matches_direct_sum(pkg, dev, width, tol, L):
    rng = np.random.default_rng(L + width)
    vol = rng.standard_normal((3, L, L, L)).astype(np.float32)
    R = O.rotvec_to_rotmat(rng.standard_normal((4, 3)))
    pts = O.rotated_points(R, L).astype(np.float32)
    plan = pkg.NufftPlan((L,) * 3, batch_size=3, device=dev, width=width)
    plan.setpts(T(pts, dev))
    out = plan.execute_forward(T(vol, dev))
    exact = O.nudft_type2(vol, pts.astype(np.float64)).reshape(out.shape)
    assert rel(out, exact) < tol
    sig = (rng.standard_normal((3, 4 * L * L)) + 1j * rng.standard_normal((3, 4 * L * L))).astype(np.complex64)
    adj = plan.execute_adjoint(T(sig, dev))
    assert rel(adj, O.nudft_type1(sig, pts.astype(np.float64), L)) < tol
    # same ES algorithm in float64: only float32 rounding remains
    assert rel(out, O.es_type2(vol, pts.astype(np.float64), 2, width).reshape(out.shape)) < 3e-6


@pytest.mark.parametrize("kind", ["nufft", "bilinear"])
def test_crowded_bins_match_oracle(pkg, dev, kind):
    """512 images at L = 16: every slice passes through the centre, so the central bins hold
    thousands of points and the interpolation takes them in several chunks of one block."""
    L, B, C = 16, 512, 3
    rng = np.random.default_rng(9)
    R = O.rotvec_to_rotmat(rng.standard_normal((B, 3)))
    if kind == "nufft":
        pts = O.rotated_points(R, L).astype(np.float32)
        vol = rng.standard_normal((C, L, L, L)).astype(np.float32)
        plan = pkg.NufftPlan((L,) * 3, batch_size=C, device=dev, width=6)
        plan.setpts(T(pts, dev))
        out = plan.execute_forward(T(vol, dev))
        assert rel(out, O.es_type2(vol, pts.astype(np.float64), 2, 6).reshape(out.shape)) < 3e-6
    else:
        pts = np.ascontiguousarray(O.rotated_points(R, L, wrap=False))
        n = 2 * L
        grid = (rng.standard_normal((C, n, n, n)) + 1j * rng.standard_normal((C, n, n, n))).astype(np.complex64)
        plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=2, mode="bilinear")
        plan.setpts(T(pts, dev, torch.float32))
        out = plan._plan.interp(T(grid, dev))
        assert rel(out.reshape(C, B, -1), O.interp_discretized(grid, pts, "bilinear")) < TOL_FP32


def test_es_adjointness_and_known_slice(pkg, dev):
    rng = np.random.default_rng(5)
    L = 15
    vol = rng.standard_normal((1, L, L, L)).astype(np.float32)
    plan = pkg.NufftPlan((L,) * 3, batch_size=1, device=dev, width=7)
    eye = np.eye(3, dtype=np.float32)[None]
    plan.setrot(T(eye, dev))
    img = pkg.vol_forward(T(vol, dev), plan)
    slice_ = pkg.centered_fft2(img) * L
    truth = O.centered_fft3(vol.astype(np.float64))[0][L // 2]
    assert rel(slice_, truth) < 5e-6  # reference tests/test_torch_wraps.py:266-278 uses 5e-3
    R = O.rotvec_to_rotmat(rng.standard_normal((6, 3)))
    plan.setpts(T(O.rotated_points(R, L).astype(np.float32), dev))
    v = T(rng.standard_normal((1, L, L, L)) + 1j * rng.standard_normal((1, L, L, L)), dev, torch.complex64)
    s = T(rng.standard_normal((1, 6 * L * L)) + 1j * rng.standard_normal((1, 6 * L * L)), dev, torch.complex64)
    # float64 inner products of the float32 operator outputs
    a = torch.vdot(s.reshape(-1).to(torch.complex128), plan.execute_forward(v).reshape(-1).to(torch.complex128))
    b = torch.vdot(plan.execute_adjoint(s).reshape(-1).to(torch.complex128), v.reshape(-1).to(torch.complex128))
    assert abs(a - b) / abs(a) < 5e-5


@pytest.mark.parametrize("disc", ["nufft", "bilinear"])
def test_rotations_equal_explicit_points(pkg, dev, disc):
    rng = np.random.default_rng(7)
    L, us = 16, 2
    R = O.rotvec_to_rotmat(rng.standard_normal((5, 3))).astype(np.float32)
    pts = O.rotated_points(R.astype(np.float64), L).astype(np.float32)
    if disc == "nufft":
        vol = T(rng.standard_normal((2, L, L, L)), dev, torch.float32)
        p1 = pkg.NufftPlan((L,) * 3, batch_size=2, device=dev)
        p2 = pkg.NufftPlan((L,) * 3, batch_size=2, device=dev)
    else:
        vol = T(rng.standard_normal((2, L * us, L * us, L * us)) + 1j, dev, torch.complex64)
        p1 = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=us)
        p2 = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=us)
    p1.setrot(T(R, dev))
    p2.setpts(T(pts, dev))
    assert rel(p1.execute_forward(vol), p2.execute_forward(vol)) < 2e-6


def test_batched_equals_looped(pkg, dev):
    """Reference tests/test_torch_wraps.py:280-309: B single-image plans == one batched plan,
    values and gradients."""
    rng = np.random.default_rng(8)
    L, B = 15, 6
    R = O.rotvec_to_rotmat(rng.standard_normal((B, 3)))
    pts = T(O.rotated_points(R, L).astype(np.float32), dev)
    base = rng.standard_normal((3, L, L, L)).astype(np.float32)
    v1 = T(base, dev).requires_grad_(True)
    plans = [pkg.NufftPlan((L,) * 3, 3, device=dev) for _ in range(B)]
    fw = torch.zeros((B, 3, L, L), device=dev)
    for i in range(B):
        plans[i].setpts(pts[i:i + 1])
        fw[i] = pkg.vol_forward(v1, plans[i])  # (1, 3, L, L): one image, three volumes, as the reference
    torch.norm(fw).backward()
    v2 = T(base, dev).requires_grad_(True)
    bp = pkg.NufftPlan((L,) * 3, 3, device=dev)
    bp.setpts(pts)
    fb = pkg.vol_forward(v2, bp)
    torch.norm(fb).backward()
    assert rel(fw, fb) < 1e-6
    assert rel(v1.grad, v2.grad) < 1e-5


@pytest.mark.parametrize("kernel", ["nufft", "bilinear"])
def test_full_size_adjointness(pkg, dev, kernel):
    """Size-independent property at L=128: <A v, s> == <v, A* s> through the fused kernels."""
    L, B = 128, 32
    g = torch.Generator(device=dev).manual_seed(0)
    R = torch.linalg.qr(torch.randn((B, 3, 3), device=dev, generator=g))[0].contiguous()
    if kernel == "nufft":
        plan = pkg.NufftPlan((L,) * 3, batch_size=2, device=dev, width=6)
        plan.setrot(R)
        v = torch.randn((2, L, L, L), device=dev, generator=g, dtype=torch.complex64)
        s = torch.randn((2, B * L * L), device=dev, generator=g, dtype=torch.complex64)
        a = torch.vdot(s.reshape(-1).to(torch.complex128), plan.execute_forward(v).reshape(-1).to(torch.complex128))
        b = torch.vdot(plan.execute_adjoint(s).reshape(-1).to(torch.complex128), v.reshape(-1).to(torch.complex128))
    else:
        plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=2)
        plan.setrot(R)
        v = torch.randn((2, 2 * L, 2 * L, 2 * L), device=dev, generator=g, dtype=torch.complex64)
        s = torch.randn((B, L, L), device=dev, generator=g, dtype=torch.complex64)
        ctf = torch.rand((B, L, L), device=dev, generator=g)
        fwd = pkg.vol_forward(v, plan, ctf, fourier_domain=True)  # (B, 2, L, L)
        a = torch.vdot(s.unsqueeze(1).expand(-1, 2, -1, -1).reshape(-1).to(torch.complex128),
                       fwd.reshape(-1).to(torch.complex128))
        back = pkg.im_backward(s, plan, ctf, fourier_domain=True)  # (1, n, n, n)
        b = torch.vdot(back.reshape(-1).to(torch.complex128), v.sum(0).reshape(-1).to(torch.complex128))
    assert abs(a - b) / abs(a) < 5e-5
