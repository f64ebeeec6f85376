"""The BF16 tensor-core Gram (tcgen05, csrc/gram_tc.cu) against the FP32 CUDA-core Gram.

With inputs exactly representable in BF16 whose products and sums are exact in FP32, the
two must agree bit for bit (this pins the operand layout, the descriptors and the TMEM
read-out); with general inputs the difference is the BF16 rounding of the inputs."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def fp32_gram(pkg, Q, y):
    lib = pkg._lib
    n, r, P = Q.shape
    gram = torch.empty((n, r, r), dtype=torch.complex64, device=Q.device)
    h = torch.empty((n, r), dtype=torch.complex64, device=Q.device)
    yy = torch.empty((n,), dtype=torch.float32, device=Q.device)
    s = Q.stride()
    lib.call("cov3d_gram", lib.stream_ptr(Q.device), n, P, r, lib.ptr(Q), s[0], s[2], s[1], lib.ptr(y), lib.ptr(gram),
             lib.ptr(h), lib.ptr(yy))
    return gram, h, yy


@pytest.mark.parametrize("n,r,P", [(7, 10, 4096), (33, 3, 1000), (4, 20, 2304)])
def test_exact_inputs_match_bit_for_bit(pkg, dev, n, r, P):
    g = torch.Generator(device=dev).manual_seed(n + r)
    q = torch.randint(-32, 33, (n, r, P, 2), generator=g, device=dev).float() / 4
    yv = torch.randint(-32, 33, (n, P, 2), generator=g, device=dev).float() / 4
    Q = torch.view_as_complex(q.contiguous())
    y = torch.view_as_complex(yv.contiguous())
    ref = fp32_gram(pkg, Q, y)
    out = pkg.covar_sgd.gram_bf16(Q, y)
    torch.cuda.synchronize()
    for a, b in zip(out, ref):
        assert torch.equal(a, b)


@pytest.mark.parametrize("n,P", [(7, 4096), (11, 1000), (5, 16384)])
def test_point_major_r10_matches_bit_for_bit(pkg, dev, n, P):
    """The fused step's layout (Q point-major, r = 10, the staged FP32 Gram's fast path on the
    other side): bit for bit against the FP32 Gram with BF16-exact inputs, including a pixel
    count that is not a multiple of the 128-pixel stage."""
    r = 10
    g = torch.Generator(device=dev).manual_seed(n + P)
    q = torch.randint(-32, 33, (n, P, r, 2), generator=g, device=dev).float() / 4
    yv = torch.randint(-32, 33, (n, P, 2), generator=g, device=dev).float() / 4
    Q = torch.view_as_complex(q.contiguous()).permute(0, 2, 1)  # (n, r, P), point stride r
    y = torch.view_as_complex(yv.contiguous())
    ref = fp32_gram(pkg, Q, y)
    out = pkg.covar_sgd.gram_bf16(Q, y)
    torch.cuda.synchronize()
    for a, b in zip(out, ref):
        assert torch.equal(a, b)


def test_general_inputs_within_bf16_rounding(pkg, dev):
    g = torch.Generator(device=dev).manual_seed(5)
    n, r, P = 40, 10, 16384
    Q = torch.randn((n, r, P), dtype=torch.complex64, device=dev, generator=g)
    y = torch.randn((n, P), dtype=torch.complex64, device=dev, generator=g) * 3
    ref = fp32_gram(pkg, Q, y)
    out = pkg.covar_sgd.gram_bf16(Q, y)
    for a, b in zip(out, ref):
        assert (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item() < 1e-2


def test_fused_step_with_bf16_gram(pkg, dev):
    from oracle import nufft_oracle as O

    L, r, B = 16, 3, 24
    rng = np.random.default_rng(3)
    vec = torch.tensor(rng.standard_normal((r, L, L, L)), dtype=torch.float32, device=dev) / L**1.5
    logs = torch.tensor(np.log(np.linspace(1.0, 0.5, r)) + np.log(L**1.5), dtype=torch.float32, device=dev)
    R = torch.tensor(O.rotvec_to_rotmat(rng.standard_normal((B, 3))), dtype=torch.float32, device=dev)
    imgs = torch.tensor(rng.standard_normal((B, L * L)) + 1j * rng.standard_normal((B, L * L)), dtype=torch.complex64,
                        device=dev) * L
    out = {}
    for prec in ("fp32", "bf16"):
        step = pkg.FusedCovarStep(L, r, "nufft", 2, device=dev, gram_precision=prec)
        step.set_rotations(R)
        c, gv, gl = step(vec, logs, imgs, None, float(L * L), sync_cost=True)
        out[prec] = (c, gv.clone(), gl.clone())
    c32, g32, _ = out["fp32"]
    c16, g16, _ = out["bf16"]
    assert abs(c16 - c32) / abs(c32) < 1e-2
    assert (torch.linalg.vector_norm(g16 - g32) / torch.linalg.vector_norm(g32)).item() < 5e-2


def _principal_angles_deg(A, B):
    qa, _ = np.linalg.qr(A.T)
    qb, _ = np.linalg.qr(B.T)
    s = np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1.0, 1.0)
    return np.degrees(np.arccos(s))


def _fsc(a, b):
    """Fourier shell correlation of two volumes (shells of the centered integer grid)."""
    L = a.shape[-1]
    fa, fb = np.fft.fftshift(np.fft.fftn(a)), np.fft.fftshift(np.fft.fftn(b))
    k = np.arange(L) - L // 2
    z, y, x = np.meshgrid(k, k, k, indexing="ij")
    sh = np.rint(np.sqrt(x * x + y * y + z * z)).astype(int)
    out = []
    for i in range(L // 2):
        m = sh == i
        out.append(np.real(np.vdot(fa[m], fb[m])) / np.sqrt(np.vdot(fa[m], fa[m]).real * np.vdot(fb[m], fb[m]).real))
    return np.array(out)


def test_bf16_training_recovers_the_fp32_subspace(pkg, dev):
    """Covariance SGD with the BF16 tensor-core Gram against the same run with the FP32 Gram
    (whose gradient is pinned to the float64 oracle): principal angles between the learned
    eigen-subspaces and the FSC of the leading eigenvolume."""
    syn = pkg.synthetic
    L, r, B, nb, steps = 16, 3, 128, 6, 120
    g = torch.Generator(device=dev).manual_seed(11)
    eig = syn.gaussian_blob_volumes(r, L, blobs=12, generator=g, device=dev)
    eig = syn.orthonormalize(eig.reshape(r, -1)).reshape(r, L, L, L) * torch.tensor([3.0, 2.0, 1.0], device=dev).reshape(
        r, 1, 1, 1) * L**1.5
    plan = pkg.NufftPlan((L,) * 3, batch_size=r, device=dev)
    batches = []
    for _ in range(nb):
        R = syn.uniform_rotations(B, generator=g, device=dev)
        plan.setrot(R)
        proj = pkg.vol_forward(eig, plan, None, fourier_domain=True)  # (B, r, L, L)
        z = torch.randn((B, r, 1, 1), generator=g, device=dev)
        img = (proj * z).sum(1).reshape(B, -1)
        img = img + torch.randn(img.shape, generator=g, device=dev, dtype=torch.complex64) * 0.5 * img.abs().mean()
        batches.append((R, img.contiguous()))
    noise_var = float((0.5 * batches[0][1].abs().mean()) ** 2)
    learned = {}
    for prec in ("fp32", "bf16"):
        torch.manual_seed(0)
        covar = pkg.Covar(L, r).to(dev)
        covar.vectors.grad = torch.zeros_like(covar.vectors)
        covar.log_sqrt_eigenvals.grad = torch.zeros_like(covar.log_sqrt_eigenvals)
        groups = covar.grad_lr_factor()
        for gp in groups:
            gp["lr"] *= 2e-3
        opt = torch.optim.Adam(groups)
        step = pkg.FusedCovarStep(L, r, "nufft", 2, device=dev, gram_precision=prec)
        for k in range(steps):
            R, img = batches[k % nb]
            step.set_rotations(R)
            step(covar.vectors.detach(), covar.log_sqrt_eigenvals.detach(), img, None, noise_var,
                 grad_vectors=covar.vectors.grad, grad_log_sqrt=covar.log_sqrt_eigenvals.grad)
            opt.step()
        learned[prec] = covar.get_vectors_spatial_domain().detach().reshape(r, -1).double().cpu().numpy()
    ang = _principal_angles_deg(learned["fp32"], learned["bf16"])
    assert ang.max() < 5.0, ang
    a, b = learned["fp32"][0].reshape((L,) * 3), learned["bf16"][0].reshape((L,) * 3)
    if np.dot(a.ravel(), b.ravel()) < 0:
        b = -b
    assert _fsc(a, b)[: L // 4].min() > 0.95


def test_bf16_training_at_rank_20_matches_the_fp64_oracle(pkg, dev):
    """The precision configuration's check at its rank, r = 20: the same covariance SGD (same
    initial parameters, batches, Adam settings) run with the BF16 tensor-core Gram on the GPU
    and in float64 by the oracle (ES cost and gradient from oracle/cpu_step.py, Adam in numpy);
    the principal angles between the two learned 20-dimensional eigen-subspaces and the FSC of
    the leading eigenvolume (L = 24, 40 steps of 64 images)."""
    from oracle import cpu_step

    syn = pkg.synthetic
    L, r, B, nb, steps = 24, 20, 64, 8, 40
    g = torch.Generator(device=dev).manual_seed(21)
    eig = syn.gaussian_blob_volumes(r, L, blobs=12, generator=g, device=dev)
    scales = torch.linspace(3.0, 0.5, r, device=dev).reshape(r, 1, 1, 1)
    eig = syn.orthonormalize(eig.reshape(r, -1)).reshape(r, L, L, L) * scales * L**1.5
    plan = pkg.NufftPlan((L,) * 3, batch_size=r, device=dev)
    batches = []
    for _ in range(nb):
        R = syn.uniform_rotations(B, generator=g, device=dev)
        plan.setrot(R)
        proj = pkg.vol_forward(eig, plan, None, fourier_domain=True)
        z = torch.randn((B, r, 1, 1), generator=g, device=dev)
        img = (proj * z).sum(1).reshape(B, -1)
        img = img + torch.randn(img.shape, generator=g, device=dev, dtype=torch.complex64) * 0.5 * img.abs().mean()
        batches.append((R, img.contiguous()))
    noise_var = float((0.5 * batches[0][1].abs().mean()) ** 2)
    torch.manual_seed(0)
    covar = pkg.Covar(L, r).to(dev)
    v0 = covar.vectors.detach().double().cpu().numpy()
    l0 = covar.log_sqrt_eigenvals.detach().double().cpu().numpy()
    lr_v, lr_l = 1e-3, 1e-1
    # GPU, BF16 Gram
    covar.vectors.grad = torch.zeros_like(covar.vectors)
    covar.log_sqrt_eigenvals.grad = torch.zeros_like(covar.log_sqrt_eigenvals)
    opt = torch.optim.Adam([{"params": covar.vectors, "lr": lr_v}, {"params": covar.log_sqrt_eigenvals, "lr": lr_l}])
    step = pkg.FusedCovarStep(L, r, "nufft", 2, device=dev, gram_precision="bf16")
    for k in range(steps):
        R, img = batches[k % nb]
        step.set_rotations(R)
        step(covar.vectors.detach(), covar.log_sqrt_eigenvals.detach(), img, None, noise_var,
             grad_vectors=covar.vectors.grad, grad_log_sqrt=covar.log_sqrt_eigenvals.grad)
        opt.step()
    gpu = covar.get_vectors_spatial_domain().detach().reshape(r, -1).double().cpu().numpy()
    # float64 oracle with the same Adam (torch's update rule, bias-corrected)
    host = [(R.double().cpu().numpy(), img.cpu().numpy().reshape(B, L, L)) for R, img in batches]
    theta = [v0.copy(), l0.copy()]
    m = [np.zeros_like(t) for t in theta]
    v = [np.zeros_like(t) for t in theta]
    for k in range(steps):
        R, img = host[k % nb]
        _, gv, gl = cpu_step.covar_cost_grad_es(theta[0], theta[1], R, img, np.ones((B, L, L)), noise_var, width=6)
        for i, (gr, lr) in enumerate(((gv, lr_v), (gl, lr_l))):
            m[i] = 0.9 * m[i] + 0.1 * gr
            v[i] = 0.999 * v[i] + 0.001 * gr * gr
            mh, vh = m[i] / (1 - 0.9 ** (k + 1)), v[i] / (1 - 0.999 ** (k + 1))
            theta[i] = theta[i] - lr * mh / (np.sqrt(vh) + 1e-8)
    ref = (theta[0] * np.exp(theta[1])[:, None, None, None]).reshape(r, -1)
    ang = _principal_angles_deg(ref, gpu)
    assert ang.max() < 5.0, ang
    a, b = ref[0].reshape((L,) * 3), gpu[0].reshape((L,) * 3)
    if np.dot(a.ravel(), b.ravel()) < 0:
        b = -b
    assert _fsc(a, b)[: L // 4].min() > 0.95
