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
