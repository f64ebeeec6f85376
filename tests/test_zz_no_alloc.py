"""The allocation-free latent-MAP entry point (cov3d_latent_map_noalloc) against the
allocating path (cov3d_gram + cov3d_cost_solve, as used by compute_latentMAP_batch).

It exists for callers that must not let the library allocate device memory (their own pool
owns the GPU, or cudaMalloc's device-wide synchronisation is not acceptable on their call
path); its intermediates live in a fixed 4 MiB device array shared by every call.  This file
is named to be collected last."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-5  # same float32 kernels on both paths; the tolerance of the other parity tests


def _noalloc(pkg, Q, y, noise_var, linv):
    lib = pkg._lib.load()
    n, r, P = Q.shape
    z = torch.empty((n, r), dtype=torch.complex64, device=Q.device)
    m = torch.empty((n, r, r), dtype=torch.complex64, device=Q.device)
    bad = torch.full((1,), -1, dtype=torch.int32, device=Q.device)
    s = Q.stride()
    st = lib.cov3d_latent_map_noalloc(pkg._lib.stream_ptr(Q.device), n, P, r, ctypes.c_void_p(Q.data_ptr()), s[0],
                                      s[2], s[1], ctypes.c_void_p(y.data_ptr()), float(noise_var),
                                      ctypes.c_void_p(linv.data_ptr()), ctypes.c_void_p(z.data_ptr()),
                                      ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(bad.data_ptr()))
    pkg._lib.check(st)
    return z, m, bad


def _case(dev, n, r, P, seed):
    g = torch.Generator(device=dev).manual_seed(seed)
    Q = torch.randn((n, r, P), dtype=torch.complex64, device=dev, generator=g)
    y = torch.randn((n, P), dtype=torch.complex64, device=dev, generator=g) * 3
    lam = torch.rand((r,), device=dev, generator=g, dtype=torch.float64) * 2 + 0.5
    linv = torch.diag(1.0 / lam).contiguous()
    return Q, y, linv


def test_noalloc_matches_allocating_path_twice(pkg, dev):
    for call, (n, r, P) in enumerate([(300, 10, 1024), (97, 6, 2304)]):
        Q, y, linv = _case(dev, n, r, P, seed=call + 1)
        z_ref, m_ref, _ = pkg.wiener_coords.compute_latentMAP_batch(y, Q, 7.5, linv)
        z, m, bad = _noalloc(pkg, Q, y, 7.5, linv)
        torch.cuda.synchronize()
        assert int(bad.item()) == 0
        z_ref = z_ref.squeeze(-1)
        assert (torch.linalg.norm(z - z_ref) / torch.linalg.norm(z_ref)).item() < TOL
        assert (torch.linalg.norm(m - m_ref) / torch.linalg.norm(m_ref)).item() < TOL


def test_noalloc_rejects_sizes_beyond_its_scratch(pkg, dev):
    lib = pkg._lib.load()
    dummy = torch.zeros((1,), dtype=torch.complex64, device=dev)
    p = ctypes.c_void_p(dummy.data_ptr())
    st = lib.cov3d_latent_map_noalloc(None, 100000, 16, 10, p, 160, 10, 1, p, 1.0, None, p, None, None)
    assert st == pkg._lib.EINVAL
    assert "scratch" in pkg._lib.last_error()
