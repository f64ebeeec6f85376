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


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _noalloc(pkg, Q, y, noise_var, linv, want_z=True, want_m=True, out=None, point_major=False):
    """Call the entry point through the C ABI.  Q is (n, r, P) channel-major, or with
    ``point_major`` a (n, P, r) tensor read with point stride r and channel stride 1."""
    lib = pkg._lib.load()
    if point_major:
        n, P, r = Q.shape
        s = Q.stride()
        strides = (s[0], s[1], s[2])
    else:
        n, r, P = Q.shape
        s = Q.stride()
        strides = (s[0], s[2], s[1])
    if out is None:
        out = (torch.empty((n, r), dtype=torch.complex64, device=Q.device),
               torch.empty((n, r, r), dtype=torch.complex64, device=Q.device),
               torch.full((1,), -1, dtype=torch.int32, device=Q.device))
    z, m, bad = out
    st = lib.cov3d_latent_map_noalloc(pkg._lib.stream_ptr(Q.device), n, P, r, _vp(Q), *strides, _vp(y),
                                      float(noise_var), _vp(linv), _vp(z) if want_z else None,
                                      _vp(m) if want_m else None, _vp(bad))
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


def _rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def test_noalloc_failure_flag_is_cleared_by_the_next_call(pkg, dev):
    """An indefinite m (prior -1e6 I) sets the shared flag; the next, valid call reports 0."""
    Q, y, linv = _case(dev, 64, 4, 256, seed=5)
    _, _, bad = _noalloc(pkg, Q, y, 7.5, -1e6 * torch.eye(4, dtype=torch.float64, device=dev))
    torch.cuda.synchronize()
    assert int(bad.item()) == 1
    _, _, bad = _noalloc(pkg, Q, y, 7.5, linv)
    torch.cuda.synchronize()
    assert int(bad.item()) == 0


def test_noalloc_single_outputs_and_point_major_layout(pkg, dev):
    """z alone, m alone, and projections stored point-major (n, P, r) at r = 10."""
    Q, y, linv = _case(dev, 200, 10, 1024, seed=6)
    z_ref, m_ref, _ = pkg.wiener_coords.compute_latentMAP_batch(y, Q, 7.5, linv)
    z_ref = z_ref.squeeze(-1)
    z, _, _ = _noalloc(pkg, Q, y, 7.5, linv, want_m=False)
    _, m, _ = _noalloc(pkg, Q, y, 7.5, linv, want_z=False)
    torch.cuda.synchronize()
    assert _rel(z, z_ref) < TOL and _rel(m, m_ref) < TOL
    Qp = Q.transpose(1, 2).contiguous()  # (n, P, r)
    z, m, bad = _noalloc(pkg, Qp, y, 7.5, linv, point_major=True)
    torch.cuda.synchronize()
    assert int(bad.item()) == 0 and _rel(z, z_ref) < TOL and _rel(m, m_ref) < TOL


def test_noalloc_device_memory_is_unchanged_after_warm_up(pkg, dev):
    """After one warm-up call at the rank used (the driver may size its per-thread local memory
    on a kernel's first launch), repeated calls leave the free device memory unchanged."""
    Q, y, linv = _case(dev, 500, 10, 1024, seed=7)
    out = (torch.empty((500, 10), dtype=torch.complex64, device=dev),
           torch.empty((500, 10, 10), dtype=torch.complex64, device=dev),
           torch.zeros((1,), dtype=torch.int32, device=dev))
    _noalloc(pkg, Q, y, 7.5, linv, out=out)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(5):
        _noalloc(pkg, Q, y, 7.5, linv, out=out)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0
