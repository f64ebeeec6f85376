"""Seeded synthetic cryo-EM data on the GPU (stands in for the reference's ``SimulatedSource``,
``source.py:312-542``, and its ASPIRE/cryoDRGN CTF code, which are not part of this library).

Volumes are sums of isotropic 3D Gaussians; rotations are uniform on SO(3) (normalised
Gaussian quaternions); the CTF is the standard weak-phase form
``-(sqrt(1-A^2) sin chi + A cos chi)``, ``chi = pi*lambda*df*k^2 - pi/2*Cs*lambda^3*k^4`` with
the relativistic electron wavelength.  CTF values are therefore not bit-identical to ASPIRE's
``RadialCTFFilter``; every parity test feeds the same CTF array to both sides.
"""

import math

import torch


def gaussian_blob_volumes(count, L, blobs=50, radius=0.35, width=(1.0, 3.0), amp=(0.5, 1.0), generator=None,
                          device="cuda"):
    """(count, L, L, L) float32 sums of ``blobs`` Gaussians, centres uniform in a ball."""
    g = generator
    dev = torch.device(device)
    ax = torch.arange(L, device=dev, dtype=torch.float32) - L // 2
    z, y, x = torch.meshgrid(ax, ax, ax, indexing="ij")
    out = torch.zeros((count, L, L, L), device=dev)
    grid = torch.stack([z, y, x]).reshape(3, -1)
    for c in range(count):
        d = torch.randn((blobs, 3), generator=g, device=dev)
        d = d / d.norm(dim=1, keepdim=True)
        rr = torch.rand((blobs, 1), generator=g, device=dev) ** (1.0 / 3.0) * radius * L
        centres = d * rr
        sig = torch.rand((blobs,), generator=g, device=dev) * (width[1] - width[0]) + width[0]
        a = torch.rand((blobs,), generator=g, device=dev) * (amp[1] - amp[0]) + amp[0]
        # all blobs at once, in slabs of voxels to bound the (blobs, voxels) temporary
        for lo in range(0, grid.shape[1], 1 << 20):
            pts = grid[:, lo:lo + (1 << 20)]
            r2 = ((pts[None] - centres[:, :, None]) ** 2).sum(1)
            out[c].view(-1)[lo:lo + pts.shape[1]] = (a[:, None] * torch.exp(-r2 / (2 * sig[:, None] ** 2))).sum(0)
    return out


def uniform_rotations(n, generator=None, device="cuda"):
    """(n, 3, 3) rotation matrices from normalised Gaussian quaternions."""
    q = torch.randn((n, 4), generator=generator, device=device, dtype=torch.float64)
    q = q / q.norm(dim=1, keepdim=True)
    w, x, y, z = q.unbind(1)
    R = torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                     2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                     2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], dim=1)
    return R.reshape(n, 3, 3).to(torch.float32)


def electron_wavelength(voltage_kv):
    v = voltage_kv * 1e3
    return 12.2643247 / math.sqrt(v * (1 + 0.978466e-6 * v))  # Angstrom


def ctf_images(defocus_um, L, pixel_size, voltage_kv=300.0, cs_mm=2.7, amplitude_contrast=0.1, device="cuda"):
    """(n, L, L) float32 CTFs on the centered Fourier grid of an L x L image."""
    dev = torch.device(device)
    lam = electron_wavelength(voltage_kv)
    f = (torch.arange(L, device=dev, dtype=torch.float64) - L // 2) / (L * pixel_size)
    ky, kx = torch.meshgrid(f, f, indexing="ij")
    k2 = kx * kx + ky * ky
    df = defocus_um.to(dev, torch.float64).reshape(-1, 1, 1) * 1e4  # Angstrom
    cs = cs_mm * 1e7
    chi = math.pi * lam * df * k2 - 0.5 * math.pi * cs * lam**3 * k2 * k2
    A = amplitude_contrast
    return (-(math.sqrt(1 - A * A) * torch.sin(chi) + A * torch.cos(chi))).to(torch.float32)


def ctf_params(defocus_um, pixel_size, voltage_kv=300.0, cs_mm=2.7, amplitude_contrast=0.1, defocus_v_um=None,
               astigmatism_deg=None, phase_shift_deg=None, device="cuda"):
    """(n, 8) CTF parameters (pixel size, defocus u and v in A, astigmatism angle, kV, Cs, amplitude
    contrast, phase shift) in the column order of the reference's ``ctf_params``
    (``source.py:157-172``), for the kernels to compute the CTF from."""
    dev = torch.device(device)
    du = defocus_um.to(dev, torch.float32).reshape(-1) * 1e4
    n = du.shape[0]
    dv = du if defocus_v_um is None else defocus_v_um.to(dev, torch.float32).reshape(-1) * 1e4
    z = torch.zeros((n,), device=dev)
    ang = z if astigmatism_deg is None else astigmatism_deg.to(dev, torch.float32).reshape(-1)
    ph = z if phase_shift_deg is None else phase_shift_deg.to(dev, torch.float32).reshape(-1)
    cols = [torch.full((n,), float(pixel_size), device=dev), du, dv, ang, torch.full((n,), float(voltage_kv), device=dev),
            torch.full((n,), float(cs_mm), device=dev), torch.full((n,), float(amplitude_contrast), device=dev), ph]
    return torch.stack(cols, dim=1).contiguous()


def ctf_from_params(params, L):
    """(n, L, L) float32 CTF images from (n, 8) parameters, computed by the library's kernel
    (``cov3d_ctf_images``): the CTF the fused step evaluates in-kernel with ``ctf_params``."""
    from . import _lib

    params = params.to(torch.float32).contiguous()
    out = torch.empty((params.shape[0], L, L), dtype=torch.float32, device=params.device)
    with torch.cuda.device(params.device):
        _lib.call("cov3d_ctf_images", _lib.stream_ptr(params.device), _lib.ptr(params), params.shape[0], int(L),
                  _lib.ptr(out))
    return out


def vmf_cluster_rotations(n, clusters=8, kappa=5.0, generator=None, device="cuda"):
    """(n, 3, 3) rotations whose viewing directions (third column, the normal of the projected
    Fourier plane) follow an equal-weight mixture of ``clusters`` von Mises-Fisher
    distributions on the sphere with concentration ``kappa`` (centres uniform), with a uniform
    in-plane angle.  Gives an anisotropic sampling of Fourier space."""
    g = generator
    dev = torch.device(device)
    cen = torch.randn((clusters, 3), generator=g, device=dev, dtype=torch.float64)
    cen = cen / cen.norm(dim=1, keepdim=True)
    mu = cen[torch.randint(0, clusters, (n,), generator=g, device=dev)]
    # Wood's method on S^2: w = 1 + log(u + (1 - u) e^{-2 kappa}) / kappa
    u = torch.rand((n,), generator=g, device=dev, dtype=torch.float64)
    w = 1.0 + torch.log(u + (1.0 - u) * math.exp(-2.0 * kappa)) / kappa
    v = torch.randn((n, 3), generator=g, device=dev, dtype=torch.float64)
    v = v - (v * mu).sum(1, keepdim=True) * mu
    v = v / v.norm(dim=1, keepdim=True)
    d = w[:, None] * mu + torch.sqrt(torch.clamp(1.0 - w * w, min=0.0))[:, None] * v
    a = torch.randn((n, 3), generator=g, device=dev, dtype=torch.float64)
    a = a - (a * d).sum(1, keepdim=True) * d
    a = a / a.norm(dim=1, keepdim=True)
    b = torch.cross(d, a, dim=1)
    th = torch.rand((n, 1), generator=g, device=dev, dtype=torch.float64) * (2 * math.pi)
    e1 = torch.cos(th) * a + torch.sin(th) * b
    e2 = torch.cross(d, e1, dim=1)
    return torch.stack([e1, e2, d], dim=2).to(torch.float32)


def orthonormalize(v):
    """Rows of v (k, m) orthonormalised by modified Gram-Schmidt in float64 (returns float32)."""
    out = []
    for i in range(v.shape[0]):
        w = v[i].to(torch.float64)
        for u in out:
            w = w - torch.dot(u, w) * u
        out.append(w / torch.linalg.vector_norm(w))
    return torch.stack(out).to(torch.float32)
