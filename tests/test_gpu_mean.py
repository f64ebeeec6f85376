"""GPU parity of the mean reconstruction (backprojection, regularize_lhs, the padding CG and its
preconditioners) through the C ABI, against the reference's float64 outputs (golden fixtures)
and the float64 oracle."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import nufft_oracle as O

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5  # float32 kernels against float64 truths, same arithmetic
# A CG stopped at ||r|| < rtol ||b|| leaves an error up to cond(A) * rtol in x; the float32
# and float64 runs stop at slightly different iterates.
TOL_CG = 1e-4


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def T(x, dev, dtype=None):
    t = torch.as_tensor(np.asarray(x))
    return t.to(device=dev, dtype=dtype) if dtype is not None else t.to(dev)


def test_backprojection_matches_reference(pkg, dev):
    g = load_golden("mean_L10.npz")
    L, us = int(g["L"]), int(g["us"])
    acc = pkg.MeanBackprojector(L, us, dev)
    for lo in range(0, len(g["images"]), 32):  # the reference's batches of 32
        sl = slice(lo, lo + 32)
        acc.add(T(g["images"][sl], dev), T(g["filters"][sl], dev), T(g["offsets"][sl], dev),
                T(g["contrasts"][sl], dev), pts_rot=T(g["pts"][sl], dev, torch.float32))
    assert rel(acc.rhs, g["rhs"]) < TOL_FP32
    assert rel(acc.lhs, g["lhs"]) < TOL_FP32


def test_regularize_lhs_matches_reference(pkg, dev):
    g = load_golden("cg_L8.npz")
    reg = pkg.regularize_lhs(T(g["lhs"], dev).to(torch.complex64))
    assert rel(reg, g["reg_lhs"]) < 1e-6


def test_mean_init_matches_oracle(pkg, dev):
    g = load_golden("cg_L8.npz")
    L, us = int(g["L"]), int(g["us"])
    plan = pkg.mean._MeanSolver.get(L, us, dev)
    rhs = T(g["rhs"], dev)
    reg = T(g["reg_lhs"], dev, torch.float32)
    b = torch.empty((L,) * 3, dtype=torch.complex64, device=dev)
    x0 = torch.empty_like(b)
    pkg._lib.call("cov3d_mean_init", plan.bind(), pkg._lib.ptr(rhs), pkg._lib.ptr(reg), pkg._lib.ptr(b),
                  pkg._lib.ptr(x0))
    assert rel(b, g["b"]) < TOL_FP32
    assert rel(x0.real, g["init"]) < TOL_FP32
    assert x0.imag.abs().max().item() == 0.0


def test_cg_matches_reference(pkg, dev):
    g = load_golden("cg_L8.npz")
    L = int(g["L"])
    x, info = pkg.cg_solve(T(g["reg_lhs"], dev), T(g["b"], dev), T(g["init"], dev).to(torch.complex64), L, rtol=1e-6,
                           history=True)
    assert info.converged
    assert rel(x.real.reshape((L,) * 3), g["x"]) < TOL_CG
    # same iteration as the reference: the count can move by one or two at float32
    assert abs(info.iters - int(g["iters"][0])) <= 2
    assert info.history[0] > info.history[-1] and info.history[-1] < 1e-6
    # the wrapper with the reference signature
    xr = pkg.correct_upsampling_padding(T(g["reg_lhs"], dev), T(g["rhs"], dev), T(g["init"], dev), L, int(g["us"]))
    assert rel(xr, g["x"]) < TOL_CG


def test_generic_cg_on_a_callable(pkg, dev):
    g = load_golden("cg_L8.npz")
    L, n = int(g["L"]), int(g["L"]) * int(g["us"])
    reg = T(g["reg_lhs"], dev).to(torch.complex128)

    def A(x):
        X = pkg.centered_fft3(x.reshape((L,) * 3), padding_size=(n,) * 3)
        return pkg.centered_ifft3(reg * X, cropping_size=(L,) * 3).reshape(-1)

    x = pkg.complex_conjugate_gradient(A, T(g["b"], dev).reshape(-1), x0=T(g["init"], dev).reshape(-1).to(
        torch.complex128))
    assert rel(x.real.reshape((L,) * 3), g["x"]) < 1e-10


def test_circulant_symbol_matches_oracle(pkg, dev):
    g = load_golden("cg_L8.npz")
    L = int(g["L"])
    sym = pkg.circulant_symbol(T(g["reg_lhs"], dev), L)
    assert rel(sym, O.circulant_symbol(g["reg_lhs"], L)) < TOL_FP32


def _clustered_case(L=12, N=160, seed=5):
    """Poses in a few tight clusters: an anisotropic kernel whose CG needs many iterations."""
    rng = np.random.default_rng(seed)
    centres = O.rotvec_to_rotmat(rng.standard_normal((4, 3)))
    R = []
    for i in range(N):
        jitter = O.rotvec_to_rotmat(0.15 * rng.standard_normal((1, 3)))[0]
        R.append(jitter @ centres[i % 4])
    R = np.array(R)
    pts = O.rotated_points(R, L).astype(np.float32)
    images = (rng.standard_normal((N, L, L)) + 1j * rng.standard_normal((N, L, L))).astype(np.complex64)
    filters = rng.uniform(0.3, 1.2, (N, L, L)).astype(np.float32)
    offsets = rng.uniform(-1.5, 1.5, (N, 2)).astype(np.float32)
    contrasts = rng.uniform(0.8, 1.2, N).astype(np.float32)
    return L, pts, images, filters, offsets, contrasts


@pytest.mark.parametrize("precond", [None, "diagonal", "circulant"])
def test_mean_pipeline_matches_oracle(pkg, dev, precond):
    L, pts, images, filters, offsets, contrasts = _clustered_case()
    acc = pkg.MeanBackprojector(L, 2, dev)
    acc.add(T(images, dev), T(filters, dev), T(offsets, dev), T(contrasts, dev), pts_rot=T(pts, dev))
    vol, info = pkg.solve_mean(acc.rhs, acc.lhs, L, 2, rtol=1e-6, precond=precond, return_info=True)
    ref, rhs, lhs, it = O.reconstruct_mean(images, pts.astype(np.float64), filters, offsets, contrasts, L, 2,
                                           rtol=1e-6)
    assert rel(acc.rhs, rhs) < TOL_FP32 and rel(acc.lhs, lhs) < TOL_FP32
    assert info.converged
    assert rel(vol, ref) < TOL_CG


def test_preconditioners_cut_iterations(pkg, dev):
    L, pts, images, filters, offsets, contrasts = _clustered_case()
    acc = pkg.MeanBackprojector(L, 2, dev)
    acc.add(T(images, dev), T(filters, dev), T(offsets, dev), T(contrasts, dev), pts_rot=T(pts, dev))
    its = {}
    for pc in (None, "diagonal", "circulant"):
        _, info = pkg.solve_mean(acc.rhs, acc.lhs, L, 2, rtol=1e-5, precond=pc, return_info=True)
        assert info.converged
        its[pc] = info.iters
    assert its["circulant"] < its[None]
    assert its["diagonal"] < its[None]


def test_cg_reports_maxiter(pkg, dev):
    g = load_golden("cg_L8.npz")
    L = int(g["L"])
    x, info = pkg.cg_solve(T(g["reg_lhs"], dev), T(g["b"], dev), T(g["init"], dev), L, rtol=1e-12, maxiter=3)
    assert not info.converged and info.iters == 2
    assert np.isfinite(info.relres) and info.relres > 1e-12


@pytest.mark.parametrize("L,precond", [(32, None), (32, "diagonal"), (64, None), (64, "diagonal"), (64, "symbol"),
                                       (128, None), (128, "symbol")])
def test_cg_iterates_match_oracle_on_fused_grids(pkg, dev, L, precond):
    """Grids of n = 64, 128, 256 take the fused axis-0 transform (four-step FFT, diagonal,
    inverse in one kernel), and so do the L^3 preconditioner's transforms at L = 64, 128: three
    CG iterations from zero against the float64 oracle's."""
    rng = np.random.default_rng(L)
    n = 2 * L
    reg = rng.uniform(0.5, 3.0, (n, n, n))
    b = (rng.standard_normal((L, L, L)) + 1j * rng.standard_normal((L, L, L))).reshape(-1)
    A = O.padding_operator(reg, L)
    M, pc = None, precond
    if precond == "diagonal":
        M = O.fine_diagonal_preconditioner(reg, L)
    elif precond == "symbol":
        sym = rng.uniform(0.5, 3.0, (L, L, L))
        M, pc = O.circulant_preconditioner(sym), T(sym, dev, torch.float32)
    ref, _, _ = O.conjugate_gradient(A, b, x0=np.zeros_like(b), rtol=1e-12, maxiter=3, precond=M)
    x, info = pkg.cg_solve(T(reg, dev, torch.float32), T(b, dev, torch.complex64),
                           torch.zeros(L**3, dtype=torch.complex64, device=dev), L, rtol=1e-12, maxiter=3,
                           precond=pc)
    assert not info.converged and info.iters == 2
    assert rel(x.reshape(-1), ref) < TOL_CG


@pytest.mark.parametrize("precond", [None, "diagonal", "symbol"])
def test_cg_iterates_at_n512_match_torch_fft_cg(pkg, dev, precond):
    """L = 256 (the fine grid of 512 takes the 32 x 16 line DFTs, the L^3 preconditioner the
    16 x 16 axis-0 kernel on every other twiddle): three CG iterations against the same
    iterations written with torch's float64 FFTs."""
    L, n = 256, 512
    g = torch.Generator(device=dev).manual_seed(3)
    reg = torch.rand((n,) * 3, generator=g, device=dev, dtype=torch.float64) * 2.5 + 0.5
    b = torch.randn((L,) * 3, generator=g, device=dev, dtype=torch.complex128).reshape(-1)
    sym = torch.rand((L,) * 3, generator=g, device=dev, dtype=torch.float64) * 2.5 + 0.5

    def A(x, d=reg):
        X = pkg.centered_fft3(x.reshape((L,) * 3), padding_size=(n,) * 3)
        return pkg.centered_ifft3(d * X, cropping_size=(L,) * 3).reshape(-1)

    if precond == "diagonal":
        M = lambda v: A(v, 1.0 / reg)  # noqa: E731
    elif precond == "symbol":
        M = lambda v: pkg.centered_ifft3(pkg.centered_fft3(v.reshape((L,) * 3)) / sym).reshape(-1)  # noqa: E731
    else:
        M = lambda v: v  # noqa: E731
    x = torch.zeros_like(b)
    r = b - A(x)
    z = M(r)
    p = z.clone()
    rz = torch.vdot(r, z).real
    for _ in range(3):
        Ap = A(p)
        alpha = rz / torch.vdot(p, Ap)
        x = x + alpha * p
        r = r - alpha * Ap
        z = M(r)
        rz_new = torch.vdot(r, z).real
        p = z + (rz_new / rz) * p
        rz = rz_new
    pc = sym.to(torch.float32) if precond == "symbol" else precond
    xd, info = pkg.cg_solve(reg.to(torch.float32), b.to(torch.complex64),
                            torch.zeros(L**3, dtype=torch.complex64, device=dev), L, rtol=1e-12, maxiter=3,
                            precond=pc)
    assert not info.converged and info.iters == 2
    assert rel(xd.reshape(-1).to(torch.complex128), x) < TOL_CG


class _MeanData(torch.utils.data.Dataset):
    """What reconstruct_mean reads from its dataset (the reference's CovarDataset contract)."""

    def __init__(self, g, dev):
        self.images = torch.tensor(g["images"], device=dev)
        self.pts_rot = torch.tensor(g["pts"], dtype=torch.float32, device=dev)
        self.filters = torch.tensor(g["filters"], device=dev)
        self.offsets = torch.tensor(g["offsets"], device=dev)
        self.contrasts = torch.tensor(g["contrasts"], device=dev)
        self.resolution = int(g["L"])
        self.noise_var = float(g["noise_var"])

    def __len__(self):
        return len(self.images)

    def __getitem__(self, i):
        return self.images[i], self.pts_rot[i], self.filters[i], i


def test_reconstruct_mean_with_initial_volume_matches_reference(pkg, dev):
    """reconstruct_mean with init_vol (mean.py:220-233): the kernel regularised by noise_var
    over the initial volume's radial PSD instead of regularize_lhs; backprojections to 1e-5,
    the CG solution to the CG tolerance (fixture from the reference in float64)."""
    g = load_golden("mean_initvol_L10.npz")
    ds = _MeanData(g, dev)
    loader = torch.utils.data.DataLoader(ds, batch_size=32, shuffle=False)
    vol, rhs, lhs = pkg.reconstruct_mean(loader, init_vol=torch.tensor(g["init_vol"], device=dev).unsqueeze(0),
                                         upsampling_factor=int(g["us"]), return_lhs_rhs=True, device=dev)
    assert rel(rhs, g["rhs"]) < TOL_FP32 and rel(lhs, g["lhs"]) < TOL_FP32
    assert rel(vol, g["volume"]) < TOL_CG
