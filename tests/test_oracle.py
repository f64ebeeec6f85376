"""The float64 oracle against the reference's own outputs (golden fixtures produced by running
the reference, tests/golden/make_golden.py) and against the reference's invariants."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from oracle import nufft_oracle as O


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


@pytest.mark.parametrize("L", [12, 15])
def test_poses(L):
    g = load_golden("poses.npz")
    R = O.rotvec_to_rotmat(g[f"L{L}_rotvecs"])
    assert rel(R, g[f"L{L}_rotmat"]) < 1e-14
    assert rel(O.rotated_points(R, L), g[f"L{L}_pts"]) < 1e-14
    assert rel(O.phase_shift(-g[f"L{L}_offsets"], L), g[f"L{L}_phase"]) < 1e-14


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "disc_*.npz"))))
def test_discretized_plan(path):
    d = np.load(path)
    mode = "bilinear" if "bilinear" in path else "nearest"
    L, us = int(d["L"]), int(d["us"])
    n, pts = L * us, d["pts"]
    fwd = O.interp_discretized(d["vol"].astype(np.complex128), pts, mode)
    assert rel(fwd, d["fwd"].reshape(fwd.shape)) < 1e-13
    assert rel(O.spread_discretized(d["sig"].reshape(1, pts.shape[0], -1), pts, n, mode), d["adj"]) < 1e-13
    assert rel(O.vol_forward_fourier(fwd, d["filters"], L), d["vol_forward"]) < 1e-13
    pro = O.im_backward_fourier_prologue(d["sig"], d["filters"], L)
    assert rel(O.spread_discretized(pro.reshape(1, pts.shape[0], -1), pts, n, mode) / L, d["im_backward"]) < 1e-13
    if "adj_unagg" in d:
        u = O.spread_discretized(d["sig"].reshape(1, pts.shape[0], -1), pts, n, mode, aggregate=False)[:, 0]
        assert rel(u, d["adj_unagg"]) < 1e-13


@pytest.mark.parametrize("objective", ["ml", "ls"])
@pytest.mark.parametrize("with_reg", [False, True])
def test_cost_and_gradient(objective, with_reg):
    c = load_golden("cost_L10_r3.npz")
    tag = objective + ("_reg" if with_reg else "")
    cost, gv, gl = O.covar_cost_grad(c["vectors_normalised"], c["log_sqrt_eigenvals"], c["images"], c["pts"],
                                     c["filters"], float(c["noise_var"]), objective=objective,
                                     reg_scale=float(c["reg_scale"]) if with_reg else 0.0,
                                     fourier_reg=c["fourier_reg"] if with_reg else None)
    assert rel(cost, c[tag + "_cost"]) < 1e-12
    assert rel(gv, c[tag + "_grad_vectors"]) < 1e-12
    assert rel(gl, c[tag + "_grad_logsqrt"]) < 1e-12


def test_latent_map():
    g = load_golden("latent_L10_r3.npz")
    z, m, b = O.latent_map_batch(g["images"], g["eigen_forward"], float(g["noise_var"]), g["eigenvals_inv"])
    assert rel(z, g["z"]) < 1e-13 and rel(m, g["m"]) < 1e-13 and rel(b, g["b"]) < 1e-13
    z, m, b = O.latent_map_batch(g["images"].real, g["eigen_forward"].real, float(g["noise_var"]), g["eigenvals_inv"])
    assert rel(z, g["z_real"]) < 1e-13 and rel(m, g["m_real"]) < 1e-13


def test_cg_and_regularize_lhs():
    g = load_golden("cg_L8.npz")
    L = int(g["L"])
    assert rel(O.regularize_lhs(g["lhs"].astype(np.complex128)), np.abs(g["reg_lhs"])) < 1e-14
    A = O.padding_operator(g["reg_lhs"], L)
    x, it, _ = O.conjugate_gradient(A, g["b"].reshape(-1), x0=g["init"].reshape(-1).astype(np.complex128))
    assert rel(x.real.reshape((L,) * 3), g["x"]) < 1e-12
    assert it == int(g["iters"][0])


def test_fourier_slice_known_answer():
    """Identity rotation: the NUDFT at the central plane equals the central slice of the
    centered 3D FFT (reference tests/test_torch_wraps.py:266-278)."""
    rng = np.random.default_rng(0)
    L = 12
    vol = rng.standard_normal((1, L, L, L))
    p0 = O.rotated_points(np.eye(3)[None], L)
    f = O.nudft_type2(vol, p0)[0, 0].reshape(L, L)
    # the plane coordinates are float32-rounded like the reference's, hence 1e-6
    assert rel(f, O.centered_fft3(vol[0])[L // 2]) < 1e-6
    exact = O.rotated_points(np.eye(3)[None], L, wrap=False)
    assert np.allclose(exact[0, 0], 0.0)


@pytest.mark.parametrize("width,tol", [(6, 5e-5), (7, 5e-6)])
def test_es_algorithm_matches_direct_sum(width, tol):
    rng = np.random.default_rng(1)
    L = 10
    vol = rng.standard_normal((2, L, L, L))
    R = O.rotvec_to_rotmat(rng.standard_normal((3, 3)))
    pts = O.rotated_points(R, L)
    assert rel(O.es_type2(vol, pts, 2, width), O.nudft_type2(vol, pts)) < tol
    sig = rng.standard_normal((2, 3, L * L)) + 1j * rng.standard_normal((2, 3, L * L))
    assert rel(O.es_type1(sig, pts, L, 2, width), O.nudft_type1(sig, pts, L)) < tol


def test_es_adjointness():
    rng = np.random.default_rng(2)
    L = 8
    vol = rng.standard_normal((1, L, L, L)) + 1j * rng.standard_normal((1, L, L, L))
    pts = O.rotated_points(O.rotvec_to_rotmat(rng.standard_normal((2, 3))), L)
    sig = rng.standard_normal((1, 2, L * L)) + 1j * rng.standard_normal((1, 2, L * L))
    a = np.vdot(sig, O.es_type2(vol, pts, 2, 6))
    b = np.vdot(O.es_type1(sig, pts, L, 2, 6), vol)
    assert abs(a - b) / abs(a) < 1e-13


def test_gradient_matches_finite_differences():
    """Closed-form ML gradient of the oracle against central differences (float64)."""
    rng = np.random.default_rng(3)
    L, r, B = 6, 2, 3
    vec = rng.standard_normal((r, L, L, L))
    vec /= np.linalg.norm(vec.reshape(r, -1), axis=1)[:, None, None, None]
    ls = np.log(rng.uniform(0.5, 2.0, r))
    pts = O.rotated_points(O.rotvec_to_rotmat(rng.standard_normal((B, 3))), L)
    imgs = rng.standard_normal((B, L, L)) + 1j * rng.standard_normal((B, L, L))
    ctf = rng.uniform(0.3, 1.2, (B, L, L))
    for kind in ("es", "bilinear"):
        f = lambda v, s: O.covar_cost_grad(v, s, imgs, pts, ctf, 2.0, kind=kind, width=6)[0]
        _, gv, gl = O.covar_cost_grad(vec, ls, imgs, pts, ctf, 2.0, kind=kind, width=6)
        eps = 1e-6
        for idx in [(0, 1, 2, 3), (1, 3, 3, 2), (0, 0, 5, 1)]:
            d = np.zeros_like(vec)
            d[idx] = eps
            fd = (f(vec + d, ls) - f(vec - d, ls)) / (2 * eps)
            assert abs(fd - gv[idx]) <= 1e-6 * max(1.0, abs(fd))
        d = np.zeros_like(ls)
        d[1] = eps
        fd = (f(vec, ls + d) - f(vec, ls - d)) / (2 * eps)
        assert abs(fd - gl[1]) <= 1e-6 * max(1.0, abs(fd))


def test_reconstruct_mean_pipeline():
    """Backprojection, regularize_lhs, Fourier-diagonal start, padding CG, sphere mask and
    grid correction against reconstruct_mean run by the reference in float64.  rhs / lhs are
    exact; the volume agrees to the accuracy an rtol=1e-6 CG of ~5,500 iterations allows (the
    two FFT libraries round differently, so the iterates drift apart slowly)."""
    g = load_golden("mean_L10.npz")
    L = int(g["L"])
    vol, rhs, lhs, it = O.reconstruct_mean(g["images"], g["pts"], g["filters"], g["offsets"], g["contrasts"], L,
                                           int(g["us"]))
    assert rel(rhs, g["rhs"]) < 1e-12
    assert rel(lhs, g["lhs"]) < 1e-12
    assert rel(vol, g["volume"]) < 1e-4
    assert abs(it - int(g["iters"][0])) < 0.02 * int(g["iters"][0])


def test_circulant_symbol_is_the_operator_diagonal_in_fourier():
    """T. Chan's optimal circulant has eigenvalues diag(F A F^-1): check a few Fourier modes."""
    g = load_golden("cg_L8.npz")
    L = int(g["L"])
    reg = g["reg_lhs"]
    sym = O.circulant_symbol(reg, L)
    A = O.padding_operator(reg, L)
    rng = np.random.default_rng(0)
    native = np.fft.ifftshift(sym)
    for _ in range(6):
        k = tuple(rng.integers(0, L, 3))
        e = np.zeros((L, L, L), np.complex128)
        e[k] = 1.0
        f = np.fft.ifftn(e).reshape(-1) * np.sqrt(L**3)
        assert abs(np.vdot(f, A(f)) - native[k]) < 1e-12 * np.abs(sym).max()


def test_preconditioned_cg_reaches_the_same_solution():
    g = load_golden("cg_L8.npz")
    L = int(g["L"])
    reg = g["reg_lhs"]
    A = O.padding_operator(reg, L)
    b = g["b"].reshape(-1)
    x0 = g["init"].reshape(-1).astype(np.complex128)
    ref, it0, _ = O.conjugate_gradient(A, b, x0=x0, rtol=1e-10)
    for M in (O.fine_diagonal_preconditioner(reg, L), O.circulant_preconditioner(O.circulant_symbol(reg, L))):
        x, it, h = O.conjugate_gradient(A, b, x0=x0, rtol=1e-10, precond=M)
        assert rel(x, ref) < 1e-8
        assert h[-1] < 1e-10


def test_halfset_regularisation_functions():
    """fsc_utils, the Fourier regularisers, the dataset gains and regularize_mean_from_halfsets
    against the reference run in float64 (the last to CG tolerance, like the mean pipeline)."""
    g = load_golden("halfsets_L10.npz")
    L = int(g["L"])
    assert rel(O.shell_average_batch(g["spec"]), g["avg_shell"]) < 1e-12
    assert rel(O.rpsd_batch(g["e1"]), g["rpsd"]) < 1e-12
    assert rel(O.expand_shells(g["shells"], L), g["expand"]) < 1e-12
    assert rel(O.upsample_expand_shells(g["shells"], 2 * L), g["upexpand"]) < 1e-12
    assert rel(O.vol_fsc(g["v1"], g["v2"]), g["vol_fsc"]) < 1e-12
    assert rel(O.covar_rpsd(g["e1"]), g["covar_rpsd"]) < 1e-12
    assert rel(O.covar_fsc(g["e1"], g["e2"]), g["covar_fsc"]) < 1e-12
    assert rel(O.total_gain(g["gain_pts"], g["gain_filters"], L), g["total_gain"]) < 1e-12
    assert rel(O.total_covar_gain(g["gain_pts"], g["gain_filters"], L), g["total_covar_gain"]) < 1e-12
    reg, fsc = O.updated_fourier_reg(g["e1"], g["e2"], g["total_covar_gain"], L, True)
    assert rel(reg, g["updated_reg"]) < 1e-12 and rel(fsc, g["updated_reg_fsc"]) < 1e-12
    assert rel(O.updated_fourier_reg(g["e1"], g["e2"], g["total_covar_gain"], L, False)[0],
               g["updated_reg_spatial"]) < 1e-12
    assert rel(O.fourier_reg_term(g["e1"], 2, L, 0.7), g["fourier_reg_term"]) < 1e-12
    assert rel(O.fourier_reg_halfsets(g["updated_reg"], 2, L), g["fourier_reg_halfsets"]) < 1e-12
    vol, it = O.regularize_mean_from_halfsets(g["m1"], g["rhs1"], g["lhs1"], g["m2"], g["rhs2"], g["lhs2"])
    assert rel(vol, g["mean_halfsets"]) < 1e-5
    assert abs(it - int(g["mean_halfsets_iters"][0])) <= 2
