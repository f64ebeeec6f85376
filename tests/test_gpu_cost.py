"""GPU parity of the covariance cost and its hand-written gradient: the drop-in cost
functions and the fused single-call step, against the reference's own outputs (golden
fixture, float64 autograd) and the float64 oracle."""
import numpy as np
import pytest
import torch

from conftest import cost_scale, load_golden
from oracle import nufft_oracle as O

pytestmark = pytest.mark.gpu

TOL_COST = 1e-5   # FP32 path vs FP64 reference, relative
TOL_GRAD = 1e-4   # gradient vs FP64, relative (the stated gradient bound)


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("objective", ["ml", "ls"])
@pytest.mark.parametrize("with_reg", [False, True])
def test_dropin_cost_matches_reference(pkg, dev, objective, with_reg):
    c = load_golden("cost_L10_r3.npz")
    L, r, us = int(c["L"]), int(c["r"]), int(c["us"])
    covar = pkg.Covar(L, r, upsampling_factor=us, vectors=torch.tensor(c["vectors"])).to(dev)
    covar.init_grid_correction("bilinear")
    plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=us, mode="bilinear")
    plan.setpts(torch.tensor(c["pts"], dtype=torch.float32, device=dev))
    fn = pkg.cost_maximum_liklihood_fourier_domain if objective == "ml" else pkg.cost_fourier_domain
    kw = dict(reg_scale=float(c["reg_scale"]), fourier_reg=torch.tensor(c["fourier_reg"], device=dev)) if with_reg else {}
    val = fn(covar.get_vectors_fourier_domain(), torch.tensor(c["images"], device=dev),
             plan, torch.tensor(c["filters"], device=dev), float(c["noise_var"]), **kw)
    val.backward()
    tag = objective + ("_reg" if with_reg else "")
    assert rel(val, c[tag + "_cost"]) < TOL_COST
    assert rel(covar.vectors.grad, c[tag + "_grad_vectors"]) < TOL_GRAD
    assert rel(covar.log_sqrt_eigenvals.grad, c[tag + "_grad_logsqrt"]) < TOL_GRAD
    # per-image (mean_aggregate=False) data term
    per = fn(covar.get_vectors_fourier_domain(), torch.tensor(c["images"], device=dev), plan,
             torch.tensor(c["filters"], device=dev), float(c["noise_var"]), mean_aggregate=False)
    if not with_reg:
        assert rel(per, c[tag + "_per_image"]) < TOL_COST


@pytest.mark.parametrize("objective", ["ml", "ls"])
@pytest.mark.parametrize("with_reg", [False, True])
def test_fused_step_matches_reference(pkg, dev, objective, with_reg):
    c = load_golden("cost_L10_r3.npz")
    L, r, us = int(c["L"]), int(c["r"]), int(c["us"])
    step = pkg.FusedCovarStep(L, r, "bilinear", us, device=dev)
    step.set_points(torch.tensor(c["pts"], dtype=torch.float32, device=dev))
    B = c["images"].shape[0]
    per = torch.empty((B,), dtype=torch.float64, device=dev)
    val, gv, gl = step(torch.tensor(c["vectors_normalised"], device=dev), torch.tensor(c["log_sqrt_eigenvals"], device=dev),
                       torch.tensor(c["images"], device=dev).reshape(B, -1),
                       torch.tensor(c["filters"], device=dev).reshape(B, -1), float(c["noise_var"]),
                       reg_scale=float(c["reg_scale"]) if with_reg else 0.0,
                       fourier_reg=torch.tensor(c["fourier_reg"], device=dev) if with_reg else None,
                       objective=0 if objective == "ml" else 1, per_image=per, sync_cost=True)
    tag = objective + ("_reg" if with_reg else "")
    assert rel(val, c[tag + "_cost"]) < TOL_COST
    assert rel(gv, c[tag + "_grad_vectors"]) < TOL_GRAD
    assert rel(gl, c[tag + "_grad_logsqrt"]) < TOL_GRAD


@pytest.mark.parametrize("per_channel", [False, True])
def test_fused_ls_regulariser_matches_dropin(pkg, dev, per_channel):
    """The least-squares cost with its Fourier regulariser (the |X X^H|^2 term of the
    reshape to (n, r n^2), r = 5 not dividing n = 128) in the fused step (line transforms, GEMMs
    before the spread) against the drop-in cost through torch autograd, with one regulariser
    for all eigenvolumes or one each; reg_scale makes the regulariser as large as the data term."""
    L, r, B = 64, 5, 8
    n = 2 * L
    g = torch.Generator(device=dev).manual_seed(5)
    torch.manual_seed(5)  # the Covar's random initial eigenvolumes
    covar = pkg.Covar(L, r, upsampling_factor=2).to(dev)
    covar.init_grid_correction("bilinear")
    R = torch.linalg.qr(torch.randn((B, 3, 3), device=dev, generator=g))[0].contiguous()
    imgs = torch.randn((B, L, L), device=dev, generator=g, dtype=torch.complex64) * 50
    ctf = torch.rand((B, L, L), device=dev, generator=g) + 0.2
    shape = (r, n, n, n) if per_channel else (n, n, n)
    fr = torch.rand(shape, device=dev, generator=g) + 0.5
    plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=2, mode="bilinear")
    plan.setrot(R)
    with torch.no_grad():
        vols = covar.get_vectors_fourier_domain()
        c0 = pkg.cost_fourier_domain(vols, imgs, plan, ctf, 300.0).item()
        c1 = pkg.cost_fourier_domain(vols, imgs, plan, ctf, 300.0, reg_scale=1.0, fourier_reg=fr).item()
    reg_scale = abs(c0) / abs(c1 - c0)
    val = pkg.cost_fourier_domain(covar.get_vectors_fourier_domain(), imgs, plan, ctf, 300.0, reg_scale=reg_scale,
                                  fourier_reg=fr)
    val.backward()
    step = pkg.FusedCovarStep(L, r, "bilinear", 2, device=dev)
    step.set_rotations(R)
    v2, gv, gl = step(covar.vectors.detach(), covar.log_sqrt_eigenvals.detach(), imgs.reshape(B, -1),
                      ctf.reshape(B, -1), 300.0, reg_scale=reg_scale, fourier_reg=fr, objective=1, sync_cost=True)
    assert rel(v2, val.item()) < 1e-5
    assert rel(gv, covar.vectors.grad) < 1e-4
    assert rel(gl, covar.log_sqrt_eigenvals.grad) < 1e-4


# r = 10 takes the staged Gram and per-pixel W-pass kernels, r = 20 two channel groups of the
# spreading, two interpolation passes and the rank-20 solve; L = 64 and 128 (fine grids of 128,
# 256) the hand-written line transforms with the pack, regulariser and unpack fused in
@pytest.mark.parametrize("L,r,B", [(16, 3, 8), (24, 5, 12), (16, 10, 6), (16, 20, 4), (64, 3, 2), (128, 2, 1)])
def test_fused_es_step_matches_fp64_oracle(pkg, dev, L, r, B):
    rng = np.random.default_rng(L * r)
    vec = rng.standard_normal((r, L, L, L))
    vec /= np.linalg.norm(vec.reshape(r, -1), axis=1)[:, None, None, None]
    vec = vec.astype(np.float32)
    ls = np.log(rng.uniform(2.0, 6.0, r)).astype(np.float32)
    R = O.rotvec_to_rotmat(rng.standard_normal((B, 3))).astype(np.float32)
    imgs = ((rng.standard_normal((B, L, L)) + 1j * rng.standard_normal((B, L, L))) * 3).astype(np.complex64)
    ctf = rng.uniform(0.2, 1.3, (B, L, L)).astype(np.float32)
    fr = rng.uniform(0.5, 2.0, (2 * L,) * 3).astype(np.float32)
    step = pkg.FusedCovarStep(L, r, "nufft", 2, width=6, device=dev)
    step.set_rotations(torch.tensor(R, device=dev))
    val, gv, gl = step(torch.tensor(vec, device=dev), torch.tensor(ls, device=dev),
                       torch.tensor(imgs, device=dev).reshape(B, -1), torch.tensor(ctf, device=dev).reshape(B, -1),
                       5.0, reg_scale=0.01, fourier_reg=torch.tensor(fr, device=dev), sync_cost=True)
    pts = O.rotated_points(R.astype(np.float64), L)
    ref = O.covar_cost_grad(vec, ls, imgs, pts, ctf, 5.0, kind="es", width=6, reg_scale=0.01, fourier_reg=fr)
    assert rel(val, ref[0]) < TOL_COST
    assert rel(gv, ref[1]) < TOL_GRAD
    assert rel(gl, ref[2]) < TOL_GRAD


@pytest.mark.parametrize("L,r,B", [(64, 4, 16), (256, 2, 2)])
def test_fused_step_equals_dropin_autograd_full_size(pkg, dev, L, r, B):
    """Two independent code paths: the single-call fused step (line-DFT transforms with the
    pack and unpack fused; n = 128 and 512) and the drop-in cost (torch's FFT of the volumes,
    vol_forward + ProjectedCost autograd) on the same discretized plan."""
    g = torch.Generator(device=dev).manual_seed(1)
    torch.manual_seed(1)  # the Covar's random initial eigenvolumes
    covar = pkg.Covar(L, r, upsampling_factor=2).to(dev)
    covar.init_grid_correction("bilinear")
    R = torch.linalg.qr(torch.randn((B, 3, 3), device=dev, generator=g))[0].contiguous()
    imgs = torch.randn((B, L, L), device=dev, generator=g, dtype=torch.complex64) * 50
    ctf = torch.rand((B, L, L), device=dev, generator=g) + 0.2
    plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=2, mode="bilinear")
    plan.setrot(R)
    val = pkg.cost_maximum_liklihood_fourier_domain(covar.get_vectors_fourier_domain(), imgs, plan, ctf, 300.0)
    val.backward()
    with torch.no_grad():
        per_image = pkg.cost_maximum_liklihood_fourier_domain(covar.get_vectors_fourier_domain(), imgs, plan, ctf,
                                                              300.0, mean_aggregate=False)
    step = pkg.FusedCovarStep(L, r, "bilinear", 2, device=dev)
    step.set_rotations(R)
    v2, gv, gl = step(covar.vectors.detach(), covar.log_sqrt_eigenvals.detach(), imgs.reshape(B, -1),
                      ctf.reshape(B, -1), 300.0, sync_cost=True)
    assert abs(v2 - val.item()) < 1e-5 * cost_scale(val.item(), per_image)
    assert rel(gv, covar.vectors.grad) < 1e-4
    assert rel(gl, covar.log_sqrt_eigenvals.grad) < 1e-4


def test_latent_map_matches_reference(pkg, dev):
    g = load_golden("latent_L10_r3.npz")
    z, m, b = pkg.wiener_coords.compute_latentMAP_batch(torch.tensor(g["images"], device=dev),
                                                        torch.tensor(g["eigen_forward"], device=dev),
                                                        float(g["noise_var"]),
                                                        torch.tensor(g["eigenvals_inv"], device=dev))
    assert rel(z, g["z"]) < TOL_COST and rel(m, g["m"]) < TOL_COST and rel(b, g["b"]) < TOL_COST
    z, m, b = pkg.wiener_coords.compute_latentMAP_batch(torch.tensor(g["images"].real, device=dev),
                                                        torch.tensor(g["eigen_forward"].real, device=dev),
                                                        float(g["noise_var"]),
                                                        torch.tensor(g["eigenvals_inv"], device=dev))
    assert rel(z, g["z_real"]) < TOL_COST and rel(m, g["m_real"]) < TOL_COST


def _es_case(L, r, B, seed):
    rng = np.random.default_rng(seed)
    vec = rng.standard_normal((r, L, L, L))
    vec /= np.linalg.norm(vec.reshape(r, -1), axis=1)[:, None, None, None]
    vec = vec.astype(np.float32)
    ls = np.log(rng.uniform(2.0, 6.0, r)).astype(np.float32)
    R = O.rotvec_to_rotmat(rng.standard_normal((B, 3))).astype(np.float32)
    imgs = ((rng.standard_normal((B, L, L)) + 1j * rng.standard_normal((B, L, L))) * 3).astype(np.complex64)
    ctf = rng.uniform(0.2, 1.3, (B, L, L)).astype(np.float32)
    fr = rng.uniform(0.5, 2.0, (2 * L,) * 3).astype(np.float32)
    return vec, ls, R, imgs, ctf, fr


# the benchmark's own kernels at the benchmark's shapes: L = 128 (fine grid 256^3) with r = 10
# (interp_kernel<ES,6,5>, spread_rows_kernel<ES,6,5,3,1>, the n = 256 line DFTs) and r = 20, and
# L = 256 (fine grid 512^3, the full-pipeline configuration); the float64 reference is the
# channel-streamed ES step of oracle/cpu_step.py (C loops + scipy FFTs)
@pytest.mark.parametrize("L,r,B", [(128, 10, 4), (128, 20, 2), (256, 10, 1)])
def test_fused_es_step_headline_shapes_match_fp64(pkg, dev, L, r, B):
    from oracle import cpu_step

    vec, ls, R, imgs, ctf, fr = _es_case(L, r, B, 7 * L + r)
    step = pkg.FusedCovarStep(L, r, "nufft", 2, width=6, device=dev)
    step.set_rotations(torch.tensor(R, device=dev))
    val, gv, gl = step(torch.tensor(vec, device=dev), torch.tensor(ls, device=dev),
                       torch.tensor(imgs, device=dev).reshape(B, -1), torch.tensor(ctf, device=dev).reshape(B, -1),
                       5.0, reg_scale=0.01, fourier_reg=torch.tensor(fr, device=dev), sync_cost=True)
    gv, gl = gv.cpu().numpy(), gl.cpu().numpy()
    del step
    torch.cuda.empty_cache()
    ref = cpu_step.covar_cost_grad_es(vec, ls, R.astype(np.float64), imgs, ctf, 5.0, width=6, reg_scale=0.01,
                                      fourier_reg=fr)
    assert rel(val, ref[0]) < TOL_COST
    assert rel(gv, ref[1]) < TOL_GRAD
    assert rel(gl, ref[2]) < TOL_GRAD


def test_fused_gradient_matches_fp64_finite_differences(pkg, dev):
    """The hand-written adjoint against float64 central differences of the oracle's cost on
    the L = 32, r = 5, N = 512 instance: <grad, d> for three random directions d of the
    parameters (vectors and log-scales)."""
    from oracle import cpu_step

    L, r, B = 32, 5, 512
    vec, ls, R, imgs, ctf, fr = _es_case(L, r, B, 3205)
    step = pkg.FusedCovarStep(L, r, "nufft", 2, width=6, device=dev)
    step.set_rotations(torch.tensor(R, device=dev))
    _, gv, gl = step(torch.tensor(vec, device=dev), torch.tensor(ls, device=dev),
                     torch.tensor(imgs, device=dev).reshape(B, -1), torch.tensor(ctf, device=dev).reshape(B, -1),
                     5.0, reg_scale=0.01, fourier_reg=torch.tensor(fr, device=dev), sync_cost=True)
    gv, gl = gv.cpu().numpy().astype(np.float64), gl.cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(11)
    R64, v64, l64 = R.astype(np.float64), vec.astype(np.float64), ls.astype(np.float64)

    def f(v, l):
        return cpu_step.covar_cost_grad_es(v, l, R64, imgs, ctf, 5.0, width=6, reg_scale=0.01, fourier_reg=fr,
                                           cost_only=True)

    for _ in range(3):
        dv = rng.standard_normal(v64.shape)
        dv /= np.linalg.norm(dv)
        dl = rng.standard_normal(r) * 0.1
        h = 1e-4
        fd = (f(v64 + h * dv, l64 + h * dl) - f(v64 - h * dv, l64 - h * dl)) / (2 * h)
        an = float(np.sum(gv * dv) + np.sum(gl * dl))
        assert abs(an - fd) / abs(fd) < TOL_GRAD, (an, fd)


@pytest.mark.parametrize("objective", ["ml", "ls"])
@pytest.mark.parametrize("with_reg", [False, True])
def test_spatial_costs_match_reference(pkg, dev, objective, with_reg):
    """cost / cost_maximum_liklihood (spatial eigenvolumes through the exact NufftPlan, spatial
    images) against the reference run in float64 on the exact NUDFT (fixture)."""
    c = load_golden("spatial_cost_L10_r3.npz")
    L, r = int(c["L"]), int(c["r"])
    covar = pkg.Covar(L, r, vectors=torch.tensor(c["vectors"])).to(dev)
    plan = pkg.NufftPlan((L,) * 3, batch_size=r, device=dev, width=8)
    plan.setpts(torch.tensor(c["pts"], dtype=torch.float32, device=dev))
    fn = pkg.cost_maximum_liklihood if objective == "ml" else pkg.cost
    kw = dict(reg_scale=float(c["reg_scale"]), fourier_reg=torch.tensor(c["fourier_reg"], device=dev)) if with_reg else {}
    ims = torch.tensor(c["images"], device=dev)
    filt = torch.tensor(c["filters"], device=dev)
    val = fn(covar.get_vectors_spatial_domain(), ims, plan, filt, float(c["noise_var"]), **kw)
    val.backward()
    tag = objective + ("_reg" if with_reg else "")
    assert rel(val, c[tag + "_cost"]) < TOL_COST
    assert rel(covar.vectors.grad, c[tag + "_grad_vectors"]) < TOL_GRAD
    assert rel(covar.log_sqrt_eigenvals.grad, c[tag + "_grad_logsqrt"]) < TOL_GRAD
    per = fn(covar.get_vectors_spatial_domain(), ims, plan, filt, float(c["noise_var"]), mean_aggregate=False, **kw)
    assert rel(per, c[tag + "_per_image"]) < TOL_COST


@pytest.mark.parametrize("L", [16, 64])
def test_fused_step_per_channel_regulariser(pkg, dev, L):
    """One Fourier regulariser per eigenvolume, (r, n^3), as CovarTrainer.compute_fourier_reg_term
    builds it: the fallback regulariser kernel (L = 16) and the one fused in the line transform
    (L = 64), against the float64 oracle."""
    r, B = 3, 6
    vec, ls, R, imgs, ctf, _ = _es_case(L, r, B, 99 + L)
    fr = np.random.default_rng(L).uniform(0.5, 2.0, (r,) + (2 * L,) * 3).astype(np.float32)
    step = pkg.FusedCovarStep(L, r, "nufft", 2, width=6, device=dev)
    step.set_rotations(torch.tensor(R, device=dev))
    val, gv, gl = step(torch.tensor(vec, device=dev), torch.tensor(ls, device=dev),
                       torch.tensor(imgs, device=dev).reshape(B, -1), torch.tensor(ctf, device=dev).reshape(B, -1),
                       5.0, reg_scale=0.05, fourier_reg=torch.tensor(fr, device=dev), sync_cost=True)
    ref = O.covar_cost_grad(vec, ls, imgs, O.rotated_points(R.astype(np.float64), L), ctf, 5.0, kind="es", width=6,
                            reg_scale=0.05, fourier_reg=fr)
    assert rel(val, ref[0]) < TOL_COST
    assert rel(gv, ref[1]) < TOL_GRAD
    assert rel(gl, ref[2]) < TOL_GRAD


def _ctf_params(rng, B):
    apix = np.full(B, 1.5)
    dfu = rng.uniform(1e4, 3e4, B)
    dfv = dfu * rng.uniform(0.9, 1.1, B)
    ang = rng.uniform(0, 180, B)
    ps = rng.uniform(0, 30, B)
    return np.stack([apix, dfu, dfv, ang, np.full(B, 300.0), np.full(B, 2.7), np.full(B, 0.1), ps], 1).astype(np.float32)


@pytest.mark.parametrize("L", [32, 128, 129])
def test_ctf_from_params_matches_fp64_formula(pkg, dev, L):
    """The in-kernel CTF (double-float phase, reduced modulo 2 pi) against the float64 formula,
    with astigmatism and phase shifts, up to Nyquist at 1.5 A pixels (phases of hundreds of
    radians): absolute error below 2e-6 (the float32 rounding of the reduced angle)."""
    rng = np.random.default_rng(L)
    prm = _ctf_params(rng, 16)
    got = pkg.synthetic.ctf_from_params(torch.tensor(prm, device=dev), L).cpu().numpy()
    want = O.ctf_from_params(prm, L)
    assert np.abs(got - want).max() < 2e-6


def test_fused_step_with_ctf_params_matches_fp64(pkg, dev):
    """The fused step with the CTF computed in-kernel from parameters against the float64
    oracle given the float64 CTF images (r = 10: the grouped interpolation path)."""
    L, r, B = 64, 10, 6
    vec, ls, R, imgs, _, fr = _es_case(L, r, B, 64)
    prm = _ctf_params(np.random.default_rng(3), B)
    ctf64 = O.ctf_from_params(prm, L)
    step = pkg.FusedCovarStep(L, r, "nufft", 2, width=6, device=dev)
    step.set_rotations(torch.tensor(R, device=dev))
    val, gv, gl = step(torch.tensor(vec, device=dev), torch.tensor(ls, device=dev),
                       torch.tensor(imgs, device=dev).reshape(B, -1), None, 5.0, reg_scale=0.01,
                       fourier_reg=torch.tensor(fr, device=dev), sync_cost=True,
                       ctf_params=torch.tensor(prm, device=dev))
    ref = O.covar_cost_grad(vec, ls, imgs, O.rotated_points(R.astype(np.float64), L), ctf64, 5.0, kind="es", width=6,
                            reg_scale=0.01, fourier_reg=fr)
    assert rel(val, ref[0]) < TOL_COST
    assert rel(gv, ref[1]) < TOL_GRAD
    assert rel(gl, ref[2]) < TOL_GRAD
