"""Edge cases of the CUDA path: the exceptions the reference raises for bad input (ValueError
for arguments, FloatingPointError for a non-positive-definite per-image matrix), a call before
the points are set, the CG stopping at maxiter, the largest rank the kernels take (r = 32)
against the float64 oracle, and a single-image batch."""
import numpy as np
import pytest
import torch

from oracle import nufft_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_bad_arguments_raise_value_errors(pkg, dev):
    L = 12
    plan = pkg.NufftPlan((L,) * 3, batch_size=2, device=dev)
    with pytest.raises(ValueError):  # points must be (N, 3, L^2)
        plan.setpts(torch.zeros((3, 2, L * L), device=dev))
    plan.setpts(torch.zeros((3, 3, L * L), device=dev))
    with pytest.raises(ValueError):  # no CPU tensors
        plan.execute_forward(torch.zeros((2, L, L, L)))
    step = pkg.FusedCovarStep(L, 2, "nufft", 2, device=dev)
    R = torch.eye(3, device=dev).expand(4, 3, 3).contiguous()
    step.set_rotations(R)
    vec = torch.zeros((2, L, L, L), device=dev)
    logs = torch.zeros((2,), device=dev)
    imgs = torch.zeros((4, L * L), dtype=torch.complex64, device=dev)
    with pytest.raises(ValueError):  # a regulariser of neither n^3 nor r n^3 values
        step(vec, logs, imgs, None, 1.0, reg_scale=1.0, fourier_reg=torch.ones((5, 5, 5), device=dev))
    with pytest.raises(ValueError):  # noise_var must be positive
        step(vec, logs, imgs, None, 0.0, sync_cost=True)
    with pytest.raises(ValueError):  # CTF parameters of the wrong shape
        step(vec, logs, imgs, None, 1.0, ctf_params=torch.zeros((4, 3), device=dev))


def test_cost_before_points_is_a_state_error(pkg, dev):
    L = 12
    step = pkg.FusedCovarStep(L, 2, "nufft", 2, device=dev)
    with pytest.raises(pkg._lib.Cov3dError):
        step(torch.zeros((2, L, L, L), device=dev), torch.zeros((2,), device=dev),
             torch.zeros((4, L * L), dtype=torch.complex64, device=dev), None, 1.0, sync_cost=True)


def test_indefinite_latent_matrix_raises_floating_point_error(pkg, dev):
    n, r, P = 3, 2, 64
    g = torch.Generator(device=dev).manual_seed(2)
    q = torch.randn((n, r, P), dtype=torch.complex64, device=dev, generator=g) * 1e-3
    y = torch.randn((n, P), dtype=torch.complex64, device=dev, generator=g)
    linv = -torch.eye(r, device=dev)  # m = Q^H Q / s + Linv is not positive definite
    with pytest.raises(FloatingPointError):
        pkg.wiener_coords.compute_latentMAP_batch(y, q, 1.0, linv)


def test_cg_stops_at_maxiter_with_its_last_iterate(pkg, dev):
    L, n = 16, 32
    g = torch.Generator(device=dev).manual_seed(3)
    reg = torch.rand((n, n, n), device=dev, generator=g) + 0.01
    b = torch.randn((L, L, L), dtype=torch.complex64, device=dev, generator=g)
    x0 = torch.zeros_like(b)
    x, info = pkg.cg_solve(reg, b, x0, L, rtol=1e-12, maxiter=5)
    assert not info.converged and info.iters <= 5 and info.relres > 1e-12
    assert torch.isfinite(torch.view_as_real(x)).all() and x.abs().sum() > 0


def test_largest_rank_matches_fp64_oracle(pkg, dev):
    """r = 32, the most channels the per-image solve takes (the interpolation runs in several
    channel passes and the spreading in several channel groups)."""
    from oracle import cpu_step

    L, r, B = 16, 32, 3
    rng = np.random.default_rng(32)
    vec = rng.standard_normal((r, L, L, L)).astype(np.float32)
    vec /= np.linalg.norm(vec.reshape(r, -1), axis=1)[:, None, None, None]
    ls = np.log(rng.uniform(2.0, 6.0, r)).astype(np.float32)
    R = O.rotvec_to_rotmat(rng.standard_normal((B, 3))).astype(np.float32)
    imgs = ((rng.standard_normal((B, L, L)) + 1j * rng.standard_normal((B, L, L))) * 3).astype(np.complex64)
    ctf = rng.uniform(0.2, 1.3, (B, L, L)).astype(np.float32)
    step = pkg.FusedCovarStep(L, r, "nufft", 2, width=6, device=dev)
    step.set_rotations(torch.tensor(R, device=dev))
    val, gv, gl = step(torch.tensor(vec, device=dev), torch.tensor(ls, device=dev),
                       torch.tensor(imgs, device=dev).reshape(B, -1), torch.tensor(ctf, device=dev).reshape(B, -1),
                       5.0, sync_cost=True)
    ref = cpu_step.covar_cost_grad_es(vec, ls, R.astype(np.float64), imgs, ctf, 5.0, width=6)
    assert rel(val, ref[0]) < 1e-5
    assert rel(gv, ref[1]) < 1e-4
    assert rel(gl, ref[2]) < 1e-4
    with pytest.raises(ValueError):  # beyond the largest rank
        pkg.FusedCovarStep(L, 33, "nufft", 2, device=dev)(
            torch.zeros((33, L, L, L), device=dev), torch.zeros((33,), device=dev),
            torch.zeros((B, L * L), dtype=torch.complex64, device=dev), None, 5.0, sync_cost=True)


def test_single_image_batch(pkg, dev):
    """One image: the projections keep their (1, r, L, L) layout through the fused step and the
    drop-in cost (the reference squeezes only the volume axis of a single volume)."""
    L, r = 16, 3
    g = torch.Generator(device=dev).manual_seed(4)
    torch.manual_seed(4)  # the Covar's random initial eigenvolumes
    covar = pkg.Covar(L, r, upsampling_factor=2).to(dev)
    covar.init_grid_correction("bilinear")
    R = torch.linalg.qr(torch.randn((1, 3, 3), device=dev, generator=g))[0].contiguous()
    imgs = torch.randn((1, L, L), device=dev, generator=g, dtype=torch.complex64) * 30
    ctf = torch.rand((1, L, L), device=dev, generator=g) + 0.2
    plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=2, mode="bilinear")
    plan.setrot(R)
    val = pkg.cost_maximum_liklihood_fourier_domain(covar.get_vectors_fourier_domain(), imgs, plan, ctf, 300.0)
    val.backward()
    step = pkg.FusedCovarStep(L, r, "bilinear", 2, device=dev)
    step.set_rotations(R)
    v2, gv, gl = step(covar.vectors.detach(), covar.log_sqrt_eigenvals.detach(), imgs.reshape(1, -1),
                      ctf.reshape(1, -1), 300.0, sync_cost=True)
    assert rel(v2, val.item()) < 1e-5 or abs(v2 - val.item()) < 1e-6  # one term: relative unless near zero
    assert rel(gv, covar.vectors.grad) < 1e-4
    assert rel(gl, covar.log_sqrt_eigenvals.grad) < 1e-4


@pytest.mark.parametrize("L", [32, 16])
def test_reserved_step_allocates_nothing(pkg, dev, L):
    """A step built with ``max_batch`` (and ``ls_regulariser`` for the least-squares objective
    with its Fourier regulariser) allocates no device memory in its calls: the workspaces, the
    transforms' cuFFT plans (n = 64, 32: outside the line DFTs) and the cuBLAS handle are made
    at construction.  A step built without ``ls_regulariser`` grows the regulariser's 2 r n^3
    complex workspace on its first such call (the control that the measurement sees it)."""
    r, B, n = 3, 8, 2 * L
    g = torch.Generator(device=dev).manual_seed(5)
    vec = (torch.randn((r, L, L, L), device=dev, generator=g) / L**1.5).contiguous()
    ls = torch.zeros((r,), device=dev)
    imgs = torch.randn((B, L * L), dtype=torch.complex64, device=dev, generator=g)
    ctf = torch.rand((B, L * L), device=dev, generator=g) + 0.2
    R = torch.linalg.qr(torch.randn((B, 3, 3), device=dev, generator=g))[0].contiguous()
    fr = torch.rand((n, n, n), device=dev, generator=g) + 0.1
    gv, gl = torch.empty_like(vec), torch.empty_like(ls)

    def run(step):
        step.set_rotations(R)
        step(vec, ls, imgs, ctf, 5.0, reg_scale=0.1, fourier_reg=fr, objective=1, grad_vectors=gv, grad_log_sqrt=gl)
        torch.cuda.synchronize(dev)

    run(pkg.FusedCovarStep(L, r, "nufft", 2, device=dev, max_batch=B, ls_regulariser=True))  # loads the kernels
    free = {}
    for flag in (True, False):
        step = pkg.FusedCovarStep(L, r, "nufft", 2, device=dev, max_batch=B, ls_regulariser=flag)
        torch.cuda.synchronize(dev)
        before, _ = torch.cuda.mem_get_info(dev)
        run(step)
        run(step)
        after, _ = torch.cuda.mem_get_info(dev)
        free[flag] = before - after
        del step
    assert free[True] == 0
    if L == 32:  # a 12.6 MB workspace: new pages whatever the allocator keeps
        assert free[False] >= 2 * r * n**3 * 8
