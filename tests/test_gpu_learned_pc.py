"""What the trained preconditioner network gains over the method without it: CG iterations to
relative residual 1e-5 with the circulant symbol (the untrained network's output, delta = 0)
against the learned symbol, on problems the network was not trained on."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _mean(rows, key):
    return float(np.mean([r[key] for r in rows]))


def test_training_on_the_gpu_lowers_the_held_out_loss(pkg, dev):
    """Training runs on the GPU through the library's kernels and lowers the trained quantity
    (the energy-norm error after K preconditioned CG steps) on problems it has not seen."""
    lp = pkg.learned_pc
    gen = lp.ProblemGenerator(32, 2000, dev)
    train = [gen(100 + i) for i in range(12)]
    held_out = [gen(9000 + i) for i in range(3)]
    net = lp.UNet3D(4, 16, dev)
    before = lp.evaluate(net, held_out)
    assert all(r["learned"] == r["circulant"] for r in before)  # zero-initialised head

    def held_out_loss():
        with torch.no_grad():
            return float(np.mean([float(lp.pcg_energy_loss(p, lp.symbol_from_features(net, p.feats, p.log_a, 32), 20))
                                  for p in held_out]))

    l0 = held_out_loss()
    hist = lp.train(net, train, epochs=4, lr=1e-3, K=20)
    assert hist[-1] < hist[0]
    assert held_out_loss() < l0


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                                    "3dcovarestimation_gb300", "learned_pc_weights.npz")),
                    reason="no trained weights")
def test_committed_network_beats_the_circulant_preconditioner(pkg, dev):
    lp = pkg.learned_pc
    pc = lp.LearnedPreconditioner(device=dev)
    gen = lp.ProblemGenerator(128, 60000, dev)
    prob = gen(77, solve_rtol=1e-5)
    rows = lp.evaluate(pc.net, [prob])
    assert rows[0]["learned"] is not None
    assert rows[0]["learned"] < rows[0]["circulant"]
    x, info = pkg.cg_solve(prob.reg, prob.b, prob.x0, 128, rtol=1e-5, precond=pc.symbol(prob.reg, 128))
    assert info.converged and info.relres < 1e-5
    # the true residual, recomputed in float64 (the CG tracks a recursively updated one); the
    # solutions themselves may differ by up to cond(A) * rtol, cond(A) ~ 1e7 here
    n = prob.reg.shape[-1]
    reg = prob.reg.double()
    xx = x.reshape((128,) * 3).to(torch.complex128)
    ax = pkg.centered_ifft3(reg * pkg.centered_fft3(xx, padding_size=(n,) * 3), cropping_size=(128,) * 3)
    b = prob.b.to(torch.complex128)
    assert float(torch.linalg.vector_norm(b - ax) / torch.linalg.vector_norm(b)) < 2e-5


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                                    "3dcovarestimation_gb300", "learned_pc_weights.npz")),
                    reason="no trained weights")
def test_committed_network_against_the_diagonal_preconditioner(pkg, dev):
    """The fallback the learned preconditioner is measured against: the Fourier-diagonal 1/reg_lhs
    on the fine grid.  Same problem, same rtol, both converge; the learned symbol (features +
    network + the L^3 symbol, timed inside the solve) takes less wall time than the diagonal
    preconditioner, whose every iteration costs a second fine-grid transform pair."""
    import time

    lp = pkg.learned_pc
    pc = lp.LearnedPreconditioner(device=dev)
    gen = lp.ProblemGenerator(128, 60000, dev)
    prob = gen(78, solve_rtol=1e-5)
    # warm both paths (transform plans, network kernels)
    pkg.cg_solve(prob.reg, prob.b, prob.x0, 128, rtol=1e-1, maxiter=2, precond="diagonal")
    pkg.cg_solve(prob.reg, prob.b, prob.x0, 128, rtol=1e-1, maxiter=2, precond=pc.symbol(prob.reg, 128))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, info_d = pkg.cg_solve(prob.reg, prob.b, prob.x0, 128, rtol=1e-5, maxiter=20000, precond="diagonal")
    torch.cuda.synchronize()
    t_diag = time.perf_counter() - t0
    t0 = time.perf_counter()
    sym = pc.symbol(prob.reg, 128)
    _, info_l = pkg.cg_solve(prob.reg, prob.b, prob.x0, 128, rtol=1e-5, maxiter=20000, precond=sym)
    torch.cuda.synchronize()
    t_learned = time.perf_counter() - t0
    assert info_d.converged and info_l.converged
    print(f"diagonal PC {info_d.iters} iterations {t_diag:.3f} s; learned {info_l.iters} iterations {t_learned:.3f} s")
    assert t_learned < t_diag
