"""Output formats (CPU): the Covar checkpoint is interchangeable with the reference's
(``covar.py:82-112``), in both directions, and the trainer's ``training_results.bin``
dictionary (``covar_sgd.py:524-545``) round-trips through torch.save.  The reference-side
checks import the reference copy under ``oracle/_ref`` (skipped where it is absent)."""
import io

import numpy as np
import pytest
import torch

from conftest import load_golden


@pytest.fixture(scope="module")
def cpkg():
    import importlib

    return importlib.import_module("3dcovarestimation_gb300")


def test_covar_state_dict_matches_reference_fixture(cpkg):
    g = load_golden("state_dict_L6_r2.npz")
    L, r = int(g["L"]), int(g["r"])
    cov = cpkg.Covar(L, r, dtype=torch.float64, fourier_domain=True, vectors=torch.tensor(g["vectors_init"]))
    cov.init_grid_correction("bilinear")
    sd = cov.state_dict()
    assert sorted(sd.keys()) == list(g["keys"])
    for k in g["keys"]:
        if "sd_" + k in g:
            np.testing.assert_allclose(np.asarray(sd[k]), g["sd_" + k], rtol=1e-6, atol=0)
    eig, lam = cov.eigenvecs
    # eigenvectors up to sign
    s = np.sign(np.sum(eig.numpy().reshape(r, -1) * g["eigenvecs"].reshape(r, -1), axis=1))
    np.testing.assert_allclose(eig.numpy() * s[:, None, None, None], g["eigenvecs"], atol=1e-10)
    np.testing.assert_allclose(lam.numpy(), g["eigenvals"], rtol=1e-10)


def test_results_dict_round_trip(cpkg):
    cov = cpkg.Covar(8, 3, fourier_domain=True)
    tr = cpkg.CovarTrainer(cov, [], "cpu", noise_var=1.0, dataset_size=10)
    tr.training_log["cost_val"] = [3.0, 2.0]
    tr.fourier_reg = torch.ones((16, 16, 16))
    buf = io.BytesIO()
    torch.save(tr.results_dict(), buf)
    buf.seek(0)
    ckp = torch.load(buf, weights_only=False)
    assert {"vectors", "log_sqrt_eigenvals", "_in_spatial_domain", "grid_correction", "vectorsGT", "fourier_reg",
            "epoch_ind", "lr_history", "cost_val", "epoch_run_time"} <= set(ckp)
    cov2 = cpkg.Covar(8, 3, fourier_domain=True)
    cov2.load_state_dict({k: ckp[k] for k in ("vectors", "log_sqrt_eigenvals", "_in_spatial_domain",
                                              "grid_correction")})
    assert torch.equal(cov2.vectors, cov.vectors)


def _reference_covar():
    from oracle import ref_step

    if not ref_step.available():
        pytest.skip("reference copy not installed under oracle/_ref")
    return ref_step.load_reference()["covar"].Covar


def test_state_dict_loads_into_reference_and_back(cpkg):
    RefCovar = _reference_covar()
    ours = cpkg.Covar(6, 2, fourier_domain=True)
    ours.init_grid_correction("bilinear")
    ref = RefCovar(6, 2, fourier_domain=True)
    ref.load_state_dict(ours.state_dict())
    assert torch.equal(ref.get_vectors_spatial_domain(), ours.get_vectors_spatial_domain())
    assert torch.equal(ref.grid_correction, ours.grid_correction)
    back = cpkg.Covar(6, 2)
    back.load_state_dict(ref.state_dict())
    assert torch.equal(back.get_vectors_spatial_domain(), ref.get_vectors_spatial_domain())
    assert back._in_spatial_domain == ref._in_spatial_domain
