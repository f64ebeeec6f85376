"""GPU half-set machinery (fsc_utils, the Fourier regularisers, dataset gains,
regularize_mean_from_halfsets) against the reference's float64 outputs."""
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from conftest import load_golden

pytestmark = pytest.mark.gpu

TOL64 = 1e-10   # float64 torch on the GPU against the reference's float64 (different FFTs)
TOL_FP32 = 1e-5  # float32 spreading kernels
TOL_CG = 1e-4    # a CG stopped at rtol 1e-6, float32 against float64


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def g():
    return load_golden("halfsets_L10.npz")


def T(x, dev):
    return torch.as_tensor(np.asarray(x)).to(dev)


def test_fsc_utils(pkg, dev, g):
    F = pkg.fsc_utils
    L = int(g["L"])
    assert rel(F.average_fourier_shell(T(g["spec"], dev)), g["avg_shell"]) < TOL64
    assert rel(F.rpsd(*T(g["e1"], dev)), g["rpsd"]) < TOL64
    assert rel(F.expand_fourier_shell(T(g["shells"], dev), L, 3), g["expand"]) < TOL64
    assert rel(F.upsample_and_expand_fourier_shell(T(g["shells"], dev), 2 * L, 3), g["upexpand"]) < TOL64
    assert rel(F.vol_fsc(T(g["v1"], dev), T(g["v2"], dev)), g["vol_fsc"]) < TOL64
    assert rel(F.covar_rpsd(T(g["e1"], dev)), g["covar_rpsd"]) < TOL64
    assert rel(F.covar_fsc(T(g["e1"], dev), T(g["e2"], dev)), g["covar_fsc"]) < TOL64


def test_fourier_regularisers(pkg, dev, g):
    L = int(g["L"])
    reg, fsc = pkg.covar_sgd.compute_updated_fourier_reg(T(g["e1"], dev), T(g["e2"], dev),
                                                          T(g["total_covar_gain"], dev).clone(), None, L, True)
    assert rel(reg, g["updated_reg"]) < TOL64 and rel(fsc, g["updated_reg_fsc"]) < TOL64
    reg_s, _ = pkg.covar_sgd.compute_updated_fourier_reg(T(g["e1"], dev), T(g["e2"], dev),
                                                          T(g["total_covar_gain"], dev).clone(), None, L, False)
    assert rel(reg_s, g["updated_reg_spatial"]) < TOL64
    fake = SimpleNamespace(covar=SimpleNamespace(upsampling_factor=2, resolution=L), noise_var=0.7, device=dev)
    pkg.CovarTrainer.compute_fourier_reg_term(fake, T(g["e1"], dev))
    assert rel(fake.fourier_reg, g["fourier_reg_term"]) < TOL64
    pkg.CovarTrainer.update_fourier_reg_halfsets(fake, T(g["updated_reg"], dev))
    assert rel(fake.fourier_reg, g["fourier_reg_halfsets"]) < TOL64


class _DS:
    def __init__(self, pts, filters, L):
        self.pts, self.filters, self.resolution = pts, filters, L

    def __len__(self):
        return len(self.pts)

    def __getitem__(self, sl):
        return None, self.pts[sl], self.filters[sl], None


def test_dataset_gains(pkg, dev, g):
    L = int(g["L"])
    ds = _DS(T(g["gain_pts"], dev).float(), T(g["gain_filters"], dev).float(), L)
    assert rel(pkg.dataset.get_total_gain(ds, batch_size=16, device=dev), g["total_gain"]) < TOL_FP32
    assert rel(pkg.dataset.get_total_covar_gain(ds, batch_size=16, device=dev), g["total_covar_gain"]) < TOL_FP32


def test_mean_from_halfsets(pkg, dev, g):
    args = [T(g[k], dev) for k in ("m1", "rhs1", "lhs1", "m2", "rhs2", "lhs2")]
    vol = pkg.mean.regularize_mean_from_halfsets(*args)
    assert rel(vol, g["mean_halfsets"]) < TOL_CG
