"""GPU parity of the functions around the cost: the trainer loop (two run_batch steps with
Adam), latentMAP / wiener_coords over a dataset in ragged batches, image preprocessing, and
the device-resident training schedule, against fixtures produced by the reference itself
(float64) and against the float64 oracle."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import nufft_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


class _Data(torch.utils.data.Dataset):
    def __init__(self, images, pts, filters, noise_var):
        self.images, self.pts_rot, self.filters, self.noise_var = images, pts, filters, noise_var
        self.mask = None

    def __len__(self):
        return len(self.images)

    def __getitem__(self, idx):
        return self.images[idx], self.pts_rot[idx], self.filters[idx], idx

    def to_fourier_domain(self):
        pass

    def to_spatial_domain(self):
        pass


def test_trainer_two_steps_match_reference(pkg, dev):
    """CovarTrainer (reference DataLoader input, bilinear plan, ML objective, Adam, Fourier
    regulariser from compute_fourier_reg_term): the cost of each run_batch and the parameters
    after each Adam update."""
    g = load_golden("trainer_L10_r3.npz")
    L, r, B = int(g["L"]), int(g["r"]), int(g["B"])
    ds = _Data(torch.tensor(g["images"]), torch.tensor(g["pts"], dtype=torch.float32), torch.tensor(g["filters"]),
               float(g["noise_var"]))
    loader = torch.utils.data.DataLoader(ds, batch_size=B, shuffle=False)
    covar = pkg.Covar(L, r, vectors=torch.tensor(g["vectors"]), fourier_domain=True)
    tr = pkg.CovarTrainer(covar, loader, dev)
    tr.setup_training(lr=float(g["lr"]), optim_type="Adam", reg=float(g["reg"]), nufft_disc="bilinear",
                      objective_func="ml")
    assert tr.reg_scale == pytest.approx(float(g["reg_scale"]))
    tr.compute_fourier_reg_term(torch.tensor(g["reg_vecs"], device=dev))
    assert rel(tr.fourier_reg, g["fourier_reg"]) < 1e-6
    for k, batch in enumerate(loader):
        im, p, f = tr.prepare_batch(batch)
        c = tr.run_batch(im, p, f)
        assert rel(float(c), g["costs"][k]) < 1e-5
        assert rel(covar.vectors, g[f"step{k}_vectors"]) < 1e-5
        assert rel(covar.log_sqrt_eigenvals, g[f"step{k}_log_sqrt"]) < 1e-5


class _Latent:
    def __init__(self, images, pts, filters, noise_var):
        self.images, self.pts, self.filters, self.noise_var = images, pts, filters, noise_var

    def __len__(self):
        return len(self.images)

    def __getitem__(self, idx):
        return self.images[idx], self.pts[idx], self.filters[idx], idx


def _latent_dataset(g, dev):
    return _Latent(torch.tensor(g["images"], dtype=torch.float32, device=dev),
                   torch.tensor(g["pts"], dtype=torch.float32, device=dev),
                   torch.tensor(g["filters"], dtype=torch.float32, device=dev), float(g["noise_var"]))


def test_latent_map_dataset_matches_reference(pkg, dev):
    """latentMAP over 40 images in batches of 16 (16, 16, 8): with the discretized bilinear plan
    against the reference's discretized run, and with the exact (ES) NufftPlan against the
    reference run on the exact NUDFT; coordinates and the per-image m."""
    g = load_golden("latent_dataset_L10_r3.npz")
    ds = _latent_dataset(g, dev)
    eig = torch.tensor(g["eigenvecs"], dtype=torch.float32, device=dev)
    lam = torch.tensor(g["eigenvals"], dtype=torch.float32, device=dev)
    bs = int(g["batch"])
    c, cov = pkg.wiener_coords.latentMAP(ds, eig, lam, batch_size=bs, return_coords_covar=True,
                                         nufft_plan=pkg.NufftPlanDiscretized)
    assert rel(c, g["map_bilinear"]) < 1e-5 and rel(cov, g["map_bilinear_covar"]) < 1e-5
    c, cov = pkg.wiener_coords.latentMAP(ds, eig, lam, batch_size=bs, return_coords_covar=True, width=8)
    assert rel(c, g["map_exact"]) < 1e-4 and rel(cov, g["map_exact_covar"]) < 1e-4


def test_wiener_coords_match_reference(pkg, dev):
    """wiener_coords (the reference's per-image QR form, run on the exact NUDFT) against the
    Gram + FP64 Cholesky formulation on the ES plan, also with a singular eigenvalue matrix."""
    g = load_golden("latent_dataset_L10_r3.npz")
    ds = _latent_dataset(g, dev)
    eig = torch.tensor(g["eigenvecs"], dtype=torch.float32, device=dev)
    lam = torch.tensor(g["eigenvals"], dtype=torch.float32, device=dev)
    c = pkg.wiener_coords.wiener_coords(ds, eig, lam, batch_size=int(g["batch"]), width=8)
    assert rel(c, g["wiener_exact"]) < 1e-4
    # a zero eigenvalue: the reference's formula gives a zero coordinate there, as does ours
    lam0 = lam.clone()
    lam0[-1] = 0
    c0 = pkg.wiener_coords.wiener_coords(ds, eig, lam0, batch_size=int(g["batch"]), width=8)
    assert torch.all(c0[:, -1] == 0)
    # against the oracle restatement of the QR form with the same projections
    plan = pkg.NufftPlan((10,) * 3, batch_size=3, device=dev, width=8)
    plan.setpts(ds.pts)
    A = pkg.vol_forward(eig, plan, ds.filters).reshape(len(ds), 3, -1).double().cpu().numpy()
    y = ds.images.reshape(len(ds), -1).double().cpu().numpy()
    L0 = np.diag(lam0.double().cpu().numpy())
    ref = []
    for j in range(len(ds)):
        q, rr = np.linalg.qr(A[j].T)
        cov = rr @ L0 @ rr.T + ds.noise_var * np.eye(3)
        ref.append(L0 @ rr.T @ np.linalg.inv(cov) @ (y[j] @ q))
    assert rel(c0, np.array(ref)) < 1e-5


_RAGGED = {}


def _ragged_case():
    """5000 images at L = 32, r = 10 and their float64 latent-MAP coordinates (cached)."""
    if _RAGGED:
        return _RAGGED
    from oracle import cpu_step

    L, r, N = 32, 10, 5000
    rng = np.random.default_rng(5)
    eig = rng.standard_normal((r, L**3))
    eig = np.linalg.qr(eig.T)[0].T.reshape(r, L, L, L)
    lam = np.linspace(3.0, 0.5, r)
    R = O.rotvec_to_rotmat(rng.standard_normal((N, 3)))
    pts = O.rotated_points(R, L).astype(np.float32)
    ctf = rng.uniform(0.3, 1.2, (N, L, L))
    noise_var = 0.02
    # images from the oracle's own float64 ES projections of random latent coordinates
    n = 2 * L
    beta = O.es_beta(7, 2)
    gc = O.grid_correction_es(L, n, 7, beta)
    grid = np.stack([O.centered_fft3(e / gc, pad_to=n) for e in eig])
    t = O.es_index(pts.astype(np.float64), n)
    samp = cpu_step.c_interp(np.ascontiguousarray(np.moveaxis(grid, 0, -1)), t, 7, beta)  # (N*P, r)
    Q = O.vol_forward_fourier(samp.T.reshape(r, N, L * L), ctf, L).reshape(N, r, L, L)
    Qs = np.real(O.centered_ifft2(Q)).reshape(N, r, -1)
    z = rng.standard_normal((N, r)) * np.sqrt(lam)
    y = np.einsum("nr,nrp->np", z, Qs) + rng.standard_normal((N, L * L)) * np.sqrt(noise_var)
    linv = np.linalg.inv(np.diag(lam) + 1e-6 * np.eye(r))
    zr, _, _ = O.latent_map_batch(y, Qs, noise_var, linv)
    _RAGGED.update(L=L, r=r, N=N, eig=eig, lam=lam, pts=pts, ctf=ctf, y=y, noise_var=noise_var, z=zr[..., 0].real)
    return _RAGGED


@pytest.mark.parametrize("batch", [256, 1000, 4096])
def test_latent_map_ragged_batches(pkg, dev, batch):
    """Config-5-style ragged batches: 5000 images at L = 32, r = 10 in batches of 256, 1000 and
    4096 (last batches 136, 1000, 904) give the coordinates of the float64 oracle (ES
    projections by the C oracle, latent_map_batch) to 1e-4."""
    d = _ragged_case()
    L, r, N, y, pts, ctf, eig, lam, noise_var = (d[k] for k in ("L", "r", "N", "y", "pts", "ctf", "eig", "lam",
                                                                  "noise_var"))
    ds = _Latent(torch.tensor(y.reshape(N, L, L), dtype=torch.float32, device=dev),
                 torch.tensor(pts, device=dev), torch.tensor(ctf, dtype=torch.float32, device=dev), noise_var)
    c = pkg.wiener_coords.latentMAP(ds, torch.tensor(eig, dtype=torch.float32, device=dev),
                                    torch.tensor(lam, dtype=torch.float32, device=dev), batch_size=batch, width=7)
    assert c.shape == (N, r)
    assert rel(c, d["z"]) < 1e-4


def test_fine_grid_reuse_equals_vol_forward(pkg, dev):
    """The eigenvolumes transformed once (cov3d_fine_grid) and interpolated per batch give the
    projections vol_forward gives with the full type 2 per batch, in both domains, over two
    batches of different poses and sizes."""
    L, r = 24, 6
    g = torch.Generator(device=dev).manual_seed(21)
    vols = torch.randn((r, L, L, L), device=dev, generator=g)
    plan = pkg.NufftPlan((L,) * 3, batch_size=r, device=dev)
    project = pkg.wiener_coords._EigenProjector(plan, vols)
    for n in (7, 13):
        R = torch.linalg.qr(torch.randn((n, 3, 3), device=dev, generator=g))[0].contiguous()
        ctf = torch.rand((n, L, L), device=dev, generator=g) + 0.2
        plan.setrot(R)
        for fourier in (True, False):
            want = pkg.vol_forward(vols, plan, ctf, fourier_domain=fourier)
            got = project(ctf, fourier_domain=fourier)
            assert got.shape == want.shape
            assert rel(got, want) < 1e-6


@pytest.mark.parametrize("masked,fourier", [(False, False), (True, False), (True, True)])
def test_preprocess_image_batch_matches_reference(pkg, dev, masked, fourier):
    g = load_golden("preprocess_L10.npz")
    L, us = int(g["L"]), int(g["us"])
    n = L * us
    plan = pkg.NufftPlanDiscretized((L,) * 3, upsample_factor=us, mode="bilinear")
    mean_f = pkg.centered_fft3(torch.tensor(g["mean_vol"], device=dev).unsqueeze(0), padding_size=(n,) * 3)
    mask_f = pkg.centered_fft3(torch.tensor(g["mask_vol"], device=dev).unsqueeze(0), padding_size=(n,) * 3)
    pts = torch.tensor(g["pts"], dtype=torch.float32, device=dev)
    phase = torch.tensor(g["phase"], device=dev).to(torch.complex64)
    ims = torch.tensor(g["images"], device=dev)
    filt = torch.tensor(g["filters"], device=dev)
    plan.setpts(pts)
    thr = pkg.get_mask_threshold(mask_f, plan)
    assert abs(thr - float(g["mask_threshold"])) <= 1e-5 * abs(float(g["mask_threshold"]))
    thr = float(g["mask_threshold"])  # the same threshold on both sides of the comparison below
    soft = pkg.utils.soft_edged_kernel(radius=5, L=L, dim=2, in_fourier=True).to(dev)
    if not masked:
        out = pkg.preprocess_image_batch(ims, plan, filt, (pts, phase), mean_f)
        assert rel(out, g["nomask"]) < 1e-5
    else:
        out = pkg.preprocess_image_batch(ims, plan, filt, (pts, phase), mean_f, mask_f, thr, soft,
                                         fourier_domain=fourier)
        assert rel(out, g["masked_fourier" if fourier else "masked"]) < 1e-5


def test_train_covar_halfsets_on_resident_dataset(pkg, dev):
    """trainCovar's half-set schedule on a device-resident dataset (rotations, no point
    arrays): both half-set trainers run, the regulariser is updated from their covariance FSC,
    and the full-data run lowers the epoch cost."""
    syn = pkg.synthetic
    gen = torch.Generator(device=dev).manual_seed(3)
    torch.manual_seed(3)  # the Covar's random initial eigenvolumes and the batch order
    L, r, N = 16, 2, 512
    eig = syn.gaussian_blob_volumes(r, L, blobs=10, generator=gen, device=dev)
    rot = syn.uniform_rotations(N, generator=gen, device=dev)
    ctf = syn.ctf_images(torch.rand((N,), generator=gen, device=dev) + 1.0, L, 3.0, device=dev)
    plan = pkg.NufftPlan((L,) * 3, batch_size=r, device=dev)
    plan.setrot(rot)
    proj = pkg.vol_forward(eig, plan, ctf)
    z = torch.randn((N, r, 1, 1), generator=gen, device=dev) * 3
    images = (proj * z).sum(1)
    noise_var = float(images.var()) * 0.5
    images = images + torch.randn(images.shape, generator=gen, device=dev) * noise_var**0.5
    ds = pkg.ResidentDataset(images, rot, ctf, noise_var)
    covar = pkg.Covar(L, r, pixel_var_estimate=float(images.var()) / L**2, fourier_domain=True).to(dev)
    tr = pkg.trainCovar(covar, ds, batch_size=128, max_epochs=3, lr=1e-5, nufft_disc="bilinear",
                        use_halfsets=True, num_reg_update_iters=1)
    assert tr.fourier_reg is not None and torch.isfinite(tr.fourier_reg).all()
    assert "covariance_fsc_halfset" in tr.training_log
    costs = tr.training_log["cost_val"]
    assert len(costs) == 6 and np.isfinite(costs).all()  # 3 half-set epochs, then 3 on all the data
    assert costs[5] < costs[3]
    assert ds._in_spatial_domain  # complete_training switched the data back


def test_recorded_data_has_the_reference_fields(pkg, dev):
    """recorded_data (workflow.py:477-518) for a Covar on the latent fixture's dataset: the
    reference's keys, and coordinates equal to latentMAP's for the same eigenvectors."""
    g = load_golden("latent_dataset_L10_r3.npz")
    ds = _latent_dataset(g, dev)
    cov = pkg.Covar(10, 3, vectors=torch.tensor(g["eigenvecs"] * np.sqrt(g["eigenvals"])[:, None, None, None],
                                                 dtype=torch.float32)).to(dev)
    gt = torch.tensor(g["eigenvecs"] * np.sqrt(g["eigenvals"])[:, None, None, None], dtype=torch.float32, device=dev)
    rec = pkg.results.recorded_data(cov, ds, gt_eigenvecs=gt, batch_size=16)
    keys = {"eigen_est", "eigenval_est", "coords_est", "coords_covar_inv_est", "mean_est", "particles_path", "ctf_path",
            "poses_path", "ind", "data_sign_inverted", "lazy", "eigenvals_GT", "eigenvectors_GT", "coords_GT",
            "coords_covar_inv_GT"}
    assert set(rec) == keys
    e, lam = cov.eigenvecs
    c = pkg.wiener_coords.latentMAP(ds, e, lam, batch_size=16)
    assert rel(rec["coords_est"], c) < 1e-6
    assert rec["coords_covar_inv_est"].shape == (len(ds), 3, 3)
    assert rel(np.sort(rec["eigenvals_GT"]), np.sort(g["eigenvals"])) < 1e-5
