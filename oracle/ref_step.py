"""The reference's own covariance-SGD step on the host cores (test infrastructure: the timed
CPU baseline of ``bench.py`` and of ``bench.py --impl reference``).

Runs the unmodified reference package copied by ``oracle/build_ref.py`` to
``oracle/_ref/cov3d``, imported through ``oracle/ref_shim.py``: ``CovarTrainer.run_batch``
(``covar_sgd.py:199-229``) with the trainer set up as ``CovarTrainer.setup_training``
(``covar_sgd.py:302-358``) does for the command-line defaults (``workflow.py:374-385``:
``nufft_disc="bilinear"``, ``objective_func="ml"``, Adam, lr 1e-6 x batch, reg 1), i.e. per
step ``NufftPlanDiscretized.setpts`` + ``Covar`` Fourier view + ``grid_sample`` projection +
``cost_maximum_liklihood_fourier_domain`` + autograd backward + Adam.  torch runs on the CPU
with every host core.

The synthetic batch has the shapes and value distributions of the GPU workload (Gaussian-blob
eigenvolumes, uniform SO(3) poses, weak-phase CTFs, SNR 0.05), generated here with numpy and
projected by the reference's own plan.
"""

import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.path.join(HERE, "_ref")


def available():
    return os.path.exists(os.path.join(REF_ROOT, "cov3d", "covar_sgd.py"))


def load_reference():
    """Import the copied reference package (raises ImportError when it is not installed)."""
    if not available():
        raise ImportError("reference package not installed under oracle/_ref (run oracle/build_ref.py)")
    if HERE not in sys.path:
        sys.path.insert(0, os.path.dirname(HERE))
    from oracle import ref_shim

    ref_shim.install(REF_ROOT)
    import importlib

    mods = {}
    for name in ("covar_sgd", "covar", "nufft_plan", "projection_funcs", "poses"):
        mods[name] = importlib.import_module("cov3d." + name)
    return mods


# ----------------------------------------------------------------------------- synthetic data


def blob_volumes(rng, count, L, blobs=50, radius=0.35, width=(1.0, 3.0), amp=(0.5, 1.0)):
    """(count, L, L, L) sums of isotropic Gaussians (centres uniform in a ball of radius
    radius*L), each evaluated on the voxels within 6 widths of its centre."""
    out = np.zeros((count, L, L, L))
    for c in range(count):
        d = rng.standard_normal((blobs, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        cen = d * (rng.uniform(size=(blobs, 1)) ** (1.0 / 3.0) * radius * L) + L // 2
        sig = rng.uniform(width[0], width[1], blobs)
        a = rng.uniform(amp[0], amp[1], blobs)
        for k in range(blobs):
            lo = np.maximum(np.floor(cen[k] - 6 * sig[k]).astype(int), 0)
            hi = np.minimum(np.ceil(cen[k] + 6 * sig[k]).astype(int) + 1, L)
            z, y, x = np.meshgrid(*[np.arange(lo[i], hi[i]) for i in range(3)], indexing="ij")
            r2 = (z - cen[k, 0]) ** 2 + (y - cen[k, 1]) ** 2 + (x - cen[k, 2]) ** 2
            out[c, lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += a[k] * np.exp(-r2 / (2 * sig[k] ** 2))
    return out


def uniform_rotvecs(rng, n):
    """Rotation vectors of uniform SO(3) rotations (normalised Gaussian quaternions)."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    angle = 2 * np.arccos(np.clip(q[:, 0], -1, 1))
    axis = q[:, 1:] / np.maximum(np.linalg.norm(q[:, 1:], axis=1, keepdims=True), 1e-12)
    return axis * angle[:, None]


def weak_phase_ctf(defocus_um, L, pixel_size, voltage_kv=300.0, cs_mm=2.7, amplitude_contrast=0.1):
    v = voltage_kv * 1e3
    lam = 12.2643247 / math.sqrt(v * (1 + 0.978466e-6 * v))
    f = (np.arange(L) - L // 2) / (L * pixel_size)
    ky, kx = np.meshgrid(f, f, indexing="ij")
    k2 = kx * kx + ky * ky
    df = np.asarray(defocus_um).reshape(-1, 1, 1) * 1e4
    chi = math.pi * lam * df * k2 - 0.5 * math.pi * cs_mm * 1e7 * lam**3 * k2 * k2
    A = amplitude_contrast
    return -(math.sqrt(1 - A * A) * np.sin(chi) + A * np.cos(chi))


class _Batches:
    """What CovarTrainer reads from its data: a dataset with ``mask``, ``noise_var`` and the
    domain switches (the images are generated in the Fourier domain already)."""

    def __init__(self, n, noise_var):
        self.n = n
        self.mask = None
        self.noise_var = noise_var

    def __len__(self):
        return self.n

    def __getitem__(self, i):
        return i

    def to_fourier_domain(self):
        pass

    def to_spatial_domain(self):
        pass


class RefCovarStep:
    """The reference trainer with ``nb`` resident batches of ``batch`` synthetic images."""

    def __init__(self, L=128, rank=10, batch=32, nb=2, seed=2000, threads=None, snr=0.05, pixel=1.5,
                 dataset_size=100000):
        import torch

        self.torch = torch
        self.threads = threads or os.cpu_count()
        torch.set_num_threads(self.threads)
        mods = load_reference()
        self.mods = mods
        rng = np.random.default_rng(seed)
        self.L, self.rank, self.batch, self.nb = L, rank, batch, nb
        eig = blob_volumes(rng, rank, L).reshape(rank, -1)
        eig, _ = np.linalg.qr(eig.T)
        eig = eig.T.reshape(rank, L, L, L)
        sqrt_lam = np.linspace(1.0, 0.3, rank) * L**1.5
        n_img = batch * nb
        rotvecs = uniform_rotvecs(rng, n_img)
        shifts = np.zeros((n_img, 2))
        PoseModule = mods["poses"].PoseModule
        pose = PoseModule(torch.tensor(rotvecs, dtype=torch.float32), torch.tensor(shifts, dtype=torch.float32), L)
        with torch.no_grad():
            pts, _ = pose(torch.arange(n_img))
        self.pts = pts.detach().to(torch.float32).contiguous()
        ctf = weak_phase_ctf(rng.uniform(1.0, 3.0, n_img), L, pixel)
        self.ctf = torch.tensor(ctf, dtype=torch.float32)
        # clean images: the reference's own projection of the eigenvolumes, weighted by
        # N(0, lambda) latent coordinates, plus white noise at the given SNR
        plan = mods["nufft_plan"].NufftPlanDiscretized((L,) * 3, upsample_factor=2, mode="bilinear")
        vols = mods["projection_funcs"].centered_fft3(torch.tensor(eig, dtype=torch.float32),
                                                      padding_size=(2 * L,) * 3)
        images = torch.empty((n_img, L, L), dtype=torch.complex64)
        with torch.no_grad():
            for i in range(0, n_img, batch):
                plan.setpts(self.pts[i:i + batch])
                proj = mods["projection_funcs"].vol_forward(vols, plan, self.ctf[i:i + batch], fourier_domain=True)
                if proj.ndim == 3:
                    proj = proj.unsqueeze(0)
                z = torch.tensor(rng.standard_normal((proj.shape[0], rank, 1, 1)) * sqrt_lam.reshape(1, rank, 1, 1),
                                 dtype=torch.float32)
                images[i:i + proj.shape[0]] = (proj * z).sum(1)
        noise_var = float((images.abs() ** 2).mean()) / snr
        noise = (rng.standard_normal(images.shape) + 1j * rng.standard_normal(images.shape)) * math.sqrt(noise_var / 2)
        self.images = images + torch.tensor(noise, dtype=torch.complex64)
        self.noise_var = noise_var
        # the trainer, set up like the command line's defaults
        covar = mods["covar"].Covar(L, rank, pixel_var_estimate=float(self.images.real.var()) / L**2,
                                    fourier_domain=True, upsampling_factor=2)
        loader = torch.utils.data.DataLoader(_Batches(n_img, noise_var), batch_size=batch)
        trainer = mods["covar_sgd"].CovarTrainer(covar, loader, torch.device("cpu"))
        trainer.setup_training(lr=1e-6, optim_type="Adam", reg=1, nufft_disc="bilinear", objective_func="ml")
        trainer.reg_scale = 1.0 / dataset_size
        # the Fourier regulariser the trainer installs before its first epoch
        # (compute_fourier_reg_term, covar_sgd.py:420-430) from an eigenvector estimate
        trainer.compute_fourier_reg_term(torch.tensor(eig * sqrt_lam.reshape(-1, 1, 1, 1), dtype=torch.float32))
        self.trainer = trainer

    def step(self, k):
        """One reference ``run_batch`` on resident batch k mod nb; returns the cost."""
        b = k % self.nb
        s = slice(b * self.batch, (b + 1) * self.batch)
        cost = self.trainer.run_batch(self.images[s], self.pts[s], self.ctf[s])
        return float(cost.detach())


def time_steps(L=128, rank=10, batch=1024, steps=20, warmup=3, seed=2000, threads=None, budget_s=150.0):
    """Images/s of whole reference steps of ``batch`` images.  Runs min(warmup, 1) untimed
    steps, then as many of the ``steps`` requested as fit in ``budget_s`` seconds at the
    warm-up step's pace (at least one).  Returns (images_per_s, detail dict with the steps
    actually run)."""
    t0 = time.perf_counter()
    st = RefCovarStep(L, rank, batch, nb=2, seed=seed, threads=threads)
    setup_s = time.perf_counter() - t0
    w = min(max(warmup, 0), 1)
    t_w = None
    for k in range(w):
        t1 = time.perf_counter()
        st.step(k)
        t_w = time.perf_counter() - t1
    n = steps if t_w is None else max(1, min(steps, int(budget_s // max(t_w, 1e-9))))
    costs = []
    t1 = time.perf_counter()
    for k in range(n):
        costs.append(st.step(w + k))
    sec = time.perf_counter() - t1
    return batch * n / sec, {"seconds": sec, "steps": n, "warmup": w, "batch": batch, "threads": st.threads,
                             "setup_s": setup_s, "warmup_step_s": t_w, "final_cost": costs[-1]}
