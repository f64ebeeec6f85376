"""Generate the golden fixtures under ``tests/golden/`` by running the reference COV3D code
(pure PyTorch, CPU, float64) on small seeded inputs.

Run where the reference source tree is available (it is not needed by the tests):

    python tests/golden/make_golden.py /path/to/reference [case_function]

The reference is imported unmodified through ``oracle/ref_shim.py`` (placeholder modules for
its unused third-party dependencies).  Every fixture stores its inputs next to the reference's
outputs, so the tests never need the reference itself.

Cases (reference file:line of the function that produced each output):

* ``poses.npz``          rotvec_to_rotmat (poses.py:44-67), PoseModule.forward
                         (poses.py:237-269), offset_to_phase_shift (poses.py:92-125)
* ``disc_*.npz``         NufftPlanDiscretized.setpts/execute_forward/execute_adjoint/
                         execute_adjoint_unaggregated (nufft_plan.py:94-242), vol_forward /
                         im_backward (projection_funcs.py:321-399)
* ``cost_*.npz``         cost_maximum_liklihood_fourier_domain and cost_fourier_domain
                         (covar_sgd.py:1290-1399) through Covar.get_vectors_fourier_domain
                         (covar.py:440-446) with autograd gradients
* ``latent_*.npz``       compute_latentMAP_batch (wiener_coords.py:168-203)
* ``cg_*.npz``           regularize_lhs + correct_upsampling_padding +
                         complex_conjugate_gradient (mean.py:43-142)
* ``mean_*.npz``         reconstruct_mean (mean.py:145-259), whole pipeline
* ``halfsets_*.npz``     fsc_utils (average_fourier_shell, rpsd, expand_fourier_shell,
                         upsample_and_expand_fourier_shell, vol_fsc, covar_rpsd, covar_fsc;
                         fsc_utils.py:116-367), CovarTrainer.compute_fourier_reg_term /
                         update_fourier_reg_halfsets (covar_sgd.py:420-447),
                         compute_updated_fourier_reg (covar_sgd.py:1155-1187),
                         regularize_mean_from_halfsets (mean.py:359-421), CovarDataset
                         get_total_gain / get_total_covar_gain (dataset.py:322-421)
"""

import io
import logging
import os
import re
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
if len(sys.argv) < 2:
    sys.exit("usage: make_golden.py /path/to/reference [case_function]")
REF = sys.argv[1]

sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import ref_shim  # noqa: E402

ref_shim.install(REF)

from cov3d import covar_sgd, mean, nufft_plan, poses, projection_funcs, wiener_coords  # noqa: E402
from cov3d.covar import Covar  # noqa: E402

torch.set_default_dtype(torch.float64)


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
    print(f"wrote {name}: {os.path.getsize(path) / 1024:.1f} KiB")


def random_rotvecs(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    angle = 2 * np.arccos(np.clip(q[:, 0], -1, 1))
    axis = q[:, 1:] / np.maximum(np.linalg.norm(q[:, 1:], axis=1, keepdims=True), 1e-12)
    return (axis * angle[:, None]).astype(np.float32)


def c32(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def ref_points(rotvecs, offsets, L):
    pose = poses.PoseModule(torch.tensor(rotvecs, dtype=torch.float64), torch.tensor(offsets, dtype=torch.float64), L,
                            dtype=torch.float64)
    with torch.no_grad():
        pts, phase = pose(torch.arange(len(rotvecs)))
    return pts, phase


def case_poses():
    rng = np.random.default_rng(11)
    out = {}
    for L in (12, 15):
        n = 7
        rotvecs = random_rotvecs(rng, n)
        offsets = (rng.uniform(-3, 3, (n, 2))).astype(np.float32)
        rotmat = poses.rotvec_to_rotmat(torch.tensor(rotvecs, dtype=torch.float64))
        pts, phase = ref_points(rotvecs, offsets, L)
        out.update({f"L{L}_rotvecs": rotvecs, f"L{L}_offsets": offsets, f"L{L}_rotmat": rotmat.numpy(),
                    f"L{L}_pts": pts.numpy(), f"L{L}_phase": phase.numpy()})
    save("poses.npz", **out)


def case_disc(L, us, mode, n_img, chans, seed, unaggregated=False):
    rng = np.random.default_rng(seed)
    n = L * us
    rotvecs = random_rotvecs(rng, n_img)
    pts, _ = ref_points(rotvecs, np.zeros((n_img, 2), np.float32), L)
    vol = c32(rng, (chans, n, n, n))
    sig = c32(rng, (n_img, L, L))
    filters = rng.uniform(0.2, 1.5, (n_img, L, L)).astype(np.float32)

    plan = nufft_plan.NufftPlanDiscretized((L,) * 3, upsample_factor=us, mode=mode)
    plan.setpts(pts)
    vol_t = torch.tensor(vol).to(torch.complex128)
    sig_t = torch.tensor(sig).to(torch.complex128)
    filt_t = torch.tensor(filters, dtype=torch.float64)
    fwd = plan.execute_forward(vol_t)
    adj = plan.execute_adjoint(sig_t)
    vf = projection_funcs.vol_forward(vol_t, plan, filt_t, fourier_domain=True)
    ib = projection_funcs.im_backward(sig_t, plan, filt_t, fourier_domain=True)
    arrays = dict(L=L, us=us, pts=pts.numpy(), rotvecs=rotvecs, vol=vol, sig=sig, filters=filters,
                  fwd=fwd.numpy(), adj=adj.numpy(), vol_forward=vf.numpy(), im_backward=ib.numpy())
    if unaggregated:
        arrays["adj_unagg"] = plan.execute_adjoint_unaggregated(sig_t).numpy()
    save(f"disc_{mode}_L{L}_us{us}.npz", **arrays)


def case_cost(L=10, r=3, B=6, us=2, seed=5):
    rng = np.random.default_rng(seed)
    n = L * us
    vectors = rng.standard_normal((r, L, L, L)).astype(np.float32) * 0.1
    rotvecs = random_rotvecs(rng, B)
    pts, _ = ref_points(rotvecs, np.zeros((B, 2), np.float32), L)
    images = c32(rng, (B, L, L)) * np.float32(3.0)
    filters = rng.uniform(0.2, 1.5, (B, L, L)).astype(np.float32)
    fourier_reg = rng.uniform(0.5, 2.0, (n, n, n)).astype(np.float32)
    noise_var = 7.5
    reg_scale = 0.3

    out = dict(L=L, r=r, us=us, vectors=vectors, rotvecs=rotvecs, pts=pts.numpy(), images=images, filters=filters,
               fourier_reg=fourier_reg, noise_var=noise_var, reg_scale=reg_scale)
    plan = nufft_plan.NufftPlanDiscretized((L,) * 3, upsample_factor=us, mode="bilinear")
    plan.setpts(pts)
    ims = torch.tensor(images).to(torch.complex128)
    filt = torch.tensor(filters, dtype=torch.float64)
    freg = torch.tensor(fourier_reg, dtype=torch.float64)
    for name, fn in (("ml", covar_sgd.cost_maximum_liklihood_fourier_domain), ("ls", covar_sgd.cost_fourier_domain)):
        for with_reg in (False, True):
            covar = Covar(L, r, dtype=torch.float64, upsampling_factor=us, vectors=torch.tensor(vectors, dtype=torch.float64))
            covar.init_grid_correction("bilinear")
            vols = covar.get_vectors_fourier_domain()
            kw = dict(reg_scale=reg_scale, fourier_reg=freg) if with_reg else {}
            cost = fn(vols, ims, plan, filt, noise_var, **kw)
            cost.backward()
            tag = f"{name}{'_reg' if with_reg else ''}"
            out[f"{tag}_cost"] = cost.detach().numpy()
            out[f"{tag}_grad_vectors"] = covar.vectors.grad.numpy()
            out[f"{tag}_grad_logsqrt"] = covar.log_sqrt_eigenvals.grad.numpy()
            # per-image (unaggregated) data term
            covar.zero_grad()
            vols = covar.get_vectors_fourier_domain()
            per_img = fn(vols, ims, plan, filt, noise_var, mean_aggregate=False)
            out[f"{tag}_per_image"] = per_img.detach().numpy()
    out["log_sqrt_eigenvals"] = covar.log_sqrt_eigenvals.detach().numpy()
    out["vectors_normalised"] = covar.vectors.detach().numpy()
    out["grid_correction"] = covar.grid_correction.numpy()
    save(f"cost_L{L}_r{r}.npz", **out)


def case_latent(L=10, r=3, B=9, seed=9):
    rng = np.random.default_rng(seed)
    images = c32(rng, (B, L, L))
    eig = c32(rng, (B, r, L, L)) * np.float32(0.5)
    lam = np.diag(rng.uniform(0.5, 3.0, r))
    lam_inv = np.linalg.inv(lam + 1e-6 * np.eye(r))
    noise_var = 2.5
    z, m, b = wiener_coords.compute_latentMAP_batch(
        torch.tensor(images).to(torch.complex128), torch.tensor(eig).to(torch.complex128), noise_var,
        torch.tensor(lam_inv).to(torch.complex128))
    zr, mr, br = wiener_coords.compute_latentMAP_batch(
        torch.tensor(images.real.astype(np.float64)), torch.tensor(eig.real.astype(np.float64)), noise_var,
        torch.tensor(lam_inv))
    z0, m0, b0 = wiener_coords.compute_latentMAP_batch(
        torch.tensor(images).to(torch.complex128), torch.tensor(eig).to(torch.complex128), noise_var)
    save(f"latent_L{L}_r{r}.npz", images=images, eigen_forward=eig, eigenvals=np.diag(lam), eigenvals_inv=lam_inv,
         noise_var=noise_var, z=z.numpy(), m=m.numpy(), b=b.numpy(), z_real=zr.numpy(), m_real=mr.numpy(),
         b_real=br.numpy(), z_identity=z0.numpy(), m_identity=m0.numpy(), b_identity=b0.numpy())


class _CGCounter(logging.Handler):
    def __init__(self):
        super().__init__()
        self.iters = []

    def emit(self, record):
        m = re.search(r"CG converged in (\d+) iterations", record.getMessage())
        if m:
            self.iters.append(int(m.group(1)))


def case_cg(L=8, us=2, seed=3):
    rng = np.random.default_rng(seed)
    n = L * us
    lhs = (rng.uniform(0.0, 4.0, (n, n, n)) ** 2).astype(np.float32)
    lhs[rng.uniform(size=lhs.shape) < 0.05] = 0.0  # unobserved frequencies, exercised by regularize_lhs's floor
    rhs = c32(rng, (n, n, n))
    lhs_t = torch.tensor(lhs).to(torch.complex128)
    rhs_t = torch.tensor(rhs).to(torch.complex128)
    reg_lhs = mean.regularize_lhs(lhs_t)
    init = projection_funcs.centered_ifft3(rhs_t / reg_lhs, cropping_size=(L,) * 3).real
    handler = _CGCounter()
    mean.logger.addHandler(handler)
    mean.logger.setLevel(logging.DEBUG)
    x = mean.correct_upsampling_padding(reg_lhs, rhs_t, init, L, us)
    mean.logger.removeHandler(handler)
    b = projection_funcs.centered_ifft3(rhs_t, cropping_size=(L,) * 3)
    save(f"cg_L{L}.npz", L=L, us=us, lhs=lhs, rhs=rhs, reg_lhs=reg_lhs.numpy(), init=init.numpy(), x=x.numpy(),
         b=b.numpy(), iters=np.array(handler.iters))


class _MeanDataset(torch.utils.data.Dataset):
    """Minimal stand-in for CovarDataset with the attributes reconstruct_mean reads."""

    def __init__(self, images, pts, filters, offsets, contrasts, L):
        self.images = images
        self.pts_rot = pts
        self.filters = filters
        self.offsets = offsets
        self.contrasts = contrasts
        self.resolution = L
        self._in_spatial_domain = False
        self.dtype = images.real.dtype
        self.noise_var = 1.0

    def __len__(self):
        return len(self.images)

    def __getitem__(self, idx):
        return self.images[idx], self.pts_rot[idx], self.filters[idx], idx

    def to_fourier_domain(self):
        pass

    def to_spatial_domain(self):
        pass


def case_mean(L=10, us=2, N=96, seed=21):
    rng = np.random.default_rng(seed)
    rotvecs = random_rotvecs(rng, N)
    offsets = rng.uniform(-2, 2, (N, 2)).astype(np.float32)
    contrasts = rng.uniform(0.7, 1.3, N).astype(np.float32)
    pts, _ = ref_points(rotvecs, np.zeros((N, 2), np.float32), L)
    images = c32(rng, (N, L, L))
    filters = rng.uniform(0.2, 1.5, (N, L, L)).astype(np.float32)
    ds = _MeanDataset(torch.tensor(images).to(torch.complex128), pts, torch.tensor(filters, dtype=torch.float64),
                      torch.tensor(offsets, dtype=torch.float64), torch.tensor(contrasts, dtype=torch.float64), L)
    loader = torch.utils.data.DataLoader(ds, batch_size=32, shuffle=False)
    handler = _CGCounter()
    mean.logger.addHandler(handler)
    mean.logger.setLevel(logging.DEBUG)
    vol, rhs, lhs = mean.reconstruct_mean(loader, upsampling_factor=us, return_lhs_rhs=True)
    mean.logger.removeHandler(handler)
    save(f"mean_L{L}.npz", L=L, us=us, rotvecs=rotvecs, offsets=offsets, contrasts=contrasts, pts=pts.numpy(),
         images=images, filters=filters, volume=vol.numpy(), rhs=rhs.numpy(), lhs=lhs.numpy(),
         iters=np.array(handler.iters))


def case_mean_initvol(L=10, us=2, N=96, seed=23):
    """reconstruct_mean with an initial volume (mean.py:220-233): the regulariser
    noise_var / (radial PSD of init_vol, upsampled) / L added to the kernel instead of
    regularize_lhs, then the same solve."""
    rng = np.random.default_rng(seed)
    rotvecs = random_rotvecs(rng, N)
    offsets = rng.uniform(-2, 2, (N, 2)).astype(np.float32)
    contrasts = rng.uniform(0.7, 1.3, N).astype(np.float32)
    pts, _ = ref_points(rotvecs, np.zeros((N, 2), np.float32), L)
    images = c32(rng, (N, L, L))
    filters = rng.uniform(0.2, 1.5, (N, L, L)).astype(np.float32)
    init_vol = rng.standard_normal((L, L, L)) * 0.5
    ds = _MeanDataset(torch.tensor(images).to(torch.complex128), pts, torch.tensor(filters, dtype=torch.float64),
                      torch.tensor(offsets, dtype=torch.float64), torch.tensor(contrasts, dtype=torch.float64), L)
    ds.noise_var = 2.0
    loader = torch.utils.data.DataLoader(ds, batch_size=32, shuffle=False)
    vol, rhs, lhs = mean.reconstruct_mean(loader, init_vol=torch.tensor(init_vol).unsqueeze(0), upsampling_factor=us,
                                          return_lhs_rhs=True)
    save(f"mean_initvol_L{L}.npz", L=L, us=us, rotvecs=rotvecs, offsets=offsets, contrasts=contrasts, pts=pts.numpy(),
         images=images, filters=filters, init_vol=init_vol, noise_var=2.0, volume=vol.numpy(), rhs=rhs.numpy(),
         lhs=lhs.numpy())


class _GainDataset:
    """Stand-in for CovarDataset with what get_total_gain / get_total_covar_gain read."""

    def __init__(self, pts, filters, L):
        self.pts_rot, self.filters, self.resolution, self.dtype = pts, filters, L, filters.dtype

    def __len__(self):
        return len(self.pts_rot)

    def __getitem__(self, idx):
        return None, self.pts_rot[idx], self.filters[idx].clone(), idx


def case_halfsets(L=10, r=3, seed=31):
    from types import SimpleNamespace

    from cov3d import dataset, fsc_utils

    rng = np.random.default_rng(seed)
    n = 2 * L
    e1 = rng.standard_normal((r, L, L, L))
    e2 = e1 + 0.3 * rng.standard_normal((r, L, L, L))
    v1 = rng.standard_normal((L, L, L))
    v2 = v1 + 0.5 * rng.standard_normal((L, L, L))
    spec = rng.uniform(0.5, 2.0, (L, L, L))
    shells = rng.uniform(0.5, 2.0, 9)
    t = torch.tensor
    out = dict(L=L, r=r, e1=e1, e2=e2, v1=v1, v2=v2, spec=spec, shells=shells)
    out["avg_shell"] = fsc_utils.average_fourier_shell(t(spec)).numpy()
    out["rpsd"] = fsc_utils.rpsd(*t(e1)).numpy()
    out["expand"] = fsc_utils.expand_fourier_shell(t(shells), L, 3).numpy()
    out["upexpand"] = fsc_utils.upsample_and_expand_fourier_shell(t(shells), n, 3).numpy()
    out["vol_fsc"] = fsc_utils.vol_fsc(t(v1), t(v2)).numpy()
    out["covar_rpsd"] = fsc_utils.covar_rpsd(t(e1)).numpy()
    out["covar_fsc"] = fsc_utils.covar_fsc(t(e1), t(e2)).numpy()
    # dataset gains from 40 images with poses
    N = 40
    rotvecs = random_rotvecs(rng, N)
    pts, _ = ref_points(rotvecs, np.zeros((N, 2), np.float32), L)
    filters = rng.uniform(0.2, 1.5, (N, L, L))
    ds = _GainDataset(pts, t(filters), L)
    out["gain_filters"], out["gain_pts"] = filters, pts.numpy()
    out["total_gain"] = dataset.CovarDataset.get_total_gain(ds, batch_size=16, device="cpu").numpy()
    covar_gain = dataset.CovarDataset.get_total_covar_gain(ds, batch_size=16, device="cpu")
    out["total_covar_gain"] = covar_gain.numpy()
    reg, cfsc = covar_sgd.compute_updated_fourier_reg(t(e1), t(e2), covar_gain, None, L, True)
    out["updated_reg"], out["updated_reg_fsc"] = reg.numpy(), cfsc.numpy()
    reg_s, _ = covar_sgd.compute_updated_fourier_reg(t(e1), t(e2), covar_gain, None, L, False)
    out["updated_reg_spatial"] = reg_s.numpy()
    fake = SimpleNamespace(covar=SimpleNamespace(upsampling_factor=2, resolution=L), noise_var=0.7,
                           device="cpu", optimize_in_fourier_domain=True)
    covar_sgd.CovarTrainer.compute_fourier_reg_term(fake, t(e1))
    out["fourier_reg_term"] = fake.fourier_reg.numpy()
    covar_sgd.CovarTrainer.update_fourier_reg_halfsets(fake, reg)
    out["fourier_reg_halfsets"] = fake.fourier_reg.numpy()
    # mean from half-sets (half-set backprojections of the mean_L10 case)
    g = np.load(os.path.join(HERE, "mean_L10.npz"))
    lhs = g["lhs"]
    rhs = g["rhs"]
    lhs1, lhs2 = 0.45 * lhs, 0.55 * lhs + 0.02 * np.abs(lhs).mean()
    rhs1, rhs2 = 0.5 * rhs, 0.5 * rhs + 0.05 * c32(rng, rhs.shape) * np.abs(rhs).mean()
    m1 = rng.standard_normal((L, L, L))
    m2 = m1 + 0.4 * rng.standard_normal((L, L, L))
    handler = _CGCounter()
    mean.logger.addHandler(handler)
    mean.logger.setLevel(logging.DEBUG)
    vol = mean.regularize_mean_from_halfsets(t(m1), t(rhs1), t(lhs1), t(m2), t(rhs2), t(lhs2))
    mean.logger.removeHandler(handler)
    out.update(m1=m1, m2=m2, lhs1=lhs1, lhs2=lhs2, rhs1=rhs1, rhs2=rhs2, mean_halfsets=vol.numpy(),
               mean_halfsets_iters=np.array(handler.iters))
    save(f"halfsets_L{L}.npz", **out)


class ExactNufftPlan(nufft_plan.NufftPlan):
    """Float64 stand-in for the reference's cuFINUFFT plan, used only to generate fixtures for
    the reference functions that construct or expect a ``NufftPlan`` (the spatial-domain costs,
    ``wiener_coords``, ``latentMAP`` with its default plan): the exact NUDFT
    ``F(w) = sum_k V[k] exp(-i w.k)``, ``k = j - L//2`` per axis, which cuFINUFFT approximates
    to ``eps`` (modes centered, point row d paired with volume axis d).  It keeps the reference
    plan's attributes, point wrapping and output shapes (``nufft_plan.py:318-392``); being a
    subclass, the reference's ``nufft_forward`` / ``nufft_adjoint`` wrap it in their autograd
    functions exactly as they wrap the real plan."""

    def __init__(self, sz, batch_size=1, eps=1e-6, dtype=torch.float64, device=torch.device("cpu"), **kwargs):
        self.sz, self.batch_size, self.device = sz, batch_size, device
        self.dtype, self.complex_dtype = torch.float64, torch.complex128

    def setpts(self, points):
        self.points_N = points.shape[0]
        self.points_L = int(round(points.shape[-1] ** 0.5))
        pts = points.transpose(0, 1).reshape((3, -1)).to(torch.float64)
        self.points = (torch.remainder(pts + torch.pi, 2 * torch.pi) - torch.pi).contiguous()
        L = self.sz[0]
        k = torch.arange(L, dtype=torch.float64) - L // 2
        k0, k1, k2 = torch.meshgrid(k, k, k, indexing="ij")
        ph = (self.points[0][:, None] * k0.reshape(1, -1) + self.points[1][:, None] * k1.reshape(1, -1)
              + self.points[2][:, None] * k2.reshape(1, -1))
        self._E = torch.exp(-1j * ph)

    def execute_forward(self, signal):
        B = signal.shape[0]
        out = signal.reshape(B, -1).to(torch.complex128) @ self._E.T
        return out.reshape(B, self.points_N, self.points_L, self.points_L)

    def execute_adjoint(self, signal):
        B = signal.shape[0]
        out = signal.reshape(B, -1).to(torch.complex128) @ self._E.conj()
        return out.reshape((B, *self.sz))


def case_spatial_costs(L=10, r=3, B=6, seed=41):
    """cost / cost_maximum_liklihood (covar_sgd.py:1190-1286): spatial eigenvolumes through an
    exact plan, spatial images, with and without the Fourier regulariser, autograd gradients."""
    rng = np.random.default_rng(seed)
    vectors = rng.standard_normal((r, L, L, L)).astype(np.float32) * 0.1
    rotvecs = random_rotvecs(rng, B)
    pts, _ = ref_points(rotvecs, np.zeros((B, 2), np.float32), L)
    images = (rng.standard_normal((B, L, L)) * 3).astype(np.float32)
    filters = rng.uniform(0.2, 1.5, (B, L, L)).astype(np.float32)
    fourier_reg = rng.uniform(0.5, 2.0, (L, L, L)).astype(np.float32)
    noise_var, reg_scale = 2.5, 0.3
    out = dict(L=L, r=r, vectors=vectors, rotvecs=rotvecs, pts=pts.numpy(), images=images, filters=filters,
               fourier_reg=fourier_reg, noise_var=noise_var, reg_scale=reg_scale)
    plan = ExactNufftPlan((L,) * 3, batch_size=r)
    plan.setpts(pts)
    ims = torch.tensor(images, dtype=torch.float64)
    filt = torch.tensor(filters, dtype=torch.float64)
    freg = torch.tensor(fourier_reg, dtype=torch.float64)
    for name, fn in (("ml", covar_sgd.cost_maximum_liklihood), ("ls", covar_sgd.cost)):
        for with_reg in (False, True):
            covar = Covar(L, r, dtype=torch.float64, vectors=torch.tensor(vectors, dtype=torch.float64))
            kw = dict(reg_scale=reg_scale, fourier_reg=freg) if with_reg else {}
            c = fn(covar.get_vectors_spatial_domain(), ims, plan, filt, noise_var, **kw)
            c.backward()
            tag = f"{name}{'_reg' if with_reg else ''}"
            out[f"{tag}_cost"] = c.detach().numpy()
            out[f"{tag}_grad_vectors"] = covar.vectors.grad.numpy()
            out[f"{tag}_grad_logsqrt"] = covar.log_sqrt_eigenvals.grad.numpy()
            per = fn(covar.get_vectors_spatial_domain(), ims, plan, filt, noise_var, mean_aggregate=False, **kw)
            out[f"{tag}_per_image"] = per.detach().numpy()
    out["log_sqrt_eigenvals"] = covar.log_sqrt_eigenvals.detach().numpy()
    out["vectors_normalised"] = covar.vectors.detach().numpy()
    save(f"spatial_cost_L{L}_r{r}.npz", **out)


class _TrainData(torch.utils.data.Dataset):
    """What CovarTrainer reads from its dataset (images, pts_rot, filters, idx; mask; noise_var)."""

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


def case_trainer(L=10, r=3, B=4, nbatch=2, seed=51):
    """Two CovarTrainer.run_batch steps (covar_sgd.py:199-229) after setup_training
    (covar_sgd.py:302-358; bilinear plan, ML objective, Adam) and compute_fourier_reg_term
    (covar_sgd.py:420-430): cost of each step and the parameters after each Adam update."""
    rng = np.random.default_rng(seed)
    N = B * nbatch
    vectors = rng.standard_normal((r, L, L, L)).astype(np.float32) * 0.1
    reg_vecs = rng.standard_normal((r, L, L, L)).astype(np.float32) * 0.1
    rotvecs = random_rotvecs(rng, N)
    pts, _ = ref_points(rotvecs, np.zeros((N, 2), np.float32), L)
    images = c32(rng, (N, L, L)) * np.float32(3.0)
    filters = rng.uniform(0.2, 1.5, (N, L, L)).astype(np.float32)
    noise_var, lr, reg = 7.5, 1e-3, 1.0
    ds = _TrainData(torch.tensor(images).to(torch.complex128), pts, torch.tensor(filters, dtype=torch.float64),
                    noise_var)
    loader = torch.utils.data.DataLoader(ds, batch_size=B, shuffle=False)
    covar = Covar(L, r, dtype=torch.float64, fourier_domain=True, vectors=torch.tensor(vectors, dtype=torch.float64))
    trainer = covar_sgd.CovarTrainer(covar, loader, torch.device("cpu"))
    trainer.setup_training(lr=lr, optim_type="Adam", reg=reg, nufft_disc="bilinear", objective_func="ml")
    trainer.compute_fourier_reg_term(torch.tensor(reg_vecs, dtype=torch.float64))
    out = dict(L=L, r=r, B=B, vectors=vectors, reg_vecs=reg_vecs, rotvecs=rotvecs, pts=pts.numpy(), images=images,
               filters=filters, noise_var=noise_var, lr=lr, reg=reg, reg_scale=trainer.reg_scale,
               fourier_reg=trainer.fourier_reg.numpy())
    costs = []
    for k, batch in enumerate(loader):
        im, p, f = trainer.prepare_batch(batch)
        costs.append(float(trainer.run_batch(im, p, f)))
        out[f"step{k}_vectors"] = covar.vectors.detach().numpy().copy()
        out[f"step{k}_log_sqrt"] = covar.log_sqrt_eigenvals.detach().numpy().copy()
    out["costs"] = np.array(costs)
    save(f"trainer_L{L}_r{r}.npz", **out)


class _LatentData:
    """What latentMAP / wiener_coords read from their dataset."""

    def __init__(self, images, pts, filters, noise_var):
        self.images, self.pts, self.filters, self.noise_var = images, pts, filters, noise_var

    def __len__(self):
        return len(self.images)

    def __getitem__(self, idx):
        return self.images[idx], self.pts[idx], self.filters[idx], idx


def case_latent_dataset(L=10, r=3, N=40, batch=16, seed=61):
    """latentMAP (wiener_coords.py:85-165) over a small dataset in ragged batches (16, 16, 8),
    with the discretized bilinear plan and with the exact plan; wiener_coords
    (wiener_coords.py:13-82, the per-image QR form) with the exact plan."""
    rng = np.random.default_rng(seed)
    rotvecs = random_rotvecs(rng, N)
    pts, _ = ref_points(rotvecs, np.zeros((N, 2), np.float32), L)
    eig = rng.standard_normal((r, L * L * L))
    eig, _ = np.linalg.qr(eig.T)
    eig = eig.T.reshape(r, L, L, L)
    eigenvals = np.array([9.0, 4.0, 1.5])[:r]
    filters = rng.uniform(0.2, 1.5, (N, L, L))
    noise_var = 0.05
    # images: projections of the eigenvolumes with N(0, eigenvals) coordinates, plus noise
    plan = ExactNufftPlan((L,) * 3, batch_size=r)
    plan.setpts(pts)
    proj = projection_funcs.vol_forward(torch.tensor(eig), plan, torch.tensor(filters))
    z = rng.standard_normal((N, r)) * np.sqrt(eigenvals)
    images = np.einsum("nr,nrij->nij", z, proj.numpy()) + rng.standard_normal((N, L, L)) * np.sqrt(noise_var)
    ds = _LatentData(torch.tensor(images), pts, torch.tensor(filters), noise_var)
    e_t, l_t = torch.tensor(eig), torch.tensor(eigenvals)
    out = dict(L=L, r=r, N=N, batch=batch, rotvecs=rotvecs, pts=pts.numpy(), eigenvecs=eig, eigenvals=eigenvals,
               filters=filters, noise_var=noise_var, images=images, z_true=z)
    c, cov = wiener_coords.latentMAP(ds, e_t, l_t, batch_size=batch, return_coords_covar=True,
                                     nufft_plan=nufft_plan.NufftPlanDiscretized)
    out["map_bilinear"], out["map_bilinear_covar"] = c.numpy(), cov.numpy()
    saved = wiener_coords.NufftPlan
    wiener_coords.NufftPlan = ExactNufftPlan
    try:
        c, cov = wiener_coords.latentMAP(ds, e_t, l_t, batch_size=batch, return_coords_covar=True,
                                         nufft_plan=ExactNufftPlan)
        out["map_exact"], out["map_exact_covar"] = c.numpy(), cov.numpy()
        out["wiener_exact"] = wiener_coords.wiener_coords(ds, e_t, l_t, batch_size=batch).numpy()
    finally:
        wiener_coords.NufftPlan = saved
    save(f"latent_dataset_L{L}_r{r}.npz", **out)


def case_preprocess(L=10, us=2, B=6, seed=71):
    """preprocess_image_batch (projection_funcs.py:199-252) with the discretized bilinear plan:
    phase shift, projected-mean subtraction, and the soft mask from the projected volume mask
    (get_mask_threshold, projection_funcs.py:255-269; soft_edged_kernel, utils.py:258-300)."""
    from cov3d import utils

    rng = np.random.default_rng(seed)
    n = L * us
    rotvecs = random_rotvecs(rng, B)
    offsets = rng.uniform(-2, 2, (B, 2)).astype(np.float32)
    pts, phase = ref_points(rotvecs, offsets, L)
    images = (rng.standard_normal((B, L, L)) * 2).astype(np.float32)
    filters = rng.uniform(0.2, 1.5, (B, L, L)).astype(np.float32)
    mean_vol = rng.standard_normal((L, L, L)).astype(np.float32)
    ax = np.arange(L) - L // 2
    zz, yy, xx = np.meshgrid(ax, ax, ax, indexing="ij")
    mask_vol = (np.sqrt(zz**2 + yy**2 + xx**2) < 0.35 * L).astype(np.float32)
    plan = nufft_plan.NufftPlanDiscretized((L,) * 3, upsample_factor=us, mode="bilinear")
    mean_f = projection_funcs.centered_fft3(torch.tensor(mean_vol, dtype=torch.float64).unsqueeze(0),
                                            padding_size=(n,) * 3)
    mask_f = projection_funcs.centered_fft3(torch.tensor(mask_vol, dtype=torch.float64).unsqueeze(0),
                                            padding_size=(n,) * 3)
    plan.setpts(pts)
    thr = projection_funcs.get_mask_threshold(mask_f, plan)
    soft = utils.soft_edged_kernel(radius=5, L=L, dim=2, in_fourier=True)
    ims = torch.tensor(images, dtype=torch.float64)
    filt = torch.tensor(filters, dtype=torch.float64)
    nomask = projection_funcs.preprocess_image_batch(ims, plan, filt, (pts, phase), mean_f)
    masked = projection_funcs.preprocess_image_batch(ims, plan, filt, (pts, phase), mean_f, mask_f, thr, soft)
    masked_f = projection_funcs.preprocess_image_batch(ims, plan, filt, (pts, phase), mean_f, mask_f, thr, soft,
                                                       fourier_domain=True)
    save(f"preprocess_L{L}.npz", L=L, us=us, rotvecs=rotvecs, offsets=offsets, pts=pts.numpy(),
         phase=phase.numpy(), images=images, filters=filters, mean_vol=mean_vol, mask_vol=mask_vol,
         mask_threshold=np.array(thr), soft_kernel_fourier=soft.numpy(), nomask=nomask.numpy(),
         masked=masked.numpy(), masked_fourier=masked_f.numpy())


def case_state_dict(L=6, r=2, seed=81):
    """The reference Covar's state_dict (covar.py:82-112) and CovarTrainer.results_dict
    (covar_sgd.py:524-535) key sets, with values, for checkpoint compatibility tests."""
    rng = np.random.default_rng(seed)
    vectors = rng.standard_normal((r, L, L, L))
    covar = Covar(L, r, dtype=torch.float64, fourier_domain=True, vectors=torch.tensor(vectors))
    covar.init_grid_correction("bilinear")
    sd = covar.state_dict()
    out = {"L": L, "r": r, "vectors_init": vectors, "keys": np.array(sorted(sd.keys()))}
    for k, v in sd.items():
        if torch.is_tensor(v):
            out["sd_" + k] = v.numpy()
        elif v is not None:
            out["sd_" + k] = np.array(v)
    eig, lam = covar.eigenvecs
    out["eigenvecs"], out["eigenvals"] = eig.numpy(), lam.numpy()
    save(f"state_dict_L{L}_r{r}.npz", **out)


if __name__ == "__main__":
    if len(sys.argv) > 2:
        globals()[sys.argv[2]]()
        sys.exit(0)
    case_poses()
    case_disc(10, 2, "bilinear", 5, 2, seed=1)
    case_disc(10, 2, "nearest", 5, 2, seed=2)
    case_disc(9, 2, "bilinear", 4, 2, seed=3)
    case_disc(10, 1, "nearest", 4, 1, seed=4, unaggregated=True)
    case_disc(7, 1, "bilinear", 3, 1, seed=6, unaggregated=True)
    case_cost()
    case_latent()
    case_cg()
    case_mean()
    case_halfsets()
    case_spatial_costs()
    case_trainer()
    case_latent_dataset()
    case_preprocess()
    case_state_dict()
    case_mean_initvol()
