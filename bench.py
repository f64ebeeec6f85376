"""Covariance-SGD throughput on GB300 (the reference's headline path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = one covariance-SGD iteration over a batch of 1024 synthetic L=128 images with
r=10 eigenvolumes (the config of the GPU drop-in workload: ES kernel width 6 at tol 1e-6,
upsampling 2, ML objective): on-the-fly points + bin sort, deapodise/pad + FFT3, ES
interpolation with the fused projection epilogue, per-image Gram + FP64 solve, hand-written
adjoint, compensated spreading, inverse FFT3, crop, Adam update.  Prints one JSON line.

``--impl reference`` times the reference's own step on the host cores: its
``CovarTrainer.run_batch`` on ``NufftPlanDiscretized`` bilinear (the command line's default;
its exact ES plan needs cuFINUFFT, which is not installed), imported unmodified from the copy
``oracle/build_ref.py`` makes, whole steps of the same batch size.  Without that copy it
falls back to the CPU port of the ES step (oracle/cpu_step.py), labelled ``kind: "port"``.
"""

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cov-SGD images/s (L=128,r=10)"
WORKLOAD = ("cov-SGD step, GPU drop-in plain FP32 config: L=128, pixel 1.5 A, r=10 Gaussian-blob eigenvolumes, "
            "batch 1024, uniform SO(3) poses, CTF 300 kV / Cs 2.7 mm / AC 0.1 / defocus U[1,3] um (from per-image "
            "parameters), SNR 0.05, "
            "NUFFT upsampling 2, ML objective + Fourier regulariser, Adam")
GPU_INTERP = "ES kernel width 6 (tol 1e-6), periodic, compensated FP32 spreading"
REF_INTERP = ("reference NufftPlanDiscretized bilinear (grid_sample), the reference command line's default; its ES "
              "plan (cuFINUFFT) is not installed")


def shared_config(args, world):
    """The workload both arms measure (identical dicts in the two JSON lines)."""
    return {"workload": WORKLOAD, "global_batch": args.batch * world, "L": args.L, "rank": args.rank, "upsample": 2,
            "objective": "ml + Fourier regulariser", "optimizer": "Adam", "snr": 0.05, "seed": args.seed,
            "l2": "inputs larger than L2: each GPU step reads a distinct resident 1024-image batch "
                  "(134 MB images; CTF computed in the kernels from 32 bytes of parameters per image) and 1.34 GB fine grids",
            "parallelism": f"dp{world}"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--L", type=int, default=128)
    ap.add_argument("--rank", type=int, default=10)
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--width", type=int, default=6)
    ap.add_argument("--resident-batches", type=int, default=16)
    ap.add_argument("--e2e-steps", type=int, default=0, help="0 = same as --steps")
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="per-image sample of the ES CPU port")
    ap.add_argument("--ref-batch", type=int, default=128, help="images per reference step in the GPU arm's baseline")
    ap.add_argument("--ref-budget", type=float, default=150.0,
                    help="seconds of timed reference steps in --impl reference (whole steps, at least one)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--seed", type=int, default=2000)
    ap.add_argument("--uncompensated", action="store_true", help="plain FP32 spreading (no TwoSum error terms)")
    ap.add_argument("--mean-images", type=int, default=300000, help="images backprojected for the mean-CG solve")
    ap.add_argument("--mean-L", type=int, default=128)
    ap.add_argument("--mean-rtol", type=float, default=1e-5)
    ap.add_argument("--mean-maxiter", type=int, default=20000)
    ap.add_argument("--no-mean", action="store_true", help="skip the mean-CG measurement")
    ap.add_argument("--no-bf16", action="store_true", help="skip the BF16-Gram variant of the step")
    ap.add_argument("--no-wiener", action="store_true", help="skip the Wiener-coordinate measurement")
    ap.add_argument("--no-bilinear", action="store_true", help="skip the bilinear-interpolation step")
    ap.add_argument("--ragged-L", type=int, default=256, help="volume size of the ragged Wiener measurement")
    ap.add_argument("--no-ragged", action="store_true", help="skip the ragged-batch Wiener measurement")
    ap.add_argument("--no-rank20", action="store_true", help="skip the rank-20 step")
    ap.add_argument("--no-small-epoch", action="store_true", help="skip the L=32 one-epoch measurement")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def cpu_baseline_port(args):
    """The CPU port of the ES step (oracle/cpu_step.py: float32 C + OpenMP loops, scipy FFT) on a
    bounded sample: the per-step FFT part timed once, the per-image part on a sample of images."""
    from oracle import cpu_step

    threads = os.cpu_count()
    cpu_step.time_baseline(args.L, args.rank, args.batch, 2, args.width, real="float", threads=threads)
    _, probe = cpu_step.time_baseline(args.L, args.rank, args.batch, 4, args.width, real="float", threads=threads)
    sample = int(max(2, min(256, args.cpu_seconds / max(probe["t_image_s"], 1e-6))))
    ips, det = cpu_step.time_baseline(args.L, args.rank, args.batch, sample, args.width, real="float",
                                      seed=args.seed, threads=threads)
    return {"value": ips, "unit": "images/s", "cores": threads, "kind": "port",
            "sample": (f"CPU port of the ES step: per-step part (pad + FFT3 + iFFT3 + crop, {det['t_step_s']:.2f} s) "
                       f"timed once and the per-image part (points, ES interp, Gram/solve, adjoint, ES spread) on "
                       f"{sample} images ({det['t_image_s'] * 1e3:.1f} ms/image); images/s = {args.batch} / (t_step + "
                       f"{args.batch} * t_image); float32 C + OpenMP, scipy.fft workers={threads}")}


def cpu_baseline_reference(args, batch, steps, warmup, budget_s):
    """Whole steps of the reference's own trainer (oracle/ref_step.py) on the host cores."""
    from oracle import ref_step

    ips, det = ref_step.time_steps(args.L, args.rank, batch, steps, warmup, seed=args.seed, budget_s=budget_s)
    return {"value": ips, "unit": "images/s", "cores": det["threads"], "kind": "reference",
            "sample": (f"{det['steps']} whole step(s) of {batch} images after {det['warmup']} warm-up step(s): the "
                       f"reference's CovarTrainer.run_batch (setpts + Covar Fourier view + grid_sample projection + "
                       f"cost_maximum_liklihood_fourier_domain + backward + Adam) on NufftPlanDiscretized bilinear, "
                       f"torch CPU threads={det['threads']}, {det['seconds']:.1f} s timed")}, det


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    t0 = time.perf_counter()
    from oracle import ref_step

    if ref_step.available():
        cb, det = cpu_baseline_reference(args, args.batch, args.steps, args.warmup, args.ref_budget)
        steps, warmup = det["steps"], det["warmup"]
        ms_step = det["seconds"] / steps * 1e3
        interp = REF_INTERP
    else:
        cb = cpu_baseline_port(args)
        steps, warmup = 1, 0
        ms_step = args.batch / cb["value"] * 1e3
        interp = "CPU port of the ES step (reference package not installed under oracle/_ref)"
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "images/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": shared_config(args, world), "interpolation": interp,
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def load_traffic(kernel):
    """dram bytes per launch of `kernel` recorded from an ncu capture in profiles/ (or None)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def make_dataset(pkg, args, dev, n_images):
    import torch

    from importlib import import_module

    syn = import_module("3dcovarestimation_gb300.synthetic")
    g = torch.Generator(device=dev).manual_seed(args.seed)
    L, r = args.L, args.rank
    eig = syn.gaussian_blob_volumes(r, L, generator=g, device=dev)
    eig = syn.orthonormalize(eig.reshape(r, -1)).reshape(r, L, L, L).contiguous()
    sqrt_lam = torch.linspace(1.0, 0.3, r, device=dev) * L**1.5
    rot = syn.uniform_rotations(n_images, generator=g, device=dev)
    defocus = torch.rand((n_images,), generator=g, device=dev) * 2.0 + 1.0
    prm = syn.ctf_params(defocus, 1.5, device=dev)  # the CTF is computed in the kernels from these
    ctf = syn.ctf_from_params(prm, L)
    images = torch.empty((n_images, L * L), dtype=torch.complex64, device=dev)
    plan = pkg.NufftPlan((L,) * 3, batch_size=r, device=dev, width=args.width)
    B = args.batch
    for i in range(0, n_images, B):
        plan.setrot(rot[i:i + B])
        proj = pkg.vol_forward(eig, plan, ctf[i:i + B], fourier_domain=True)  # (b, r, L, L)
        z = torch.randn((proj.shape[0], r, 1, 1), generator=g, device=dev) * sqrt_lam.reshape(1, r, 1, 1)
        images[i:i + B] = (proj * z).sum(1).reshape(-1, L * L)
    signal_var = float((images.abs() ** 2).mean())
    noise_var = signal_var / 0.05
    images += torch.randn(images.shape, generator=g, device=dev, dtype=torch.complex64) * (noise_var ** 0.5)
    return images, rot, prm, noise_var


def run_wiener_ragged(pkg, args, dev):
    """Wiener / latent-MAP coordinates at the full-pipeline size: L = args.ragged_L, r = 10,
    batches of 256 .. 4096 images in a fixed ragged sequence over a resident pool of 4096
    Fourier-domain images (the solve's cost does not depend on the image values), uniform
    SO(3) poses, CTF from per-image parameters, the eigenvolumes' fine grid transformed once.
    Returns images/s over the sequence (CUDA events)."""
    import torch

    from importlib import import_module

    syn = import_module("3dcovarestimation_gb300.synthetic")
    wc = import_module("3dcovarestimation_gb300.wiener_coords")
    L, r = args.ragged_L, 10
    g = torch.Generator(device=dev).manual_seed(args.seed + 5)
    eig = syn.gaussian_blob_volumes(r, L, generator=g, device=dev)
    eig = syn.orthonormalize(eig.reshape(r, -1)).reshape(r, L, L, L)
    lam = torch.linspace(4.0, 0.5, r, device=dev, dtype=torch.float64)
    linv = torch.diag(1.0 / lam)
    pool = 4096
    images = torch.randn((pool, L, L), device=dev, generator=g, dtype=torch.complex64) * 10
    rot = syn.uniform_rotations(pool, generator=g, device=dev)
    df = torch.rand((pool,), device=dev, generator=g) * 2 + 1
    prm = syn.ctf_params(df, 1.0, device=dev)
    sizes = [256, 1000, 4096, 3000, 512, 2048, 1500, 4096, 768, 3500]
    plan = pkg.NufftPlan((L,) * 3, batch_size=r, device=dev, width=args.width)
    project = wc._EigenProjector(plan, eig)

    def batch(nimg, off):
        idx = slice(off, off + nimg)
        plan.setrot(rot[idx])
        q = project(syn.ctf_from_params(prm[idx], L), fourier_domain=True)
        return wc.compute_latentMAP_batch(images[idx], q, 1.0e4, linv)[0]

    batch(sizes[0], 0)  # warm-up: plan, fine grid, kernels
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    total = 0
    for k, nimg in enumerate(sizes):
        batch(nimg, (k * 331) % (pool - nimg + 1))
        total += nimg
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return {"images_per_s": total / (ms / 1e3), "images": total, "L": L, "rank": r, "batch_sizes": sizes,
            "note": "ragged batches of 256..4096 images (full-pipeline configuration's sizes, L=256): ES "
                    "interpolation of the eigenvolumes' fine grid, FP32 Gram, FP64 Cholesky per image"}


def run_small_epoch(pkg, args, dev, with_reference):
    """The CPU-runnable configuration's training part: one epoch of covariance SGD at L = 32,
    r = 5 over 2 000 images in batches of 256 (the last one 208), on bilinear plans, timed as
    the wall time of the whole epoch on the GPU (host-resident images copied in per batch,
    the cost read back per batch) and, when the reference is installed, the reference's own
    run_batch for the same batches on the host cores."""
    import torch

    from importlib import import_module

    syn = import_module("3dcovarestimation_gb300.synthetic")
    L, r, N, B = 32, 5, 2000, 256
    g = torch.Generator(device=dev).manual_seed(args.seed + 7)
    images = (torch.randn((N, L * L), device=dev, generator=g, dtype=torch.complex64) * 10).cpu().pin_memory()
    rot = syn.uniform_rotations(N, generator=g, device=dev).cpu().pin_memory()
    prm = syn.ctf_params(torch.rand((N,), device=dev, generator=g) * 2 + 1, 3.0, device=dev).cpu().pin_memory()
    covar = pkg.Covar(L, r, upsampling_factor=2).to(dev)
    covar.vectors.grad = torch.zeros_like(covar.vectors)
    covar.log_sqrt_eigenvals.grad = torch.zeros_like(covar.log_sqrt_eigenvals)
    opt = torch.optim.Adam([{"params": covar.vectors, "lr": 1e-6 * B}, {"params": covar.log_sqrt_eigenvals,
                                                                        "lr": 1e-4 * B}])
    step = pkg.FusedCovarStep(L, r, "bilinear", 2, device=dev, max_batch=B)

    def epoch():
        costs = []
        for i in range(0, N, B):
            j = min(N, i + B)
            step.set_rotations(rot[i:j].to(dev, non_blocking=True))
            c, _, _ = step(covar.vectors.detach(), covar.log_sqrt_eigenvals.detach(),
                           images[i:j].to(dev, non_blocking=True), None, 1.0e4, 0.0, None,
                           grad_vectors=covar.vectors.grad, grad_log_sqrt=covar.log_sqrt_eigenvals.grad,
                           ctf_params=prm[i:j].to(dev, non_blocking=True))
            opt.step()
            costs.append(float(c))
        return costs

    epoch()  # warm-up: plans, kernels
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    epoch()
    torch.cuda.synchronize()
    gpu_s = time.perf_counter() - t0
    out = {"L": L, "rank": r, "images": N, "batch": B, "gpu_epoch_s": gpu_s, "gpu_images_per_s": N / gpu_s,
           "note": "one epoch of the fused step on bilinear plans, host images copied in and the cost read back "
                   "per batch; mean CG not included"}
    if with_reference:
        from oracle import ref_step

        if ref_step.available():
            ips, det = ref_step.time_steps(L, r, B, 8, 1, seed=args.seed, budget_s=60.0)
            out["reference_images_per_s"] = ips
            out["reference_epoch_s_estimate"] = N / ips
            out["reference_sample"] = (f"{det['steps']} whole run_batch step(s) of {B} images after {det['warmup']} "
                                       f"warm-up, torch CPU threads={det['threads']}")
    return out


def run_mean_cg(pkg, args, dev):
    """Mean reconstruction at L = args.mean_L from args.mean_images images whose viewing
    directions follow a mixture of 8 von Mises-Fisher clusters (kappa 5): backprojection
    throughput, then wall time and iterations of the padding CG to relative residual
    args.mean_rtol with each preconditioner."""
    import torch

    from importlib import import_module

    syn = import_module("3dcovarestimation_gb300.synthetic")
    mean = import_module("3dcovarestimation_gb300.mean")
    L, B, N = args.mean_L, args.batch, args.mean_images
    g = torch.Generator(device=dev).manual_seed(args.seed + 4000)
    vol = syn.gaussian_blob_volumes(1, L, generator=g, device=dev)
    rot = syn.vmf_cluster_rotations(N, 8, 5.0, generator=g, device=dev)
    fwd = pkg.NufftPlan((L,) * 3, batch_size=1, device=dev, width=args.width)
    acc = mean.MeanBackprojector(L, 2, dev)
    stream = torch.cuda.current_stream()
    bp_ms = 0.0
    noise_sd = None
    for i in range(0, N, B):
        rb = rot[i:i + B]
        defocus = torch.rand((rb.shape[0],), generator=g, device=dev) * 2.0 + 1.0
        ctf = syn.ctf_images(defocus, L, 1.5, device=dev)
        fwd.setrot(rb)
        img = pkg.vol_forward(vol, fwd, ctf, fourier_domain=True)[:, 0]
        if noise_sd is None:
            noise_sd = (float((img.abs() ** 2).mean()) / 0.05) ** 0.5
        img = img + torch.randn(img.shape, generator=g, device=dev, dtype=torch.complex64) * noise_sd
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        acc.add(img, ctf, rotations=rb)
        e1.record(stream)
        e1.synchronize()
        bp_ms += e0.elapsed_time(e1)
    reg = mean.regularize_lhs(acc.lhs)
    plan = mean._MeanSolver.get(L, 2, dev)
    b = torch.empty((L,) * 3, dtype=torch.complex64, device=dev)
    x0 = torch.empty_like(b)
    pkg._lib.call("cov3d_mean_init", plan.bind(), pkg._lib.ptr(acc.rhs.contiguous()), pkg._lib.ptr(reg),
                  pkg._lib.ptr(b), pkg._lib.ptr(x0))
    out = {"workload": f"mean at L={L}, {N} images, viewing directions from 8 vMF clusters (kappa 5), "
                       f"nearest plan at upsampling 2, CG to relative residual {args.mean_rtol}",
           "backprojection_images_per_s": N / (bp_ms / 1e3), "rtol": args.mean_rtol,
           "maxiter": args.mean_maxiter}
    # warm the cuFFT plans and the symbol path once
    mean.cg_solve(reg, b, x0, L, rtol=1e-1, maxiter=2, precond="circulant")
    mean.cg_solve(reg, b, x0, L, rtol=1e-1, maxiter=2, precond="diagonal")
    for name, pc in (("plain", None), ("diagonal_pc", "diagonal"), ("circulant_pc", "circulant")):
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("mean_cg_" + name)
        t0 = time.perf_counter()
        x, info = mean.cg_solve(reg, b, x0, L, rtol=args.mean_rtol, maxiter=args.mean_maxiter, precond=pc)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        torch.cuda.nvtx.range_pop()
        out[name] = {"seconds": sec, "iters": info.iters, "relres": info.relres, "converged": info.converged,
                     "ms_per_iter": 1e3 * sec / max(1, info.iters + 1)}
    lp = import_module("3dcovarestimation_gb300.learned_pc")
    if os.path.exists(lp.WEIGHTS_PATH):
        pcn = lp.LearnedPreconditioner(device=dev)
        pcn.symbol(reg, L)  # warm
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("mean_cg_learned_pc")
        t0 = time.perf_counter()
        sym = pcn.symbol(reg, L)  # features + network + upsampling, inside the timed solve
        x, info = mean.cg_solve(reg, b, x0, L, rtol=args.mean_rtol, maxiter=args.mean_maxiter, precond=sym)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        torch.cuda.nvtx.range_pop()
        out["learned_pc"] = {"seconds": sec, "iters": info.iters, "relres": info.relres, "converged": info.converged,
                             "ms_per_iter": 1e3 * sec / max(1, info.iters + 1)}
        out["learned_vs_diagonal_pc_time"] = sec / out["diagonal_pc"]["seconds"]
    else:
        out["learned_pc"] = "no trained weights (3dcovarestimation_gb300/learned_pc_weights.npz)"
    return out


def run_gb300(args):
    import torch

    rank, world, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    pkg = importlib.import_module("3dcovarestimation_gb300")
    from importlib import import_module

    syn = import_module("3dcovarestimation_gb300.synthetic")
    L, r, B = args.L, args.rank, args.batch
    nb = max(2, args.resident_batches)
    images, rot, prm, noise_var = make_dataset(pkg, args, dev, nb * B)
    images = images.reshape(nb, B, -1)
    rot = rot.reshape(nb, B, 3, 3).contiguous()
    prm = prm.reshape(nb, B, -1)
    covar = pkg.Covar(L, r, upsampling_factor=2).to(dev)
    step_fn = pkg.FusedCovarStep(L, r, "nufft", 2, width=args.width, device=dev,
                                 compensated=not args.uncompensated, max_batch=B)
    covar.vectors.grad = torch.zeros_like(covar.vectors)
    covar.log_sqrt_eigenvals.grad = torch.zeros_like(covar.log_sqrt_eigenvals)
    groups = covar.grad_lr_factor()
    for gp in groups:
        gp["lr"] *= 1e-6 * B
    opt = torch.optim.Adam(groups)
    n = 2 * L
    shell = torch.fft.fftshift(torch.fft.fftfreq(n, device=dev)) * n
    rr = torch.sqrt(shell[:, None, None] ** 2 + shell[None, :, None] ** 2 + shell[None, None, :] ** 2)
    fourier_reg = (1.0 + rr) ** 2 / (n**3)
    reg_scale = 1.0 / 100000  # reg / N with N = 100,000 images
    cost_acc = torch.zeros((), dtype=torch.float64, device=dev)

    dp = import_module("3dcovarestimation_gb300.distributed")

    def grads_allreduce():
        dp.allreduce_mean_([covar.vectors.grad, covar.log_sqrt_eigenvals.grad])

    def step(k, imgs=None, prms=None, rots=None):
        b = (k * world + rank) % nb
        step_fn.set_rotations(rot[b] if rots is None else rots)
        c, _, _ = step_fn(covar.vectors.detach(), covar.log_sqrt_eigenvals.detach(),
                          images[b] if imgs is None else imgs, None, noise_var, reg_scale, fourier_reg,
                          grad_vectors=covar.vectors.grad, grad_log_sqrt=covar.log_sqrt_eigenvals.grad,
                          ctf_params=prm[b] if prms is None else prms)
        grads_allreduce()
        opt.step()
        return c.reshape(())

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    for k in range(args.warmup):
        cost_acc += step(k)
    barrier()
    lib = pkg._lib
    launches0 = lib.launch_count()
    step_fn.plan.timing(True)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        barrier()
        torch.cuda.nvtx.range_push("cov_sgd_steps")
        e0.record(stream)
        for k in range(args.steps):
            cost_acc += step(args.warmup + k)
        e1.record(stream)
        barrier()
        torch.cuda.nvtx.range_pop()
    ms_total = e0.elapsed_time(e1)
    launches = lib.launch_count() - launches0
    phases = step_fn.plan.timing_read()
    step_fn.plan.timing(False)
    clocks = clk.summary()
    ms_max = ms_total
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t)
    ms_step = ms_max / args.steps
    value = world * B * args.steps / (ms_max / 1e3)

    # end to end through the same C-ABI call with host (pinned) buffers: every step copies its
    # batch's images, CTF and rotations host -> device (on a copy stream, into the other of two
    # device buffers while the previous step computes) and reads the cost back
    e2e_steps = args.e2e_steps or args.steps
    nhost = min(nb, 4)
    h_images = images[:nhost].cpu().pin_memory()
    h_prm = prm[:nhost].cpu().pin_memory()
    h_rot = rot[:nhost].cpu().pin_memory()
    bufs = [(torch.empty_like(images[0]), torch.empty_like(prm[0]), torch.empty_like(rot[0])) for _ in range(2)]
    ready = [torch.cuda.Event() for _ in range(2)]
    free = [torch.cuda.Event() for _ in range(2)]
    copy_stream = torch.cuda.Stream()
    h_cost = torch.zeros((e2e_steps,), dtype=torch.float64).pin_memory()

    def h2d(k):
        j, slot = k % nhost, k % 2
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(free[slot])
            for dst, src in zip(bufs[slot], (h_images[j], h_prm[j], h_rot[j])):
                dst.copy_(src, non_blocking=True)
            ready[slot].record(copy_stream)

    barrier()
    t0 = time.perf_counter()
    h2d(0)
    for k in range(e2e_steps):
        if k + 1 < e2e_steps:
            h2d(k + 1)
        slot = k % 2
        stream.wait_event(ready[slot])
        c = step(k, *bufs[slot])
        free[slot].record(stream)
        h_cost[k:k + 1].copy_(c.reshape(1), non_blocking=True)
    barrier()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t)
    e2e_value = world * B * e2e_steps / e2e_s
    h2d_bytes = sum(t.numel() * t.element_size() for t in bufs[0])

    # the same step with the per-image Gram contractions in BF16 on the tensor cores
    bf16 = None
    if not args.no_bf16:
        step_bf = pkg.FusedCovarStep(L, r, "nufft", 2, width=args.width, device=dev,
                                     compensated=not args.uncompensated, gram_precision="bf16", max_batch=B)

        def step16(k):
            b = (k * world + rank) % nb
            step_bf.set_rotations(rot[b])
            c, _, _ = step_bf(covar.vectors.detach(), covar.log_sqrt_eigenvals.detach(), images[b], None, noise_var,
                              reg_scale, fourier_reg, grad_vectors=covar.vectors.grad,
                              grad_log_sqrt=covar.log_sqrt_eigenvals.grad, ctf_params=prm[b])
            return c

        for k in range(2):
            step16(k)
        barrier()
        step_bf.plan.timing(True)
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nbf = max(3, args.steps // 2)
        f0.record(stream)
        for k in range(nbf):
            step16(k)
        f1.record(stream)
        barrier()
        ph16 = step_bf.plan.timing_read()
        step_bf.plan.timing(False)
        ms16 = f0.elapsed_time(f1) / nbf
        bf16 = {"ms_per_step": ms16, "images_per_s": world * B / (ms16 / 1e3), "steps": nbf,
                "gram_ms": ph16["gram"][0] / nbf, "gram_ms_fp32": phases["gram"][0] / args.steps,
                "note": "Gram contractions in BF16 with FP32 accumulation (tcgen05); projections, spreading, "
                        "solve and update unchanged (FP32 / FP64)"}

    # the precision configuration's rank: r = 20 at the same L and batch, FP32 and BF16 Gram
    rank20 = None
    if not args.no_rank20:
        r2 = 20
        covar20 = pkg.Covar(L, r2, upsampling_factor=2).to(dev)
        gv20 = torch.zeros_like(covar20.vectors)
        gl20 = torch.zeros_like(covar20.log_sqrt_eigenvals)
        rank20 = {"L": L, "rank": r2, "batch": B}
        for prec in ("fp32", "bf16"):
            st20 = pkg.FusedCovarStep(L, r2, "nufft", 2, width=args.width, device=dev,
                                      compensated=not args.uncompensated, gram_precision=prec, max_batch=B)

            def step20(k):
                b = (k * world + rank) % nb
                st20.set_rotations(rot[b])
                st20(covar20.vectors.detach(), covar20.log_sqrt_eigenvals.detach(), images[b], None, noise_var,
                     reg_scale, fourier_reg, grad_vectors=gv20, grad_log_sqrt=gl20, ctf_params=prm[b])

            for k in range(2):
                step20(k)
            barrier()
            st20.plan.timing(True)
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            n20 = max(3, args.steps // 4)
            t0.record(stream)
            for k in range(n20):
                step20(k)
            t1.record(stream)
            barrier()
            ph20 = st20.plan.timing_read()
            st20.plan.timing(False)
            ms20 = t0.elapsed_time(t1) / n20
            rank20[prec] = {"images_per_s": world * B / (ms20 / 1e3), "ms_per_step": ms20, "steps": n20,
                            "phases_ms_per_step": {k: v[0] / n20 for k, v in ph20.items() if v[1]}}
            del st20
        torch.cuda.empty_cache()

    # the same step on the reference's default interpolation (NufftPlanDiscretized bilinear,
    # grid_sample semantics): the like-for-like comparison with the reference's CPU arm
    bilinear = None
    if not args.no_bilinear:
        step_bl = pkg.FusedCovarStep(L, r, "bilinear", 2, device=dev, compensated=not args.uncompensated,
                                     max_batch=B)
        covar_bl = pkg.Covar(L, r, upsampling_factor=2).to(dev)
        covar_bl.vectors.grad = torch.zeros_like(covar_bl.vectors)
        covar_bl.log_sqrt_eigenvals.grad = torch.zeros_like(covar_bl.log_sqrt_eigenvals)
        opt_bl = torch.optim.Adam([{"params": covar_bl.vectors, "lr": 1e-6 * B},
                                   {"params": covar_bl.log_sqrt_eigenvals, "lr": 1e-4 * B}])

        def step_bilinear(k, imgs=None, prms=None, rots=None):
            b = (k * world + rank) % nb
            step_bl.set_rotations(rot[b] if rots is None else rots)
            c, _, _ = step_bl(covar_bl.vectors.detach(), covar_bl.log_sqrt_eigenvals.detach(),
                              images[b] if imgs is None else imgs, None, noise_var, reg_scale, fourier_reg,
                              grad_vectors=covar_bl.vectors.grad, grad_log_sqrt=covar_bl.log_sqrt_eigenvals.grad,
                              ctf_params=prm[b] if prms is None else prms)
            dp.allreduce_mean_([covar_bl.vectors.grad, covar_bl.log_sqrt_eigenvals.grad])
            opt_bl.step()
            return c.reshape(())

        for k in range(args.warmup):
            step_bilinear(k)
        barrier()
        step_bl.plan.timing(True)
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for k in range(args.steps):
            step_bilinear(k)
        g1.record(stream)
        barrier()
        phbl = step_bl.plan.timing_read()
        step_bl.plan.timing(False)
        msbl = g0.elapsed_time(g1) / args.steps
        # end to end with host buffers, copies inside the timed region (as the headline e2e)
        barrier()
        t0 = time.perf_counter()
        h2d(0)
        for k in range(e2e_steps):
            if k + 1 < e2e_steps:
                h2d(k + 1)
            slot = k % 2
            stream.wait_event(ready[slot])
            c = step_bilinear(k, *bufs[slot])
            free[slot].record(stream)
            h_cost[k:k + 1].copy_(c.reshape(1), non_blocking=True)
        barrier()
        e2e_bl = world * B * e2e_steps / (time.perf_counter() - t0)
        bilinear = {"images_per_s": world * B / (msbl / 1e3), "ms_per_step": msbl, "steps": args.steps,
                    "e2e_images_per_s": e2e_bl,
                    "phases_ms_per_step": {k: v[0] / args.steps for k, v in phbl.items() if v[1]},
                    "note": "fused step on NufftPlanDiscretized bilinear semantics (grid_sample, 8 taps), the "
                            "same interpolation as the reference arm"}

    # Wiener / latent-MAP coordinates of the resident images with the current eigenvolumes
    # (wiener_coords.latentMAP's per-batch work: projections + FP32 Gram + FP64 Cholesky solve)
    wiener = None
    if not args.no_wiener:
        wc = import_module("3dcovarestimation_gb300.wiener_coords")
        eigv = covar.get_vectors_spatial_domain().detach()
        lam = torch.exp(2 * covar.log_sqrt_eigenvals.detach()).to(torch.float64)
        linv = torch.diag(1.0 / (lam + 1e-6))
        wplan = pkg.NufftPlan((L,) * 3, batch_size=r, device=dev, width=args.width)
        project = wc._EigenProjector(wplan, eigv)  # as latentMAP: the eigenvolumes' grid once

        def wbatch(b):
            wplan.setrot(rot[b])
            q = project(syn.ctf_from_params(prm[b], L), fourier_domain=True)
            return wc.compute_latentMAP_batch(images[b], q, noise_var, linv)[0]

        wbatch(0)
        barrier()
        w0, w1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0.record(stream)
        for b in range(nb):
            wbatch(b)
        w1.record(stream)
        barrier()
        wms = w0.elapsed_time(w1)
        wiener = {"images_per_s": nb * B / (wms / 1e3), "images": nb * B, "batch": B,
                  "note": "per batch: ES interpolation of the r eigenvolumes' fine grid (transformed once, as "
                          "latentMAP does) with CTF, FP32 Gram, FP64 Cholesky solve per image (Fourier-domain "
                          "images)"}

    if rank != 0:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()
        return

    # roofline of the dominant kernel (interp or spread), per step = per launch group
    M = B * L * L
    n3 = n**3
    # grid, samples, rotations (36 B) and CTF parameters (32 B) per image: the CTF itself is
    # evaluated in the kernels
    alg = {"interp": r * n3 * 8 + r * M * 8 + B * (9 * 4 + 8 * 4),
           "spread": r * M * 8 + 2 * r * n3 * 8 + B * (9 * 4 + 8 * 4)}
    dom = max(("interp", "spread"), key=lambda k: phases[k][0])
    dom_ms = phases[dom][0] / max(1, args.steps)
    peak, peak_kind = load_peaks()
    achieved = alg[dom] / (dom_ms / 1e3) / 1e9
    flops = M * (args.width**3) * r * 4
    sm_mhz = clocks.get("sm_mhz") or 1900.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    kernel_name = "interp_kernel" if dom == "interp" else ("spread_rows_kernel" if r >= 5 else "spread_kernel")
    line = {
        "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": shared_config(args, world),
        "interpolation": GPU_INTERP, "resident_images": nb * B,
        "spreading": "fp32" if args.uncompensated else "fp32 + TwoSum compensation",
        "roofline": {"bound": "hbm", "kernel": kernel_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": load_traffic(kernel_name),
                     "algorithmic_bytes_per_launch": alg[dom], "ms_per_launch": dom_ms,
                     "fp32_tflops": flops / (phases["interp"][0] / args.steps / 1e3) / 1e12,
                     "fp32_frac_interp": flops / (phases["interp"][0] / args.steps / 1e3) / 1e12 / fp32_peak},
        "e2e": {"value": e2e_value, "unit": "images/s", "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": 8},
        "gpu_launches": launches,
        "clocks": clocks,
        "phases_ms_per_step": {k: v[0] / args.steps for k, v in phases.items() if v[1]},
        "final_cost": float(cost_acc) / (args.warmup + args.steps),
    }
    if bf16 is not None:
        line["bf16_gram"] = bf16
    if rank20 is not None:
        line["rank20_step"] = rank20
    if wiener is not None:
        line["wiener_coords"] = wiener
    if not args.no_wiener and not args.no_ragged:
        line["wiener_ragged"] = run_wiener_ragged(pkg, args, dev)
    if not args.no_small_epoch:
        line["small_epoch"] = run_small_epoch(pkg, args, dev, with_reference=not args.no_cpu_baseline)
    if not args.no_mean:
        line["mean_cg"] = run_mean_cg(pkg, args, dev)
    if bilinear is not None:
        line["bilinear_step"] = bilinear
    if not args.no_cpu_baseline:
        cb, _ = cpu_baseline_reference(args, args.ref_batch, 1, 1, 1e9)
        line["cpu_baseline"] = cb
        line["cpu_baseline_es_port"] = cpu_baseline_port(args)
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    args = parse()
    import torch

    torch.manual_seed(args.seed)  # the Covar's random initial eigenvolumes (the data have their own generators)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
