"""The multi-rank (data-parallel) host logic on CPU with gloo ranks: uneven image shards,
the product's reductions of the covariance gradient (weighted by shard size) and of the
half-set mean backprojections (two rank groups), each equal to the single-process result of
the float64 oracle."""
import os
import socket

import numpy as np
import torch
import torch.multiprocessing as mp

from conftest import load_golden


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _init(rank, world, port):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    return dist


def _grad_case():
    from oracle import nufft_oracle as O

    rng = np.random.default_rng(4)
    L, r, B = 8, 2, 7
    vec = rng.standard_normal((r, L, L, L))
    vec /= np.linalg.norm(vec.reshape(r, -1), axis=1)[:, None, None, None]
    ls = np.log(rng.uniform(2, 5, r))
    R = O.rotvec_to_rotmat(rng.standard_normal((B, 3)))
    imgs = (rng.standard_normal((B, L, L)) + 1j * rng.standard_normal((B, L, L))) * 2
    ctf = rng.uniform(0.3, 1.2, (B, L, L))
    return vec, ls, R, imgs, ctf


def _grad_worker(rank, world, port, out):
    import importlib

    dist = _init(rank, world, port)
    from oracle import nufft_oracle as O

    D = importlib.import_module("3dcovarestimation_gb300.distributed")
    vec, ls, R, imgs, ctf = _grad_case()
    lo, hi = D.shard(len(R), rank, world)  # 4 and 3 images
    L = vec.shape[-1]
    c, gv, gl = O.covar_cost_grad(vec, ls, imgs[lo:hi], O.rotated_points(R[lo:hi], L), ctf[lo:hi], 3.0, kind="es",
                                  width=6)
    t = [torch.tensor([c]), torch.tensor(gv), torch.tensor(gl)]
    D.allreduce_mean_(t, count=hi - lo)
    out[rank] = tuple(x.numpy() for x in t)
    dist.destroy_process_group()


def _mean_worker(rank, world, port, out):
    import importlib

    dist = _init(rank, world, port)
    from oracle import nufft_oracle as O

    D = importlib.import_module("3dcovarestimation_gb300.distributed")
    g = load_golden("mean_L10.npz")
    N = 90
    lo, hi = D.shard(N, rank, world)  # 23, 23, 22, 22 images
    sl = slice(lo, hi)
    L = int(g["L"])
    rhs, lhs = O.mean_backprojection(g["images"][sl], g["pts"][sl], g["filters"][sl], g["offsets"][sl],
                                     g["contrasts"][sl], L, int(g["us"]))
    h1, h2 = D.reduce_halfset_backprojections(torch.tensor(rhs), torch.tensor(lhs), L)
    out[rank] = ([x.numpy() for x in h1], [x.numpy() for x in h2])
    dist.destroy_process_group()


def _run(target, world):
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    return dict(out)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def test_uneven_shards_reduce_to_the_full_batch_gradient():
    from oracle import nufft_oracle as O

    out = _run(_grad_worker, 2)
    vec, ls, R, imgs, ctf = _grad_case()
    c, gv, gl = O.covar_cost_grad(vec, ls, imgs, O.rotated_points(R, vec.shape[-1]), ctf, 3.0, kind="es", width=6)
    for r in range(2):
        c_r, gv_r, gl_r = out[r]
        assert abs(c_r[0] - c) / abs(c) < 1e-12
        assert rel(gv_r, gv) < 1e-12 and rel(gl_r, gl) < 1e-12


def test_halfset_groups_reduce_to_the_halfset_backprojections():
    from oracle import nufft_oracle as O

    out = _run(_mean_worker, 4)
    g = load_golden("mean_L10.npz")
    L, us = int(g["L"]), int(g["us"])
    halves = []
    for lo, hi in ((0, 46), (46, 90)):  # ranks {0, 1} and {2, 3}
        sl = slice(lo, hi)
        rhs, lhs = O.mean_backprojection(g["images"][sl], g["pts"][sl], g["filters"][sl], g["offsets"][sl],
                                         g["contrasts"][sl], L, us)
        mean = np.real(O.centered_ifft3(rhs / (lhs + 1e-1), crop_to=L))
        halves.append((mean, rhs, lhs))
    for r in range(4):
        for h in range(2):
            for got, want in zip(out[r][h], halves[h]):
                assert rel(got, want) < 1e-12


def test_shards_cover_every_item_once():
    import importlib

    D = importlib.import_module("3dcovarestimation_gb300.distributed")
    for n in (0, 1, 7, 96, 1001):
        for w in (1, 2, 3, 8):
            spans = [D.shard(n, r, w) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(w - 1))
            assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1
