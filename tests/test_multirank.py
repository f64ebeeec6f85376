"""The multi-rank (data-parallel) host logic on CPU: two gloo ranks shard the images, reduce
partial mean grids and average gradients; the result equals the single-process one."""
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


def _worker(rank, world, port, out):
    import importlib
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    from oracle import nufft_oracle as O

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    D = importlib.import_module("3dcovarestimation_gb300.distributed")
    g = load_golden("mean_L10.npz")
    L = int(g["L"])
    lo, hi = D.shard(len(g["images"]), rank, world)
    sl = slice(lo, hi)
    rhs, lhs = O.mean_backprojection(g["images"][sl], g["pts"][sl], g["filters"][sl], g["offsets"][sl],
                                     g["contrasts"][sl], L, int(g["us"]))
    grids = [torch.tensor(rhs), torch.tensor(lhs)]
    D.allreduce_sum_(grids)
    grad = torch.full((3, 4), float(rank + 1), dtype=torch.float64)
    D.allreduce_mean_([grad])
    out[rank] = (grids[0].numpy(), grids[1].numpy(), grad.numpy())
    dist.destroy_process_group()


def test_two_ranks_reduce_to_the_single_process_result():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    g = load_golden("mean_L10.npz")
    for r in range(2):
        rhs, lhs, grad = out[r]
        assert np.linalg.norm(rhs - g["rhs"]) / np.linalg.norm(g["rhs"]) < 1e-12
        assert np.linalg.norm(lhs - g["lhs"]) / np.linalg.norm(g["lhs"]) < 1e-12
        assert np.allclose(grad, 1.5)


def test_shards_cover_every_item_once():
    import importlib

    D = importlib.import_module("3dcovarestimation_gb300.distributed")
    for n in (0, 1, 7, 96, 1001):
        for w in (1, 2, 3, 8):
            spans = [D.shard(n, r, w) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(w - 1))
            assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1
