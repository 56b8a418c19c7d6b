"""Multi-rank host logic on the CPU (gloo, world size 2): view ranges of a sharded batch and the
gradient all-reduce of a sharded differentiable batch."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from ifrit_gb300.sharding import allreduce_gradients, view_range


def test_view_ranges_cover_every_view_once():
    for n in (0, 1, 5, 64, 256, 257):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                b, e = view_range(n, r, world)
                assert 0 <= b <= e <= n
                seen.extend(range(b, e))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        view_range(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n_views, V = 7, 11
        b, e = view_range(n_views, rank, world)
        # per-view gradient contributions of a shared mesh, as each rank's backward would produce
        rng = np.random.default_rng(0)
        per_view = torch.from_numpy(rng.normal(size=(n_views, V, 3)).astype(np.float32))
        g = per_view[b:e].sum(0)
        allreduce_gradients([g, None])
        out[rank] = g.numpy().tolist()
    finally:
        dist.destroy_process_group()


def test_sharded_gradient_sum_equals_unsharded_sum():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    rng = np.random.default_rng(0)
    want = rng.normal(size=(7, 11, 3)).astype(np.float32).sum(0)
    for r in range(world):
        assert np.allclose(np.array(out[r]), want, atol=1e-5)
