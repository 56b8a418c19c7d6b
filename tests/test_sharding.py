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


def _small_batch():
    from ifrit_gb300 import scenes
    return scenes.c3_batch(seed=3, num_views=5, sizes=(48, 64), tri_range=(200, 800))


def _render_views(views):
    from oracle import oracle as O
    out = []
    for v in views:
        d = O.make_draw(v["vertices"], v["indices"], v["mvp"], attr_offset=3, attr_count=v["vertices"].shape[1] - 3,
                        cull_mode=v["cull"], depth_func=3)
        r = O.render([d], v["width"], v["height"], v["samples"])
        out.append((r["color"], r["depth"], r["vis"]))
    return out


def _small_diff():
    from ifrit_gb300 import scenes
    from oracle import diff_oracle as D
    sc = scenes.c4_scene(seed=6, num_views=5, size=48, subdivisions=2, tex_size=16)
    f, mv, W, H = sc["faces"], sc["mvps"], sc["width"], sc["height"]
    nb = D.neighbors(f)
    vis_c = D.raster_visibility(sc["clean"], f, mv, W, H)
    codes_c = D.decisions(sc["clean"], f, nb, mv, vis_c)
    vis = D.raster_visibility(sc["noisy"], f, mv, W, H)
    codes = D.decisions(sc["noisy"], f, nb, mv, vis)
    return sc, vis_c, codes_c, vis, codes


def _adjoint(sc, vis_c, codes_c, vis, codes, b, e):
    """FP64 adjoint of views [b, e) of the L2 loss against the clean renders."""
    from oracle import diff_oracle as D
    f, mv, tex = sc["faces"], sc["mvps"][b:e], sc["texture"]
    as64 = lambda x: torch.as_tensor(np.asarray(x, np.float64))  # noqa: E731
    with torch.no_grad():
        target = D.forward(as64(sc["clean"]), as64(sc["colors"]), as64(sc["uvs"]), tex, f, mv, vis_c[b:e], codes_c[b:e])
        img = D.forward(as64(sc["noisy"]), as64(sc["colors"]), as64(sc["uvs"]), tex, f, mv, vis[b:e], codes[b:e])
    return D.adjoint(sc["noisy"], sc["colors"], sc["uvs"], tex, f, mv, vis[b:e], codes[b:e],
                     (2 * (img - target)).numpy())


def _render_worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        views = _small_batch()
        b, e = view_range(len(views), rank, world)
        mine = _render_views(views[b:e])
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)  # the host gather of a sharded batch's images
        if rank == 0:
            out["images"] = [img for part in gathered for img in part]
        sc, vis_c, codes_c, vis, codes = _small_diff()
        b, e = view_range(len(sc["mvps"]), rank, world)
        grads = [torch.from_numpy(np.ascontiguousarray(g)) for g in _adjoint(sc, vis_c, codes_c, vis, codes, b, e)]
        allreduce_gradients(grads)
        out[rank] = [g.numpy() for g in grads]
    finally:
        dist.destroy_process_group()


def test_sharded_batch_and_adjoint_equal_unsharded():
    """Two gloo ranks each take their view range (view_range): the images they render with the CPU
    oracle, gathered on rank 0, equal the unsharded batch's; and their FP64 adjoints of the
    differentiable loss, summed by allreduce_gradients, equal the adjoint over all views."""
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_render_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    want = _render_views(_small_batch())
    got = out["images"]
    assert len(got) == len(want) == 5
    for (cg, dg, vg), (cw, dw, vw) in zip(got, want):
        assert np.array_equal(cg, cw) and np.array_equal(dg.view(np.uint32), dw.view(np.uint32))
        assert np.array_equal(vg, vw) and (vw >= 0).any()
    sc, vis_c, codes_c, vis, codes = _small_diff()
    full = _adjoint(sc, vis_c, codes_c, vis, codes, 0, len(sc["mvps"]))
    for r in range(world):
        for g, w in zip(out[r], full):
            assert np.allclose(g, w, rtol=1e-10, atol=1e-12)
        assert np.abs(out[r][0]).max() > 0
