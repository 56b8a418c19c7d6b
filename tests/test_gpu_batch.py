"""GPU parity of the batched form (iftrDrawBatch): views of uneven size, sample count and
triangle count rendered as one pass, each view compared with the oracle rendering that view
alone.  Visibility ids (view-local) and per-sample depth bit-exact, colour within one RGBA8
step, for both tile sizes, after autotuning, and on graph replays."""
import os

import numpy as np
import pytest

import ifrit_gb300 as ig
from ifrit_gb300 import scenes
from ifrit_gb300.batch import BatchRenderer
from oracle import oracle as O
from tests.gpu_harness import FMT_TO_ORACLE, assert_parity

pytestmark = pytest.mark.gpu
NTHREADS = os.cpu_count() or 1

# (width, height, samples, scene, seed, cull)
VIEWS = [
    (128, 128, 1, "ico", 1, ig.CULL_BACK),
    (200, 120, 4, "soup", 2, ig.CULL_NONE),
    (64, 48, 8, "soup", 3, ig.CULL_NONE),
    (256, 256, 4, "ico", 4, ig.CULL_BACK),
    (100, 70, 2, "soup", 5, ig.CULL_NONE),
    (130, 257, 1, "soup", 6, ig.CULL_NONE),
    (96, 96, 16, "ico", 7, ig.CULL_BACK),
    (333, 181, 4, "soup", 8, ig.CULL_NONE),
]


def _scene(kind, seed, W, H):
    if kind == "ico":
        v, f = scenes.jittered_icosphere(4, seed)
        return v, f, scenes.orbit_camera(np.random.default_rng(seed), 3.0, W / H)
    return scenes.triangle_soup(3000 + 1500 * seed, seed, W, H)


def _build(br, views=VIEWS, fmt=ig.FORMAT_RGBA8, extra=None):
    """Adds the views and one mesh per view (plus `extra` meshes: (view, v, f, mvp, kwargs))."""
    meshes = {}
    for i, (W, H, S, kind, seed, cull) in enumerate(views):
        br.add_view(W, H, S, fmt, visibility=True, clear=True, clear_color=(0.1, 0.2, 0.3, 1.0))
        v, f, mvp = _scene(kind, seed, W, H)
        br.add_mesh(i, v, f, mvp, attr_count=v.shape[1] - 3, cull=cull)
        meshes.setdefault(i, []).append((v, f, mvp, {"cull": cull}))
    for view, v, f, mvp, kw in extra or []:
        br.add_mesh(view, v, f, mvp, attr_count=v.shape[1] - 3, **kw)
        meshes.setdefault(view, []).append((v, f, mvp, kw))
    return meshes


def _oracle_view(W, H, S, meshes, fmt=ig.FORMAT_RGBA8, clear=True, color=None, depth=None):
    draws, base = [], 0
    for v, f, mvp, kw in meshes:
        od = O.make_draw(v, f, mvp, attr_offset=3, attr_count=v.shape[1] - 3, cull_mode=kw.get("cull", ig.CULL_BACK),
                         depth_func=kw.get("depth_func", ig.LESS_OR_EQUAL), depth_write=int(kw.get("depth_write", True)),
                         blend=kw.get("blend"), prim_base=base)
        draws.append(od)
        base += f.size // 3
    return O.render(draws, W, H, S, FMT_TO_ORACLE[fmt], clear=clear, clear_color=(0.1, 0.2, 0.3, 1.0),
                    clear_depth=1.0, nthreads=NTHREADS, color=color, depth=depth)


def _check_all(br, meshes, views=VIEWS):
    for i, (W, H, S, *_rest) in enumerate(views):
        gpu = {"color": br.color(i), "depth": br.depth(i), "vis": br.visibility(i)}
        ref = _oracle_view(W, H, S, meshes[i])
        assert_parity(gpu, ref)
        assert (gpu["vis"] >= 0).any(), "view %d is empty" % i


@pytest.mark.parametrize("tile_size", [16, 8])
def test_batch_matches_oracle_per_view(tile_size):
    br = BatchRenderer()
    br.set_tuning(autotune=False, tile_size=tile_size, ctas_per_sm=0)
    meshes = _build(br)
    br.draw()
    br.finish()
    assert br.tuning()[0] == tile_size
    _check_all(br, meshes)
    br.close()


def test_batch_autotuned_and_replayed():
    br = BatchRenderer()
    meshes = _build(br)
    br.draw()  # sizes, tunes, captures
    br.finish()
    assert br.tuning()[0] in (8, 16)
    _check_all(br, meshes)
    # replays of the captured graph: same result, and new vertex contents are picked up
    for t in br.views:
        t[1]["depth"].fill_(0.5)
        t[1]["color"].zero_()
    br.draw()
    br.finish()
    _check_all(br, meshes)
    v0, f0, mvp0, kw0 = meshes[3][0]
    moved = v0.copy()
    moved[:, :3] *= 0.8
    br.keep[3][0].copy_(br.to_device(moved, br.torch.float32))
    br.draw()
    br.finish()
    meshes[3][0] = (moved, f0, mvp0, kw0)
    _check_all(br, meshes)
    br.close()


def test_batch_multi_draw_views_blending_and_accumulation():
    """Views with several draws (opaque + blended: the ordered path) next to deferred views, then
    a second batch that draws on top of the first one's targets (clear = 0)."""
    W, H = 160, 128
    views = [(W, H, 1, "soup", 11, ig.CULL_NONE), (W, H, 4, "ico", 12, ig.CULL_BACK), (W, H, 1, "soup", 13, ig.CULL_NONE)]
    rng = np.random.default_rng(3)
    v, f, mvp = scenes.triangle_soup(4000, 14, W, H)
    col = rng.uniform(0, 1, (len(v), 4)).astype(np.float32)
    col[:, 3] = rng.uniform(0.2, 0.9, len(v))
    rgba = np.concatenate([v[:, :3], col], 1)
    extra = [(0, rgba, f, mvp, {"cull": ig.CULL_NONE, "blend": (6, 7, 1, 7), "depth_write": False}),
             (1, rgba, f[:1000], mvp, {"cull": ig.CULL_NONE})]
    br = BatchRenderer()
    meshes = _build(br, views, extra=extra)
    br.draw()
    br.finish()
    _check_all(br, meshes, views)
    first = [{"color": br.color(i), "depth": br.depth(i)} for i in range(len(views))]
    # second pass on top of the first (view 2 only, 1x so the resolved colour is the whole state)
    br2 = BatchRenderer()
    br2.add_view(W, H, 1, ig.FORMAT_RGBA8, visibility=True, clear=False)
    tgt = br2.target(0)
    tgt["color"].copy_(br2.torch.from_numpy(first[2]["color"].view(np.int32)).to(br2.device))
    tgt["depth"].copy_(br2.torch.from_numpy(first[2]["depth"]).to(br2.device))
    br2.add_mesh(0, rgba, f, mvp, attr_count=4, cull=ig.CULL_NONE, blend=(6, 7, 1, 7), depth_write=False)
    br2.draw()
    br2.finish()
    gpu = {"color": br2.color(0), "depth": br2.depth(0), "vis": br2.visibility(0)}
    ref = _oracle_view(W, H, 1, [(rgba, f, mvp, {"cull": ig.CULL_NONE, "blend": (6, 7, 1, 7), "depth_write": False})],
                       clear=False, color=first[2]["color"].copy(), depth=first[2]["depth"].copy())
    assert_parity(gpu, ref)
    br.close()
    br2.close()


def test_batch_rejects_bad_descriptions():
    br = BatchRenderer()
    br.add_view(64, 64, 3)  # 3 samples: not a valid count
    with pytest.raises(ig.IfritError) as e:
        br.draw()
    assert e.value.code == 1
    br.close()


def test_c3_style_batch_subset_matches_oracle():
    """Twelve views drawn from the batched benchmark's generator (1k-200k triangles per view,
    edges 128-1024, 1x/4x), autotuned, each view against the oracle."""
    views = scenes.c3_batch(seed=5, num_views=12)
    br = BatchRenderer()
    meshes = {}
    for k, v in enumerate(views):
        br.add_view(v["width"], v["height"], v["samples"], ig.FORMAT_RGBA8, visibility=True, clear=True,
                    clear_color=(0.1, 0.2, 0.3, 1.0))
        br.add_mesh(k, v["vertices"], v["indices"], v["mvp"], attr_count=v["vertices"].shape[1] - 3, cull=v["cull"])
        meshes[k] = [(v["vertices"], v["indices"], v["mvp"], {"cull": v["cull"]})]
    br.draw()
    br.finish()
    for k, v in enumerate(views):
        gpu = {"color": br.color(k), "depth": br.depth(k), "vis": br.visibility(k)}
        ref = _oracle_view(v["width"], v["height"], v["samples"], meshes[k])
        assert_parity(gpu, ref)
    br.close()
