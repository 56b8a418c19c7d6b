"""Deferred shading of ordered fragments: the ordered stage hands each tile's passing fragments to a
shading kernel and a per-pixel blending kernel; tiles that do not fit the fragment buffer, or that
have a pixel with more than 6 fragments, are finished by the ordered stage itself.  Every route must
give the same image, bit for bit, and match the oracle."""
import os

import numpy as np
import pytest

import ifrit_gb300 as ig
from ifrit_gb300 import scenes
from oracle import oracle as O
from tests.gpu_harness import FMT_TO_ORACLE, assert_parity

pytestmark = pytest.mark.gpu


def _stress_pass(capacity, seed=9, W=320, H=180):
    sc = scenes.c5_scene(seed=seed, instances=6, frequency=12, width=W, height=H, blended=0.34, tex_size=256,
                         target_complexity=2.0)
    r = ig.Renderer(W, H, 8, ig.FORMAT_RGBA16F, visibility=True)
    r.set_ordered_fragment_capacity(capacity)
    r.set_geometry(sc["vertices"], sc["indices"], 2)
    r.set_texture(sc["texture"], max_aniso=16)
    r.begin_pass(clear=True)
    for d in sc["draws"]:
        r.set_state(cull=ig.CULL_BACK, depth_func=ig.LESS_OR_EQUAL, depth_write=not d["blend"], shading=ig.FS_TEXTURED)
        r.set_blend(d["blend"], 6, 7, 1, 7)
        r.set_mvp(d["mvp"])
        r.pass_draw(d["first"], d["count"])
    r.end_pass()
    out = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    r.close()
    return out, sc


def _same(a, b):
    for k in ("color", "depth", "vis"):
        x, y = a[k].view(np.uint8), b[k].view(np.uint8)
        assert (x == y).all(), "%s differs at %d bytes" % (k, int((x != y).sum()))


def test_deferred_inline_and_partial_capacity_agree():
    deferred, sc = _stress_pass(-1)
    inline, _ = _stress_pass(0)
    partial, _ = _stress_pass(700)  # a few tiles fit, the rest are finished by the ordered stage
    _same(deferred, inline)
    _same(deferred, partial)
    # and the oracle
    chain, levels = O.build_mips(sc["texture"])
    tex = (chain, levels, sc["texture"].shape[1], sc["texture"].shape[0])
    odraws, base = [], 0
    for d in sc["draws"]:
        f = sc["indices"][d["first"] // 3:(d["first"] + d["count"]) // 3]
        odraws.append(O.make_draw(sc["vertices"], f, d["mvp"], attr_offset=3, attr_count=2, cull_mode=2, depth_func=3,
                                  depth_write=int(not d["blend"]), blend=(6, 7, 1, 7) if d["blend"] else None,
                                  shading=O.SHADE_TEXTURED, texture=tex, sampler={"max_aniso": 16}, prim_base=base))
        base += len(f)
    ref = O.render(odraws, sc["width"], sc["height"], 8, O.FMT_RGBA16F, clear=True, nthreads=os.cpu_count() or 1)
    assert_parity(deferred, ref, fmt=ig.FORMAT_RGBA16F)


def _layers_pass(capacity, S, first_blended):
    """Twelve overlapping blended layers of large triangles (a pixel gets up to 12 fragments: those
    tiles go to the redo list and are finished by the in-stage form, which applies some fragments on
    the spot) beside small blended triangles; with `first_blended` the pass has no order-independent
    prefix."""
    rng = np.random.default_rng(77)
    W, H = 96, 80
    verts, tris = [], []
    for i in range(12):
        z = -1.5 - 0.01 * i
        cx, cy = rng.uniform(-0.3, 0.3, 2)
        p = np.array([[cx - 1.2, cy - 1.0, z], [cx + 1.0, cy - 0.9, z], [cx - 0.1, cy + 1.1, z]], np.float32)
        c = rng.uniform(0, 1, (3, 4)).astype(np.float32)
        c[:, 3] = rng.uniform(0.2, 0.8, 3)
        tris.append([len(verts), len(verts) + 1, len(verts) + 2])
        verts.extend(np.concatenate([p, c], 1))
    for i in range(300):
        cx, cy = rng.uniform(-1, 1, 2)
        z = rng.uniform(-1.6, -1.3)
        p = np.array([[cx, cy, z], [cx + 0.1, cy, z], [cx, cy + 0.1, z]], np.float32)
        c = rng.uniform(0, 1, (3, 4)).astype(np.float32)
        tris.append([len(verts), len(verts) + 1, len(verts) + 2])
        verts.extend(np.concatenate([p, c], 1))
    v = np.array(verts, np.float32)
    f = np.array(tris, np.int32)
    mvp = scenes.perspective(60.0, W / H, 0.1, 50.0).astype(np.float32)
    r = ig.Renderer(W, H, S, ig.FORMAT_RGBA32F, visibility=True)
    r.set_ordered_fragment_capacity(capacity)
    r.set_geometry(v, f, 4)
    r.set_mvp(mvp)
    r.begin_pass(clear=True)
    split = 0 if first_blended else 100
    draws = [(0, split, False), (split, len(f), True)] if split else [(0, len(f), True)]
    odraws, base = [], 0
    for a, b, blend in draws:
        r.set_state(cull=ig.CULL_NONE, depth_func=ig.LESS_OR_EQUAL, depth_write=not blend, clear_color=(0.1, 0.2, 0.3, 1.0))
        r.set_blend(blend, 6, 7, 1, 7)
        r.pass_draw(3 * a, 3 * (b - a))
        odraws.append(O.make_draw(v, f[a:b], mvp, attr_offset=3, attr_count=4, cull_mode=0, depth_func=3,
                                  depth_write=int(not blend), blend=(6, 7, 1, 7) if blend else None, prim_base=base))
        base += b - a
    r.end_pass()
    out = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    r.close()
    ref = O.render(odraws, W, H, S, FMT_TO_ORACLE[ig.FORMAT_RGBA32F], clear=True, clear_color=(0.1, 0.2, 0.3, 1.0),
                   nthreads=os.cpu_count() or 1)
    return out, ref


@pytest.mark.parametrize("S,first_blended", [(1, False), (4, False), (4, True), (8, True)])
def test_many_layers_mixed_routes(S, first_blended):
    deferred, ref = _layers_pass(-1, S, first_blended)
    inline, _ = _layers_pass(0, S, first_blended)
    _same(deferred, inline)
    assert_parity(deferred, ref, fmt=ig.FORMAT_RGBA32F)


@pytest.mark.parametrize("S,blended", [(1, 4000), (4, 4000), (4, 10000)])
def test_dense_ordered_tiles_marking_and_batches(S, blended):
    """Hundreds of small blended triangles per 16x16 tile over an opaque prefix: batches of more
    than 64 records (candidates marked from the records' side) and tiles of more than 256 ordered
    entries (several batches), through the deferring form, the in-stage form and the oracle.  With
    10,000 blended triangles the busiest tiles hold more than the 2,048 ordered entries the deferring
    form sorts and go to the redo list whole."""
    rng = np.random.default_rng(91)
    W, H = 48, 40
    verts, tris = [], []
    for i in range(20):  # opaque prefix: large triangles behind
        cx, cy = rng.uniform(-0.5, 0.5, 2)
        z = rng.uniform(-3.0, -2.5)
        p = np.array([[cx - 1.5, cy - 1.5, z], [cx + 1.5, cy - 1.2, z], [cx, cy + 1.6, z]], np.float32)
        c = rng.uniform(0, 1, (3, 4)).astype(np.float32)
        c[:, 3] = 1.0
        tris.append([len(verts), len(verts) + 1, len(verts) + 2])
        verts.extend(np.concatenate([p, c], 1))
    for i in range(blended):  # blended: ~2-pixel triangles in front
        cx, cy = rng.uniform(-0.55, 0.55, 2)
        z = rng.uniform(-1.6, -1.2)
        p = np.array([[cx, cy, z], [cx + 0.05, cy, z], [cx, cy + 0.05, z]], np.float32)
        c = rng.uniform(0, 1, (3, 4)).astype(np.float32)
        tris.append([len(verts), len(verts) + 1, len(verts) + 2])
        verts.extend(np.concatenate([p, c], 1))
    v = np.array(verts, np.float32)
    f = np.array(tris, np.int32)
    mvp = scenes.perspective(60.0, W / H, 0.1, 50.0).astype(np.float32)
    outs = []
    for capacity in (-1, 0):
        r = ig.Renderer(W, H, S, ig.FORMAT_RGBA32F, visibility=True)
        r.set_ordered_fragment_capacity(capacity)
        r.set_geometry(v, f, 4)
        r.set_mvp(mvp)
        r.begin_pass(clear=True)
        odraws, base = [], 0
        for a, b, blend in ((0, 20, False), (20, len(f), True)):
            r.set_state(cull=ig.CULL_NONE, depth_func=ig.LESS_OR_EQUAL, depth_write=not blend,
                        clear_color=(0.1, 0.2, 0.3, 1.0))
            r.set_blend(blend, 6, 7, 1, 7)
            r.pass_draw(3 * a, 3 * (b - a))
            odraws.append(O.make_draw(v, f[a:b], mvp, attr_offset=3, attr_count=4, cull_mode=0, depth_func=3,
                                      depth_write=int(not blend), blend=(6, 7, 1, 7) if blend else None,
                                      prim_base=base))
            base += b - a
        r.end_pass()
        outs.append({"color": r.color(), "depth": r.depth(), "vis": r.visibility()})
        st = r.stats()
        r.close()
        if capacity == -1:
            assert st.tile_pairs > blended  # 4,000 blended: up to 1,600 ordered entries in one tile
    _same(outs[0], outs[1])
    ref = O.render(odraws, W, H, S, FMT_TO_ORACLE[ig.FORMAT_RGBA32F], clear=True, clear_color=(0.1, 0.2, 0.3, 1.0),
                   nthreads=os.cpu_count() or 1)
    assert_parity(outs[0], ref, fmt=ig.FORMAT_RGBA32F)
