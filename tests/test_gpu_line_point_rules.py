"""The reference's own line and point pipelines (iftrSetPolygonRules REFERENCE, restated from
TileRasterCoreInvocationCuda.cu:2780-3334) against the oracle's restatement of the same rules:
visibility and depth bit-exact, colour within one RGBA8 step (1e-5 relative for float targets).

Cases: points and lines of a jittered icosphere and of a random soup (some vertices behind the
camera, so line endpoints are moved to w = 1 and points are skipped), Gouraud and primitive-id
shading, RGBA8 and RGBA32F targets, a non-square target, a draw without clear over a filled
frame (the strict depth test against the buffer), and the unsupported combinations.
"""
import os

import numpy as np
import pytest

import ifrit_gb300 as ig
from ifrit_gb300 import scenes
from oracle import oracle as O
from tests.gpu_harness import FMT_TO_ORACLE, assert_parity

pytestmark = pytest.mark.gpu


def _scene(kind):
    if kind == "icosphere":
        v, f = scenes.jittered_icosphere(3, 9)
        return v, f, scenes.default_mvp(160 / 120), 3
    rng = np.random.default_rng(12)
    n = 600
    pos = rng.uniform(-1.5, 1.5, (3 * n, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(-4.0, 1.2, 3 * n)  # some vertices behind the camera at z = 1
    col = rng.uniform(0, 1, (3 * n, 4)).astype(np.float32)
    v = np.concatenate([pos, col], 1)
    f = np.arange(3 * n, dtype=np.int32).reshape(-1, 3)
    proj = scenes.perspective(60.0, 160 / 120, 0.1, 100.0)
    view = scenes.look_at((0.0, 0.0, 1.0), (0.0, 0.0, -1.0))
    return v, f, (proj @ view).astype(np.float32), 4


def _both(kind, mode, W=160, H=120, fmt=ig.FORMAT_RGBA8, shading=ig.FS_GOURAUD, prefill=False):
    v, f, mvp, attr = _scene(kind)
    r = ig.Renderer(W, H, 1, fmt, visibility=True)
    r.set_state(cull=ig.CULL_BACK, depth_func=ig.LESS_OR_EQUAL, shading=shading)
    r.set_mvp(mvp)
    r.set_geometry(v, f, attr)
    ofmt = FMT_TO_ORACLE[fmt]
    color = depth = None
    if prefill:  # a filled frame first, then the line / point draw without clear over it
        r.draw(clear=True)
        pre = O.render([O.make_draw(v, f, mvp, attr_offset=3, attr_count=attr, cull_mode=2, depth_func=3,
                                    shading=shading)], W, H, 1, ofmt, clear=True)
        color, depth = pre["color"], pre["depth"]
    r.set_polygon_mode(mode, rules=ig.POLYGON_RULES_REFERENCE)
    r.draw(clear=not prefill)
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=attr, cull_mode=2, depth_func=3, shading=shading,
                    polygon_mode=mode, polygon_rules=1)
    ref = O.render([d], W, H, 1, ofmt, clear=not prefill, color=color, depth=depth)
    if prefill:  # the oracle's visibility output covers only this draw; take the GPU's earlier ids where kept
        keep = ref["vis"] < 0
        ref["vis"] = np.where(keep, gpu["vis"], ref["vis"])
    r.close()
    return gpu, ref


@pytest.mark.parametrize("kind", ["icosphere", "soup"])
@pytest.mark.parametrize("mode", [ig.POLYGON_LINE, ig.POLYGON_POINT])
def test_reference_rules_match_oracle(kind, mode):
    gpu, ref = _both(kind, mode)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).sum() > (40 if mode == ig.POLYGON_POINT else 300)


@pytest.mark.parametrize("mode", [ig.POLYGON_LINE, ig.POLYGON_POINT])
def test_reference_rules_float_target_primitive_ids_non_square(mode):
    gpu, ref = _both("soup", mode, W=200, H=96, fmt=ig.FORMAT_RGBA32F, shading=ig.FS_PRIMITIVE_ID)
    assert_parity(gpu, ref, fmt=ig.FORMAT_RGBA32F)


def test_reference_rules_over_filled_frame_without_clear():
    gpu, ref = _both("icosphere", ig.POLYGON_LINE, prefill=True)
    assert_parity(gpu, ref)


def test_reference_rules_unsupported_combinations():
    v, f, mvp, attr = _scene("icosphere")
    r = ig.Renderer(64, 64, 4, ig.FORMAT_RGBA8, visibility=True)
    r.set_mvp(mvp)
    r.set_geometry(v, f, attr)
    r.set_polygon_mode(ig.POLYGON_LINE, rules=ig.POLYGON_RULES_REFERENCE)
    with pytest.raises(ig.IfritError):  # multisampled target
        r.draw(clear=True)
    r.close()
