"""Pins the CPU oracle against the reference renderer's own outputs.

The fixtures in tests/golden/ were produced by the reference's multithreaded CPU tile
rasterizer (projects/softgraphics/src/engine/tileraster/, built by oracle/build_ref.py;
generator: tests/golden/make_golden.py).  The oracle runs in its reference-compatibility
mode (1x sample at the pixel corner, as TileRasterWorker.cpp:1186-1203 samples integer
pixel coordinates; depth LESS; back faces culled; clear depth 0x7f7f7f7f).

What must agree, and how:
  * visibility: every pixel whose visible primitive differs has its sample point within
    0.05 px of an edge of one of the two triangles: float edge functions with an epsilon
    bias and no fill rule vs 16.8 fixed point with a top-left rule disagree only there;
  * depth: where both pick the same primitive, the oracle's depth is within 1e-5
    (relative) of the float64 plane through the vertices snapped to 1/256 pixel, and the
    reference's within 2e-3 of the oracle's (median <= 1e-4): the reference interpolates
    through unsnapped float NDC vertices and loses precision on slivers;
  * colour: where both pick the same primitive, RGBA8 colour differs by at most one step on
    >= 99.5% of pixels (the reference interpolates with 12-bit reciprocal estimates).
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import geometry as G

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_*.npz")))
REF_CLEAR_DEPTH = float(np.frombuffer(np.uint32(0x7F7F7F7F).tobytes(), np.float32)[0])


def render_oracle(fx):
    v, f, mvp = fx["vertices"], fx["indices"], fx["mvp"]
    W, H = int(fx["width"]), int(fx["height"])
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=3, depth_func=1, cull_mode=2, front_ccw=1)
    return O.render([d], W, H, 1, O.FMT_RGBA8, clear=True, clear_color=(0, 0, 0, 0),
                    clear_depth=REF_CLEAR_DEPTH, compat=True)


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 9


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[4:-4] for p in GOLDEN])
def test_oracle_matches_reference(path):
    fx = np.load(path)
    v, f, mvp = fx["vertices"], fx["indices"], fx["mvp"]
    W, H = int(fx["width"]), int(fx["height"])
    out = render_oracle(fx)
    vis_o = out["vis"][..., 0]
    vis_r = fx["vis"]
    bad = G.mismatch_near_edges(vis_o, vis_r, v, f, mvp, W, H, tol=0.05)
    assert not bad, bad[:10]

    same = (vis_o == vis_r) & (vis_r >= 0)
    d_o = out["depth"][..., 0]
    d_r = fx["depth"]
    rel_ref = np.abs(d_o[same] - d_r[same]) / np.maximum(np.abs(d_r[same]), 1e-30)
    if same.any():
        assert rel_ref.max() <= 2e-3, rel_ref.max()
        assert np.median(rel_ref) <= 1e-4, np.median(rel_ref)
        ys, xs = np.nonzero(same)
        pick = np.random.default_rng(0).choice(len(ys), size=min(200, len(ys)), replace=False)
        for i in pick:
            y, x = ys[i], xs[i]
            ex = G.exact_depth(v, f, mvp, W, H, vis_o[y, x], float(x), float(y))
            assert abs(d_o[y, x] - ex) <= 1e-5 * max(abs(ex), 1e-3), (y, x, d_o[y, x], ex)

    c_o = out["color"].view(np.uint8).reshape(H, W, 4).astype(int)
    c_r = fx["rgba8"].astype(int)
    diff = np.abs(c_o - c_r).max(axis=-1)[same]
    if diff.size:
        assert (diff <= 1).mean() >= 0.995, (diff <= 1).mean()
    # background (uncovered by both): cleared colour
    bg = (vis_o < 0) & (vis_r < 0)
    assert (c_o[bg] == 0).all()
