"""Known-answer tests of the CPU oracle itself (fill rule, MSAA patterns, depth functions,
clipping, texture arithmetic, format conversions).  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from ifrit_gb300 import scenes

EYE = np.eye(4, dtype=np.float32)


def tri_vertices(pos, col=None):
    pos = np.asarray(pos, np.float32)
    col = np.ones((len(pos), 3), np.float32) if col is None else np.asarray(col, np.float32)
    return np.concatenate([pos, col], 1)


def test_shared_edge_covers_each_sample_once():
    # a quad split along its diagonal, both halves drawn with ALWAYS: every covered sample
    # belongs to exactly one half (top-left rule), including samples exactly on the diagonal
    v = tri_vertices([[-1, -1, 0.5], [1, -1, 0.5], [1, 1, 0.5], [-1, 1, 0.5]])
    for S in (1, 4, 8):
        cnt = np.zeros((32, 32, S), np.int64)
        for tri in ([0, 1, 2], [0, 2, 3]):
            d = O.make_draw(v, np.array([tri], np.int32), EYE, depth_func=7, cull_mode=0)
            out = O.render([d], 32, 32, S)
            cnt += out["vis"] >= 0
        assert cnt.max() == 1 and cnt.min() == 1


def test_fan_of_triangles_is_watertight():
    # 16 triangles around a centre point: every sample in the disc is covered exactly once
    n = 16
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    pos = [[0.013, -0.021, 0.5]] + [[0.9 * np.cos(a), 0.9 * np.sin(a), 0.5] for a in ang]
    idx = np.array([[0, 1 + i, 1 + (i + 1) % n] for i in range(n)], np.int32)
    v = tri_vertices(pos)
    cnt = np.zeros((64, 64, 4), np.int64)
    for t in range(n):
        d = O.make_draw(v, idx[t:t + 1], EYE, depth_func=7, cull_mode=0)
        cnt += O.render([d], 64, 64, 4)["vis"] >= 0
    assert cnt.max() == 1
    # and as one draw: the visible id set covers the same samples
    d = O.make_draw(v, idx, EYE, depth_func=7, cull_mode=0)
    vis = O.render([d], 64, 64, 4)["vis"]
    assert ((vis >= 0) == (cnt == 1)).all()


def test_msaa_sample_pattern_single_pixel():
    # a rectangle covering pixel column x in [0, 0.5] px of a 16x16 target: at 4x exactly the
    # samples left of the pixel centre are covered; the right edge (x = 0.5 px, interior to
    # its left) is not a top-left edge, so a sample on it would not be covered
    W = 16
    x0, x1 = -1.0, -1.0 + 2 * 0.5 / W
    v = tri_vertices([[x0, -1.2, 0.5], [x1, -1.2, 0.5], [x1, 1.2, 0.5], [x0, 1.2, 0.5]])
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    d = O.make_draw(v, idx, EYE, depth_func=7, cull_mode=0)
    for S in (4, 8, 16):
        vis = O.render([d], W, W, S)["vis"]
        for k, (sx, sy) in enumerate(ctypes_positions(S)):
            assert (vis[5, 0, k] >= 0) == (sx < 128), (S, k, sx, sy)
        assert (vis[:, 1:] < 0).all()


def ctypes_positions(S):
    import ctypes
    xs = (ctypes.c_int * 16)()
    ys = (ctypes.c_int * 16)()
    O.lib().ofx_sample_positions(S, 0, xs, ys)
    return [(xs[k], ys[k]) for k in range(S)]


def test_sample_patterns_are_the_standard_ones():
    assert ctypes_positions(1) == [(128, 128)]
    assert ctypes_positions(4) == [(96, 32), (224, 96), (32, 160), (160, 224)]
    p8 = ctypes_positions(8)
    assert len(set(p8)) == 8 and all(0 <= x < 256 and 0 <= y < 256 for x, y in p8)


@pytest.mark.parametrize("func,expect", [(1, 0), (3, 1), (4, 0), (6, 1), (7, 1), (2, 1), (0, -1)])
def test_depth_function_tie_break(func, expect):
    # two coincident triangles at the same depth: strict LESS/GREATER keep the first,
    # LEQUAL/GEQUAL/EQUAL/ALWAYS the last, NEVER none
    v = tri_vertices([[-0.8, -0.8, 0.4], [0.8, -0.8, 0.4], [0.0, 0.8, 0.4]])
    idx = np.array([[0, 1, 2], [0, 1, 2]], np.int32)
    d = O.make_draw(v, idx, EYE, depth_func=func, cull_mode=0)
    clear_depth = 0.4 if func == 2 else (0.0 if func in (4, 6) else 1.0)
    out = O.render([d], 16, 16, 1, clear_depth=clear_depth)
    assert out["vis"][8, 8, 0] == expect


def test_depth_test_order_independent_visibility():
    # random overlapping soup: the visible id per sample equals the argmin over (depth, id)
    rng = np.random.default_rng(3)
    pos = rng.uniform(-1, 1, (60, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(0.1, 0.9, 60)
    v = tri_vertices(pos)
    idx = np.arange(60, dtype=np.int32).reshape(-1, 3)
    d = O.make_draw(v, idx, EYE, depth_func=1, cull_mode=0)
    base = O.render([d], 48, 48, 4)
    perm = rng.permutation(len(idx))
    # render each triangle alone, then combine with the LESS/earliest rule
    best_d = np.full((48, 48, 4), 1.0, np.float32)
    best_i = np.full((48, 48, 4), -1, np.int64)
    for t in perm:
        dd = O.make_draw(v, idx[t:t + 1], EYE, depth_func=7, cull_mode=0, prim_base=int(t))
        o = O.render([dd], 48, 48, 4)
        cov = o["vis"] >= 0
        z = o["depth"]
        better = cov & ((z < best_d) | ((z == best_d) & (best_i >= 0) & (t < best_i)))
        better &= ~(cov & (z == best_d) & (best_i < 0))
        best_d = np.where(better, z, best_d)
        best_i = np.where(better, t, best_i)
    assert (best_i == base["vis"]).all()
    assert (best_d == base["depth"]).all()


def test_near_plane_clipping_keeps_visible_part():
    # a triangle crossing the camera plane renders its in-front part without NaNs
    mvp = scenes.default_mvp(1.0)
    v = tri_vertices([[-1.0, -0.5, 0.0], [1.0, -0.5, 0.0], [0.0, 0.3, 5.0]])  # last vertex behind the eye
    d = O.make_draw(v, np.array([[0, 1, 2]], np.int32), mvp, cull_mode=0)
    out = O.render([d], 64, 64, 1, fmt=O.FMT_RGBA32F)
    cov = out["vis"][..., 0] >= 0
    assert cov.sum() > 100
    assert np.isfinite(out["depth"][cov]).all()
    assert (out["depth"][cov] >= -1e-6).all() and (out["depth"][cov] <= 1 + 1e-6).all()


def test_cull_modes():
    v = tri_vertices([[-0.5, -0.5, 0.5], [0.5, -0.5, 0.5], [0.0, 0.5, 0.5]])
    ccw = np.array([[0, 1, 2]], np.int32)
    cw = ccw[:, [0, 2, 1]]
    for cull, ccw_vis, cw_vis in ((0, True, True), (1, False, True), (2, True, False), (3, False, False)):
        for idx, want in ((ccw, ccw_vis), (cw, cw_vis)):
            d = O.make_draw(v, idx, EYE, cull_mode=cull, front_ccw=1)
            assert (O.render([d], 16, 16)["vis"] >= 0).any() == want


def test_log2_accuracy():
    xs = np.concatenate([np.exp(np.linspace(-80, 80, 4001)), [1.0, 2.0, 0.5, 3.0, 1e-40, 1e30]]).astype(np.float32)
    got = np.array([O.lib().ofx_log2(float(x)) for x in xs], np.float64)
    ref = np.log2(xs.astype(np.float64))
    assert np.max(np.abs(got - ref)) < 2e-5
    assert O.lib().ofx_log2(1.0) == 0.0 and O.lib().ofx_log2(8.0) == 3.0


def test_f16_conversion_matches_numpy():
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.normal(size=2000) * 10.0 ** rng.integers(-8, 6, 2000),
                           [0.0, -0.0, 65504.0, 65520.0, 1e10, -1e10, 6e-8, 3e-8, 5.96e-8, np.inf, -np.inf]]).astype(np.float32)
    got = np.array([O.lib().ofx_f32_to_f16(float(v)) for v in vals], np.uint16)
    ref = vals.astype(np.float16).view(np.uint16)
    assert (got == ref).all()


def test_mip_chain_box_filter():
    rng = np.random.default_rng(1)
    lv0 = rng.integers(0, 2 ** 32, size=(6, 10), dtype=np.uint64).astype(np.uint32)
    chain, levels = O.build_mips(lv0)
    assert levels == 5  # 10x6 -> 5x3 -> 3x2 -> 2x1 -> 1x1
    ch = lv0.view(np.uint8).reshape(6, 10, 4).astype(np.int64)
    l1 = chain[60:75].view(np.uint8).reshape(3, 5, 4).astype(np.int64)
    exp = np.zeros((3, 5, 4), np.int64)
    for y in range(3):
        for x in range(5):
            ys, xs = [2 * y, min(2 * y + 1, 5)], [2 * x, min(2 * x + 1, 9)]
            s = sum(ch[yy, xx] for yy in ys for xx in xs)
            exp[y, x] = (s + 2) >> 2
    assert (l1 == exp).all()


def test_texture_constant_and_lod():
    lv0 = np.full((64, 64), 0xFF336699, np.uint32)
    chain, levels = O.build_mips(lv0)
    tex = O.Texture()
    import ctypes
    tex.texels = chain.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    tex.width, tex.height, tex.levels = 64, 64, levels
    for aniso in (1, 8):
        s = O.Sampler(0, 0, 1, 0, aniso, 0.0)
        out = (ctypes.c_float * 4)()
        O.lib().ofx_sample_texture(ctypes.byref(tex), ctypes.byref(s), 0.3, 0.7, 0.05, 0.0, 0.0, 0.004, out)
        assert np.allclose(list(out), [0x99 / 255, 0x66 / 255, 0x33 / 255, 1.0], atol=1e-6)


def test_scissor_rectangles_inclusive_bounds():
    # full-screen quad; scissor (2.5, 1, 3, 2): pixels with 2.5 <= x <= 5.5 and 1 <= y <= 3, i.e.
    # x in 3..5 and y in 1..3 (the reference's inclusive float test); a second rectangle adds
    # pixel column 7; enabled with no rectangle keeps everything
    v = tri_vertices([[-1, -1, 0.5], [1, -1, 0.5], [1, 1, 0.5], [-1, 1, 0.5]])
    f = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    d = O.make_draw(v, f, EYE, depth_func=7, cull_mode=0, scissor=[(2.5, 1.0, 3.0, 2.0)])
    vis = O.render([d], 8, 6, 1)["vis"][..., 0] >= 0
    want = np.zeros((6, 8), bool)
    want[1:4, 3:6] = True
    assert (vis == want).all()
    d = O.make_draw(v, f, EYE, depth_func=7, cull_mode=0, scissor=[(2.5, 1.0, 3.0, 2.0), (7.0, 0.0, 0.0, 5.0)])
    vis = O.render([d], 8, 6, 4)["vis"] >= 0
    want[0:6, 7] = True
    assert (vis == want[..., None]).all()
    d = O.make_draw(v, f, EYE, depth_func=7, cull_mode=0, scissor=[])
    assert (O.render([d], 8, 6, 1)["vis"] >= 0).all()


def _px_to_ndc(pts, W, H):
    return [[(x / W) * 2 - 1, (y / H) * 2 - 1, 0.5] for x, y in pts]


def test_point_mode_covers_the_pixel_of_each_vertex():
    W, H = 16, 12
    pts = [(2.3, 3.6), (12.7, 2.2), (6.4, 9.8)]
    v = tri_vertices(_px_to_ndc(pts, W, H))
    d = O.make_draw(v, np.array([[0, 1, 2]], np.int32), EYE, depth_func=7, cull_mode=0, polygon_mode=O.POLY_POINT)
    vis = O.render([d], W, H, 1)["vis"][..., 0] >= 0
    want = np.zeros((H, W), bool)
    for x, y in pts:
        want[int(y), int(x)] = True
    assert (vis == want).all()


def test_line_mode_one_pixel_per_column_along_an_x_major_edge():
    W, H = 32, 24
    pts = [(2.3, 5.6), (20.7, 7.1), (11.0, 22.0)]
    v = tri_vertices(_px_to_ndc(pts, W, H))
    d = O.make_draw(v, np.array([[0, 1, 2]], np.int32), EYE, depth_func=7, cull_mode=0, polygon_mode=O.POLY_LINE)
    vis = O.render([d], W, H, 1)["vis"][..., 0] >= 0
    # rows 0..9 near the top edge only hold that edge between columns 5 and 17
    col = vis[:10, 5:18].sum(0)
    assert (col == 1).all(), col
    # the interior of the triangle is not filled
    assert not vis[14, 10:13].any()
    # and the lines are there at 4x too, with every pixel they touch holding at least one sample
    vis4 = O.render([d], W, H, 4)["vis"] >= 0
    assert vis4[:10, 5:18].any(axis=2).sum(0).min() >= 1


def test_row_band_render_matches_full_frame():
    """Rendering only rows [y0, y1) of a frame (every triangle set up, only the band rasterised)
    reproduces those rows of the full render exactly, for a deferred and a blended pass."""
    from ifrit_gb300 import scenes
    v, f, mvp = scenes.triangle_soup(20000, 4, 320, 200)
    opaque = O.make_draw(v, f[:10000], mvp, attr_offset=3, attr_count=2, cull_mode=0, depth_func=3)
    blended = O.make_draw(v, f[10000:], mvp, attr_offset=3, attr_count=2, cull_mode=0, depth_func=3, depth_write=0,
                          blend=(6, 7, 1, 7), prim_base=10000)
    for draws in ([opaque], [opaque, blended]):
        full = O.render(draws, 320, 200, 4, nthreads=4)
        for y0, y1 in ((0, 64), (70, 134), (199, 200)):
            band = O.render(draws, 320, 200, 4, nthreads=3, rows=(y0, y1))
            for k in ("color", "depth", "vis"):
                assert np.array_equal(full[k][y0:y1].view(np.uint8), band[k].view(np.uint8)), (k, y0, y1)
