"""GPU parity: the sm_103a path (through the C-ABI) against the CPU oracle on the same seeded
inputs.  Visibility ids and per-sample depth must be bit-exact; colour within one RGBA8 step
(one half-float ulp for RGBA16F, 1e-5 relative for FP32 targets)."""
import glob
import os

import numpy as np
import pytest

import ifrit_gb300 as ig
from ifrit_gb300 import scenes
from tests.gpu_harness import assert_parity, render_both

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_*.npz")))


def soup(n, seed, W, H, **kw):
    return scenes.triangle_soup(n, seed, W, H, **kw)


def test_plain_frame_c1_512():
    v, f, mvp = scenes.c1_scene(1)
    gpu, ref, _ = render_both(v, f, mvp, 512, 512, depth_func=ig.LESS_OR_EQUAL)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).sum() > 50000


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[4:-4] for p in GOLDEN])
@pytest.mark.parametrize("S", [1, 4])
def test_known_answer_scenes(path, S):
    fx = np.load(path)
    W, H = int(fx["width"]), int(fx["height"])
    gpu, ref, _ = render_both(fx["vertices"], fx["indices"], fx["mvp"], W, H, S=S, depth_func=ig.LESS)
    assert_parity(gpu, ref)


@pytest.mark.parametrize("S", [1, 2, 4, 8, 16])
def test_msaa_soup(S):
    v, f, mvp = soup(20000, 5, 256, 192)
    v6 = np.concatenate([v[:, :3], np.abs(v[:, 3:5]) % 1.0, np.full((len(v), 1), 0.5, np.float32)], 1)
    gpu, ref, _ = render_both(v6, f, mvp, 256, 192, S=S, cull=ig.CULL_NONE, depth_func=ig.LESS)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).mean() > 0.5


@pytest.mark.parametrize("func", [ig.NEVER, ig.LESS, ig.EQUAL, ig.LESS_OR_EQUAL, ig.GREATER,
                                  ig.GREATER_OR_EQUAL, ig.ALWAYS])
def test_depth_functions_with_duplicates(func):
    # duplicated triangles make every depth comparison tie somewhere
    v, f, mvp = soup(3000, 9, 128, 96)
    f = np.concatenate([f, f[::3]], 0)
    v6 = np.concatenate([v[:, :3], np.abs(v[:, 3:5]) % 1.0, np.full((len(v), 1), 0.25, np.float32)], 1)
    clear_depth = 0.0 if func in (ig.GREATER, ig.GREATER_OR_EQUAL) else 1.0
    gpu, ref, _ = render_both(v6, f, mvp, 128, 96, S=4, cull=ig.CULL_NONE, depth_func=func, clear_depth=clear_depth)
    assert_parity(gpu, ref)


def test_depth_write_disabled_and_test_disabled():
    v, f, mvp = soup(3000, 10, 128, 96)
    v6 = np.concatenate([v[:, :3], np.abs(v[:, 3:5]) % 1.0, np.full((len(v), 1), 0.75, np.float32)], 1)
    gpu, ref, _ = render_both(v6, f, mvp, 128, 96, S=4, cull=ig.CULL_NONE, depth_func=ig.LESS, depth_write=False)
    assert_parity(gpu, ref)
    gpu, ref, _ = render_both(v6, f, mvp, 128, 96, S=1, cull=ig.CULL_NONE, depth_func=ig.LESS, depth_test=False)
    assert_parity(gpu, ref)


@pytest.mark.parametrize("cull,front_ccw", [(ig.CULL_NONE, True), (ig.CULL_FRONT, True), (ig.CULL_BACK, False),
                                            (ig.CULL_FRONT_AND_BACK, True)])
def test_cull_modes(cull, front_ccw):
    v, f, mvp = soup(4000, 11, 128, 128)
    v6 = np.concatenate([v[:, :3], np.abs(v[:, 3:5]) % 1.0, np.full((len(v), 1), 0.5, np.float32)], 1)
    gpu, ref, _ = render_both(v6, f, mvp, 128, 128, cull=cull, front_ccw=front_ccw, depth_func=ig.LESS)
    assert_parity(gpu, ref)


def test_clipping_near_plane_and_guard_band():
    # camera inside a large jittered sphere plus triangles far outside the guard band
    v, f = scenes.jittered_icosphere(3, 4, jitter=0.1)
    v = v.copy()
    v[:, :3] *= 3.0
    mvp = (scenes.perspective(70.0, 1.25, 0.1, 50.0) @ scenes.look_at((0.3, 0.2, 0.1), (0, 0, -1))).astype(np.float32)
    gpu, ref, _ = render_both(v, f, mvp, 160, 128, S=4, cull=ig.CULL_NONE, depth_func=ig.LESS)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).mean() > 0.9
    big = np.array([[-5000, -3000, -2.0, 1, 0, 0], [6000, -2000, -2.0, 0, 1, 0], [0, 7000, -2.5, 0, 0, 1],
                    [-0.2, -0.2, -1.0, 1, 1, 0], [0.3, -0.1, -1.0, 0, 1, 1], [0.0, 0.4, -1.0, 1, 0, 1]], np.float32)
    fi = np.array([[0, 1, 2], [3, 4, 5]], np.int32)
    mvp2 = scenes.perspective(60.0, 1.0, 0.1, 50.0).astype(np.float32)
    gpu, ref, _ = render_both(big, fi, mvp2, 96, 96, S=8, cull=ig.CULL_NONE, depth_func=ig.LESS)
    assert_parity(gpu, ref)


@pytest.mark.parametrize("fmt", [ig.FORMAT_RGBA16F, ig.FORMAT_RGBA32F, ig.FORMAT_RGB32F])
def test_float_targets(fmt):
    v, f, mvp = scenes.c1_scene(3)
    v = v.copy()
    v[:, 3:] *= 3.0  # values above 1 survive in float targets
    gpu, ref, _ = render_both(v, f, mvp, 192, 160, S=4, fmt=fmt)
    assert_parity(gpu, ref, fmt=fmt)


@pytest.mark.parametrize("aniso,address", [(1, 0), (8, 0), (16, 1), (4, 2)])
def test_textured_trilinear_anisotropic(aniso, address):
    v, f, mvp = soup(20000, 12, 256, 160)
    tex = scenes.value_noise_texture(256, 3)
    gpu, ref, _ = render_both(v, f, mvp, 256, 160, S=4, attr=2, cull=ig.CULL_NONE, depth_func=ig.LESS,
                              shading=ig.FS_TEXTURED, texture=tex, max_aniso=aniso, address=address)
    assert_parity(gpu, ref)


def _pinwheels(W, H, wedges=16, radius=2.7, seed=41):
    """Fans of `wedges` thin triangles around a centre inside a pixel, one every 6 pixels, at
    random sub-pixel offsets, depths and rotations (NDC positions, identity transform): the centre
    pixel's samples fall in up to min(S, wedges) different triangles."""
    rng = np.random.default_rng(seed)
    verts, tris = [], []
    for cy in range(3, H - 3, 6):
        for cx in range(3, W - 3, 6):
            ox, oy = rng.uniform(0.3, 0.7, 2)
            z = rng.uniform(-0.5, 0.5)
            rot = rng.uniform(0.0, 2.0 * np.pi)
            c = np.array([(cx + ox) / W * 2.0 - 1.0, (cy + oy) / H * 2.0 - 1.0, z])
            base = len(verts)
            verts.append(np.concatenate([c, rng.uniform(0, 1, 3)]))
            for i in range(wedges):
                a = rot + 2.0 * np.pi * i / wedges
                q = c + np.array([radius * np.cos(a) * 2.0 / W, radius * np.sin(a) * 2.0 / H, 0.0])
                verts.append(np.concatenate([q, rng.uniform(0, 1, 3)]))
            for i in range(wedges):
                tris.append([base, base + 1 + i, base + 1 + (i + 1) % wedges])
    return np.array(verts, np.float32), np.array(tris, np.int32), np.eye(4, dtype=np.float32)


@pytest.mark.parametrize("S", [8, 16])
@pytest.mark.parametrize("textured", [False, True])
def test_pixels_with_more_than_four_primitives(S, textured):
    """Pixels whose samples see more than the four primitives the shade stage shades together:
    the others are shaded per sample on the stage's out-of-line path."""
    W, H = 72, 54
    v, f, mvp = _pinwheels(W, H)
    kw = {}
    if textured:
        v = np.concatenate([v[:, :3], (v[:, :2] + 1.0) * 3.0], 1)
        kw = dict(attr=2, shading=ig.FS_TEXTURED, texture=scenes.value_noise_texture(128, 7), max_aniso=8)
    gpu, ref, _ = render_both(v, f, mvp, W, H, S=S, cull=ig.CULL_NONE, depth_func=ig.LESS, **kw)
    assert_parity(gpu, ref)
    vis = gpu["vis"].reshape(-1, S)
    distinct = np.array([len(set(r[r >= 0].tolist())) for r in vis])
    assert (distinct > 4).sum() >= 50


@pytest.mark.parametrize("aniso", [1, 8])
def test_textured_clipped_triangles(aniso):
    """Camera inside a textured sphere: the triangles crossing the near plane (95 of 1,280) are
    clipped into fan triangles whose set-up and vertex attributes take the general path in every
    stage (no triangle record), with anisotropic texture lookups on them."""
    v, f = scenes.jittered_icosphere(3, 9, jitter=0.1)
    v = v.copy()
    v[:, :3] *= 3.0
    uv = np.stack([0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi), 0.5 + v[:, 1] / 6.0], 1).astype(np.float32)
    vt = np.concatenate([v[:, :3], uv * 4.0], 1)
    mvp = (scenes.perspective(70.0, 1.25, 0.1, 50.0) @ scenes.look_at((0.3, 0.2, 0.1), (0, 0, -1))).astype(np.float32)
    tex = scenes.value_noise_texture(256, 5)
    gpu, ref, _ = render_both(vt, f, mvp, 160, 128, S=4, attr=2, cull=ig.CULL_NONE, depth_func=ig.LESS,
                              shading=ig.FS_TEXTURED, texture=tex, max_aniso=aniso, address=0)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).mean() > 0.9


def test_overflow_retry_gives_same_image():
    v, f, mvp = soup(20000, 13, 256, 160)
    v6 = np.concatenate([v[:, :3], np.abs(v[:, 3:5]) % 1.0, np.full((len(v), 1), 0.5, np.float32)], 1)
    r = ig.Renderer(256, 160, 4, ig.FORMAT_RGBA8, visibility=True)
    r.reserve(1000)  # forces the capacity-overflow path on the first attempt
    gpu, ref, r = render_both(v6, f, mvp, 256, 160, S=4, cull=ig.CULL_NONE, depth_func=ig.LESS, renderer=r)
    assert r.stats().retries >= 1
    assert_parity(gpu, ref)


def test_second_draw_without_clear_keeps_depth():
    v, f, mvp = soup(5000, 14, 128, 128)
    v6 = np.concatenate([v[:, :3], np.abs(v[:, 3:5]) % 1.0, np.full((len(v), 1), 0.5, np.float32)], 1)
    half = len(f) // 2
    r = ig.Renderer(128, 128, 1, ig.FORMAT_RGBA8, visibility=True)
    r.set_state(cull=ig.CULL_NONE, depth_func=ig.LESS)
    r.set_mvp(mvp)
    r.set_geometry(v6, f[:half], 3)
    r.draw(clear=True)
    r.set_geometry(v6, f[half:], 3)
    r.draw(clear=False)
    from oracle import oracle as O
    d1 = O.make_draw(v6, f[:half], mvp, cull_mode=0, depth_func=1)
    first = O.render([d1], 128, 128, 1)
    d2 = O.make_draw(v6, f[half:], mvp, cull_mode=0, depth_func=1)
    second = O.render([d2], 128, 128, 1, clear=False, color=first["color"], depth=first["depth"])
    assert (r.depth().view(np.uint32) == second["depth"].view(np.uint32)).all()
    cg, cr = r.color().view(np.uint8).astype(int), second["color"].view(np.uint8).astype(int)
    assert np.abs(cg - cr).max() <= 1


def test_full_size_textured_msaa_frame():
    """The benchmark frame at full size: 1M triangles, 1920x1080, 4x MSAA, trilinear + 8x
    anisotropic filtering of a 1024^2 value-noise texture."""
    v, f, mvp = scenes.c2_scene()
    tex = scenes.value_noise_texture(1024, 2)
    gpu, ref, _ = render_both(v, f, mvp, 1920, 1080, S=4, attr=2, cull=ig.CULL_NONE, depth_func=ig.LESS_OR_EQUAL,
                              shading=ig.FS_TEXTURED, texture=tex, max_aniso=8)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).mean() > 0.95


# ---------------------------------------------------------------- multi-draw passes, blending
def _pass_both(W, H, S, draws, fmt=ig.FORMAT_RGBA8, clear_color=(0.1, 0.2, 0.3, 1.0)):
    """draws: list of dicts(vertices, indices, mvp, attr, cull, depth_func, depth_write, blend, shading)
    sharing one vertex/index array each; renders them as one pass on both sides."""
    from oracle import oracle as O
    v = draws[0]["vertices"]
    allf = np.concatenate([d["indices"] for d in draws], 0)
    r = ig.Renderer(W, H, S, fmt, visibility=True)
    r.set_geometry(v, allf, draws[0]["attr"])
    r.set_state(cull=draws[0]["cull"], depth_func=draws[0]["depth_func"], clear_color=clear_color)
    r.begin_pass(clear=True)
    first, odraws, base = 0, [], 0
    for d in draws:
        r.set_state(cull=d["cull"], depth_func=d["depth_func"], depth_write=d.get("depth_write", True),
                    shading=d.get("shading", ig.FS_GOURAUD), clear_color=clear_color)
        r.set_mvp(d["mvp"])
        blend = d.get("blend")
        if blend:
            r.set_blend(True, *blend)
        else:
            r.set_blend(False)
        n = d["indices"].size
        r.pass_draw(first, n)
        od, keep = O.make_draw(v, d["indices"], d["mvp"], attr_offset=3, attr_count=d["attr"], cull_mode=d["cull"],
                               depth_func=d["depth_func"], depth_write=int(d.get("depth_write", True)),
                               blend=blend, shading=d.get("shading", 0), prim_base=base)
        odraws.append((od, keep))
        first += n
        base += n // 3
    r.end_pass()
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    from tests.gpu_harness import FMT_TO_ORACLE
    ref = O.render(odraws, W, H, S, FMT_TO_ORACLE[fmt], clear=True, clear_color=clear_color, clear_depth=1.0,
                   nthreads=os.cpu_count() or 1)
    return gpu, ref


def _rgba_soup(n, seed, W, H):
    v, f, mvp = soup(n, seed, W, H)
    rng = np.random.default_rng(seed)
    col = rng.uniform(0, 1, (len(v), 4)).astype(np.float32)
    col[:, 3] = rng.uniform(0.2, 0.9, len(v))
    return np.concatenate([v[:, :3], col], 1), f, mvp


@pytest.mark.parametrize("S", [1, 4, 8])
def test_multi_draw_instances_deferred(S):
    v, f, mvp = _rgba_soup(6000, 31, 160, 128)
    rng = np.random.default_rng(2)
    draws = []
    for i in range(4):
        m = mvp.copy()
        m[:, 3] += (rng.normal(size=4) * 0.05).astype(np.float32)
        draws.append(dict(vertices=v, indices=f[i * 1500:(i + 1) * 1500], mvp=m, attr=4, cull=0, depth_func=ig.LESS))
    gpu, ref = _pass_both(160, 128, S, draws)
    assert_parity(gpu, ref)


@pytest.mark.parametrize("S", [1, 4])
def test_alpha_blended_draws_in_order(S):
    v, f, mvp = _rgba_soup(6000, 32, 160, 128)
    draws = [dict(vertices=v, indices=f[:3000], mvp=mvp, attr=4, cull=0, depth_func=ig.LESS),
             dict(vertices=v, indices=f[3000:], mvp=mvp, attr=4, cull=0, depth_func=ig.LESS, depth_write=False,
                  blend=(6, 7, 1, 7))]
    gpu, ref = _pass_both(160, 128, S, draws)
    assert_parity(gpu, ref)


@pytest.mark.parametrize("factors", [(1, 1, 1, 1), (2, 3, 8, 9), (4, 5, 0, 1), (8, 9, 6, 7)])
def test_blend_factors(factors):
    v, f, mvp = _rgba_soup(3000, 33, 96, 80)
    draws = [dict(vertices=v, indices=f, mvp=mvp, attr=4, cull=0, depth_func=ig.ALWAYS, blend=factors)]
    gpu, ref = _pass_both(96, 80, 4, draws, fmt=ig.FORMAT_RGBA32F)
    assert_parity(gpu, ref, fmt=ig.FORMAT_RGBA32F)


def test_not_equal_and_mixed_depth_state_pass():
    v, f, mvp = _rgba_soup(4000, 34, 128, 96)
    f = np.concatenate([f, f[::4]], 0)
    draws = [dict(vertices=v, indices=f[:2000], mvp=mvp, attr=4, cull=0, depth_func=ig.LESS),
             dict(vertices=v, indices=f[2000:4000], mvp=mvp, attr=4, cull=0, depth_func=ig.NOT_EQUAL),
             dict(vertices=v, indices=f[4000:], mvp=mvp, attr=4, cull=0, depth_func=ig.GREATER_OR_EQUAL)]
    gpu, ref = _pass_both(128, 96, 4, draws)
    assert_parity(gpu, ref)


def test_stress_style_pass_small():
    """Every feature of the 4K stress configuration in one pass, at a size the oracle renders in
    seconds: RGBA16F, 8x MSAA, displaced geodesic instances with random transforms, 16x
    anisotropic texturing with a noise alpha, blended instances drawn last back to front."""
    from oracle import oracle as O
    sc = scenes.c5_scene(seed=9, instances=6, frequency=12, width=320, height=180, blended=0.34, tex_size=256,
                         target_complexity=2.0)
    W, H = sc["width"], sc["height"]
    assert sum(d["blend"] for d in sc["draws"]) == 2
    r = ig.Renderer(W, H, 8, ig.FORMAT_RGBA16F, visibility=True)
    r.set_geometry(sc["vertices"], sc["indices"], 2)
    r.set_texture(sc["texture"], max_aniso=16)
    r.begin_pass(clear=True)
    chain, levels = O.build_mips(sc["texture"])
    tex = (chain, levels, sc["texture"].shape[1], sc["texture"].shape[0])
    odraws, base = [], 0
    for d in sc["draws"]:
        r.set_state(cull=ig.CULL_BACK, depth_func=ig.LESS_OR_EQUAL, depth_write=not d["blend"], shading=ig.FS_TEXTURED)
        r.set_blend(d["blend"], 6, 7, 1, 7)
        r.set_mvp(d["mvp"])
        r.pass_draw(d["first"], d["count"])
        f = sc["indices"][d["first"] // 3:(d["first"] + d["count"]) // 3]
        odraws.append(O.make_draw(sc["vertices"], f, d["mvp"], attr_offset=3, attr_count=2, cull_mode=2, depth_func=3,
                                  depth_write=int(not d["blend"]), blend=(6, 7, 1, 7) if d["blend"] else None,
                                  shading=O.SHADE_TEXTURED, texture=tex, sampler={"max_aniso": 16}, prim_base=base))
        base += len(f)
    r.end_pass()
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    ref = O.render(odraws, W, H, 8, O.FMT_RGBA16F, clear=True, nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref, fmt=ig.FORMAT_RGBA16F)
    assert (gpu["vis"] >= 0).mean() > 0.5
    r.close()


def test_scissor_rectangles_single_and_multi_draw():
    """Scissor test per draw: a soup under two rectangles at 4x; then a pass whose draws carry
    different scissor state, one of them blended (in-order stage)."""
    from oracle import oracle as O
    W, H = 200, 150
    v, f, mvp = soup(8000, 31, W, H)
    rects = [(13.5, 20.0, 60.25, 40.0), (90.0, 70.5, 70.0, 60.0)]
    r = ig.Renderer(W, H, 4, ig.FORMAT_RGBA8, visibility=True)
    r.set_state(cull=ig.CULL_NONE, depth_func=ig.LESS_OR_EQUAL)
    r.set_mvp(mvp)
    r.set_geometry(v, f, 2)
    r.set_scissors(rects)
    r.draw(clear=True)
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=2, cull_mode=0, depth_func=3, scissor=rects)
    ref = O.render([d], W, H, 4, clear=True, nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref)
    inside = np.zeros((H, W), bool)
    inside[20:61, 14:74] = True
    inside[71:131, 90:161] = True
    assert not (gpu["vis"][~inside] >= 0).any() and (gpu["vis"][inside] >= 0).mean() > 0.5
    r.close()
    # multi-draw pass: opaque draw under one rectangle, opaque draw without scissor, blended draw
    # under another rectangle
    vr, fr, mvpr = _rgba_soup(6000, 32, W, H)
    half = len(fr) // 3
    r = ig.Renderer(W, H, 4, ig.FORMAT_RGBA8, visibility=True)
    r.set_geometry(vr, fr, 4)
    r.set_mvp(mvpr)
    r.begin_pass(clear=True)
    plan = [((0, 3 * half), [(10.0, 10.0, 100.0, 80.0)], None),
            ((3 * half, 3 * half), None, None),
            ((6 * half, 3 * (len(fr) - 2 * half)), [(50.0, 40.0, 120.0, 100.0)], (6, 7, 1, 7))]
    odraws, base = [], 0
    for (first, count), sc, blend in plan:
        r.set_state(cull=ig.CULL_NONE, depth_func=ig.LESS_OR_EQUAL, depth_write=blend is None,
                    clear_color=(0.1, 0.2, 0.3, 1.0))
        r.set_blend(blend is not None, *(blend or (6, 7, 1, 7)))
        r.set_scissors(sc or [], enable=sc is not None)
        r.pass_draw(first, count)
        sub = fr[first // 3:(first + count) // 3]
        odraws.append(O.make_draw(vr, sub, mvpr, attr_offset=3, attr_count=4, cull_mode=0, depth_func=3,
                                  depth_write=int(blend is None), blend=blend, scissor=sc, prim_base=base))
        base += len(sub)
    r.end_pass()
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    ref = O.render(odraws, W, H, 4, clear=True, clear_color=(0.1, 0.2, 0.3, 1.0), nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref)
    r.close()


@pytest.mark.parametrize("mode,S", [(ig.POLYGON_LINE, 1), (ig.POLYGON_LINE, 4), (ig.POLYGON_POINT, 1), (ig.POLYGON_POINT, 8)])
def test_polygon_modes_soup(mode, S):
    from oracle import oracle as O
    W, H = 160, 120
    v, f, mvp = soup(2000, 40 + S, W, H, median_px=12.0)
    r = ig.Renderer(W, H, S, ig.FORMAT_RGBA8, visibility=True)
    r.set_state(cull=ig.CULL_NONE, depth_func=ig.LESS_OR_EQUAL)
    r.set_polygon_mode(mode)
    r.set_mvp(mvp)
    r.set_geometry(v, f, 2)
    r.draw(clear=True)
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=2, cull_mode=0, depth_func=3, polygon_mode=mode)
    ref = O.render([d], W, H, S, clear=True, nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref)
    # something is drawn, and the 1-pixel points cover fewer samples than the filled triangles
    fill = O.render([O.make_draw(v, f, mvp, attr_offset=3, attr_count=2, cull_mode=0, depth_func=3)], W, H, S,
                    clear=True, nthreads=os.cpu_count() or 1)
    n_mode, n_fill = int((gpu["vis"] >= 0).sum()), int((fill["vis"] >= 0).sum())
    assert n_mode > 0 and (mode == ig.POLYGON_LINE or n_mode < n_fill)
    r.close()


def test_line_mode_icosphere_culled_and_textured():
    from oracle import oracle as O
    v, f = scenes.jittered_icosphere(3, 4)
    uv = np.stack([0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi), 0.5 + v[:, 1] / 2], 1).astype(np.float32)
    vt = np.concatenate([v[:, :3], uv], 1)
    mvp = scenes.default_mvp(4 / 3)
    tex = scenes.value_noise_texture(128, 3)
    W, H = 256, 192
    r = ig.Renderer(W, H, 4, ig.FORMAT_RGBA8, visibility=True)
    r.set_state(cull=ig.CULL_BACK, depth_func=ig.LESS_OR_EQUAL, shading=ig.FS_TEXTURED)
    r.set_polygon_mode(ig.POLYGON_LINE)
    r.set_mvp(mvp)
    r.set_geometry(vt, f, 2)
    r.set_texture(tex, max_aniso=4)
    r.draw(clear=True)
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    chain, levels = O.build_mips(tex)
    d = O.make_draw(vt, f, mvp, attr_offset=3, attr_count=2, cull_mode=2, depth_func=3, polygon_mode=O.POLY_LINE,
                    shading=O.SHADE_TEXTURED, texture=(chain, levels, 128, 128), sampler={"max_aniso": 4})
    ref = O.render([d], W, H, 4, clear=True, nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).any()
    r.close()


@pytest.mark.parametrize("case", ["soup1", "soup4", "soup8", "greater", "always", "textured", "icosphere",
                                  "scissor_lines"])
def test_atomic_visibility_path_matches_oracle(case):
    """The atomics-only raster path (no binning; per-triangle threads resolve global 64-bit keys)
    gives the tile path's image: visibility and depth bit-exact against the oracle."""
    from oracle import oracle as O
    W, H = 192, 144
    S, func, shading, tex, attr, cull, mode, sc = 4, ig.LESS_OR_EQUAL, ig.FS_GOURAUD, None, 2, ig.CULL_NONE, 0, None
    v, f, mvp = soup(15000, 50, W, H)
    if case == "soup1":
        S = 1
    elif case == "soup8":
        S = 8
    elif case == "greater":
        func = ig.GREATER
    elif case == "always":
        f = np.concatenate([f, f[::2]], 0)
        func = ig.ALWAYS
    elif case == "textured":
        shading, tex = ig.FS_TEXTURED, scenes.value_noise_texture(128, 9)
    elif case == "icosphere":
        v, f, mvp = scenes.c1_scene(2)
        attr, cull = 3, ig.CULL_BACK
    elif case == "scissor_lines":
        mode, sc = ig.POLYGON_LINE, [(20.5, 10.0, 90.0, 70.0)]
    r = ig.Renderer(W, H, S, ig.FORMAT_RGBA8, visibility=True)
    r.set_raster_path(ig.RASTER_ATOMIC)
    r.set_state(cull=cull, depth_func=func, shading=shading, clear_depth=0.0 if func == ig.GREATER else 1.0)
    r.set_polygon_mode(mode)
    if sc:
        r.set_scissors(sc)
    r.set_mvp(mvp)
    r.set_geometry(v, f, attr)
    tex_arg = None
    if tex is not None:
        r.set_texture(tex, max_aniso=8)
        chain, levels = O.build_mips(tex)
        tex_arg = (chain, levels, 128, 128)
    r.draw(clear=True)
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=attr, cull_mode=cull, depth_func=func, shading=shading,
                    texture=tex_arg, sampler={"max_aniso": 8}, polygon_mode=mode, scissor=sc)
    ref = O.render([d], W, H, S, clear=True, clear_depth=0.0 if func == ig.GREATER else 1.0,
                   nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).any()
    r.close()


@pytest.mark.parametrize("S", [4, 16])
def test_dense_large_triangles_defer_span_batches(S):
    """Hundreds of large overlapping triangles per tile: a batch of up to 256 records then holds
    more row spans than one batch takes (2,048), so records are deferred to further batches, and
    most records need the 64-bit coverage test (vertex spans of 32 pixels and more)."""
    rng = np.random.default_rng(77)
    n = 700
    c = rng.uniform(-0.6, 0.6, (n, 1, 2))
    p = c + rng.normal(size=(n, 3, 2)) * rng.uniform(0.3, 1.2, (n, 1, 1))
    z = rng.uniform(-6.0, -2.0, (n, 1, 1)) + rng.normal(size=(n, 3, 1)) * 0.2
    pos = np.concatenate([p * -z, z], 2).reshape(-1, 3)
    col = rng.uniform(0, 1, (3 * n, 3))
    v = np.concatenate([pos, col], 1).astype(np.float32)
    f = np.arange(3 * n, dtype=np.int32).reshape(-1, 3)
    mvp = scenes.perspective(60.0, 1.0, 0.1, 100.0).astype(np.float32)
    gpu, ref, _ = render_both(v, f, mvp, 96, 96, S=S, cull=ig.CULL_NONE, depth_func=ig.LESS)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).mean() > 0.9
