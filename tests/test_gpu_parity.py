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
