"""Pins the oracle's texture sampler and blending against the reference's own code.

Sampler: tests/golden/sampler.npz holds what the reference's TextureSampleImpl functions
(include/ifrit/softgraphics/engine/math/ShaderBuiltinCuda.cuh:96-272, compiled for the host by
oracle/build_ref.py, generator tests/golden/make_golden.py) return for seeded UVs and quad
derivatives over two RGBA8 textures, every filter / address mode / border colour and anisotropy
off, 2, 8 and 16.  The oracle's reference-compatible sampler (oracle_fx.c, `compat`) must return
the same FP32 bits for every one of them.  Its default sampler, which the GPU path implements,
differs from it only by the switches listed in oracle_fx.c; the test shows that those switches
change results (so the fixtures do exercise them).

Blending: tests/golden/blend_*.npz hold the reference CPU renderer's FP32 colour for overlapping
translucent triangles, one blend-factor set each (TileRasterRenderer::setBlendFunc,
TileRasterRenderer.cpp:212-333; applied per fragment in order, TileRasterWorker.cpp:2346-2373).
The oracle draws the same scene with the reference's coefficient table (`blend_compat`) at the
reference's sample point (pixel corner) and must agree within one RGBA8 step everywhere (the
reference interpolates colours with 12-bit reciprocal estimates); with the factors by their names
(the default, as the GPU path blends) the alpha-weighted sets differ by far more.
"""
import ctypes
import glob
import os

import numpy as np
import pytest

from oracle import build_ref
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
REF_CLEAR_DEPTH = float(np.frombuffer(np.uint32(0x7F7F7F7F).tobytes(), np.float32)[0])
BLEND = sorted(glob.glob(os.path.join(GOLDEN, "blend_*.npz")))


def oracle_sample(level0, params, cfg, compat=1):
    chain, levels = O.build_mips(level0)
    h, w = level0.shape
    tex = O.Texture()
    tex.texels = chain.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    tex.width, tex.height, tex.levels = w, h, levels
    s = O.Sampler()
    s.filter, s.address_u, s.address_v, s.border_white, s.max_aniso = (int(x) for x in cfg)
    s.compat = compat
    out = np.zeros((len(params), 4), np.float32)
    o = (ctypes.c_float * 4)()
    fn = O.lib().ofx_sample_texture
    for i, p in enumerate(params):
        s.lod_bias = float(p[6])
        fn(ctypes.byref(tex), ctypes.byref(s), float(p[0]), float(p[1]), float(p[2]), float(p[3]), float(p[4]),
           float(p[5]), o)
        out[i] = o[:]
    return out


def test_sampler_matches_reference_bit_exact():
    fx = np.load(os.path.join(GOLDEN, "sampler.npz"))
    params, cfgs, results = fx["params"], fx["configs"], fx["results"]
    texs = [fx["tex0"], fx["tex1"]]
    assert results.shape == (2, len(cfgs), len(params), 4) and len(cfgs) >= 56
    for ti, t in enumerate(texs):
        for ci, cfg in enumerate(cfgs):
            got = oracle_sample(t, params, cfg)
            same = (got.view(np.uint32) == results[ti, ci].view(np.uint32)).all(axis=1)
            assert same.all(), (ti, tuple(cfg), int((~same).sum()), params[~same][:2], got[~same][:2],
                                results[ti, ci][~same][:2])


def test_sampler_default_differs_from_reference_quirks():
    """The default sampler's documented fixes (y footprint, centred taps, footprint axes) do
    change results on these inputs, so the bit-exact pin above is not vacuous."""
    fx = np.load(os.path.join(GOLDEN, "sampler.npz"))
    params, t = fx["params"], fx["tex1"]
    for cfg in ((1, 2, 2, 0, 1), (1, 2, 2, 0, 8)):
        a = oracle_sample(t, params, cfg, compat=1)
        b = oracle_sample(t, params, cfg, compat=0)
        assert (np.abs(a - b).max(axis=1) > 1e-4).mean() > 0.2, cfg


@pytest.mark.skipif(not build_ref.have_checkout(), reason="needs the reference checkout (IFRIT_REFERENCE_ROOT)")
def test_sampler_matches_live_reference_on_fresh_inputs():
    from tests.golden import make_golden as MG
    lib = ctypes.CDLL(build_ref.build_sampler())
    params = MG.sampler_inputs(seed=101, n=600)
    rng = np.random.default_rng(5)
    level0 = rng.integers(0, 2 ** 32, (40, 17), dtype=np.uint64).astype(np.uint32)
    for cfg in MG.sampler_configs()[::3]:
        ref = MG.ref_sample(lib, level0, params, cfg)
        got = oracle_sample(level0, params, cfg)
        assert (got.view(np.uint32) == ref.view(np.uint32)).all(), cfg


def render_blend(fx, compat):
    v, f = fx["vertices"], fx["indices"]
    W, H = int(fx["width"]), int(fx["height"])
    d = O.make_draw(v, f, fx["mvp"], attr_offset=3, attr_count=4, depth_func=1, cull_mode=2,
                    blend=tuple(int(x) for x in fx["factors"]), blend_compat=compat)
    return O.render([d], W, H, 1, O.FMT_RGBA32F, clear=True, clear_color=(0, 0, 0, 0),
                    clear_depth=REF_CLEAR_DEPTH, compat=True)["color"]


def test_blend_fixtures_present():
    assert len(BLEND) >= 5


@pytest.mark.parametrize("path", BLEND, ids=[os.path.basename(p)[6:-4] for p in BLEND])
def test_blend_matches_reference(path):
    fx = np.load(path)
    ref = fx["rgba"]
    got = render_blend(fx, compat=1)
    diff = np.abs(got - ref).max(axis=-1)
    assert (ref.max(axis=-1) > 0).mean() > 0.3  # the translucent triangles cover a third of the target
    assert diff.max() <= 1.0 / 255, diff.max()
    assert np.median(diff[ref.max(axis=-1) > 0]) <= 1e-4


def test_blend_named_factors_deviate_from_reference_table():
    fx = np.load(os.path.join(GOLDEN, "blend_src_alpha_over.npz"))
    diff = np.abs(render_blend(fx, compat=0) - fx["rgba"]).max(axis=-1)
    assert diff.max() > 0.1
