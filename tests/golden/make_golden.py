"""Generates the golden fixtures in tests/golden/ from the reference itself.

* ``ref_<scene>.npz``: the reference's own multithreaded CPU tile rasterizer
  (TileRasterRenderer, built by oracle/build_ref.py from the reference checkout into
  oracle/_ref/) on small seeded scenes: the FP32 colour quantised to RGBA8, the FP32 depth and
  the visible primitive id per pixel.  The id comes from a second render of the same geometry
  with unshared vertices whose only varying is the primitive index.
* ``blend_<name>.npz``: the same renderer drawing overlapping translucent triangles (per-vertex
  RGBA, alpha in [0.2, 0.9]) with blending enabled through TileRasterRenderer::setBlendFunc,
  one factor set per fixture: the FP32 colour (its in-order path's depth write-back is not
  compared, see oracle/build_ref.py).
* ``sampler.npz``: the reference's texture sampler (TextureSampleImpl, ShaderBuiltinCuda.cuh,
  compiled for the host by oracle/build_ref.py) on seeded UVs and derivatives over two RGBA8
  textures (37x23 and 64x64 with full mip chains), for both filters, every address mode, border
  colours and anisotropy off / 2 / 8 / 16: the FP32 RGBA results.

The reference needs the checkout (IFRIT_REFERENCE_ROOT) and, for the renderer's SIMD build, an
x86 host, so this script runs only in the build container; the fixtures it writes are what the
CPU tests read.  Usage:  python tests/golden/make_golden.py [scenes|blend|sampler|all]
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "ifrit-v2_gb300"))

from oracle import build_ref  # noqa: E402
from ifrit_gb300 import scenes  # noqa: E402

REF_CLEAR_DEPTH = np.frombuffer(np.uint32(0x7F7F7F7F).tobytes(), np.float32)[0]


def kat_scenes():
    """Hand-built known-answer scenes: (name, vertices (V,6), indices (T,3), mvp, W, H)."""
    eye = np.eye(4, dtype=np.float32)
    out = []

    def mk(pos, col, idx):
        v = np.concatenate([np.asarray(pos, np.float32), np.asarray(col, np.float32)], 1)
        return v, np.asarray(idx, np.int32).reshape(-1, 3)

    # single triangle
    v, i = mk([[-0.8, -0.7, 0.5], [0.7, -0.6, 0.3], [-0.1, 0.8, 0.7]], [[1, 0, 0], [0, 1, 0], [0, 0, 1]], [0, 1, 2])
    out.append(("single", v, i, eye, 64, 64))
    # two triangles sharing an edge (fill rule)
    v, i = mk([[-0.9, -0.9, 0.2], [0.9, -0.8, 0.4], [0.8, 0.9, 0.6], [-0.85, 0.85, 0.3]],
              [[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0]], [0, 1, 2, 0, 2, 3])
    out.append(("shared_edge", v, i, eye, 64, 64))
    # T-junction: one big triangle beside two smaller ones that split its edge
    v, i = mk([[-0.9, -0.9, 0.5], [0.0, -0.9, 0.5], [0.0, 0.9, 0.5], [0.9, 0.0, 0.5], [0.0, 0.0, 0.5]],
              [[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1]], [0, 1, 2, 1, 3, 4, 4, 3, 2])
    out.append(("t_junction", v, i, eye, 64, 64))
    # overlapping pair with different depth (early-Z order)
    v, i = mk([[-0.8, -0.8, 0.3], [0.6, -0.7, 0.3], [-0.2, 0.7, 0.3], [-0.6, -0.5, 0.6], [0.8, -0.2, 0.1],
               [0.2, 0.9, 0.6]], [[1, 0, 0]] * 3 + [[0, 0, 1]] * 3, [0, 1, 2, 3, 4, 5])
    out.append(("overlap", v, i, eye, 64, 64))
    # sub-pixel slivers and tiny triangles
    rng = np.random.default_rng(7)
    pos, col, idx = [], [], []
    for t in range(40):
        c = rng.uniform(-0.9, 0.9, 2)
        d = rng.normal(size=(3, 2)) * rng.choice([0.005, 0.02, 0.05])
        p = np.concatenate([c + d, np.full((3, 1), rng.uniform(0.1, 0.9))], 1)
        a = (p[1, 0] - p[0, 0]) * (p[2, 1] - p[0, 1]) - (p[2, 0] - p[0, 0]) * (p[1, 1] - p[0, 1])
        if a < 0:
            p = p[[0, 2, 1]]
        pos += list(p)
        col += list(rng.uniform(0, 1, (3, 3)))
        idx += [3 * t, 3 * t + 1, 3 * t + 2]
    v, i = mk(pos, col, idx)
    out.append(("slivers", v, i, eye, 64, 64))
    # full-screen pair
    v, i = mk([[-1, -1, 0.5], [1, -1, 0.5], [1, 1, 0.5], [-1, 1, 0.5]], [[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]],
              [0, 1, 2, 0, 2, 3])
    out.append(("fullscreen", v, i, eye, 32, 32))
    # the plain-frame icosphere at reduced resolutions
    v, f, mvp = scenes.c1_scene(1)
    out.append(("c1_128", v, f, mvp, 128, 128))
    out.append(("c1_256", v, f, mvp, 256, 256))
    v, f = scenes.jittered_icosphere(3, 11)
    mvp = scenes.orbit_camera(np.random.default_rng(5), 2.5, 96 / 80)
    out.append(("ico3_orbit_96x80", v, f, mvp, 96, 80))
    return out


def ref_lib():
    path = build_ref.build()
    if path is None:
        raise SystemExit("reference CPU renderer unavailable on this host")
    lib = ctypes.CDLL(path)
    lib.ref_render.restype = ctypes.c_double
    return lib


def ref_render(lib, v8, idx, mvp, W, H, depth_func=1):
    fp = ctypes.POINTER(ctypes.c_float)
    v8 = np.ascontiguousarray(v8, np.float32)
    idx = np.ascontiguousarray(idx, np.int32)
    rgba = np.zeros((H, W, 4), np.float32)
    depth = np.zeros((H, W), np.float32)
    m = np.ascontiguousarray(mvp, np.float32)
    lib.ref_render(v8.ctypes.data_as(fp), len(v8), idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), idx.size // 3,
                   m.ctypes.data_as(fp), W, H, depth_func, 0, rgba.ctypes.data_as(fp), depth.ctypes.data_as(fp), 0, 0)
    return rgba, depth


def render_reference(lib, v, f, mvp, W, H):
    """Returns (rgba8 (H,W,4) uint8, depth (H,W) f32, vis (H,W) int32) from the reference."""
    v8 = np.zeros((len(v), 8), np.float32)
    v8[:, :3] = v[:, :3]
    v8[:, 4:7] = v[:, 3:6]
    v8[:, 7] = 1.0
    rgba, depth = ref_render(lib, v8, f, mvp, W, H)
    T = len(f)
    vd = np.zeros((3 * T, 8), np.float32)
    vd[:, :3] = v[f.reshape(-1), :3]
    vd[:, 4] = np.repeat(np.arange(T, dtype=np.float32), 3)
    vd[:, 7] = 1.0
    rgba_id, depth_id = ref_render(lib, vd, np.arange(3 * T, dtype=np.int32), mvp, W, H)
    covered = depth_id < 1e30
    vis = np.where(covered, np.rint(rgba_id[..., 0]).astype(np.int64), -1).astype(np.int32)
    rgba8 = np.rint(np.clip(rgba, 0, 1) * 255).astype(np.uint8)
    return rgba8, depth, vis


BLEND_SETS = {  # (srcColor, dstColor, srcAlpha, dstAlpha), IfritBlendFactor numbering
    "src_alpha_over": (6, 7, 6, 7),
    "additive": (1, 1, 1, 1),
    "dst_alpha": (8, 9, 1, 0),
    "one_minus_dst_alpha": (9, 1, 7, 6),
    "inverse_over": (7, 6, 8, 9),
}


def blend_scene(seed=3, n=10):
    """Overlapping counter-clockwise triangles at random depths with per-vertex RGBA colour."""
    rng = np.random.default_rng(seed)
    pos, col, idx = [], [], []
    for t in range(n):
        c = rng.uniform(-0.5, 0.5, 2)
        p = c + rng.normal(size=(3, 2)) * 0.5
        p = np.concatenate([p, np.full((3, 1), rng.uniform(0.1, 0.9))], 1)
        a = (p[1, 0] - p[0, 0]) * (p[2, 1] - p[0, 1]) - (p[2, 0] - p[0, 0]) * (p[1, 1] - p[0, 1])
        if a < 0:
            p = p[[0, 2, 1]]
        cc = rng.uniform(0, 1, (3, 4))
        cc[:, 3] = rng.uniform(0.2, 0.9, 3)
        pos += list(p)
        col += list(cc)
        idx += [3 * t, 3 * t + 1, 3 * t + 2]
    v = np.concatenate([np.asarray(pos, np.float32), np.asarray(col, np.float32)], 1)
    return v, np.asarray(idx, np.int32).reshape(-1, 3)


def make_blend(lib):
    fp = ctypes.POINTER(ctypes.c_float)
    lib.ref_render_ex.restype = ctypes.c_double
    v, f = blend_scene()
    W = H = 64
    eye = np.eye(4, dtype=np.float32)
    for name, factors in BLEND_SETS.items():
        v8 = np.zeros((len(v), 8), np.float32)
        v8[:, :3] = v[:, :3]
        v8[:, 4:8] = v[:, 3:7]
        rgba = np.zeros((H, W, 4), np.float32)
        depth = np.zeros((H, W), np.float32)
        b = np.asarray((1,) + factors, np.int32)
        lib.ref_render_ex(v8.ctypes.data_as(fp), len(v8), f.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(f),
                          eye.ctypes.data_as(fp), W, H, 1, 1, b.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                          rgba.ctypes.data_as(fp), depth.ctypes.data_as(fp), 0, 0)
        path = os.path.join(HERE, "blend_%s.npz" % name)
        np.savez_compressed(path, rgba=rgba, vertices=v, indices=f, mvp=eye, width=W, height=H,
                            factors=np.asarray(factors, np.int32))
        print("wrote", path)


SAMPLER_N = 256
INV255 = np.float32(float.fromhex("0x1.010102p-8"))  # texel = byte * (1/255), as the oracle decodes RGBA8


def sampler_inputs(seed=11, n=SAMPLER_N):
    """UV in [-0.9, 1.9] and derivatives of magnitude 1e-4 .. 0.2 (a probe then stays above one
    period below 0, where the reference's repeat modes would read out of range), 5 % exact
    zeros, 30 % with LOD bias 0.5."""
    rng = np.random.default_rng(seed)
    uv = rng.uniform(-0.9, 1.9, (n, 2))
    d = 10 ** rng.uniform(-4, np.log10(0.2), (n, 4)) * rng.choice([-1, 1], (n, 4))
    d[rng.random((n, 4)) < 0.05] = 0
    bias = np.where(rng.random(n) < 0.3, 0.5, 0.0)
    return np.concatenate([uv, d, bias[:, None]], 1).astype(np.float32)


def sampler_configs():
    """(filter, address_u, address_v, border_white, max_aniso); max_aniso 1 = anisotropy off."""
    out = []
    for filt in (0, 1):
        for au, av, bw in ((0, 0, 0), (1, 1, 0), (2, 2, 0), (3, 3, 0), (3, 3, 1), (4, 4, 0), (0, 2, 0)):
            for aniso in (1, 2, 8, 16):
                out.append((filt, au, av, bw, aniso))
    return out


def ref_sample(lib, level0, params, cfg):
    from oracle import oracle as O
    chain, _ = O.build_mips(level0)
    padded = np.concatenate([chain, np.repeat(chain[-1:], 64)])  # levels past the chain read as the last one
    tex4 = (padded.view(np.uint8).reshape(-1, 4).astype(np.float32) * INV255).astype(np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    out = np.zeros((len(params), 4), np.float32)
    filt, au, av, bw, aniso = cfg
    h, w = level0.shape
    lib.ref_sample_batch(len(params), params.ctypes.data_as(fp), tex4.ctypes.data_as(fp), w, h, filt, au, av, bw,
                         int(aniso > 1), ctypes.c_float(aniso), out.ctypes.data_as(fp))
    return out


def sampler_textures():
    rng = np.random.default_rng(23)
    return [rng.integers(0, 2 ** 32, (23, 37), dtype=np.uint64).astype(np.uint32),
            rng.integers(0, 2 ** 32, (64, 64), dtype=np.uint64).astype(np.uint32)]


def make_sampler():
    path = build_ref.build_sampler()
    if path is None:
        raise SystemExit("reference sampler unavailable (IFRIT_REFERENCE_ROOT)")
    lib = ctypes.CDLL(path)
    params = sampler_inputs()
    texs = sampler_textures()
    cfgs = sampler_configs()
    results = np.zeros((len(texs), len(cfgs), len(params), 4), np.float32)
    for ti, t in enumerate(texs):
        for ci, cfg in enumerate(cfgs):
            results[ti, ci] = ref_sample(lib, t, params, cfg)
    out = os.path.join(HERE, "sampler.npz")
    np.savez_compressed(out, params=params, tex0=texs[0], tex1=texs[1], configs=np.asarray(cfgs, np.int32),
                        results=results)
    print("wrote", out)


def main():
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("sampler", "all"):
        make_sampler()
    if what == "sampler":
        return
    lib = ref_lib()
    if what in ("blend", "all"):
        make_blend(lib)
    if what == "blend":
        return
    for name, v, f, mvp, W, H in kat_scenes():
        rgba8, depth, vis = render_reference(lib, v, f, mvp, W, H)
        path = os.path.join(HERE, "ref_%s.npz" % name)
        np.savez_compressed(path, rgba8=rgba8, depth=depth, vis=vis, vertices=v, indices=f,
                            mvp=np.asarray(mvp, np.float32), width=W, height=H,
                            ref_threads=lib.ref_num_threads())
        print("wrote", path, "covered", int((vis >= 0).sum()))


if __name__ == "__main__":
    main()
