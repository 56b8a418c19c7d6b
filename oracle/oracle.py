"""Test infrastructure only: ctypes front end of the C oracle (oracle_fx.c).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module.  It is the checker the GPU rasterizer is compared against, never a code path of
the product.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_fx.so")

FMT_RGBA8, FMT_RGBA16F, FMT_RGBA32F, FMT_RGB32F = 0, 1, 2, 3
SHADE_GOURAUD, SHADE_TEXTURED, SHADE_PRIMID = 0, 1, 2
POLY_FILL, POLY_LINE, POLY_POINT = 0, 1, 2


def build(force=False):
    src = os.path.join(HERE, "oracle_fx.c")
    hdr = os.path.join(HERE, "oracle_fx.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-o", LIB_PATH, src, "-lm", "-lpthread"]
    subprocess.run(cmd, check=True)
    return LIB_PATH


class Sampler(ctypes.Structure):
    _fields_ = [("address_u", ctypes.c_int), ("address_v", ctypes.c_int), ("filter", ctypes.c_int),
                ("border_white", ctypes.c_int), ("max_aniso", ctypes.c_int), ("lod_bias", ctypes.c_float),
                ("compat", ctypes.c_int)]


class Texture(ctypes.Structure):
    _fields_ = [("texels", ctypes.POINTER(ctypes.c_uint32)), ("width", ctypes.c_int),
                ("height", ctypes.c_int), ("levels", ctypes.c_int)]


class Draw(ctypes.Structure):
    _fields_ = [("vertices", ctypes.POINTER(ctypes.c_float)), ("vertex_stride", ctypes.c_int),
                ("num_vertices", ctypes.c_int), ("attr_offset", ctypes.c_int), ("attr_count", ctypes.c_int),
                ("indices", ctypes.POINTER(ctypes.c_int)), ("num_triangles", ctypes.c_int),
                ("prim_base", ctypes.c_int), ("mvp", ctypes.c_float * 16),
                ("cull_mode", ctypes.c_int), ("front_ccw", ctypes.c_int), ("depth_test", ctypes.c_int),
                ("depth_func", ctypes.c_int), ("depth_write", ctypes.c_int), ("blend_enable", ctypes.c_int),
                ("blend_src_color", ctypes.c_int), ("blend_dst_color", ctypes.c_int),
                ("blend_src_alpha", ctypes.c_int), ("blend_dst_alpha", ctypes.c_int),
                ("shading", ctypes.c_int), ("tex", Texture), ("sampler", Sampler),
                ("scissor_enable", ctypes.c_int), ("scissor_count", ctypes.c_int),
                ("scissor", (ctypes.c_float * 4) * 16), ("polygon_mode", ctypes.c_int),
                ("blend_compat", ctypes.c_int), ("polygon_rules", ctypes.c_int)]


class Target(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("samples", ctypes.c_int),
                ("format", ctypes.c_int), ("sample_compat", ctypes.c_int), ("color", ctypes.c_void_p),
                ("depth", ctypes.POINTER(ctypes.c_float)), ("vis", ctypes.POINTER(ctypes.c_int)),
                ("row0", ctypes.c_int), ("rows", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.ofx_render_pass.restype = ctypes.c_int
        _lib.ofx_render_pass.argtypes = [ctypes.POINTER(Draw), ctypes.c_int, ctypes.POINTER(Target), ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_int]
        _lib.ofx_build_mips.restype = ctypes.c_int
        _lib.ofx_build_mips.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int, ctypes.c_int]
        _lib.ofx_mip_chain_texels.restype = ctypes.c_int
        _lib.ofx_mip_chain_texels.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        _lib.ofx_log2.restype = ctypes.c_float
        _lib.ofx_log2.argtypes = [ctypes.c_float]
        _lib.ofx_f32_to_f16.restype = ctypes.c_uint16
        _lib.ofx_f32_to_f16.argtypes = [ctypes.c_float]
        _lib.ofx_sample_texture.restype = None
        _lib.ofx_sample_texture.argtypes = [ctypes.POINTER(Texture), ctypes.POINTER(Sampler)] + \
            [ctypes.c_float] * 6 + [ctypes.POINTER(ctypes.c_float)]
    return _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def build_mips(level0):
    """level0: (h, w) uint32 RGBA8 -> (flat uint32 mip chain, levels)."""
    h, w = level0.shape
    lv = ctypes.c_int()
    total = lib().ofx_mip_chain_texels(w, h, ctypes.byref(lv))
    chain = np.zeros(total, np.uint32)
    chain[:w * h] = level0.reshape(-1)
    lib().ofx_build_mips(chain.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), w, h)
    return chain, lv.value


def make_draw(vertices, indices, mvp, *, attr_offset=3, attr_count=3, prim_base=0, cull_mode=2,
              front_ccw=1, depth_test=1, depth_func=3, depth_write=1, blend=None, shading=SHADE_GOURAUD,
              texture=None, sampler=None, scissor=None, polygon_mode=0, blend_compat=0, polygon_rules=0):
    """Returns (Draw, keepalive) for numpy vertices (V, stride) float32 and indices (T, 3) int32.
    blend_compat / sampler["compat"] select the reference's blend table and sampler as written
    (pinning only; see oracle_fx.h)."""
    vertices = np.ascontiguousarray(vertices, np.float32)
    indices = np.ascontiguousarray(indices, np.int32).reshape(-1)
    d = Draw()
    d.vertices = _fp(vertices)
    d.vertex_stride = vertices.shape[1]
    d.num_vertices = vertices.shape[0]
    d.attr_offset, d.attr_count = attr_offset, attr_count
    d.indices = indices.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.num_triangles = indices.size // 3
    d.prim_base = prim_base
    m = np.ascontiguousarray(mvp, np.float32).reshape(-1)
    for i in range(16):
        d.mvp[i] = float(m[i])
    d.cull_mode, d.front_ccw = cull_mode, front_ccw
    d.depth_test, d.depth_func, d.depth_write = depth_test, depth_func, depth_write
    if blend is not None:
        d.blend_enable = 1
        d.blend_src_color, d.blend_dst_color, d.blend_src_alpha, d.blend_dst_alpha = blend
    d.shading = shading
    keep = [vertices, indices]
    if texture is not None:
        chain, levels, w, h = texture
        chain = np.ascontiguousarray(chain, np.uint32)
        d.tex.texels = chain.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        d.tex.width, d.tex.height, d.tex.levels = w, h, levels
        keep.append(chain)
    s = sampler or {}
    d.sampler.address_u = s.get("address_u", 0)
    d.sampler.address_v = s.get("address_v", 0)
    d.sampler.filter = s.get("filter", 1)
    d.sampler.border_white = s.get("border_white", 0)
    d.sampler.max_aniso = s.get("max_aniso", 1)
    d.sampler.lod_bias = s.get("lod_bias", 0.0)
    d.sampler.compat = int(s.get("compat", 0))
    d.polygon_mode = polygon_mode
    d.blend_compat = int(blend_compat)
    d.polygon_rules = int(polygon_rules)
    if scissor is not None:  # list of (x, y, w, h) rectangles; [] = enabled with none (passes all)
        d.scissor_enable = 1
        d.scissor_count = min(len(scissor), 16)
        for i, r in enumerate(scissor[:16]):
            for k in range(4):
                d.scissor[i][k] = float(r[k])
    return d, keep


def color_dtype(fmt):
    return {FMT_RGBA8: (np.uint32, 1), FMT_RGBA16F: (np.uint64, 1), FMT_RGBA32F: (np.float32, 4),
            FMT_RGB32F: (np.float32, 3)}[fmt]


def render(draws, width, height, samples=1, fmt=FMT_RGBA8, clear=True, clear_color=(0, 0, 0, 0),
           clear_depth=1.0, compat=False, nthreads=1, color=None, depth=None, with_vis=True, rows=None):
    """Renders a pass of draws ((Draw, keep) pairs).  Returns dict(color, depth, vis).
    rows=(y0, y1): only that band of the height-row frame is rendered, into buffers of y1 - y0
    rows."""
    dt, ch = color_dtype(fmt)
    nrows = height if rows is None else rows[1] - rows[0]
    if color is None:
        color = np.zeros((nrows, width, ch) if ch > 1 else (nrows, width), dt)
    if depth is None:
        depth = np.zeros((nrows, width, samples), np.float32)
    vis = np.zeros((nrows, width, samples), np.int32) if with_vis else None
    t = Target()
    t.width, t.height, t.samples, t.format, t.sample_compat = width, height, samples, fmt, int(compat)
    if rows is not None:
        t.row0, t.rows = int(rows[0]), int(rows[1] - rows[0])
    t.color = color.ctypes.data_as(ctypes.c_void_p)
    t.depth = _fp(depth)
    t.vis = vis.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if with_vis else None
    arr = (Draw * len(draws))(*[d for d, _ in draws])
    cc = np.asarray(clear_color, np.float32)
    rc = lib().ofx_render_pass(arr, len(draws), ctypes.byref(t), int(clear), _fp(cc), float(clear_depth), nthreads)
    if rc != 0:
        raise ValueError("oracle render failed: %d" % rc)
    return {"color": color, "depth": depth, "vis": vis}
