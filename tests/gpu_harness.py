"""Shared helpers of the GPU parity tests: render one scene through the C-ABI and through
the CPU oracle with identical state (test infrastructure)."""
import os

import numpy as np

import ifrit_gb300 as ig
from oracle import oracle as O

FMT_TO_ORACLE = {ig.FORMAT_RGBA8: O.FMT_RGBA8, ig.FORMAT_RGBA16F: O.FMT_RGBA16F,
                 ig.FORMAT_RGBA32F: O.FMT_RGBA32F, ig.FORMAT_RGB32F: O.FMT_RGB32F}


def render_both(vertices, indices, mvp, W, H, *, S=1, fmt=ig.FORMAT_RGBA8, attr=3, cull=ig.CULL_BACK,
                front_ccw=True, depth_func=ig.LESS_OR_EQUAL, depth_test=True, depth_write=True,
                shading=ig.FS_GOURAUD, texture=None, max_aniso=1, address=0, filter_mode=1, lod_bias=0.0,
                clear_color=(0.0, 0.0, 0.0, 0.0), clear_depth=1.0, reserve=None, renderer=None):
    """Returns (gpu dict, oracle dict, renderer) with color / depth / vis."""
    r = renderer or ig.Renderer(W, H, S, fmt, visibility=True)
    r.set_state(cull=cull, front_ccw=front_ccw, depth_func=depth_func, depth_test=depth_test,
                depth_write=depth_write, shading=shading, clear_color=clear_color, clear_depth=clear_depth)
    r.set_mvp(mvp)
    r.set_geometry(vertices, indices, attr)
    tex_arg = None
    if texture is not None:
        r.set_texture(texture, max_aniso=max_aniso, address=address, filter_mode=filter_mode, lod_bias=lod_bias)
        chain, levels = O.build_mips(texture)
        tex_arg = (chain, levels, texture.shape[1], texture.shape[0])
    if reserve is not None:
        r.reserve(reserve)
    r.draw(clear=True)
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    d = O.make_draw(vertices, indices, mvp, attr_offset=3, attr_count=attr, cull_mode=cull,
                    front_ccw=int(front_ccw), depth_test=int(depth_test), depth_func=depth_func,
                    depth_write=int(depth_write), shading=shading, texture=tex_arg,
                    sampler={"address_u": address, "address_v": address, "filter": filter_mode,
                             "max_aniso": max_aniso, "lod_bias": lod_bias})
    ref = O.render([d], W, H, S, FMT_TO_ORACLE[fmt], clear=True, clear_color=clear_color,
                   clear_depth=clear_depth, nthreads=os.cpu_count() or 1)
    return gpu, ref, r


def assert_parity(gpu, ref, fmt=ig.FORMAT_RGBA8, color_tol=1):
    """Visibility and per-sample depth bit-exact; colour within one RGBA8 step (or one
    half-float ulp / 1e-5 relative for float targets)."""
    vis_mism = int((gpu["vis"] != ref["vis"]).sum())
    assert vis_mism == 0, "visibility mismatches: %d" % vis_mism
    dg, dr = gpu["depth"].view(np.uint32), ref["depth"].view(np.uint32)
    assert (dg == dr).all(), "depth mismatches: %d" % int((dg != dr).sum())
    if fmt == ig.FORMAT_RGBA8:
        cg = gpu["color"].view(np.uint8).astype(np.int32)
        cr = ref["color"].view(np.uint8).astype(np.int32)
        diff = np.abs(cg - cr).max()
        assert diff <= color_tol, "colour max diff %d" % diff
    elif fmt == ig.FORMAT_RGBA16F:
        hg = gpu["color"].view(np.uint16).astype(np.int32)
        hr = ref["color"].view(np.uint16).astype(np.int32)
        assert np.abs(hg - hr).max() <= 1
    else:
        cg, cr = gpu["color"], ref["color"]
        assert np.allclose(cg, cr, rtol=1e-5, atol=1e-6, equal_nan=True)
