"""The allocation-free entry point, iftrDrawNoAlloc, against the renderer's own entry point.

iftrDrawNoAlloc exists for callers that cannot allocate device memory while they draw: a
plugin living inside a host application that owns every GPU allocation, or a real-time loop
that runs with a zero allocation budget.  Such a caller hands in device inputs and outputs it
already owns, and the pass keeps all of its intermediate data in one fixed-size device array
inside the library (IFTR_NOALLOC_SCRATCH_BYTES, limits IFTR_NOALLOC_MAX_*).

This test (the caller here may allocate; the entry point must not) renders two different
scenes back to back through the C-ABI, so the second call runs on scratch that still holds
the first call's data, and compares each result with what iftrDrawLegacy produces for the
same inputs: visibility ids and per-sample depth bit-exact, colour within one RGBA8 step.
"""
import ctypes

import numpy as np
import pytest

import ifrit_gb300 as ig
from ifrit_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def reference_render(v, f, mvp, W, H, S, attr, cull, depth_func, shading, texture=None, aniso=1):
    r = ig.Renderer(W, H, S, ig.FORMAT_RGBA8, visibility=True)
    r.set_state(cull=cull, depth_func=depth_func, shading=shading)
    r.set_mvp(mvp)
    r.set_geometry(v, f, attr)
    if texture is not None:
        r.set_texture(texture, max_aniso=aniso)
    r.draw(clear=True)
    out = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    r.close()
    return out


def no_alloc_render(torch, v, f, mvp, W, H, S, attr, cull, depth_func, shading, texture=None, aniso=1, expect=0):
    dev = torch.device("cuda")
    dv = torch.from_numpy(np.ascontiguousarray(v, np.float32)).to(dev)
    di = torch.from_numpy(np.ascontiguousarray(f, np.int32).reshape(-1)).to(dev)
    color = torch.empty((H, W), dtype=torch.int32, device=dev)
    depth = torch.empty((H, W, S), dtype=torch.float32, device=dev)
    vis = torch.empty((H, W, S), dtype=torch.int32, device=dev)
    p = ig.NoAllocPass()
    p.vertices, p.strideFloats, p.numVertices = dv.data_ptr(), v.shape[1], v.shape[0]
    p.attrOffsetFloats, p.attrCount = 3, attr
    p.indices, p.numIndices = di.data_ptr(), int(f.size)
    for i, x in enumerate(np.asarray(mvp, np.float32).reshape(-1)):
        p.mvp[i] = float(x)
    p.width, p.height, p.samples, p.colorFormat = W, H, S, ig.FORMAT_RGBA8
    p.color, p.depth, p.visibility = color.data_ptr(), depth.data_ptr(), vis.data_ptr()
    p.clear, p.clearDepth = 1, 1.0
    p.depthFunc, p.depthTest, p.depthWrite = depth_func, 1, 1
    p.cullMode, p.frontCounterClockwise, p.shadingModel = cull, 1, shading
    keep = [dv, di]
    if texture is not None:
        chain, levels = O.build_mips(texture)
        dt = torch.from_numpy(chain.view(np.int32)).to(dev)
        keep.append(dt)
        p.texels, p.texWidth, p.texHeight, p.texLevels = dt.data_ptr(), texture.shape[1], texture.shape[0], levels
        p.sampler = ig.SamplerState(1, 0, 0, 0, 0, int(aniso > 1), float(aniso), 0.0)
    stream = torch.cuda.current_stream(dev)
    rc = ig.load().iftrDrawNoAlloc(ctypes.byref(p), ctypes.c_void_p(stream.cuda_stream))
    assert rc == expect, ig.load().iftrGetErrorString(rc)
    torch.cuda.synchronize()
    return {"color": color.cpu().numpy().view(np.uint32), "depth": depth.cpu().numpy(), "vis": vis.cpu().numpy()}


def assert_same(got, want):
    assert (got["vis"] == want["vis"]).all(), int((got["vis"] != want["vis"]).sum())
    assert (got["depth"].view(np.uint32) == want["depth"].view(np.uint32)).all()
    diff = np.abs(got["color"].view(np.uint8).astype(int) - want["color"].view(np.uint8).astype(int)).max()
    assert diff <= 1, diff


def test_no_alloc_matches_renderer_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    # call 1: textured 4x MSAA soup
    v, f, mvp = scenes.triangle_soup(20000, 21, 256, 160)
    tex = scenes.value_noise_texture(256, 5)
    args = (v, f, mvp, 256, 160, 4, 2, ig.CULL_NONE, ig.LESS_OR_EQUAL, ig.FS_TEXTURED)
    first = no_alloc_render(torch, *args, texture=tex, aniso=8)
    assert_same(first, reference_render(*args, texture=tex, aniso=8))
    assert (first["vis"] >= 0).mean() > 0.5
    # call 2: the plain Gouraud icosphere frame, on scratch left over from call 1
    v2, f2, mvp2 = scenes.c1_scene(1)
    args2 = (v2, f2, mvp2, 512, 512, 1, 3, ig.CULL_BACK, ig.LESS_OR_EQUAL, ig.FS_GOURAUD)
    second = no_alloc_render(torch, *args2)
    assert_same(second, reference_render(*args2))
    assert (second["vis"] >= 0).sum() > 50000


def test_no_alloc_matches_the_oracle():
    torch = pytest.importorskip("torch")
    v, f, mvp = scenes.triangle_soup(6000, 33, 192, 128)
    got = no_alloc_render(torch, v, f, mvp, 192, 128, 8, 2, ig.CULL_NONE, ig.LESS, ig.FS_GOURAUD)
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=2, cull_mode=0, depth_func=ig.LESS)
    assert_same(got, O.render([d], 192, 128, 8))


def test_no_alloc_overflow_then_next_call_is_correct():
    """More (triangle, tile) overlaps than IFTR_NOALLOC_MAX_TILE_PAIRS: the call reports
    IFTR_ERR_OVERFLOW (its outputs are undefined), and the next call on the same scratch is right."""
    torch = pytest.importorskip("torch")
    W, H = 2048, 1024  # 8,192 tiles and 2,097,152 samples: both at their limits
    n = 100  # each triangle covers every tile: 819,200 overlaps > 524,288
    z = np.linspace(0.2, 0.8, n, dtype=np.float32)
    v = np.zeros((3 * n, 6), np.float32)
    for i in range(n):
        v[3 * i:3 * i + 3, 0:3] = [[-1, -1, z[i]], [3, -1, z[i]], [-1, 3, z[i]]]
        v[3 * i:3 * i + 3, 3:6] = (i % 7) / 7.0
    f = np.arange(3 * n, dtype=np.int32).reshape(-1, 3)
    no_alloc_render(torch, v, f, np.eye(4, dtype=np.float32), W, H, 1, 3, ig.CULL_NONE, ig.LESS_OR_EQUAL,
                    ig.FS_GOURAUD, expect=4)
    v2, f2, mvp2 = scenes.triangle_soup(3000, 8, 256, 128)
    args = (v2, f2, mvp2, 256, 128, 4, 2, ig.CULL_NONE, ig.LESS_OR_EQUAL, ig.FS_GOURAUD)
    assert_same(no_alloc_render(torch, *args), reference_render(*args))


def test_no_alloc_rejects_sizes_over_its_limits():
    p = ig.NoAllocPass()
    p.width, p.height, p.samples = 4096, 4096, 4  # far above IFTR_NOALLOC_MAX_SAMPLES
    p.strideFloats, p.color, p.depth = 3, 1, 1
    assert ig.load().iftrDrawNoAlloc(ctypes.byref(p), None) == 1
    # within the sample and tile limits, but wider than the 16384-pixel cap of every entry point
    p.width, p.height, p.samples = 40000, 48, 1
    assert ig.load().iftrDrawNoAlloc(ctypes.byref(p), None) == 1
