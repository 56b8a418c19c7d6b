"""ctypes front end of the reference CPU renderer built by oracle/build_ref.py (test and
baseline infrastructure only: the golden-fixture script, the pinning tests and bench.py's
CPU-baseline legs use it; the product never does).

The library is ``oracle/_ref/libifrit_ref.so`` (x86, the reference's AVX2 build) or
``oracle/_ref/libifrit_ref_scalar.so`` (any host, SIMD switches off).  ``oracle/ref_driver.cpp``
drives the reference's own ``TileRasterRenderer::drawElements`` (TileRasterRenderer.cpp:436-457)
with a vertex shader applying the MVP and a fragment shader passing the vertex colour through.
"""
import ctypes
import os

import numpy as np

from . import build_ref

REF_CLEAR_DEPTH = float(np.frombuffer(np.uint32(0x7F7F7F7F).tobytes(), np.float32)[0])


def load(build=True):
    """Returns (ctypes library, build kind) or (None, reason)."""
    simd = build_ref.is_x86()
    name = "libifrit_ref.so" if simd else "libifrit_ref_scalar.so"
    path = os.path.join(build_ref.OUT, name)
    if build and build_ref.available():
        try:
            path = build_ref.build(simd=simd)
        except Exception as e:  # noqa: BLE001 - reported to the caller as the reason
            return None, "reference build failed: %s" % str(e).splitlines()[0][:200]
    if not path or not os.path.exists(path):
        return None, "reference CPU renderer not built (no staged reference tree)"
    lib = ctypes.CDLL(path)
    lib.ref_render_ex.restype = ctypes.c_double
    lib.ref_render.restype = ctypes.c_double
    return lib, ("x86 AVX2 build" if simd else "scalar build (SIMD switches off)")


def render(lib, vertices, indices, mvp, width, height, depth_func=1, deterministic=False, blend=None, warm=0, timed=0):
    """Draws indexed triangles through the reference renderer.  vertices: (V, >=6) float32 with
    xyz then RGB(A) from column 3.  Returns (rgba (H,W,4) f32, depth (H,W) f32, median ms)."""
    fp = ctypes.POINTER(ctypes.c_float)
    v = np.asarray(vertices, np.float32)
    v8 = np.zeros((len(v), 8), np.float32)
    v8[:, :3] = v[:, :3]
    nc = min(v.shape[1] - 3, 4)
    v8[:, 4:4 + nc] = v[:, 3:3 + nc]
    if nc < 4:
        v8[:, 7] = 1.0
    idx = np.ascontiguousarray(indices, np.int32).reshape(-1)
    m = np.ascontiguousarray(mvp, np.float32)
    rgba = np.zeros((height, width, 4), np.float32)
    depth = np.zeros((height, width), np.float32)
    b = None if blend is None else np.asarray((1,) + tuple(blend), np.int32)
    ms = lib.ref_render_ex(v8.ctypes.data_as(fp), len(v8), idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                           idx.size // 3, m.ctypes.data_as(fp), width, height, depth_func, int(deterministic),
                           None if b is None else b.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                           rgba.ctypes.data_as(fp), depth.ctypes.data_as(fp), warm, timed)
    return rgba, depth, ms


def num_threads(lib):
    return int(lib.ref_num_threads())
