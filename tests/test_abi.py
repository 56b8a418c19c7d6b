"""C-ABI checks that need no GPU: the library builds and loads, exports every entry point
include/ifrit_gb300.h declares, and its host-only objects behave (no compute calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

import ifrit_gb300 as ig

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ifrit_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"IFTR_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    return ig.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert len(syms) >= 60
    assert set(ig.EXPORTED) == set(syms), set(ig.EXPORTED) ^ set(syms)


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_error_strings(lib):
    assert lib.iftrGetErrorString(0) == b"ok"
    assert lib.iftrGetErrorString(4) == b"scratch capacity exceeded"


def test_host_function_shaders_are_unsupported(lib):
    h = lib.iftrCreateInstance()
    assert h
    assert lib.iftrBindVertexShaderFunc(h, None, None) == 2
    assert lib.iftrBindFragmentShaderFunc(h, None) == 2
    assert lib.iftrBindVertexShader(h, None) == 2
    assert lib.iftrBindFragmentShader(h, None) == 2
    assert lib.iftrBindFragmentShaderBuiltin(h, ig.FS_TEXTURED) == 0
    assert lib.iftrBindFragmentShaderBuiltin(h, 99) == 1
    assert lib.iftrSetMsaaSamples(h, 3) == 1
    assert lib.iftrSetMsaaSamples(h, 8) == 0
    assert lib.iftrSetDepthFunc(h, 8) == 1
    assert lib.iftrSetCullMode(h, 4) == 1
    assert lib.iftrDestroyInstance(h) == 0


def test_host_objects(lib):
    img = lib.ifcrCreateImageFP32(8, 4, 4)
    data = lib.ifcrGetImageRawDataFP32(img)
    assert data[0] == 0.0 and data[8 * 4 * 4 - 1] == 0.0
    fb = lib.iftrCreateFrameBuffer()
    arr = (ctypes.c_void_p * 1)(img)
    assert lib.iftrSetFrameBufferColorAttachmentFP32(fb, arr, 1) == 0
    assert lib.iftrSetFrameBufferColorAttachmentDevice(fb, 7, 8, 8) == 1
    vb = lib.iftrCreateVertexBuffer()
    layout = (ctypes.c_int * 2)(ig.IFTP_FLOAT3, ig.IFTP_FLOAT2)
    assert lib.iftrSetVertexBufferLayout(vb, layout, 2) == 0
    assert lib.iftrSetVertexBufferSize(vb, 3) == 0
    assert lib.iftrAllocateVertexBuffer(vb) == 0
    v = np.array([1, 2, 3, 4], np.float32)
    assert lib.iftrSetVertexBufferValueFloat4(vb, 2, 1, ctypes.c_void_p(v.ctypes.data)) == 0
    assert lib.iftrSetVertexBufferValueFloat4(vb, 3, 0, ctypes.c_void_p(v.ctypes.data)) == 1
    assert lib.iftrSetVertexBufferData(vb, ctypes.c_void_p(v.ctypes.data), 4) == 1  # wrong size
    bad = (ctypes.c_int * 1)(ig.IFTP_FLOAT2)
    assert lib.iftrSetVertexBufferLayout(vb, bad, 1) == 2  # position needs >= 3 floats
    mgr = lib.ifbufCreateBufferManager()
    buf = lib.ifbufCreateBuffer(mgr, 16)
    assert lib.ifbufBufferData(buf, ctypes.c_void_p(v.ctypes.data), 0, 16) == 0
    assert lib.ifbufBufferData(buf, ctypes.c_void_p(v.ctypes.data), 8, 16) == 1
    vd = lib.iftrCreateVaryingDescriptor()
    desc = (ctypes.c_int * 1)(ig.IFTP_FLOAT4)
    assert lib.iftrWriteVaryingDescriptor(vd, desc, 1) == 0
    for call, obj in ((lib.iftrDestroyVaryingDescriptor, vd), (lib.ifbufDestroyBufferManager, mgr),
                      (lib.iftrDestroyVertexBuffer, vb), (lib.iftrDestroyFrameBuffer, fb), (lib.ifcrDestroyImageFP32, img)):
        assert call(obj) == 0


def test_null_handles_rejected(lib):
    assert lib.iftrDrawLegacy(None, 3, 1) == 1
    assert lib.iftrDestroyInstance(None) == 1
    assert lib.iftrFinish(None) == 1


def test_mesh_outputs_argument_checks(lib):
    """iftrDrawMeshOutputs validates its arguments before any device work."""
    h = lib.iftrCreateInstance()
    assert h
    buf = (ctypes.c_float * 16)()
    ib = (ctypes.c_int * 8)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    q = ctypes.cast(ib, ctypes.c_void_p)
    # negative group count, attribute count above 4, varyings requested without an array, bad maxima
    assert lib.iftrDrawMeshOutputs(h, -1, p, None, 0, q, q, q, 4, 3, 1) == 1
    assert lib.iftrDrawMeshOutputs(h, 1, p, p, 5, q, q, q, 4, 3, 1) == 1
    assert lib.iftrDrawMeshOutputs(h, 1, p, None, 3, q, q, q, 4, 3, 1) == 1
    assert lib.iftrDrawMeshOutputs(h, 1, p, None, 0, q, q, q, 0, 3, 1) == 1
    assert lib.iftrDrawMeshOutputs(h, 1, None, None, 0, q, q, q, 4, 3, 1) == 1
    assert lib.iftrDrawMeshOutputs(None, 0, None, None, 0, None, None, None, 4, 3, 1) == 1
    assert lib.iftrDestroyInstance(h) == 0


@pytest.mark.skipif(not os.path.exists(os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")), reason="nvcc absent")
def test_extension_header_builds(lib):
    """The device-side extension point (include/ifrit_gb300_ext.cuh) compiles for sm_103a with a
    fragment functor and a mesh-stage functor, links against the library and loads (no calls)."""
    from ifrit_gb300 import build as ibuild
    here = os.path.dirname(os.path.abspath(__file__))
    out = os.path.join(ibuild.BUILD, "ext", "libext_shaders.so")
    ibuild.build_extension([os.path.join(here, "ext", "ext_shaders.cu")], out)
    ext = ctypes.CDLL(out)
    assert ext.ext_shade and ext.ext_draw_grid


def test_ordered_fragment_capacity_argument_checks(lib):
    h = lib.iftrCreateInstance()
    assert h
    assert lib.iftrSetOrderedFragmentCapacity(h, -2) == 1
    assert lib.iftrSetOrderedFragmentCapacity(h, 1 << 40) == 1
    for n in (-1, 0, 1000):
        assert lib.iftrSetOrderedFragmentCapacity(h, n) == 0
    assert lib.iftrSetOrderedFragmentCapacity(None, 0) == 1
    assert lib.iftrDestroyInstance(h) == 0
