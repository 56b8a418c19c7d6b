"""GB300-native software triangle rasterizer (Ifrit-v2 soft renderer drop-in).

Python front end over the C-ABI of ``libifrit_gb300.so`` (declared in
include/ifrit_gb300.h).  Every call goes through the exported ``iftr*`` / ``ifcr*`` /
``ifbuf*`` entry points; there is no Python or CPU fallback: if the CUDA library cannot be
loaded, :func:`load` raises.
"""
import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

IFTR_OK = 0
ERRORS = {1: "invalid argument", 2: "unsupported", 3: "CUDA error", 4: "scratch capacity exceeded",
          5: "no CUDA device", 6: "missing binding", 7: "ordered tile list limit"}
FORMAT_RGBA8, FORMAT_RGBA16F, FORMAT_RGBA32F, FORMAT_RGB32F = 0, 1, 2, 3
FS_GOURAUD, FS_TEXTURED, FS_PRIMITIVE_ID = 0, 1, 2
IFTP_FLOAT1, IFTP_FLOAT2, IFTP_FLOAT3, IFTP_FLOAT4 = 1, 2, 3, 4
CULL_NONE, CULL_FRONT, CULL_BACK, CULL_FRONT_AND_BACK = 0, 1, 2, 3
NEVER, LESS, EQUAL, LESS_OR_EQUAL, GREATER, NOT_EQUAL, GREATER_OR_EQUAL, ALWAYS = range(8)
POLYGON_FILL, POLYGON_LINE, POLYGON_POINT = 0, 1, 2
POLYGON_RULES_FILL_PARTS, POLYGON_RULES_REFERENCE = 0, 1
RASTER_TILED, RASTER_ATOMIC = 0, 1

EXPORTED = [
    "iftrCreateInstance", "iftrDestroyInstance", "iftrInit", "iftrBindFrameBuffer", "iftrBindVertexBuffer",
    "iftrBindIndexBuffer", "iftrBindVertexShaderFunc", "iftrBindFragmentShaderFunc", "iftrBindVertexShader",
    "iftrBindFragmentShader", "iftrBindVertexShaderBuiltin", "iftrBindFragmentShaderBuiltin",
    "iftrBindUniformBuffer", "iftrSetBlendFunc", "iftrSetDepthFunc", "iftrOptsetForceDeterministic",
    "iftrOptSetDepthTestEnable", "iftrDrawLegacy", "iftrClear", "iftrSetCullMode", "iftrSetFrontFace",
    "iftrSetMsaaSamples", "iftrSetClearValues", "iftrSetDepthWriteEnable", "iftrCreateTexture",
    "iftrCopyHostBufferToImage", "iftrGenerateMipmap", "iftrCreateSampler", "iftrBindTexture", "iftrSetStream",
    "iftrDrawAsync", "iftrFinish", "iftrBindVertexBufferDevice", "iftrBindIndexBufferDevice",
    "iftrSetUniformMatrix", "iftrSetVisibilityOutput", "iftrReserve", "iftrGetDeviceAttachments",
    "iftrReadbackColor", "iftrReadbackDepth", "iftrReadbackVisibility", "iftrGetStats", "iftrGetErrorString",
    "iftrCreateFrameBuffer", "iftrDestroyFrameBuffer", "iftrSetFrameBufferColorAttachmentFP32",
    "iftrSetFrameBufferDepthAttachmentFP32", "iftrSetFrameBufferColorAttachmentDevice", "ifcrCreateImageFP32",
    "ifcrDestroyImageFP32", "ifcrGetImageRawDataFP32", "iftrCreateVaryingDescriptor",
    "iftrDestroyVaryingDescriptor", "iftrWriteVaryingDescriptor", "iftrCreateVertexBuffer",
    "iftrDestroyVertexBuffer", "iftrSetVertexBufferLayout", "iftrSetVertexBufferSize",
    "iftrAllocateVertexBuffer", "iftrSetVertexBufferValueFloat4", "iftrSetVertexBufferData",
    "ifbufCreateBufferManager", "ifbufDestroyBufferManager", "ifbufCreateBuffer", "ifbufDestroyBuffer",
    "ifbufBufferData", "iftrSetStageTiming", "iftrGetStageTimes", "iftrGetVertexBufferRawData",
    "iftrSetVertexBufferDirty", "ifbufGetBufferRawData", "ifbufSetBufferDirty", "iftrDrawNoAlloc",
    "iftrBeginPass", "iftrPassDraw", "iftrEndPass", "iftrDrawBatch", "iftrSetBatchTuning", "iftrGetBatchTuning",
    "iftrDiffForward", "iftrDiffBackward", "iftrSetScissors", "iftrSetScissorTestEnable",
    "iftrSetRasterizerPolygonMode", "iftrSetRasterPath", "iftrDrawMeshOutputs", "iftrSetOrderedFragmentCapacity", "iftrSetPolygonRules",
]


class BlendState(ctypes.Structure):
    _fields_ = [("blendEnable", ctypes.c_int), ("srcColorBlendFactor", ctypes.c_int),
                ("dstColorBlendFactor", ctypes.c_int), ("srcAlphaBlendFactor", ctypes.c_int),
                ("dstAlphaBlendFactor", ctypes.c_int)]


class SamplerState(ctypes.Structure):
    _fields_ = [("filterMode", ctypes.c_int), ("addressModeU", ctypes.c_int), ("addressModeV", ctypes.c_int),
                ("addressModeW", ctypes.c_int), ("borderColor", ctypes.c_int), ("anisotropyEnable", ctypes.c_int),
                ("maxAnisotropy", ctypes.c_float), ("lodBias", ctypes.c_float)]


class NoAllocPass(ctypes.Structure):
    """IfritGbNoAllocPass (include/ifrit_gb300.h)."""
    _fields_ = [("vertices", ctypes.c_void_p), ("strideFloats", ctypes.c_int), ("numVertices", ctypes.c_int),
                ("attrOffsetFloats", ctypes.c_int), ("attrCount", ctypes.c_int), ("indices", ctypes.c_void_p),
                ("numIndices", ctypes.c_int), ("mvp", ctypes.c_float * 16), ("width", ctypes.c_int),
                ("height", ctypes.c_int), ("samples", ctypes.c_int), ("colorFormat", ctypes.c_int),
                ("color", ctypes.c_void_p), ("depth", ctypes.c_void_p), ("visibility", ctypes.c_void_p),
                ("clear", ctypes.c_int), ("clearColor", ctypes.c_float * 4), ("clearDepth", ctypes.c_float),
                ("depthFunc", ctypes.c_int), ("depthTest", ctypes.c_int), ("depthWrite", ctypes.c_int),
                ("cullMode", ctypes.c_int), ("frontCounterClockwise", ctypes.c_int), ("shadingModel", ctypes.c_int),
                ("texels", ctypes.c_void_p), ("texWidth", ctypes.c_int), ("texHeight", ctypes.c_int),
                ("texLevels", ctypes.c_int), ("sampler", SamplerState)]


class BatchView(ctypes.Structure):
    """IfritGbBatchView (include/ifrit_gb300.h)."""
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("samples", ctypes.c_int),
                ("colorFormat", ctypes.c_int), ("color", ctypes.c_void_p), ("depth", ctypes.c_void_p),
                ("visibility", ctypes.c_void_p), ("clear", ctypes.c_int), ("clearColor", ctypes.c_float * 4),
                ("clearDepth", ctypes.c_float)]


class BatchDraw(ctypes.Structure):
    """IfritGbBatchDraw (include/ifrit_gb300.h)."""
    _fields_ = [("view", ctypes.c_int), ("vertices", ctypes.c_void_p), ("strideFloats", ctypes.c_int),
                ("numVertices", ctypes.c_int), ("attrOffsetFloats", ctypes.c_int), ("attrCount", ctypes.c_int),
                ("indices", ctypes.c_void_p), ("numIndices", ctypes.c_int), ("mvp", ctypes.c_float * 16),
                ("depthFunc", ctypes.c_int), ("depthTest", ctypes.c_int), ("depthWrite", ctypes.c_int),
                ("cullMode", ctypes.c_int), ("frontCounterClockwise", ctypes.c_int), ("shadingModel", ctypes.c_int),
                ("blend", BlendState), ("texels", ctypes.c_void_p), ("texWidth", ctypes.c_int),
                ("texHeight", ctypes.c_int), ("texLevels", ctypes.c_int), ("sampler", SamplerState)]


class DiffPass(ctypes.Structure):
    """IfritGbDiffPass (include/ifrit_gb300.h)."""
    _fields_ = [("numViews", ctypes.c_int), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("mvp", ctypes.c_void_p), ("positions", ctypes.c_void_p), ("colors", ctypes.c_void_p),
                ("uvs", ctypes.c_void_p), ("faces", ctypes.c_void_p), ("neighbors", ctypes.c_void_p),
                ("numVertices", ctypes.c_int), ("numTriangles", ctypes.c_int), ("texture", ctypes.c_void_p),
                ("texWidth", ctypes.c_int), ("texHeight", ctypes.c_int), ("visibility", ctypes.c_void_p),
                ("shaded", ctypes.c_void_p), ("image", ctypes.c_void_p), ("aaCodes", ctypes.c_void_p),
                ("gradImage", ctypes.c_void_p), ("gradPositions", ctypes.c_void_p), ("gradColors", ctypes.c_void_p),
                ("gradUvs", ctypes.c_void_p)]


class Stats(ctypes.Structure):
    _fields_ = [("triangles_in", ctypes.c_uint64), ("tile_pairs", ctypes.c_uint64),
                ("pair_capacity", ctypes.c_uint64), ("retries", ctypes.c_int), ("deferred_tiles", ctypes.c_int),
                ("deferred_fragments", ctypes.c_uint64)]


_lib = None


def load(build_if_missing=True):
    """Loads libifrit_gb300.so (building it in-tree if needed) and declares signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and not os.path.exists(LIB_PATH):
        _build.build()
    lib = ctypes.CDLL(LIB_PATH)
    vp, ip, fp, sz = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_size_t
    for name in EXPORTED:
        getattr(lib, name).restype = ctypes.c_int
    for name in ("iftrCreateInstance", "iftrCreateFrameBuffer", "ifcrCreateImageFP32", "iftrCreateVaryingDescriptor",
                 "iftrCreateVertexBuffer", "ifbufCreateBufferManager", "ifbufCreateBuffer", "iftrGetVertexBufferRawData",
                 "ifbufGetBufferRawData"):
        getattr(lib, name).restype = vp
    lib.ifcrGetImageRawDataFP32.restype = fp
    lib.iftrGetErrorString.restype = ctypes.c_char_p
    sig = {
        "iftrDestroyInstance": [vp], "iftrInit": [vp], "iftrBindFrameBuffer": [vp, vp],
        "iftrBindVertexBuffer": [vp, vp], "iftrBindIndexBuffer": [vp, vp],
        "iftrBindVertexShaderFunc": [vp, vp, vp], "iftrBindFragmentShaderFunc": [vp, vp],
        "iftrBindVertexShader": [vp, vp], "iftrBindFragmentShader": [vp, vp],
        "iftrBindVertexShaderBuiltin": [vp, ip, vp], "iftrBindFragmentShaderBuiltin": [vp, ip],
        "iftrBindUniformBuffer": [vp, ip, ip, vp], "iftrSetBlendFunc": [vp, ctypes.POINTER(BlendState)],
        "iftrSetDepthFunc": [vp, ip], "iftrOptsetForceDeterministic": [vp, ip], "iftrOptSetDepthTestEnable": [vp, ip],
        "iftrDrawLegacy": [vp, ip, ip], "iftrClear": [vp], "iftrSetCullMode": [vp, ip], "iftrSetFrontFace": [vp, ip],
        "iftrSetMsaaSamples": [vp, ip], "iftrSetClearValues": [vp, fp, ctypes.c_float],
        "iftrSetDepthWriteEnable": [vp, ip], "iftrCreateTexture": [vp, ip, ip, ip, ip],
        "iftrCopyHostBufferToImage": [vp, vp, ip], "iftrGenerateMipmap": [vp, ip, ip],
        "iftrCreateSampler": [vp, ip, ctypes.POINTER(SamplerState)], "iftrBindTexture": [vp, ip, ip],
        "iftrSetStream": [vp, vp], "iftrDrawAsync": [vp, ip, ip], "iftrFinish": [vp],
        "iftrBindVertexBufferDevice": [vp, vp, ip, ip, ip, ip], "iftrBindIndexBufferDevice": [vp, vp, ip],
        "iftrSetUniformMatrix": [vp, fp], "iftrSetVisibilityOutput": [vp, ip], "iftrReserve": [vp, sz],
        "iftrGetDeviceAttachments": [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)],
        "iftrReadbackColor": [vp, vp, sz], "iftrReadbackDepth": [vp, vp, sz], "iftrReadbackVisibility": [vp, vp, sz],
        "iftrGetStats": [vp, ctypes.POINTER(Stats)], "iftrGetErrorString": [ip],
        "iftrDestroyFrameBuffer": [vp], "iftrSetFrameBufferColorAttachmentFP32": [vp, ctypes.POINTER(vp), sz],
        "iftrSetFrameBufferDepthAttachmentFP32": [vp, vp], "iftrSetFrameBufferColorAttachmentDevice": [vp, ip, ip, ip],
        "ifcrCreateImageFP32": [sz, sz, sz], "ifcrDestroyImageFP32": [vp], "ifcrGetImageRawDataFP32": [vp],
        "iftrDestroyVaryingDescriptor": [vp], "iftrWriteVaryingDescriptor": [vp, ctypes.POINTER(ctypes.c_int), sz],
        "iftrDestroyVertexBuffer": [vp], "iftrSetVertexBufferLayout": [vp, ctypes.POINTER(ctypes.c_int), sz],
        "iftrSetVertexBufferSize": [vp, sz], "iftrAllocateVertexBuffer": [vp],
        "iftrSetVertexBufferValueFloat4": [vp, ip, ip, vp], "iftrSetVertexBufferData": [vp, vp, sz],
        "ifbufDestroyBufferManager": [vp], "ifbufCreateBuffer": [vp, sz], "ifbufDestroyBuffer": [vp],
        "ifbufBufferData": [vp, vp, sz, sz], "iftrSetStageTiming": [vp, ip], "iftrGetStageTimes": [vp, fp, ip],
        "iftrGetVertexBufferRawData": [vp], "iftrSetVertexBufferDirty": [vp], "ifbufGetBufferRawData": [vp],
        "ifbufSetBufferDirty": [vp], "iftrDrawNoAlloc": [ctypes.POINTER(NoAllocPass), vp],
        "iftrBeginPass": [vp, ip], "iftrPassDraw": [vp, ip, ip], "iftrEndPass": [vp],
        "iftrDrawBatch": [vp, ctypes.POINTER(BatchView), ip, ctypes.POINTER(BatchDraw), ip],
        "iftrSetBatchTuning": [vp, ip, ip, ip],
        "iftrGetBatchTuning": [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
        "iftrDiffForward": [ctypes.POINTER(DiffPass), vp], "iftrDiffBackward": [ctypes.POINTER(DiffPass), vp],
        "iftrSetScissors": [vp, fp, ip], "iftrSetScissorTestEnable": [vp, ip],
        "iftrSetRasterizerPolygonMode": [vp, ip], "iftrSetRasterPath": [vp, ip],
        "iftrDrawMeshOutputs": [vp, ip, vp, vp, ip, vp, vp, vp, ip, ip, ip],
        "iftrSetOrderedFragmentCapacity": [vp, ctypes.c_longlong],
    }
    for name, args in sig.items():
        getattr(lib, name).argtypes = args
    lib.iftrCreateInstance.argtypes = []
    lib.iftrCreateFrameBuffer.argtypes = []
    lib.iftrCreateVaryingDescriptor.argtypes = []
    lib.iftrCreateVertexBuffer.argtypes = []
    lib.ifbufCreateBufferManager.argtypes = []
    _lib = lib
    return lib


class IfritError(RuntimeError):
    def __init__(self, call, code):
        super().__init__("%s failed: %s (%d)" % (call, ERRORS.get(code, "?"), code))
        self.code = code


def check(call, rc):
    if rc != IFTR_OK:
        raise IfritError(call, rc)
    return rc


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Renderer:
    """Owns one renderer instance plus the objects the reference API expects the caller to
    own (framebuffer, vertex buffer, index/uniform buffers), and exposes a numpy-friendly
    draw.  Every method is a thin sequence of C-ABI calls."""

    def __init__(self, width, height, samples=1, fmt=FORMAT_RGBA8, visibility=True):
        self.lib = L = load()
        self.h = L.iftrCreateInstance()
        if not self.h:
            raise MemoryError("iftrCreateInstance")
        check("iftrInit", L.iftrInit(self.h))
        self.width, self.height, self.samples, self.fmt = width, height, samples, fmt
        self.fb = L.iftrCreateFrameBuffer()
        check("iftrSetFrameBufferColorAttachmentDevice",
              L.iftrSetFrameBufferColorAttachmentDevice(self.fb, fmt, width, height))
        check("iftrBindFrameBuffer", L.iftrBindFrameBuffer(self.h, self.fb))
        check("iftrSetMsaaSamples", L.iftrSetMsaaSamples(self.h, samples))
        check("iftrSetVisibilityOutput", L.iftrSetVisibilityOutput(self.h, int(visibility)))
        check("iftrBindVertexShaderBuiltin", L.iftrBindVertexShaderBuiltin(self.h, 0, None))
        self.vb = L.iftrCreateVertexBuffer()
        self.mgr = L.ifbufCreateBufferManager()
        self.ib = None
        self.ib_bytes = 0
        self.vb_layout = None
        self.vb_count = -1

    def close(self):
        L = self.lib
        if self.h:
            L.iftrDestroyInstance(self.h)
            L.iftrDestroyFrameBuffer(self.fb)
            L.iftrDestroyVertexBuffer(self.vb)
            L.ifbufDestroyBufferManager(self.mgr)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state
    def set_state(self, *, cull=CULL_BACK, front_ccw=True, depth_func=LESS_OR_EQUAL, depth_test=True,
                  depth_write=True, shading=FS_GOURAUD, clear_color=(0, 0, 0, 0), clear_depth=1.0):
        L, h = self.lib, self.h
        check("iftrSetCullMode", L.iftrSetCullMode(h, cull))
        check("iftrSetFrontFace", L.iftrSetFrontFace(h, int(front_ccw)))
        check("iftrSetDepthFunc", L.iftrSetDepthFunc(h, depth_func))
        check("iftrOptSetDepthTestEnable", L.iftrOptSetDepthTestEnable(h, int(depth_test)))
        check("iftrSetDepthWriteEnable", L.iftrSetDepthWriteEnable(h, int(depth_write)))
        check("iftrBindFragmentShaderBuiltin", L.iftrBindFragmentShaderBuiltin(h, shading))
        cc = (ctypes.c_float * 4)(*clear_color)
        check("iftrSetClearValues", L.iftrSetClearValues(h, cc, ctypes.c_float(clear_depth)))

    def set_texture(self, level0, max_aniso=1, address=0, filter_mode=1, lod_bias=0.0, slot=0):
        """level0: (h, w) uint32 RGBA8; builds the full mip chain on the device."""
        L, h = self.lib, self.h
        th, tw = level0.shape
        check("iftrCreateTexture", L.iftrCreateTexture(h, slot, tw, th, 0))
        data = np.ascontiguousarray(level0, np.uint32)
        check("iftrCopyHostBufferToImage", L.iftrCopyHostBufferToImage(h, _ptr(data), slot))
        check("iftrGenerateMipmap", L.iftrGenerateMipmap(h, slot, 1))
        s = SamplerState(filter_mode, address, address, address, 0, int(max_aniso > 1), float(max_aniso), lod_bias)
        check("iftrCreateSampler", L.iftrCreateSampler(h, slot, ctypes.byref(s)))
        check("iftrBindTexture", L.iftrBindTexture(h, slot, slot))

    def set_blend(self, enable, src_color=6, dst_color=7, src_alpha=1, dst_alpha=7):
        """Blend factors use the IfritBlendFactor numbering (6 SRC_ALPHA, 7 ONE_MINUS_SRC_ALPHA)."""
        s = BlendState(int(enable), src_color, dst_color, src_alpha, dst_alpha)
        check("iftrSetBlendFunc", self.lib.iftrSetBlendFunc(self.h, ctypes.byref(s)))

    def draw_mesh_outputs(self, positions, indices, num_vertices, num_indices, attributes=None, attr_count=0,
                          clear=True):
        """Draws a mesh (or geometry) stage's per-work-group outputs (iftrDrawMeshOutputs): CUDA
        tensors positions (G, maxV, 4) float32 clip space, attributes (G, maxV, 4) float32 or None,
        indices (G, maxI) int32 group-local, num_vertices / num_indices (G,) int32."""
        G, max_v = int(positions.shape[0]), int(positions.shape[1])
        max_i = int(indices.shape[1])
        for t in (positions, indices, num_vertices, num_indices) + ((attributes,) if attributes is not None else ()):
            if not (t.is_cuda and t.is_contiguous()):
                raise ValueError("mesh outputs must be contiguous CUDA tensors")
        check("iftrDrawMeshOutputs", self.lib.iftrDrawMeshOutputs(
            self.h, G, positions.data_ptr(), attributes.data_ptr() if attributes is not None else None, attr_count,
            indices.data_ptr(), num_vertices.data_ptr(), num_indices.data_ptr(), max_v, max_i, int(clear)))

    def set_ordered_fragment_capacity(self, fragments=-1):
        """-1: automatic deferred shading of ordered fragments; 0: shaded inside the ordered stage;
        n > 0: a fragment buffer of exactly n (tiles that do not fit are finished in the stage)."""
        check("iftrSetOrderedFragmentCapacity", self.lib.iftrSetOrderedFragmentCapacity(self.h, int(fragments)))

    def set_raster_path(self, path):
        check("iftrSetRasterPath", self.lib.iftrSetRasterPath(self.h, path))

    def set_polygon_mode(self, mode, rules=None):
        """rules: POLYGON_RULES_FILL_PARTS or POLYGON_RULES_REFERENCE (iftrSetPolygonRules)."""
        check("iftrSetRasterizerPolygonMode", self.lib.iftrSetRasterizerPolygonMode(self.h, mode))
        if rules is not None:
            check("iftrSetPolygonRules", self.lib.iftrSetPolygonRules(self.h, rules))

    def set_scissors(self, rects, enable=True):
        """rects: list of (x, y, w, h); enable False switches the test off."""
        arr = (ctypes.c_float * (4 * max(1, len(rects))))(*[float(x) for r in rects for x in r])
        check("iftrSetScissors", self.lib.iftrSetScissors(self.h, arr, len(rects)))
        check("iftrSetScissorTestEnable", self.lib.iftrSetScissorTestEnable(self.h, int(enable)))

    def begin_pass(self, clear=True):
        check("iftrBeginPass", self.lib.iftrBeginPass(self.h, int(clear)))

    def pass_draw(self, first_index, num_indices):
        check("iftrPassDraw", self.lib.iftrPassDraw(self.h, first_index, num_indices))

    def end_pass(self):
        check("iftrEndPass", self.lib.iftrEndPass(self.h))

    def set_mvp(self, mvp):
        m = np.ascontiguousarray(mvp, np.float32).reshape(-1)
        check("iftrSetUniformMatrix", self.lib.iftrSetUniformMatrix(self.h, m.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    # ---- geometry through the reference-style host objects
    def set_geometry(self, vertices, indices, attr_components):
        """vertices: (V, 3 + attr_components) float32 AoS; indices: (T, 3) int32."""
        L, h = self.lib, self.h
        vertices = np.ascontiguousarray(vertices, np.float32)
        indices = np.ascontiguousarray(indices, np.int32)
        layout = (IFTP_FLOAT3,) + ((attr_components,) if attr_components else ())
        if layout != self.vb_layout or len(vertices) != self.vb_count:
            arr = (ctypes.c_int * len(layout))(*layout)
            check("iftrSetVertexBufferLayout", L.iftrSetVertexBufferLayout(self.vb, arr, len(layout)))
            check("iftrSetVertexBufferSize", L.iftrSetVertexBufferSize(self.vb, len(vertices)))
            check("iftrAllocateVertexBuffer", L.iftrAllocateVertexBuffer(self.vb))
            self.vb_layout, self.vb_count = layout, len(vertices)
        check("iftrSetVertexBufferData", L.iftrSetVertexBufferData(self.vb, _ptr(vertices), vertices.nbytes))
        if self.ib is None or self.ib_bytes != indices.nbytes:
            self.ib = L.ifbufCreateBuffer(self.mgr, indices.nbytes)
            self.ib_bytes = indices.nbytes
        check("ifbufBufferData", L.ifbufBufferData(self.ib, _ptr(indices), 0, indices.nbytes))
        check("iftrBindVertexBuffer", L.iftrBindVertexBuffer(h, self.vb))
        check("iftrBindIndexBuffer", L.iftrBindIndexBuffer(h, self.ib))
        self.num_indices = indices.size

    def bind_device_geometry(self, vert_ptr, stride_floats, num_vertices, attr_offset, attr_count, idx_ptr, num_indices):
        L, h = self.lib, self.h
        check("iftrBindVertexBufferDevice",
              L.iftrBindVertexBufferDevice(h, ctypes.c_void_p(vert_ptr), stride_floats, num_vertices, attr_offset, attr_count))
        check("iftrBindIndexBufferDevice", L.iftrBindIndexBufferDevice(h, ctypes.c_void_p(idx_ptr), num_indices))
        self.num_indices = num_indices

    def reserve(self, pairs):
        check("iftrReserve", self.lib.iftrReserve(self.h, pairs))

    def set_stream(self, stream_ptr):
        check("iftrSetStream", self.lib.iftrSetStream(self.h, ctypes.c_void_p(stream_ptr)))

    # ---- draw
    def draw(self, clear=True, num_indices=None):
        n = self.num_indices if num_indices is None else num_indices
        check("iftrDrawLegacy", self.lib.iftrDrawLegacy(self.h, n, int(clear)))

    def draw_async(self, clear=True, num_indices=None):
        n = self.num_indices if num_indices is None else num_indices
        check("iftrDrawAsync", self.lib.iftrDrawAsync(self.h, n, int(clear)))

    def finish(self):
        check("iftrFinish", self.lib.iftrFinish(self.h))

    # ---- readback
    def color(self):
        if self.fmt == FORMAT_RGBA8:
            out = np.empty((self.height, self.width), np.uint32)
        elif self.fmt == FORMAT_RGBA16F:
            out = np.empty((self.height, self.width), np.uint64)
        elif self.fmt == FORMAT_RGBA32F:
            out = np.empty((self.height, self.width, 4), np.float32)
        else:
            out = np.empty((self.height, self.width, 3), np.float32)
        check("iftrReadbackColor", self.lib.iftrReadbackColor(self.h, _ptr(out), out.nbytes))
        return out

    def color_into(self, out):
        check("iftrReadbackColor", self.lib.iftrReadbackColor(self.h, _ptr(out), out.nbytes))

    def depth(self):
        out = np.empty((self.height, self.width, self.samples), np.float32)
        check("iftrReadbackDepth", self.lib.iftrReadbackDepth(self.h, _ptr(out), out.size))
        return out

    def visibility(self):
        out = np.empty((self.height, self.width, self.samples), np.int32)
        check("iftrReadbackVisibility", self.lib.iftrReadbackVisibility(self.h, _ptr(out), out.size))
        return out

    def device_attachments(self):
        c, d, v = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check("iftrGetDeviceAttachments", self.lib.iftrGetDeviceAttachments(self.h, ctypes.byref(c), ctypes.byref(d), ctypes.byref(v)))
        return c.value, d.value, v.value

    def set_stage_timing(self, enable=True):
        check("iftrSetStageTiming", self.lib.iftrSetStageTiming(self.h, int(enable)))

    def stage_times(self):
        """[count, scan, scatter, raster, shade, ordered] device milliseconds of the last pass."""
        ms = (ctypes.c_float * 6)()
        check("iftrGetStageTimes", self.lib.iftrGetStageTimes(self.h, ms, 6))
        return list(ms)

    def mark_geometry_dirty(self):
        """Marks the host vertex and index buffers as rewritten (the next draw uploads both)."""
        check("iftrSetVertexBufferDirty", self.lib.iftrSetVertexBufferDirty(self.vb))
        check("ifbufSetBufferDirty", self.lib.ifbufSetBufferDirty(self.ib))

    def stats(self):
        s = Stats()
        check("iftrGetStats", self.lib.iftrGetStats(self.h, ctypes.byref(s)))
        return s
