"""Batched views through ``iftrDrawBatch``: many independent views of uneven size, sample
count and triangle count rendered as one pass from device-resident inputs.

PyTorch provides the device storage (inputs and render targets are CUDA tensors) and the
stream; every render call goes through the C-ABI.  The first :meth:`BatchRenderer.draw` of a
new description sizes the scratch, autotunes the launch parameters and captures a CUDA graph;
later calls with the same description replay the graph.
"""
import ctypes

import numpy as np

from . import (BatchDraw, BatchView, BlendState, SamplerState, FORMAT_RGBA8, FORMAT_RGBA16F, FORMAT_RGBA32F,
               FS_GOURAUD, FS_TEXTURED, CULL_BACK, LESS_OR_EQUAL, check, load)


def _color_shape(fmt, H, W):
    import torch
    if fmt == FORMAT_RGBA8:
        return (H, W), torch.int32
    if fmt == FORMAT_RGBA16F:
        return (H, W), torch.int64
    if fmt == FORMAT_RGBA32F:
        return (H, W, 4), torch.float32
    return (H, W, 3), torch.float32


class BatchRenderer:
    """One renderer instance used for batched passes.  Views own CUDA tensors (colour,
    per-sample depth, optional per-sample visibility); meshes reference CUDA tensors of
    vertices (V, stride) float32 and indices (T, 3) int32."""

    def __init__(self, device="cuda"):
        import torch
        self.torch = torch
        self.device = torch.device(device)
        self.lib = L = load()
        self.h = L.iftrCreateInstance()
        if not self.h:
            raise MemoryError("iftrCreateInstance")
        check("iftrInit", L.iftrInit(self.h))
        self.stream = torch.cuda.current_stream(self.device)
        check("iftrSetStream", L.iftrSetStream(self.h, ctypes.c_void_p(self.stream.cuda_stream)))
        self.views, self.draws, self.keep = [], [], []
        self._arrays = None

    def close(self):
        if self.h:
            self.lib.iftrDestroyInstance(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- description
    def add_view(self, width, height, samples=1, fmt=FORMAT_RGBA8, visibility=False, clear=True,
                 clear_color=(0.0, 0.0, 0.0, 0.0), clear_depth=1.0, targets=None):
        """targets: optional dict of caller-owned CUDA tensors (color, depth, vis) to render into."""
        torch = self.torch
        shape, dt = _color_shape(fmt, height, width)
        if targets is not None:
            t = dict(targets)
            visibility = t.get("vis") is not None
        else:
            t = {"color": torch.zeros(shape, dtype=dt, device=self.device),
                 "depth": torch.full((height, width, samples), float(clear_depth), dtype=torch.float32,
                                     device=self.device),
                 "vis": torch.full((height, width, samples), -1, dtype=torch.int32, device=self.device)
                 if visibility else None}
        v = BatchView()
        v.width, v.height, v.samples, v.colorFormat = width, height, samples, fmt
        v.color, v.depth = t["color"].data_ptr(), t["depth"].data_ptr()
        v.visibility = t["vis"].data_ptr() if visibility else None
        v.clear = int(clear)
        for i in range(4):
            v.clearColor[i] = float(clear_color[i])
        v.clearDepth = float(clear_depth)
        self.views.append((v, t))
        self._arrays = None
        return len(self.views) - 1

    def set_view_clear(self, view, clear):
        self.views[view][0].clear = int(clear)
        self._arrays = None

    def to_device(self, a, dtype):
        torch = self.torch
        if isinstance(a, torch.Tensor):
            return a.to(self.device, dtype).contiguous()
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32 if dtype == torch.float32 else np.int32)).to(self.device)

    def add_mesh(self, view, vertices, indices, mvp, attr_count=3, attr_offset=3, *, cull=CULL_BACK,
                 front_ccw=True, depth_func=LESS_OR_EQUAL, depth_test=True, depth_write=True, shading=FS_GOURAUD,
                 blend=None, texture=None, sampler=None):
        """vertices / indices: numpy or torch; texture: (device uint32 mip chain, levels, w, h)."""
        torch = self.torch
        dv = self.to_device(vertices, torch.float32)
        di = self.to_device(indices, torch.int32).reshape(-1)
        d = BatchDraw()
        d.view = view
        d.vertices, d.strideFloats, d.numVertices = dv.data_ptr(), dv.shape[1], dv.shape[0]
        d.attrOffsetFloats, d.attrCount = attr_offset, attr_count
        d.indices, d.numIndices = di.data_ptr(), di.numel()
        for i, x in enumerate(np.asarray(mvp, np.float32).reshape(-1)):
            d.mvp[i] = float(x)
        d.depthFunc, d.depthTest, d.depthWrite = depth_func, int(depth_test), int(depth_write)
        d.cullMode, d.frontCounterClockwise, d.shadingModel = cull, int(front_ccw), shading
        if blend:
            d.blend = BlendState(1, *blend)
        else:
            d.blend = BlendState(0, 1, 0, 1, 0)
        keep = [dv, di]
        if shading == FS_TEXTURED:
            chain, levels, tw, th = texture
            keep.append(chain)
            d.texels, d.texWidth, d.texHeight, d.texLevels = chain.data_ptr(), tw, th, levels
            s = sampler or {}
            aniso = s.get("max_aniso", 1)
            d.sampler = SamplerState(s.get("filter", 1), s.get("address", 0), s.get("address", 0), 0, 0,
                                     int(aniso > 1), float(aniso), float(s.get("lod_bias", 0.0)))
        self.draws.append(d)
        self.keep.append(keep)
        self._arrays = None
        return len(self.draws) - 1, dv, di

    # ---- tuning
    def set_tuning(self, autotune=True, tile_size=16, ctas_per_sm=0):
        check("iftrSetBatchTuning", self.lib.iftrSetBatchTuning(self.h, int(autotune), tile_size, ctas_per_sm))

    def tuning(self):
        ts, cp = ctypes.c_int(), ctypes.c_int()
        check("iftrGetBatchTuning", self.lib.iftrGetBatchTuning(self.h, ctypes.byref(ts), ctypes.byref(cp)))
        return ts.value, cp.value

    # ---- render
    def _build_arrays(self):
        if self._arrays is None:
            va = (BatchView * len(self.views))(*[v for v, _ in self.views])
            da = (BatchDraw * max(1, len(self.draws)))(*self.draws)
            self._arrays = (va, da)
        return self._arrays

    def draw(self):
        """Enqueues the batch on the renderer's stream (asynchronous after the first call)."""
        va, da = self._build_arrays()
        check("iftrDrawBatch", self.lib.iftrDrawBatch(self.h, va, len(self.views), da, len(self.draws)))

    def finish(self):
        check("iftrFinish", self.lib.iftrFinish(self.h))

    def target(self, view):
        return self.views[view][1]

    def color(self, view):
        c = self.views[view][1]["color"].cpu().numpy()
        fmt = self.views[view][0].colorFormat
        if fmt == FORMAT_RGBA8:
            return c.view(np.uint32)
        if fmt == FORMAT_RGBA16F:
            return c.view(np.uint64)
        return c

    def depth(self, view):
        return self.views[view][1]["depth"].cpu().numpy()

    def visibility(self, view):
        return self.views[view][1]["vis"].cpu().numpy()
