"""Differentiable rendering of many views of one triangle mesh.

Forward: the batched rasterizer (``iftrDrawBatch``, 1x, back-face culling, depth LESS) writes
one triangle id per pixel and view; ``iftrDiffForward`` shades every pixel (perspective-correct
per-vertex colour times a bilinear RGB texture at the interpolated UV) and antialiases
silhouette edges.  Backward: ``iftrDiffBackward`` recomputes everything it needs from the saved
visibility buffer and antialiasing decisions and accumulates gradients with respect to
per-vertex positions, colours and UVs.  :class:`RenderFunction` is the
``torch.autograd.Function`` over both.
"""
import ctypes

import numpy as np

from . import (CULL_BACK, FORMAT_RGBA8, FS_PRIMITIVE_ID, LESS, DiffPass, check, load)
from .batch import BatchRenderer


def mesh_neighbors(faces):
    """(T, 3) int32: for triangle t and vertex k, the triangle sharing the edge opposite k
    (vertices k+1, k+2), or -1 when the edge has no second triangle."""
    f = np.asarray(faces, np.int64).reshape(-1, 3)
    T = len(f)
    a = np.concatenate([f[:, 1], f[:, 2], f[:, 0]])
    b = np.concatenate([f[:, 2], f[:, 0], f[:, 1]])
    owner = np.concatenate([np.arange(T)] * 3)
    slot = np.repeat(np.arange(3), T)
    key = np.minimum(a, b) * (int(f.max()) + 1) + np.maximum(a, b)
    order = np.argsort(key, kind="stable")
    ks = key[order]
    out = np.full((T, 3), -1, np.int32)
    same = np.nonzero(ks[1:] == ks[:-1])[0]
    # only edges shared by exactly two triangles get a neighbour
    single = np.ones(len(same), bool)
    if len(same) > 1:
        run = np.diff(same) == 1
        single[1:] &= ~run
        single[:-1] &= ~run
    i = same[single]
    o0, o1 = order[i], order[i + 1]
    out[owner[o0], slot[o0]] = owner[o1]
    out[owner[o1], slot[o1]] = owner[o0]
    return out


class DiffRenderer:
    """Views (N cameras, one resolution) of one mesh with fixed topology and texture."""

    def __init__(self, faces, num_vertices, width, height, mvps, texture, device="cuda"):
        import torch
        self.torch = torch
        self.device = torch.device(device)
        self.lib = load()
        self.W, self.H = int(width), int(height)
        self.mvps = torch.as_tensor(np.asarray(mvps, np.float32).reshape(-1, 16), device=self.device).contiguous()
        self.N = self.mvps.shape[0]
        faces = np.ascontiguousarray(np.asarray(faces, np.int32).reshape(-1, 3))
        self.T, self.V = len(faces), int(num_vertices)
        self.faces = torch.from_numpy(faces).to(self.device)
        self.neighbors = torch.from_numpy(mesh_neighbors(faces)).to(self.device)
        tex = np.ascontiguousarray(np.asarray(texture, np.float32))
        self.tex_h, self.tex_w = tex.shape[:2]
        self.texture = torch.from_numpy(tex).to(self.device)
        N, H, W = self.N, self.H, self.W
        self.pos_buf = torch.zeros((self.V, 3), dtype=torch.float32, device=self.device)
        self.vis = torch.full((N, H, W), -1, dtype=torch.int32, device=self.device)
        self.depth = torch.ones((N, H, W, 1), dtype=torch.float32, device=self.device)
        self.color = torch.zeros((N, H, W), dtype=torch.int32, device=self.device)
        self.raster = BatchRenderer(device)
        mv = self.mvps.cpu().numpy()
        for n in range(N):
            self.raster.add_view(W, H, 1, FORMAT_RGBA8, clear=True, clear_depth=1.0,
                                 targets={"color": self.color[n], "depth": self.depth[n], "vis": self.vis[n]})
        for n in range(N):
            self.raster.add_mesh(n, self.pos_buf, self.faces, mv[n].reshape(4, 4), attr_count=0, cull=CULL_BACK,
                                 depth_func=LESS, shading=FS_PRIMITIVE_ID)

    def rasterize(self, positions):
        """Visibility of all views for float32 positions (V, 3); returns the (N, H, W) ids."""
        self.pos_buf.copy_(positions.detach().reshape(-1, 3))
        self.raster.draw()
        return self.vis

    def _pass(self, pos, col, uv, vis, shaded, image, codes):
        p = DiffPass()
        p.numViews, p.width, p.height = self.N, self.W, self.H
        p.mvp = self.mvps.data_ptr()
        p.positions, p.colors, p.uvs = pos.data_ptr(), col.data_ptr(), uv.data_ptr()
        p.faces, p.neighbors = self.faces.data_ptr(), self.neighbors.data_ptr()
        p.numVertices, p.numTriangles = self.V, self.T
        p.texture, p.texWidth, p.texHeight = self.texture.data_ptr(), self.tex_w, self.tex_h
        p.visibility, p.shaded, p.image, p.aaCodes = vis.data_ptr(), shaded.data_ptr(), image.data_ptr(), codes.data_ptr()
        return p

    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    def forward(self, pos, col, uv):
        """Non-differentiable forward: (image, shaded, visibility copy, aa codes)."""
        torch = self.torch
        N, H, W = self.N, self.H, self.W
        pos = pos.detach().float().contiguous()
        col = col.detach().float().contiguous()
        uv = uv.detach().float().contiguous()
        vis = self.rasterize(pos).clone()
        shaded = torch.empty((N, H, W, 3), dtype=torch.float32, device=self.device)
        image = torch.empty_like(shaded)
        codes = torch.empty((N, H, W, 2), dtype=torch.int8, device=self.device)
        p = self._pass(pos, col, uv, vis, shaded, image, codes)
        check("iftrDiffForward", self.lib.iftrDiffForward(ctypes.byref(p), self.stream()))
        return image, shaded, vis, codes

    def backward(self, pos, col, uv, vis, shaded, codes, grad_image):
        torch = self.torch
        pos = pos.detach().float().contiguous()
        col = col.detach().float().contiguous()
        uv = uv.detach().float().contiguous()
        g = grad_image.detach().float().contiguous()
        gp, gc, gu = torch.zeros_like(pos), torch.zeros_like(col), torch.zeros_like(uv)
        p = self._pass(pos, col, uv, vis, shaded, shaded, codes)
        p.gradImage, p.gradPositions, p.gradColors, p.gradUvs = g.data_ptr(), gp.data_ptr(), gc.data_ptr(), gu.data_ptr()
        check("iftrDiffBackward", self.lib.iftrDiffBackward(ctypes.byref(p), self.stream()))
        return gp, gc, gu

    def render(self, pos, col, uv):
        """Differentiable images (N, H, W, 3) of the mesh with vertex positions, colours and UVs."""
        return RenderFunction.apply(pos, col, uv, self)

    def close(self):
        self.raster.close()


def _autograd_function():
    import torch

    class _Render(torch.autograd.Function):
        @staticmethod
        def forward(ctx, pos, col, uv, renderer):
            image, shaded, vis, codes = renderer.forward(pos, col, uv)
            ctx.renderer = renderer
            ctx.save_for_backward(pos, col, uv, vis, shaded, codes)
            return image

        @staticmethod
        def backward(ctx, grad_image):
            pos, col, uv, vis, shaded, codes = ctx.saved_tensors
            gp, gc, gu = ctx.renderer.backward(pos, col, uv, vis, shaded, codes, grad_image)
            return gp.to(pos.dtype), gc.to(col.dtype), gu.to(uv.dtype), None

    return _Render


class _LazyFunction:
    """torch.autograd.Function created on first use (keeps torch an optional import)."""
    _fn = None

    def apply(self, *args):
        if _LazyFunction._fn is None:
            _LazyFunction._fn = _autograd_function()
        return _LazyFunction._fn.apply(*args)


RenderFunction = _LazyFunction()
