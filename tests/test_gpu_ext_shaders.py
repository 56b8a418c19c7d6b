"""GPU tests of the device-side shader extension point (include/ifrit_gb300_ext.cuh), the
replacement for the reference's host shader objects (engine/base/Shaders.h:46-120; device copies
with vtable fix-ups in core/cuda/CudaUtils.cuh:26-38).

tests/ext/ext_shaders.cu is compiled at test time with ifrit_gb300.build.build_extension (sm_103a,
linked against libifrit_gb300.so) and called through ctypes:

* the GOURAUD functor shading a draw's visibility buffer reproduces the built-in shade stage's
  output bit for bit (RGBA8 and RGBA32F, 1x and 4x, including near-plane-clipped fan triangles);
* a test functor reading every fragment field (attribute, quad derivatives, triangle) equals a
  numpy restatement over the built-in RGBA32F image bit for bit, and that image matches the oracle
  (so the chain oracle -> built-in -> functor is pinned);
* a functor-driven mesh stage (a grid, some groups empty or short) drawn through
  iftrDrawMeshOutputs matches the oracle drawing the same indexed mesh;
* a vertex functor over an indexed mesh matches the oracle drawing the host-transformed mesh;
* a task functor spawning 0-3 mesh groups per task group, with the mesh functor run per (task, sub),
  matches the oracle drawing the cells in (task, sub) order, and too many spawned groups return
  IFTR_ERR_OVERFLOW."""
import ctypes
import os

import numpy as np
import pytest
import torch

import ifrit_gb300 as ig
from ifrit_gb300 import build as ibuild
from ifrit_gb300 import scenes
from oracle import oracle as O
from tests.gpu_harness import FMT_TO_ORACLE, assert_parity

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
BG = (0.125, 0.25, 0.5, 1.0)


@pytest.fixture(scope="module")
def ext():
    out = os.path.join(ibuild.BUILD, "ext", "libext_shaders.so")
    ibuild.build_extension([os.path.join(HERE, "ext", "ext_shaders.cu")], out)
    lib = ctypes.CDLL(out)
    vp, ip = ctypes.c_void_p, ctypes.c_int
    lib.ext_shade.argtypes = [ip, vp, ip, ip, ip, ip, vp, ip, vp, ip, ip, ip, ip, ip, vp, ip, vp, vp, vp]
    lib.ext_shade.restype = ip
    lib.ext_draw_grid.argtypes = [vp, ip, ip, vp, vp, vp, vp, vp, vp, ip, vp]
    lib.ext_draw_grid.restype = ip
    lib.ext_draw_task_grid.argtypes = [vp, ip, ip, vp, vp, vp, vp, vp, vp, vp, ip, ip, vp]
    lib.ext_draw_task_grid.restype = ip
    lib.ext_draw_vertices.argtypes = [vp, vp, ip, vp, ip, vp, vp, vp, vp, ip, vp]
    lib.ext_draw_vertices.restype = ip
    return lib


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def draw_and_shade(lib, which, v, f, mvp, W, H, S, fmt, cull, attr):
    """Built-in draw through device geometry, then the functor over its visibility buffer.
    Returns (built-in colour, functor colour, visibility) as numpy arrays."""
    dev = torch.device("cuda")
    dv = torch.from_numpy(_f32(v)).to(dev)
    di = torch.from_numpy(np.ascontiguousarray(f, np.int32)).to(dev)
    r = ig.Renderer(W, H, S, fmt, visibility=True)
    r.set_state(cull=cull, depth_func=ig.LESS, shading=ig.FS_GOURAUD, clear_color=BG)
    r.bind_device_geometry(dv.data_ptr(), v.shape[1], len(v), 3, attr, di.data_ptr(), f.size)
    r.set_mvp(mvp)
    r.draw(clear=True)
    builtin = r.color()
    _, _, vis_ptr = r.device_attachments()
    out = torch.zeros(builtin.shape, dtype={np.uint32: torch.int32, np.uint64: torch.int64,
                                            np.float32: torch.float32}[builtin.dtype.type], device=dev)
    m = _f32(mvp).reshape(-1)
    bg = np.array(BG, np.float32)
    rc = lib.ext_shade(which, dv.data_ptr(), v.shape[1], len(v), 3, attr, di.data_ptr(), len(f), m.ctypes.data,
                       cull, 1, W, H, S, vis_ptr, fmt, out.data_ptr(), bg.ctypes.data,
                       torch.cuda.current_stream().cuda_stream)
    assert rc == 0, "ext_shade returned CUDA error %d" % rc
    functor = out.cpu().numpy().view(builtin.dtype).reshape(builtin.shape)
    vis = r.visibility()
    r.close()
    return builtin, functor, vis


def inside_sphere():
    """Camera inside a large jittered sphere: many triangles cross the near plane and are drawn
    as clipped fan sub-triangles."""
    v, f = scenes.jittered_icosphere(3, 4, jitter=0.1)
    v = v.copy()
    v[:, :3] *= 3.0
    mvp = (scenes.perspective(70.0, 1.25, 0.1, 50.0) @ scenes.look_at((0.3, 0.2, 0.1), (0, 0, -1))).astype(np.float32)
    return v, f, mvp


@pytest.mark.parametrize("S", [1, 4])
@pytest.mark.parametrize("fmt", [ig.FORMAT_RGBA8, ig.FORMAT_RGBA32F])
@pytest.mark.parametrize("scene", ["orbit", "inside"])
def test_gouraud_functor_matches_builtin(ext, S, fmt, scene):
    if scene == "orbit":
        v, f, mvp = scenes.c1_scene(7)
        W, H, cull = 192, 160, ig.CULL_BACK
    else:
        v, f, mvp = inside_sphere()
        W, H, cull = 160, 128, ig.CULL_NONE
    builtin, functor, vis = draw_and_shade(ext, 0, v, f, mvp, W, H, S, fmt, cull, 3)
    assert (vis >= 0).mean() > 0.3
    assert (vis < 0).any() or scene == "inside"
    bad = builtin.view(np.uint32) != functor.view(np.uint32)
    assert not bad.any(), "functor differs from the built-in shading at %d words" % int(bad.sum())


def test_fragment_fields_match_builtin_and_oracle(ext):
    v, f, mvp = scenes.c1_scene(8)
    W, H = 192, 160
    builtin, functor, vis = draw_and_shade(ext, 1, v, f, mvp, W, H, 1, ig.FORMAT_RGBA32F, ig.CULL_BACK, 3)
    vis = vis[..., 0]
    # the built-in RGBA32F image against the oracle (the attribute at every pixel centre)
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=3, cull_mode=ig.CULL_BACK, depth_func=ig.LESS)
    ref = O.render([d], W, H, 1, FMT_TO_ORACLE[ig.FORMAT_RGBA32F], clear=True, clear_color=BG,
                   nthreads=os.cpu_count() or 1)
    assert (ref["vis"][..., 0] == vis).all()
    assert np.allclose(builtin, ref["color"], rtol=1e-5, atol=1e-6)
    # numpy restatement of the functor over the built-in image, on pixels whose quad partners
    # show the same triangle (there the partner's own colour is the partner attribute)
    a = builtin
    cov = vis >= 0
    exp0 = (a[..., 0] * a[..., 0] + a[..., 2]).astype(np.float32)
    assert (functor[..., 0][cov] == exp0[cov]).all()
    assert (functor[..., 3][cov] == vis[cov].astype(np.float32)).all()
    assert (functor[~cov] == np.array(BG, np.float32)).all()
    ys, xs = np.nonzero(cov)
    hx, vy = xs ^ 1, ys ^ 1
    okx = (hx < W) & (vis[ys, np.minimum(hx, W - 1)] == vis[ys, xs])
    oky = (vy < H) & (vis[np.minimum(vy, H - 1), xs] == vis[ys, xs])
    assert okx.sum() > 1000 and oky.sum() > 1000
    yx, xx = ys[okx], xs[okx]
    ddx = np.where(xx & 1, a[yx, xx, 0] - a[yx, xx ^ 1, 0], a[yx, xx ^ 1, 0] - a[yx, xx, 0]).astype(np.float32)
    assert (functor[yx, xx, 2] == ddx * np.float32(64.0)).all()
    yy, xy = ys[oky], xs[oky]
    ddy = np.where(yy & 1, a[yy, xy, 1] - a[yy ^ 1, xy, 1], a[yy ^ 1, xy, 1] - a[yy, xy, 1]).astype(np.float32)
    assert (functor[yy, xy, 1] == ddy * np.float32(64.0)).all()


def _cell(verts, tris, nx, cell, one_triangle):
    """Host restatement of cell_vertex / quad_index (tests/ext/ext_shaders.cu)."""
    cx, cy = cell % nx, cell // nx
    base = len(verts)
    z = np.float32(-2.0) - np.float32((cx * 3 + cy * 5) % 8) * np.float32(0.0625)
    for i in range(4):
        vx, vy = cx + (i & 1), cy + (i >> 1)
        verts.append([np.float32(vx) * np.float32(0.125) - np.float32(1.0),
                      np.float32(vy) * np.float32(0.125) - np.float32(1.0), z,
                      np.float32(vx) * np.float32(0.0625), np.float32(vy) * np.float32(0.0625),
                      np.float32((cell * 5) % 9) * np.float32(0.125), 1.0])
    tris.append([base, base + 1, base + 2])
    if not one_triangle:
        tris.append([base + 2, base + 1, base + 3])


def grid_mesh(nx, ny):
    """GridMesh's groups: per-group vertices (x, y, z, r, g, b, a) and the triangles of the
    non-empty groups in group order."""
    verts, tris = [], []
    for g in range(nx * ny):
        if g % 7 == 3:
            continue
        _cell(verts, tris, nx, g, g % 5 == 1)
    return np.array(verts, np.float32), np.array(tris, np.int32)


def task_grid(tasks, nx):
    """TaskSpawn + TaskGrid: task t spawns t % 4 groups; group (t, sub) draws cell 3 t + sub."""
    verts, tris = [], []
    for t in range(tasks):
        for sub in range(t % 4):
            _cell(verts, tris, nx, 3 * t + sub, (t + sub) % 3 == 1)
    return np.array(verts, np.float32), np.array(tris, np.int32)


@pytest.mark.parametrize("S", [1, 4])
def test_functor_mesh_stage_matches_oracle(ext, S):
    nx, ny, W, H = 24, 16, 160, 128
    mvp = scenes.perspective(60.0, W / H, 0.1, 50.0).astype(np.float32)
    G = nx * ny
    dev = torch.device("cuda")
    pos = torch.full((G, 4, 4), 7.0, dtype=torch.float32, device=dev)
    att = torch.zeros((G, 4, 4), dtype=torch.float32, device=dev)
    idx = torch.full((G, 6), -1, dtype=torch.int32, device=dev)
    nv = torch.zeros(G, dtype=torch.int32, device=dev)
    ni = torch.zeros(G, dtype=torch.int32, device=dev)
    r = ig.Renderer(W, H, S, ig.FORMAT_RGBA8, visibility=True)
    r.set_state(cull=ig.CULL_NONE, depth_func=ig.LESS, shading=ig.FS_GOURAUD, clear_color=BG)
    m = _f32(mvp).reshape(-1)
    rc = ext.ext_draw_grid(r.h, nx, ny, m.ctypes.data, pos.data_ptr(), att.data_ptr(), idx.data_ptr(),
                           nv.data_ptr(), ni.data_ptr(), 1, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, "draw_mesh_stage returned %d" % rc
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    r.close()
    v, f = grid_mesh(nx, ny)
    assert int(ni.sum().item()) == f.size
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=4, cull_mode=ig.CULL_NONE, depth_func=ig.LESS)
    ref = O.render([d], W, H, S, FMT_TO_ORACLE[ig.FORMAT_RGBA8], clear=True, clear_color=BG,
                   nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).sum() > W * H // 4


@pytest.mark.parametrize("S", [1, 4])
def test_functor_task_stage_matches_oracle(ext, S):
    tasks, nx, W, H = 120, 24, 160, 128
    mvp = scenes.perspective(60.0, W / H, 0.1, 50.0).astype(np.float32)
    G = sum(t % 4 for t in range(tasks))
    dev = torch.device("cuda")
    pos = torch.full((G, 4, 4), 7.0, dtype=torch.float32, device=dev)
    att = torch.zeros((G, 4, 4), dtype=torch.float32, device=dev)
    idx = torch.full((G, 6), -1, dtype=torch.int32, device=dev)
    nv = torch.zeros(G, dtype=torch.int32, device=dev)
    ni = torch.zeros(G, dtype=torch.int32, device=dev)
    offs = torch.zeros(tasks + 1, dtype=torch.int32, device=dev)
    r = ig.Renderer(W, H, S, ig.FORMAT_RGBA8, visibility=True)
    r.set_state(cull=ig.CULL_NONE, depth_func=ig.LESS, shading=ig.FS_GOURAUD, clear_color=BG)
    m = _f32(mvp).reshape(-1)
    stream = torch.cuda.current_stream().cuda_stream
    # one group too few: nothing drawn, IFTR_ERR_OVERFLOW
    rc = ext.ext_draw_task_grid(r.h, tasks, nx, m.ctypes.data, pos.data_ptr(), att.data_ptr(), idx.data_ptr(),
                                nv.data_ptr(), ni.data_ptr(), offs.data_ptr(), G - 1, 1, stream)
    assert rc == 4  # IFTR_ERR_OVERFLOW
    rc = ext.ext_draw_task_grid(r.h, tasks, nx, m.ctypes.data, pos.data_ptr(), att.data_ptr(), idx.data_ptr(),
                                nv.data_ptr(), ni.data_ptr(), offs.data_ptr(), G, 1, stream)
    assert rc == 0, "draw_task_mesh_stage returned %d" % rc
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    r.close()
    v, f = task_grid(tasks, nx)
    assert int(ni.sum().item()) == f.size
    assert offs.cpu().numpy()[-1] == G
    d = O.make_draw(v, f, mvp, attr_offset=3, attr_count=4, cull_mode=ig.CULL_NONE, depth_func=ig.LESS)
    ref = O.render([d], W, H, S, FMT_TO_ORACLE[ig.FORMAT_RGBA8], clear=True, clear_color=BG,
                   nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).sum() > W * H // 8


@pytest.mark.parametrize("S", [1, 4])
def test_functor_vertex_stage_matches_oracle(ext, S):
    v, f, mvp = scenes.c1_scene(9)
    W, H = 192, 160
    V = len(v)
    dev = torch.device("cuda")
    dv = torch.from_numpy(_f32(v)).to(dev)
    di = torch.from_numpy(np.ascontiguousarray(f, np.int32).reshape(-1)).to(dev)
    pos = torch.zeros((V, 4), dtype=torch.float32, device=dev)
    att = torch.zeros((V, 4), dtype=torch.float32, device=dev)
    counts = torch.zeros(2, dtype=torch.int32, device=dev)
    r = ig.Renderer(W, H, S, ig.FORMAT_RGBA32F, visibility=True)
    r.set_state(cull=ig.CULL_BACK, depth_func=ig.LESS, shading=ig.FS_GOURAUD, clear_color=BG)
    m = _f32(mvp).reshape(-1)
    rc = ext.ext_draw_vertices(r.h, dv.data_ptr(), V, di.data_ptr(), f.size, m.ctypes.data, pos.data_ptr(),
                               att.data_ptr(), counts.data_ptr(), 1, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, "draw_vertex_stage returned %d" % rc
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    r.close()
    # host restatement of ScaleVertex: scaled positions, colour + alpha 0.5 as the varying
    fac = (np.float32(1.0) + (np.arange(V) % 3).astype(np.float32) * np.float32(0.125)).astype(np.float32)
    vh = np.concatenate([(v[:, :3] * fac[:, None]).astype(np.float32), v[:, 3:6],
                         np.full((V, 1), 0.5, np.float32)], 1).astype(np.float32)
    d = O.make_draw(vh, f, mvp, attr_offset=3, attr_count=4, cull_mode=ig.CULL_BACK, depth_func=ig.LESS)
    ref = O.render([d], W, H, S, FMT_TO_ORACLE[ig.FORMAT_RGBA32F], clear=True, clear_color=BG,
                   nthreads=os.cpu_count() or 1)
    assert_parity(gpu, ref, fmt=ig.FORMAT_RGBA32F)
    assert (gpu["vis"] >= 0).mean() > 0.2
