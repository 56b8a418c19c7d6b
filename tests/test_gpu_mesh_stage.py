"""GPU parity of the mesh / geometry stage boundary (iftrDrawMeshOutputs): per-work-group
clip-space outputs, compacted in group order and drawn, against the oracle drawing the same
indexed mesh through its vertex transform.

The host forms each vertex's clip position with the vertex stage's own float32 expression,
((m0 x + m1 y) + m2 z) + m3 per row, so both sides rasterise identical clip coordinates; the
groups cover consecutive triangles, so triangle ids (group order, then local order) equal the
mesh's.  Unused vertex / index slots hold garbage, one group is empty, and group sizes vary."""
import numpy as np
import pytest
import torch

import ifrit_gb300 as ig
from ifrit_gb300 import scenes
from tests.gpu_harness import assert_parity, render_both

pytestmark = pytest.mark.gpu


def clip_of(v, mvp):
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    m = mvp.astype(np.float32)
    return np.stack([((m[r, 0] * x + m[r, 1] * y) + m[r, 2] * z) + m[r, 3] for r in range(4)], 1).astype(np.float32)


def mesh_groups(v, f, mvp, rng, max_tris=48):
    groups, t = [], 0
    while t < len(f):
        n = int(rng.integers(1, max_tris + 1))
        groups.append(f[t:t + n])
        t += n
    groups.insert(len(groups) // 2, f[:0])  # an empty work group
    max_v = max(len(np.unique(g)) for g in groups) + 5
    max_i = max_tris * 3 + 6
    G = len(groups)
    pos = rng.uniform(-1e3, 1e3, (G, max_v, 4)).astype(np.float32)  # garbage in unused slots
    att = rng.uniform(-9, 9, (G, max_v, 4)).astype(np.float32)
    idx = rng.integers(-5, 1000, (G, max_i)).astype(np.int32)
    nv = np.zeros(G, np.int32)
    ni = np.zeros(G, np.int32)
    clip = clip_of(v, mvp)
    for gi, g in enumerate(groups):
        ids, local = np.unique(g.reshape(-1), return_inverse=True)
        nv[gi], ni[gi] = len(ids), g.size
        pos[gi, :len(ids)] = clip[ids]
        att[gi, :len(ids), :3] = v[ids, 3:6]
        att[gi, :len(ids), 3] = 0.0
        idx[gi, :g.size] = local.astype(np.int32)
    return pos, att, idx, nv, ni


@pytest.mark.parametrize("S", [1, 4])
def test_mesh_outputs_match_indexed_draw(S):
    rng = np.random.default_rng(40 + S)
    v, f = scenes.jittered_icosphere(4, 41, jitter=0.03)
    W, H = 192, 160
    mvp = scenes.default_mvp(W / H)
    pos, att, idx, nv, ni = mesh_groups(v, f, mvp, rng)
    # the oracle (and the plain GPU path) on the indexed mesh
    _, ref, _ = render_both(v, f, mvp, W, H, S=S, cull=ig.CULL_BACK, depth_func=ig.LESS)
    r = ig.Renderer(W, H, S, ig.FORMAT_RGBA8, visibility=True)
    r.set_state(cull=ig.CULL_BACK, depth_func=ig.LESS, shading=ig.FS_GOURAUD)
    dev = torch.device("cuda")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    r.draw_mesh_outputs(T(pos), T(idx), T(nv), T(ni), attributes=T(att), attr_count=3)
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).sum() > 5000


def test_mesh_outputs_reject_bad_counts():
    r = ig.Renderer(64, 64, 1, ig.FORMAT_RGBA8, visibility=True)
    dev = torch.device("cuda")
    pos = torch.zeros((2, 8, 4), dtype=torch.float32, device=dev)
    idx = torch.zeros((2, 6), dtype=torch.int32, device=dev)
    nv = torch.tensor([3, 9], dtype=torch.int32, device=dev)  # 9 > max 8
    ni = torch.tensor([3, 3], dtype=torch.int32, device=dev)
    with pytest.raises(ig.IfritError):
        r.draw_mesh_outputs(pos, idx, nv, ni)
    nv = torch.tensor([3, 3], dtype=torch.int32, device=dev)
    ni = torch.tensor([3, 4], dtype=torch.int32, device=dev)  # not a multiple of 3
    with pytest.raises(ig.IfritError):
        r.draw_mesh_outputs(pos, idx, nv, ni)
