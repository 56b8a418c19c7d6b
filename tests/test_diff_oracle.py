"""The FP64 restatement of the differentiable path (oracle/diff_oracle.py) on the CPU: its
autograd adjoint against central differences at fixed visibility, the edge adjacency, and the
oracle rasterizer's visibility ids."""
import numpy as np
import torch

from ifrit_gb300 import scenes
from ifrit_gb300.diff import mesh_neighbors
from oracle import diff_oracle as D


def _small():
    sc = scenes.c4_scene(seed=7, num_views=2, size=40, subdivisions=3, tex_size=32)
    return sc, D.neighbors(sc["faces"])


def test_neighbors_agree_with_package_adjacency():
    f = scenes.icosphere(3)[1]
    assert (D.neighbors(f) == mesh_neighbors(f)).all()
    open_mesh = f[:-7]  # removing triangles leaves boundary edges without a neighbour
    assert (D.neighbors(open_mesh) == mesh_neighbors(open_mesh)).all()
    assert (mesh_neighbors(open_mesh) < 0).any()


def test_fp64_adjoint_matches_central_differences_at_fixed_visibility():
    sc, nb = _small()
    f, mv, W, H, tex = sc["faces"], sc["mvps"], sc["width"], sc["height"], sc["texture"]
    vis_c = D.raster_visibility(sc["clean"], f, mv, W, H)
    target = D.forward(torch.tensor(sc["clean"], dtype=torch.float64), torch.tensor(sc["colors"], dtype=torch.float64),
                       torch.tensor(sc["uvs"], dtype=torch.float64), tex, f, mv, vis_c,
                       D.decisions(sc["clean"], f, nb, mv, vis_c)).numpy()
    vis = D.raster_visibility(sc["noisy"], f, mv, W, H)
    codes = D.decisions(sc["noisy"], f, nb, mv, vis)
    assert (codes >= 0).sum() > 50
    _, gp, gc, gu, _ = D.loss_and_grads(sc["noisy"], sc["colors"], sc["uvs"], tex, f, mv, vis, codes, target)
    params = {"pos": sc["noisy"].astype(np.float64), "col": sc["colors"].astype(np.float64),
              "uv": sc["uvs"].astype(np.float64)}
    grads = {"pos": gp, "col": gc, "uv": gu}
    rng = np.random.default_rng(0)
    h = 1e-6
    for name in ("pos", "col", "uv"):
        cand = np.argwhere(np.abs(grads[name]) > 0)
        for i in map(tuple, cand[rng.choice(len(cand), 6, replace=False)]):
            vals = []
            for sgn in (1, -1):
                p = {k: torch.tensor(v) for k, v in params.items()}
                p[name][i] += sgn * h
                with torch.no_grad():
                    img = D.forward(p["pos"], p["col"], p["uv"], tex, f, mv, vis, codes)
                vals.append(float(((img - torch.tensor(target)) ** 2).sum()))
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - grads[name][i]) <= 1e-5 * np.abs(grads[name]).max(), (name, i, fd, grads[name][i])


def test_oracle_visibility_ids_are_triangles_of_the_mesh():
    sc, _ = _small()
    vis = D.raster_visibility(sc["noisy"], sc["faces"], sc["mvps"], sc["width"], sc["height"])
    assert vis.shape == (2, 40, 40)
    assert vis.max() < len(sc["faces"]) and (vis >= 0).mean() > 0.2
