"""GPU parity of the differentiable path (iftrDiffForward / iftrDiffBackward behind
torch.autograd.Function) against the FP64 CPU restatement in oracle/diff_oracle.py.

  * visibility: the GPU ids equal the oracle rasterizer's (bit-exact);
  * forward: images within 5e-5 of the float64 forward on the same visibility and decisions
    (float32 perspective barycentrics; shaded values lie in [0, 1]),
    decisions agree with an independent float64 recomputation on >= 99.5% of pixel pairs;
  * gradients: max |g_gpu - g_fp64| / max |g_fp64| <= 1e-3 for positions, colours and UVs
    (L = sum((image - target)^2), target rendered from the clean positions), both for the same
    upstream gradient and end to end;
  * central differences (h = 1e-3) of the full float64 forward (visibility and decisions
    recomputed per evaluation) on 100 random parameters: colours within 1e-3 of the GPU
    gradient (normalised), UVs within 3e-2 (bilinear texture kinks), positions with matching
    sign on >= 80% and correlation >= 0.4 (antialiasing makes the image only approximately
    continuous where visibility changes; measured 88% and 0.54 on this scene).
"""
import numpy as np
import pytest
import torch

from ifrit_gb300 import scenes
from ifrit_gb300.diff import DiffRenderer, mesh_neighbors
from oracle import diff_oracle as D

pytestmark = pytest.mark.gpu


def _setup(num_views=8, size=128, subdivisions=4, tex_size=64, seed=4):
    sc = scenes.c4_scene(seed=seed, num_views=num_views, size=size, subdivisions=subdivisions, tex_size=tex_size)
    dr = DiffRenderer(sc["faces"], len(sc["clean"]), sc["width"], sc["height"], sc["mvps"], sc["texture"])
    dev = torch.device("cuda")
    t = {k: torch.from_numpy(sc[k]).to(dev) for k in ("clean", "noisy", "colors", "uvs")}
    return sc, dr, t


def _norm_err(g, ref):
    return float(np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-30))


def test_visibility_and_forward_match_fp64():
    sc, dr, t = _setup()
    img, shaded, vis, codes = dr.forward(t["noisy"], t["colors"], t["uvs"])
    torch.cuda.synchronize()
    vis_np, codes_np = vis.cpu().numpy(), codes.cpu().numpy()
    ref_vis = D.raster_visibility(sc["noisy"], sc["faces"], sc["mvps"], sc["width"], sc["height"])
    assert (vis_np == ref_vis).all()
    ref = D.forward(torch.tensor(sc["noisy"], dtype=torch.float64), torch.tensor(sc["colors"], dtype=torch.float64),
                    torch.tensor(sc["uvs"], dtype=torch.float64), sc["texture"], sc["faces"], sc["mvps"], vis_np,
                    codes_np).numpy()
    assert np.abs(img.cpu().numpy() - ref).max() <= 5e-5
    own = D.decisions(sc["noisy"], sc["faces"], D.neighbors(sc["faces"]), sc["mvps"], vis_np)
    agree = float((own == codes_np).mean())
    print("antialiasing decisions agreeing with float64: %.5f, pairs blended: %d" % (agree, int((codes_np >= 0).sum())))
    assert agree >= 0.995 and (codes_np >= 0).sum() > 1000
    dr.close()


def test_gradients_match_fp64_adjoint():
    """The adjoint for the same upstream gradient dL/dimage (the hand-written CUDA adjoint
    against float64 autograd), and end to end (each side from its own forward residual)."""
    sc, dr, t = _setup()
    with torch.no_grad():
        target = dr.forward(t["clean"], t["colors"], t["uvs"])[0]
    pos = t["noisy"].clone().requires_grad_(True)
    col = t["colors"].clone().requires_grad_(True)
    uv = t["uvs"].clone().requires_grad_(True)
    img = dr.render(pos, col, uv)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    _, _, vis, codes = dr.forward(t["noisy"], t["colors"], t["uvs"])
    args = (sc["noisy"], sc["colors"], sc["uvs"], sc["texture"], sc["faces"], sc["mvps"], vis.cpu().numpy(),
            codes.cpu().numpy())
    ap, ac, au = D.adjoint(*args, (2 * (img - target)).detach().cpu().numpy())
    adj = {"positions": _norm_err(pos.grad.cpu().numpy(), ap), "colors": _norm_err(col.grad.cpu().numpy(), ac),
           "uvs": _norm_err(uv.grad.cpu().numpy(), au)}
    L64, gp, gc, gu, _ = D.loss_and_grads(*args, target.cpu().numpy())
    e2e = {"positions": _norm_err(pos.grad.cpu().numpy(), gp), "colors": _norm_err(col.grad.cpu().numpy(), gc),
           "uvs": _norm_err(uv.grad.cpu().numpy(), gu)}
    print("loss gpu %.6f fp64 %.6f; max normalised gradient error vs the fp64 adjoint: %s; end to end: %s"
          % (float(loss.detach()), L64, adj, e2e))
    assert abs(float(loss.detach()) - L64) <= 1e-4 * L64
    for k in adj:
        assert adj[k] <= 1e-3 and e2e[k] <= 1e-3, (k, adj[k], e2e[k])
    dr.close()


def test_gradients_against_central_differences():
    sc, dr, t = _setup(num_views=4, size=96, subdivisions=4, tex_size=64, seed=5)
    f, mv, W, H, tex = sc["faces"], sc["mvps"], sc["width"], sc["height"], sc["texture"]
    nb = D.neighbors(f)
    with torch.no_grad():
        target = dr.forward(t["clean"], t["colors"], t["uvs"])[0].cpu().numpy()
    pos = t["noisy"].clone().requires_grad_(True)
    col = t["colors"].clone().requires_grad_(True)
    uv = t["uvs"].clone().requires_grad_(True)
    ((dr.render(pos, col, uv) - torch.from_numpy(target).cuda()) ** 2).sum().backward()
    grads = {"pos": pos.grad.cpu().numpy(), "col": col.grad.cpu().numpy(), "uv": uv.grad.cpu().numpy()}
    base = {"pos": sc["noisy"], "col": sc["colors"].astype(np.float64), "uv": sc["uvs"].astype(np.float64)}
    rng = np.random.default_rng(11)
    h = 1e-3
    out = {}
    for name, count in (("pos", 34), ("col", 33), ("uv", 33)):
        g = grads[name]
        cand = np.argwhere(np.abs(g) > 0)
        pick = cand[rng.choice(len(cand), count, replace=False)]
        fd, an = [], []
        for i in map(tuple, pick):
            vals, steps = [], []
            for sgn in (1, -1):
                p = dict(base)
                p[name] = base[name].copy()
                p[name][i] += sgn * (np.float32(h) if name == "pos" else h)
                steps.append(float(p[name][i]))
                vals.append(D.full_loss(p["pos"], p["col"], p["uv"], tex, f, nb, mv, W, H, target))
            fd.append((vals[0] - vals[1]) / (steps[0] - steps[1]))
            an.append(g[i])
        fd, an = np.array(fd), np.array(an)
        out[name] = (float(np.abs(fd - an).max() / np.abs(g).max()), float(np.mean(np.sign(fd) == np.sign(an))),
                     float(np.corrcoef(fd, an)[0, 1]))
    print("central differences vs GPU gradients (max normalised error, sign agreement, correlation): %s" % out)
    assert out["col"][0] <= 1e-3
    assert out["uv"][0] <= 3e-2
    assert out["pos"][1] >= 0.8 and out["pos"][2] >= 0.4
    dr.close()


def test_autograd_function_accumulates_gradients():
    sc, dr, t = _setup(num_views=2, size=64, subdivisions=3, tex_size=32)
    pos = t["noisy"].clone().requires_grad_(True)
    col = t["colors"].clone().requires_grad_(True)
    uv = t["uvs"].clone().requires_grad_(True)
    img = dr.render(pos, col, uv)
    assert img.shape == (2, 64, 64, 3) and img.requires_grad
    img.sum().backward()
    g1 = col.grad.clone()
    img = dr.render(pos, col, uv)
    img.sum().backward()
    assert torch.allclose(col.grad, 2 * g1, rtol=1e-5, atol=1e-6)
    assert (mesh_neighbors(sc["faces"]) >= 0).all()  # closed mesh
    dr.close()


def test_position_gradients_against_central_differences_where_smooth():
    """Positions whose central-difference stencil crosses no non-differentiable point of the
    forward: visibility, antialiasing decisions and the kink signature (bilinear texel cells,
    the |t - 1/2| and clamp points of the edge blend, oracle/diff_oracle.kink_signature) are the
    same at +h and -h.  There the image is smooth in the parameter, so central differences of the
    float64 loss (h = 1e-5 on float64 positions) bound the gradients: the FP64 adjoint within
    1e-4 relative per parameter, the GPU gradient within 2e-3 of the largest gradient."""
    sc, dr, t = _setup(num_views=4, size=96, subdivisions=4, tex_size=64, seed=5)
    f, mv, W, H, tex = sc["faces"], sc["mvps"], sc["width"], sc["height"], sc["texture"]
    nb = D.neighbors(f)
    with torch.no_grad():
        target = dr.forward(t["clean"], t["colors"], t["uvs"])[0].cpu().numpy()
    pos = t["noisy"].clone().requires_grad_(True)
    ((dr.render(pos, t["colors"], t["uvs"]) - torch.from_numpy(target).cuda()) ** 2).sum().backward()
    g_gpu = pos.grad.cpu().numpy()
    vis = D.raster_visibility(sc["noisy"], f, mv, W, H)
    codes = D.decisions(sc["noisy"], f, nb, mv, vis)
    _, g64, _, _, _ = D.loss_and_grads(sc["noisy"], sc["colors"], sc["uvs"], tex, f, mv, vis, codes, target)
    sig = D.kink_signature(sc["noisy"], sc["uvs"], tex, f, mv, vis, codes)
    col64, uv64 = torch.as_tensor(sc["colors"].astype(np.float64)), torch.as_tensor(sc["uvs"].astype(np.float64))
    tgt = torch.as_tensor(target.astype(np.float64))
    rng = np.random.default_rng(17)
    cand = np.argwhere(np.abs(g64) > 0)
    rng.shuffle(cand)
    h = 1e-5
    fd, a64, agpu, tried = [], [], [], 0
    for i in map(tuple, cand[:200]):
        tried += 1
        vals = []
        for sgn in (1, -1):
            p = sc["noisy"].astype(np.float64)
            p[i] += sgn * h
            v2 = D.raster_visibility(p, f, mv, W, H)
            if not (v2 == vis).all():
                break
            c2 = D.decisions(p, f, nb, mv, v2)
            if not (c2 == codes).all() or not np.array_equal(D.kink_signature(p, sc["uvs"], tex, f, mv, v2, c2), sig):
                break
            with torch.no_grad():
                img = D.forward(torch.as_tensor(p), col64, uv64, tex, f, mv, v2, c2)
            vals.append(float(((img - tgt) ** 2).sum()))
        if len(vals) < 2:
            continue
        fd.append((vals[0] - vals[1]) / (2 * h))
        a64.append(g64[i])
        agpu.append(g_gpu[i])
        if len(fd) >= 40:
            break
    fd, a64, agpu = np.array(fd), np.array(a64), np.array(agpu)
    rel64 = float((np.abs(fd - a64) / np.abs(fd)).max())
    norm_gpu = float(np.abs(fd - agpu).max() / np.abs(g_gpu).max())
    rel_gpu = float(np.median(np.abs(fd - agpu) / np.abs(fd)))
    print("positions with a smooth stencil: %d of %d tried; central differences vs FP64 adjoint: max relative "
          "%.3g; vs GPU: max normalised %.3g, median relative %.3g" % (len(fd), tried, rel64, norm_gpu, rel_gpu))
    assert len(fd) >= 30
    assert rel64 <= 1e-4
    assert norm_gpu <= 2e-3
    dr.close()
