"""Parity at full size: the paths that only trigger at scale, against the oracle.

* The 4K stress frame (3840x2160 RGBA16F, 8x MSAA, 10,035,200 triangles from 40 displaced
  geodesic instances, 4096^2 texture with 16x anisotropic filtering, 4 blended instances drawn
  last back to front in one ordered pass) rendered whole on the GPU; the oracle renders three
  64-row bands of the same frame (every triangle set up, only the band's rows rasterised) that
  cross the blended instances.  Visibility and per-sample depth bit-exact, RGBA16F colour within
  one half-float ulp; the pass must finish without a scratch re-run and without the ordered
  stage's per-tile limit.  (Blended instances sorted back to front sit mostly behind opaque ones;
  the bands are placed where they show.)
* A target of more than 32K 16x16 tiles (4096x2304), whose list-offset scan takes the
  multi-launch path, compared whole.
"""
import os

import numpy as np
import pytest

import ifrit_gb300 as ig
from ifrit_gb300 import scenes
from oracle import oracle as O
from tests.gpu_harness import assert_parity, render_both

pytestmark = pytest.mark.gpu

BAND = 64


def stress_pass(r, sc):
    r.begin_pass(clear=True)
    for d in sc["draws"]:
        r.set_state(cull=ig.CULL_BACK, depth_func=ig.LESS_OR_EQUAL, depth_write=not d["blend"], shading=ig.FS_TEXTURED)
        r.set_blend(d["blend"], 6, 7, 1, 7)  # SRC_ALPHA, ONE_MINUS_SRC_ALPHA; alpha ONE, ONE_MINUS_SRC_ALPHA
        r.set_mvp(d["mvp"])
        r.pass_draw(d["first"], d["count"])
    r.end_pass()


def test_stress_frame_full_size_bands():
    sc = scenes.c5_scene()
    W, H = sc["width"], sc["height"]
    assert len(sc["indices"]) == 10035200
    r = ig.Renderer(W, H, 8, ig.FORMAT_RGBA16F, visibility=True)
    r.set_geometry(sc["vertices"], sc["indices"], 2)
    r.set_texture(sc["texture"], max_aniso=16)
    stress_pass(r, sc)  # raises on IFTR_ERR_LIMIT or any other error status
    assert r.stats().retries == 0
    gpu = {"color": r.color(), "depth": r.depth(), "vis": r.visibility()}
    r.close()
    assert (gpu["vis"] >= 0).mean() > 0.9

    chain, levels = O.build_mips(sc["texture"])
    tex = (chain, levels, sc["texture"].shape[1], sc["texture"].shape[0])
    odraws, blended, base = [], [], 0  # primitive ids count triangles in pass order
    for d in sc["draws"]:
        f = sc["indices"][d["first"] // 3:(d["first"] + d["count"]) // 3]
        odraws.append(O.make_draw(sc["vertices"], f, d["mvp"], attr_offset=3, attr_count=2, cull_mode=2, depth_func=3,
                                  depth_write=int(not d["blend"]), blend=(6, 7, 1, 7) if d["blend"] else None,
                                  shading=O.SHADE_TEXTURED, texture=tex, sampler={"max_aniso": 16}, prim_base=base))
        if d["blend"]:
            blended.append((base, base + len(f)))
        base += len(f)
    assert len(blended) == 4
    # bands centred on where blended instances are visible (instances drawn behind opaque ones may
    # show in a few rows or not at all), topped up to three bands at fixed rows
    seen = []
    for lo, hi in blended:
        rows = np.nonzero(((gpu["vis"] >= lo) & (gpu["vis"] < hi)).any(axis=(1, 2)))[0]
        if rows.size:
            seen.append((rows.size, int(np.median(rows))))
    assert seen, "no blended instance visible"
    centres = [c for _, c in sorted(seen, reverse=True)[:3]]
    for c in (H // 3, 2 * H // 3):
        if len(centres) < 3:
            centres.append(c)
    blended_rows = 0
    for c in centres:
        y0 = int(np.clip(c - BAND // 2, 0, H - BAND))
        ref = O.render(odraws, W, H, 8, O.FMT_RGBA16F, clear=True, nthreads=os.cpu_count() or 1, rows=(y0, y0 + BAND))
        part = {k: gpu[k][y0:y0 + BAND] for k in ("color", "depth", "vis")}
        assert_parity(part, ref, fmt=ig.FORMAT_RGBA16F)
        blended_rows += sum(int(((part["vis"] >= lo) & (part["vis"] < hi)).any(axis=(1, 2)).sum()) for lo, hi in blended)
    assert blended_rows > 0

def test_target_over_32k_tiles_multi_launch_scan():
    W, H = 4096, 2304  # 256 x 144 = 36,864 tiles of 16x16
    v, f, mvp = scenes.triangle_soup(200000, 77, W, H, median_px=12.0)
    gpu, ref, r = render_both(v, f, mvp, W, H, S=1, attr=2, cull=ig.CULL_NONE)
    assert_parity(gpu, ref)
    assert (gpu["vis"] >= 0).mean() > 0.5
    r.close()


def test_differentiable_full_batch_gradients_match_fp64():
    """The differentiable configuration at full size: 64 views at 256x256 of the 20,480-triangle
    icosphere.  All 64 views are rendered and back-propagated on the GPU; the loss covers 4 of
    them (the others contribute zero upstream gradient), so the vertex gradients must equal the
    FP64 adjoint of those 4 views: max |g_gpu - g_fp64| / max |g_fp64| <= 1e-3 for positions,
    colours and UVs, for the same upstream gradient and end to end."""
    import torch

    from ifrit_gb300.diff import DiffRenderer
    from oracle import diff_oracle as D

    sc = scenes.c4_scene()
    assert sc["mvps"].shape[0] == 64 and sc["width"] == sc["height"] == 256 and len(sc["faces"]) == 20480
    dr = DiffRenderer(sc["faces"], len(sc["clean"]), sc["width"], sc["height"], sc["mvps"], sc["texture"])
    dev = torch.device("cuda")
    t = {k: torch.from_numpy(sc[k]).to(dev) for k in ("clean", "noisy", "colors", "uvs")}
    with torch.no_grad():
        target = dr.forward(t["clean"], t["colors"], t["uvs"])[0]
    pos, col, uv = (t[k].clone().requires_grad_(True) for k in ("noisy", "colors", "uvs"))
    img = dr.render(pos, col, uv)
    nv = 4
    loss = ((img[:nv] - target[:nv]) ** 2).sum()
    loss.backward()
    _, _, vis, codes = dr.forward(t["noisy"], t["colors"], t["uvs"])
    args = (sc["noisy"], sc["colors"], sc["uvs"], sc["texture"], sc["faces"], sc["mvps"][:nv],
            vis[:nv].cpu().numpy(), codes[:nv].cpu().numpy())
    err = lambda g, r: float(np.abs(g.grad.cpu().numpy() - r).max() / max(np.abs(r).max(), 1e-30))  # noqa: E731
    ap, ac, au = D.adjoint(*args, (2 * (img[:nv] - target[:nv])).detach().cpu().numpy())
    L64, gp, gc, gu, _ = D.loss_and_grads(*args, target[:nv].cpu().numpy())
    adj = {"positions": err(pos, ap), "colors": err(col, ac), "uvs": err(uv, au)}
    e2e = {"positions": err(pos, gp), "colors": err(col, gc), "uvs": err(uv, gu)}
    print("64 x 256^2: loss gpu %.6f fp64 %.6f; gradient error vs FP64 adjoint %s, end to end %s"
          % (float(loss.detach()), L64, adj, e2e))
    assert abs(float(loss.detach()) - L64) <= 1e-4 * L64
    for k in adj:
        assert adj[k] <= 1e-3 and e2e[k] <= 1e-3, (k, adj[k], e2e[k])
    dr.close()
