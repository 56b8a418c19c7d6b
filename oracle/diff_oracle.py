"""FP64 CPU restatement of the differentiable shading + silhouette antialiasing, and its adjoint.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA differentiable path.  The reference renderer
has no differentiable path, so this is written from the specification of the path itself:

  * perspective-correct barycentrics from clip coordinates: a_i = x_i - px w_i,
    b_i = y_i - py w_i, D = a x b, lambda = D / sum(D), at the pixel centre
    ((x + 0.5) / W * 2 - 1, (y + 0.5) / H * 2 - 1);
  * colour = sum lambda_i col_i, uv = sum lambda_i uv_i, bilinear RGB texture with repeat
    addressing and texel centres at (i + 0.5) / size; shaded = colour * texture;
  * silhouette antialiasing of adjacent pixel pairs: the nearer triangle of the pair covers
    pixel a; its edge crossing the segment a -> b at fraction t (first crossed edge), if it is a
    silhouette (no neighbour across it or the neighbour faces away), blends the pixel it intrudes
    on by |t - 1/2| towards the other pixel's shaded colour.

Everything is float64 (torch on the CPU); the adjoint is torch autograd of this forward, so it is
independent of the hand-written CUDA adjoint.  Visibility comes either from the GPU or from the
C oracle rasterizer (``raster_visibility``), which is bit-identical to the GPU rasterizer.
"""
import os

import numpy as np
import torch

from . import oracle as O

F64 = torch.float64


def neighbors(faces):
    """Triangle across the edge opposite vertex k (or -1), by a dictionary of edges."""
    f = np.asarray(faces).reshape(-1, 3)
    edges = {}
    for t, tri in enumerate(f.tolist()):
        for k in range(3):
            e = tuple(sorted((tri[(k + 1) % 3], tri[(k + 2) % 3])))
            edges.setdefault(e, []).append((t, k))
    out = np.full((len(f), 3), -1, np.int32)
    for owners in edges.values():
        if len(owners) == 2:
            (t0, k0), (t1, k1) = owners
            out[t0, k0] = t1
            out[t1, k1] = t0
    return out


def raster_visibility(pos, faces, mvps, W, H):
    """(N, H, W) triangle ids from the C oracle rasterizer (1x, back-face culling, depth LESS)."""
    pos = np.ascontiguousarray(pos, np.float32)
    out = []
    for m in np.asarray(mvps, np.float32).reshape(-1, 4, 4):
        d = O.make_draw(pos, faces, m, attr_offset=3, attr_count=0, cull_mode=2, depth_func=1,
                        shading=O.SHADE_PRIMID)
        r = O.render([d], W, H, 1, O.FMT_RGBA8, clear=True, clear_depth=1.0, nthreads=os.cpu_count() or 1)
        out.append(r["vis"][..., 0])
    return np.stack(out)


def _clip(pos, mvps):
    return torch.einsum("nij,vj->nvi", mvps[:, :, :3], pos) + mvps[:, None, :, 3]


def _ndc(x, y, W, H):
    return (x.to(F64) + 0.5) / W * 2 - 1, (y.to(F64) + 0.5) / H * 2 - 1


def _bary(c, px, py):
    a = c[..., 0] - px[:, None] * c[..., 3]
    b = c[..., 1] - py[:, None] * c[..., 3]
    D = torch.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1], a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1)
    return D / D.sum(1, keepdim=True)


def _bilinear(tex, uv):
    th, tw = tex.shape[:2]
    s = uv[:, 0] * tw - 0.5
    q = uv[:, 1] * th - 0.5
    fs, fq = torch.floor(s).detach(), torch.floor(q).detach()
    fx, fy = s - fs, q - fq
    i0 = torch.remainder(fs.long(), tw)
    i1 = torch.remainder(fs.long() + 1, tw)
    j0 = torch.remainder(fq.long(), th)
    j1 = torch.remainder(fq.long() + 1, th)
    fx, fy = fx[:, None], fy[:, None]
    return (1 - fy) * ((1 - fx) * tex[j0, i0] + fx * tex[j0, i1]) + fy * ((1 - fx) * tex[j1, i0] + fx * tex[j1, i1])


def shade(pos, col, uv, tex, faces, mvps, vis):
    """Shaded images (N, H, W, 3) before antialiasing."""
    N, H, W = vis.shape
    clip = _clip(pos, mvps)
    n, y, x = torch.nonzero(vis >= 0, as_tuple=True)
    t = vis[n, y, x].long()
    vtx = faces[t]
    c = clip[n[:, None], vtx]
    px, py = _ndc(x, y, W, H)
    lam = _bary(c, px, py)
    colr = (lam[..., None] * col[vtx]).sum(1)
    uvi = (lam[..., None] * uv[vtx]).sum(1)
    vals = colr * _bilinear(tex, uvi)
    s = torch.zeros((N, H, W, 3), dtype=F64)
    return s.index_put((n, y, x), vals)


def _project(c):
    X, Y = c[..., 0] / c[..., 3], c[..., 1] / c[..., 3]
    area = (X[:, 1] - X[:, 0]) * (Y[:, 2] - Y[:, 0]) - (X[:, 2] - X[:, 0]) * (Y[:, 1] - Y[:, 0])
    return X, Y, area


def _edge(X, Y, sgn, k, px, py):
    j, l = (k + 1) % 3, (k + 2) % 3
    g = lambda A, i: A.gather(1, i[:, None])[:, 0]
    Xj, Yj, Xl, Yl = g(X, j), g(Y, j), g(X, l), g(Y, l)
    return sgn * ((Xl - Xj) * (py - Yj) - (Yl - Yj) * (px - Xj))


def _pairs(vis, direction):
    """Owner pixels (n, y, x) and partner coordinates of all in-bounds pairs of a direction."""
    N, H, W = vis.shape
    dx, dy = (1, 0) if direction == 0 else (0, 1)
    n, y, x = torch.meshgrid(torch.arange(N), torch.arange(H - dy), torch.arange(W - dx), indexing="ij")
    n, y, x = n.reshape(-1), y.reshape(-1), x.reshape(-1)
    return n, y, x, x + dx, y + dy


def antialias(s, pos, faces, mvps, vis, codes):
    """Applies the recorded antialiasing decisions codes[n, y, x, dir] (owner = left / upper
    pixel; code = a_is_q * 3 + edge, or -1) to the shaded images."""
    N, H, W = vis.shape
    clip = _clip(pos, mvps)
    flat = s.reshape(-1, 3)
    delta = torch.zeros_like(flat)
    for direction in (0, 1):
        n, y, x, x2, y2 = _pairs(vis, direction)
        code = codes[n, y, x, direction].long()
        keep = code >= 0
        n, y, x, x2, y2, code = n[keep], y[keep], x[keep], x2[keep], y2[keep], code[keep]
        if len(n) == 0:
            continue
        a_is_q = code >= 3
        k = code % 3
        axp, ayp = torch.where(a_is_q, x2, x), torch.where(a_is_q, y2, y)
        bxp, byp = torch.where(a_is_q, x, x2), torch.where(a_is_q, y, y2)
        T = vis[n, ayp, axp].long()
        c = clip[n[:, None], faces[T]]
        X, Y, area = _project(c)
        sgn = torch.sign(area).detach()
        ax, ay = _ndc(axp, ayp, W, H)
        bx, by = _ndc(bxp, byp, W, H)
        ea, eb = _edge(X, Y, sgn, k, ax, ay), _edge(X, Y, sgn, k, bx, by)
        t = torch.clamp(ea / (ea - eb), 0.0, 1.0)
        w = t - 0.5
        to_b = (w >= 0).detach()
        tx, ty = torch.where(to_b, bxp, axp), torch.where(to_b, byp, ayp)
        sx, sy = torch.where(to_b, axp, bxp), torch.where(to_b, ayp, byp)
        ti = (n * H + ty) * W + tx
        si = (n * H + sy) * W + sx
        d = torch.abs(w)[:, None] * (flat[si] - flat[ti])
        delta = delta.index_add(0, ti, d)
    return (flat + delta).reshape(N, H, W, 3)


def kink_signature(pos, uv, tex, faces, mvps, vis, codes):
    """Where the forward (for fixed visibility and decisions) sits relative to its
    non-differentiable points: the bilinear texel cell of every shaded pixel's UV (floor in
    _bilinear) and, for every blended pixel pair, whether the edge crossing t is below 1/2 (the
    |t - 1/2| kink), below 0 or above 1 (the clamp).  Central differences whose stencil keeps
    visibility, decisions and this signature measure a smooth function of the parameter."""
    pos = torch.as_tensor(np.asarray(pos, np.float64))
    uv = torch.as_tensor(np.asarray(uv, np.float64))
    faces = torch.as_tensor(np.asarray(faces)).long()
    mvps = torch.as_tensor(np.asarray(mvps, np.float64)).reshape(-1, 4, 4)
    vis = torch.as_tensor(np.asarray(vis))
    codes = torch.as_tensor(np.asarray(codes))
    N, H, W = vis.shape
    th, tw = tex.shape[:2]
    out = []
    with torch.no_grad():
        clip = _clip(pos, mvps)
        n, y, x = torch.nonzero(vis >= 0, as_tuple=True)
        vtx = faces[vis[n, y, x].long()]
        px, py = _ndc(x, y, W, H)
        lam = _bary(clip[n[:, None], vtx], px, py)
        uvi = (lam[..., None] * uv[vtx]).sum(1)
        out += [torch.floor(uvi[:, 0] * tw - 0.5).long(), torch.floor(uvi[:, 1] * th - 0.5).long()]
        for direction in (0, 1):
            n, y, x, x2, y2 = _pairs(vis, direction)
            code = codes[n, y, x, direction].long()
            keep = code >= 0
            n, y, x, x2, y2, code = n[keep], y[keep], x[keep], x2[keep], y2[keep], code[keep]
            if len(n) == 0:
                continue
            a_is_q = code >= 3
            k = code % 3
            axp, ayp = torch.where(a_is_q, x2, x), torch.where(a_is_q, y2, y)
            bxp, byp = torch.where(a_is_q, x, x2), torch.where(a_is_q, y, y2)
            c = clip[n[:, None], faces[vis[n, ayp, axp].long()]]
            X, Y, area = _project(c)
            sgn = torch.sign(area)
            ax, ay = _ndc(axp, ayp, W, H)
            bx, by = _ndc(bxp, byp, W, H)
            ea, eb = _edge(X, Y, sgn, k, ax, ay), _edge(X, Y, sgn, k, bx, by)
            t = ea / (ea - eb)
            out += [(t >= 0.5).long(), (t < 0).long(), (t > 1).long()]
    return torch.cat(out).numpy()


def decisions(pos, faces, nbrs, mvps, vis):
    """The antialiasing decisions computed independently in float64: codes (N, H, W, 2)."""
    pos = torch.as_tensor(pos, dtype=F64)
    mvps = torch.as_tensor(np.asarray(mvps, np.float64).reshape(-1, 4, 4))
    faces = torch.as_tensor(np.asarray(faces, np.int64).reshape(-1, 3))
    nbrs = torch.as_tensor(np.asarray(nbrs, np.int64))
    vis = torch.as_tensor(np.asarray(vis, np.int64))
    N, H, W = vis.shape
    clip = _clip(pos, mvps)
    codes = torch.full((N, H, W, 2), -1, dtype=torch.int64)

    def depth_at(nn, tt, xx, yy):
        c = clip[nn[:, None], faces[tt]]
        px, py = _ndc(xx, yy, W, H)
        lam = _bary(c, px, py)
        return (lam * c[..., 3]).sum(1)

    for direction in (0, 1):
        n, y, x, x2, y2 = _pairs(vis, direction)
        tp, tq = vis[n, y, x], vis[n, y2, x2]
        sel = tp != tq
        n, y, x, x2, y2, tp, tq = n[sel], y[sel], x[sel], x2[sel], y2[sel], tp[sel], tq[sel]
        a_is_q = torch.zeros_like(tp, dtype=torch.bool)
        a_is_q |= tp < 0
        both = (tp >= 0) & (tq >= 0)
        if both.any():
            dq = depth_at(n[both], tq[both], x2[both], y2[both])
            dp = depth_at(n[both], tp[both], x[both], y[both])
            a_is_q[both] = dq < dp
        T = torch.where(a_is_q, tq, tp)
        c = clip[n[:, None], faces[T]]
        ok = (c[..., 3] > 0).all(1)
        X, Y, area = _project(c)
        ok &= area != 0
        sgn = torch.sign(area)
        axp, ayp = torch.where(a_is_q, x2, x), torch.where(a_is_q, y2, y)
        bxp, byp = torch.where(a_is_q, x, x2), torch.where(a_is_q, y, y2)
        ax, ay = _ndc(axp, ayp, W, H)
        bx, by = _ndc(bxp, byp, W, H)
        best = torch.full_like(tp, -1)
        best_t = torch.full(tp.shape, 2.0, dtype=F64)
        for k in range(3):
            kk = torch.full_like(tp, k)
            ea, eb = _edge(X, Y, sgn, kk, ax, ay), _edge(X, Y, sgn, kk, bx, by)
            cross = (eb < 0) & (ea > eb)
            t = torch.where(cross, ea / torch.where(cross, ea - eb, torch.ones_like(ea)), torch.full_like(ea, 2.0))
            better = cross & (t < best_t)
            best = torch.where(better, kk, best)
            best_t = torch.where(better, t, best_t)
        ok &= best >= 0
        nb = nbrs[T, best.clamp(min=0)]
        has_nb = ok & (nb >= 0)
        if has_nb.any():
            cn = clip[n[has_nb][:, None], faces[nb[has_nb]]]
            projectable = (cn[..., 3] > 0).all(1)
            _, _, an = _project(cn)
            same_facing = projectable & (an != 0) & ((an > 0) == (area[has_nb] > 0))
            idx = torch.nonzero(has_nb, as_tuple=True)[0]
            ok[idx[same_facing]] = False
        code = torch.where(ok, a_is_q.long() * 3 + best, torch.full_like(best, -1))
        codes[n, y, x, direction] = code
    return codes.numpy().astype(np.int8)


def forward(pos, col, uv, tex, faces, mvps, vis, codes):
    """Float64 images (N, H, W, 3); inputs are torch float64 tensors (grads allowed)."""
    faces = torch.as_tensor(np.asarray(faces, np.int64).reshape(-1, 3))
    vis = torch.as_tensor(np.asarray(vis, np.int64))
    codes = torch.as_tensor(np.asarray(codes, np.int64))
    mvps = torch.as_tensor(np.asarray(mvps, np.float64).reshape(-1, 4, 4))
    tex = torch.as_tensor(np.asarray(tex, np.float64))
    s = shade(pos, col, uv, tex, faces, mvps, vis)
    return antialias(s, pos, faces, mvps, vis, codes)


def loss_and_grads(pos, col, uv, tex, faces, mvps, vis, codes, target):
    """L = sum((image - target)^2) in float64 and its gradients w.r.t. pos, col, uv."""
    p = torch.tensor(np.asarray(pos, np.float64), requires_grad=True)
    c = torch.tensor(np.asarray(col, np.float64), requires_grad=True)
    u = torch.tensor(np.asarray(uv, np.float64), requires_grad=True)
    img = forward(p, c, u, tex, faces, mvps, vis, codes)
    L = ((img - torch.as_tensor(np.asarray(target, np.float64))) ** 2).sum()
    L.backward()
    return float(L.detach()), p.grad.numpy(), c.grad.numpy(), u.grad.numpy(), img.detach().numpy()


def adjoint(pos, col, uv, tex, faces, mvps, vis, codes, grad_image):
    """Gradients of sum(image * grad_image) w.r.t. pos, col, uv: the adjoint of the forward for
    a given upstream gradient dL/dimage (float64)."""
    p = torch.tensor(np.asarray(pos, np.float64), requires_grad=True)
    c = torch.tensor(np.asarray(col, np.float64), requires_grad=True)
    u = torch.tensor(np.asarray(uv, np.float64), requires_grad=True)
    img = forward(p, c, u, tex, faces, mvps, vis, codes)
    (img * torch.as_tensor(np.asarray(grad_image, np.float64))).sum().backward()
    return p.grad.numpy(), c.grad.numpy(), u.grad.numpy()


def full_loss(pos, col, uv, tex, faces, nbrs, mvps, W, H, target):
    """The whole forward in float64 with visibility and decisions recomputed for these
    positions (oracle rasterizer), for finite differences."""
    vis = raster_visibility(pos, faces, mvps, W, H)
    codes = decisions(pos, faces, nbrs, mvps, vis)
    with torch.no_grad():
        img = forward(torch.as_tensor(np.asarray(pos, np.float64)), torch.as_tensor(np.asarray(col, np.float64)),
                      torch.as_tensor(np.asarray(uv, np.float64)), tex, faces, mvps, vis, codes)
        return float(((img - torch.as_tensor(np.asarray(target, np.float64))) ** 2).sum())
