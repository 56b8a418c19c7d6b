"""Float64 helpers shared by the parity tests (test infrastructure)."""
import numpy as np


def project(vertices, mvp, W, H):
    """Pixel-space x, y, NDC z of every vertex in float64 (same mapping as the renderer)."""
    p = np.concatenate([vertices[:, :3].astype(np.float64), np.ones((len(vertices), 1))], 1)
    c = p @ np.asarray(mvp, np.float64).T
    n = c[:, :3] / c[:, 3:4]
    return (n[:, 0] * 0.5 + 0.5) * W, (n[:, 1] * 0.5 + 0.5) * H, n[:, 2]


def edge_distance(sx, sy, tri, px, py):
    """Distance (pixels) from point (px, py) to the nearest edge line segment of `tri`."""
    best = np.inf
    for a, b in ((0, 1), (1, 2), (2, 0)):
        ax, ay, bx, by = sx[tri[a]], sy[tri[a]], sx[tri[b]], sy[tri[b]]
        dx, dy = bx - ax, by - ay
        L2 = dx * dx + dy * dy
        t = 0.0 if L2 == 0 else min(1.0, max(0.0, ((px - ax) * dx + (py - ay) * dy) / L2))
        qx, qy = ax + t * dx, ay + t * dy
        best = min(best, np.hypot(px - qx, py - qy))
    return best


def mismatch_near_edges(vis_a, vis_b, vertices, indices, mvp, W, H, sample_offset=(0.0, 0.0), tol=1.0):
    """Returns the list of mismatching pixels that are NOT within `tol` px of an edge of
    either triangle involved (empty list = all mismatches are edge effects)."""
    sx, sy, _ = project(vertices, mvp, W, H)
    bad = []
    for y, x in np.argwhere(vis_a != vis_b):
        px, py = x + sample_offset[0], y + sample_offset[1]
        d = np.inf
        for pid in (vis_a[y, x], vis_b[y, x]):
            if pid >= 0:
                d = min(d, edge_distance(sx, sy, indices[pid], px, py))
        if d > tol:
            bad.append((int(y), int(x), float(d)))
    return bad


def exact_depth(vertices, indices, mvp, W, H, pid, px, py, snap=True):
    """Screen-linear NDC depth of triangle `pid` at pixel-space point (px, py), float64,
    through the vertex positions snapped to the 1/256-pixel grid when `snap` is set."""
    sx, sy, sz = project(vertices, mvp, W, H)
    if snap:
        sx, sy = np.rint(sx * 256.0) / 256.0, np.rint(sy * 256.0) / 256.0
    t = indices[pid]
    A = np.array([[sx[t[0]], sx[t[1]], sx[t[2]]], [sy[t[0]], sy[t[1]], sy[t[2]]], [1.0, 1.0, 1.0]])
    lam = np.linalg.solve(A, [px, py, 1.0])
    return float(lam @ sz[t])
