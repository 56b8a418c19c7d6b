"""Seeded synthetic scenes and cameras.

The reference's benchmark assets (bunny, sponza, character models) are not shipped with
it, so every workload here is generated: icospheres with radial jitter, log-normal
triangle soups, value-noise textures and random cameras, all from numpy's PCG64 so the
same seed gives the same bytes on x86 and Arm hosts.

Conventions (shared with the renderer): clip = M @ (x, y, z, 1) with M row-major;
NDC z in [0, 1] (near plane at 0); pixel x = (x_ndc * 0.5 + 0.5) * W and
pixel y = (y_ndc * 0.5 + 0.5) * H, so NDC y = -1 is image row 0.
"""
import math

import numpy as np

# ----------------------------------------------------------------------------- cameras


def perspective(fovy_deg, aspect, near, far):
    """Right-handed perspective projection with a [0, 1] depth range."""
    f = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    m = np.zeros((4, 4), np.float64)
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = far / (near - far)
    m[2, 3] = near * far / (near - far)
    m[3, 2] = -1.0
    return m


def look_at(eye, target, up=(0.0, 1.0, 0.0)):
    eye, target, up = (np.asarray(a, np.float64) for a in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def orbit_camera(rng, distance, aspect, fovy=60.0, near=0.1, far=100.0):
    """Random viewing direction on a sphere of radius `distance` looking at the origin."""
    v = rng.normal(size=3)
    v /= np.linalg.norm(v)
    up = (0.0, 1.0, 0.0) if abs(v[1]) < 0.95 else (1.0, 0.0, 0.0)
    return (perspective(fovy, aspect, near, far) @ look_at(v * distance, (0, 0, 0), up)).astype(np.float32)


def default_mvp(aspect=1.0):
    """Perspective fov 60 deg, camera at distance 3 on +z looking at the origin."""
    return (perspective(60.0, aspect, 0.1, 100.0) @ look_at((0, 0, 3), (0, 0, 0))).astype(np.float32)


# ----------------------------------------------------------------------------- meshes


def icosphere(subdivisions):
    """Unit icosphere: (vertices (V,3) float64, faces (T,3) int32), outward CCW winding."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    for _ in range(subdivisions):
        cache = {}
        new_faces = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    v = np.array(verts)
    f = np.array(faces, np.int32)
    # enforce outward winding: (b - a) x (c - a) points away from the centre
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = np.einsum("ij,ij->i", n, v[f].mean(axis=1)) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f


def jittered_icosphere(subdivisions, seed, jitter=0.02):
    """Icosphere with uniform radial jitter +-jitter and per-vertex RGB in [0, 1].

    Returns (vertices (V,6) float32 [x y z r g b], indices (T,3) int32)."""
    rng = np.random.default_rng(seed)
    v, f = icosphere(subdivisions)
    r = 1.0 + rng.uniform(-jitter, jitter, size=(len(v), 1))
    col = rng.uniform(0.0, 1.0, size=(len(v), 3))
    return np.concatenate([v * r, col], axis=1).astype(np.float32), f


def geodesic_mesh(frequency):
    """Class-I geodesic subdivision of the icosahedron: every base face is split into
    frequency^2 triangles and the points are pushed onto the unit sphere (20 f^2 triangles,
    10 f^2 + 2 vertices).  Points shared by neighbouring base faces are merged."""
    n = int(frequency)
    base_v, base_f = icosphere(0)
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    keep = ii + jj <= n
    ii, jj = ii[keep], jj[keep]
    kk = n - ii - jj
    local = {(a, b): t for t, (a, b) in enumerate(zip(ii.tolist(), jj.tolist()))}
    # triangles of one face in local point numbering
    tri = []
    for i in range(n):
        for j in range(n - i):
            tri.append((local[(i, j)], local[(i + 1, j)], local[(i, j + 1)]))
            if j < n - i - 1:
                tri.append((local[(i + 1, j)], local[(i + 1, j + 1)], local[(i, j + 1)]))
    tri = np.asarray(tri, np.int64)
    A, B, C = base_v[base_f[:, 0]], base_v[base_f[:, 1]], base_v[base_f[:, 2]]
    pts = (A[:, None, :] * kk[None, :, None] + B[:, None, :] * ii[None, :, None] + C[:, None, :] * jj[None, :, None]) / n
    pts = pts / np.linalg.norm(pts, axis=2, keepdims=True)
    npt = pts.shape[1]
    allp = pts.reshape(-1, 3)
    key = np.round(allp * (1 << 20)).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    v = allp[first]
    f = inv.reshape(-1)[(tri[None, :, :] + (np.arange(len(base_f)) * npt)[:, None, None]).reshape(-1, 3)]
    f = f.astype(np.int32)
    nrm = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = np.einsum("ij,ij->i", nrm, v[f].mean(axis=1)) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f


def geodesic_sphere(frequency, seed, displacement=0.05):
    """Geodesic icosphere of the given frequency (20 * f^2 triangles), radially displaced by a
    sum of random spherical waves.  Returns (positions (V,3), uv (V,2), indices)."""
    rng = np.random.default_rng(seed)
    v, f = geodesic_mesh(frequency)
    k = rng.normal(size=(6, 3)) * 4.0
    ph = rng.uniform(0, 2 * np.pi, size=6)
    disp = np.sin(v @ k.T + ph).mean(axis=1)
    v = v * (1.0 + displacement * disp)[:, None]
    uv = np.stack([0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi),
                   0.5 + np.arcsin(np.clip(v[:, 1] / np.linalg.norm(v, axis=1), -1, 1)) / np.pi], 1)
    return v.astype(np.float32), uv.astype(np.float32), f


def triangle_soup(num_tris, seed, width, height, fovy=60.0, median_px=4.0, sigma=1.0, near=0.5, far=20.0,
                  apex=0.2, uv_density=(0.5, 4.0), max_stretch=8.0):
    """Unshared random triangles with centres uniform (by volume) in the view frustum.

    Each triangle has a longest (base) edge whose on-screen length at the centre's depth is
    log-normal in pixels (median `median_px`, shape `sigma`) and an apex at `apex` x base
    length (x U[0.5, 1.5]) from the base; `apex` = 0.2 gives a depth complexity of about 6
    for 1M triangles at 1920x1080.  Each vertex carries a UV from a random anisotropic affine
    map (texel density log-uniform in `uv_density` texels per pixel of a 1024^2 texture,
    stretch up to `max_stretch`).

    Returns (vertices (3T,5) float32 [x y z u v] in view space, indices (T,3), mvp)."""
    rng = np.random.default_rng(seed)
    aspect = width / height
    th = math.tan(math.radians(fovy) / 2)
    u = rng.uniform(size=num_tris)
    d = (near ** 3 + u * (far ** 3 - near ** 3)) ** (1.0 / 3.0)  # pdf ~ d^2 on [near, far]
    xn = rng.uniform(-1, 1, num_tris)
    yn = rng.uniform(-1, 1, num_tris)
    centre = np.stack([xn * d * th * aspect, yn * d * th, -d], 1)
    px_world = 2.0 * d * th / height  # world size of one pixel at depth d
    L = median_px * np.exp(sigma * rng.normal(size=num_tris))
    theta = rng.uniform(0, 2 * np.pi, num_tris)
    ex = np.stack([np.cos(theta), np.sin(theta)], 1)
    ey = np.stack([-np.sin(theta), np.cos(theta)], 1)
    h = apex * L * rng.uniform(0.5, 1.5, num_tris)
    t = rng.uniform(-0.5, 0.5, num_tris)
    off2 = np.stack([-0.5 * L[:, None] * ex - h[:, None] * ey / 3,
                     0.5 * L[:, None] * ex - h[:, None] * ey / 3,
                     (t * L)[:, None] * ex + (2 * h / 3)[:, None] * ey], 1)  # (T, 3, 2) pixels
    # counter-clockwise in NDC for half of them, clockwise for the rest
    flip = rng.uniform(size=num_tris) < 0.5
    off2[flip] = off2[flip][:, [0, 2, 1]]
    offz = rng.uniform(-0.3, 0.3, size=(num_tris, 3)) * L[:, None]
    off = np.concatenate([off2, offz[..., None]], 2)
    pos = centre[:, None, :] + off * px_world[:, None, None]
    dens = np.exp(rng.uniform(np.log(uv_density[0]), np.log(uv_density[1]), num_tris)) / 1024.0
    stretch = np.exp(rng.uniform(0, np.log(max_stretch), num_tris))
    rot = rng.uniform(0, np.pi, num_tris)
    c, s = np.cos(rot), np.sin(rot)
    m00, m01 = c * dens * stretch, -s * dens
    m10, m11 = s * dens * stretch, c * dens
    base = rng.uniform(0, 1, size=(num_tris, 2))
    ox, oy = off[..., 0], off[..., 1]
    uu = base[:, 0:1] + m00[:, None] * ox + m01[:, None] * oy
    vv = base[:, 1:2] + m10[:, None] * ox + m11[:, None] * oy
    verts = np.concatenate([pos.reshape(-1, 3), np.stack([uu, vv], 2).reshape(-1, 2)], 1).astype(np.float32)
    idx = np.arange(3 * num_tris, dtype=np.int32).reshape(-1, 3)
    mvp = perspective(fovy, aspect, 0.1, 100.0).astype(np.float32)
    return verts, idx, mvp


def c2_scene(seed=2, num_tris=1_000_000, width=1920, height=1080):
    """1M-triangle textured soup for a 1920x1080 4x MSAA target (depth complexity ~6)."""
    return triangle_soup(num_tris, seed, width, height)


def soup_depth_complexity(verts, idx, mvp, width, height):
    """Sum of projected triangle areas over the screen area (no culling, no clipping)."""
    p = verts[:, :3].astype(np.float64)
    clip = np.concatenate([p, np.ones((len(p), 1))], 1) @ mvp.astype(np.float64).T
    xy = clip[:, :2] / clip[:, 3:4]
    sx = (xy[:, 0] * 0.5 + 0.5) * width
    sy = (xy[:, 1] * 0.5 + 0.5) * height
    a, b, c = idx[:, 0], idx[:, 1], idx[:, 2]
    area = 0.5 * np.abs((sx[b] - sx[a]) * (sy[c] - sy[a]) - (sx[c] - sx[a]) * (sy[b] - sy[a]))
    return float(area.sum() / (width * height))


# ----------------------------------------------------------------------------- textures


def value_noise_texture(size, seed, octaves=5):
    """Seeded multi-octave value noise, RGBA8 packed as uint32 (h, w), alpha 255."""
    rng = np.random.default_rng(seed)
    img = np.zeros((size, size, 3), np.float64)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = 4 * (2 ** o)
        lat = rng.uniform(0, 1, size=(cells + 1, cells + 1, 3))
        lat[-1, :, :] = lat[0, :, :]
        lat[:, -1, :] = lat[:, 0, :]
        t = (np.arange(size) + 0.5) / size * cells
        i0 = np.floor(t).astype(int)
        f = t - i0
        f = f * f * (3 - 2 * f)
        i1 = i0 + 1
        fy, fx = f[:, None, None], f[None, :, None]
        v = (lat[i0][:, i0] * (1 - fx) * (1 - fy) + lat[i0][:, i1] * fx * (1 - fy) +
             lat[i1][:, i0] * (1 - fx) * fy + lat[i1][:, i1] * fx * fy)
        img += amp * v
        total += amp
        amp *= 0.55
    img = np.clip(np.round(img / total * 255.0), 0, 255).astype(np.uint32)
    return img[..., 0] | (img[..., 1] << 8) | (img[..., 2] << 16) | (np.uint32(255) << 24)


def c1_scene(seed=1):
    """20,480-triangle icosphere (subdivision 5) with +-2% radial jitter and per-vertex RGB,
    perspective fov 60 deg at distance 3 (512x512 target in the benchmark)."""
    v, f = jittered_icosphere(5, seed)
    return v, f, default_mvp(1.0)


def c3_batch(seed=3, num_views=256, sizes=(128, 256, 512, 1024), tri_range=(1000, 200_000)):
    """Batched workload: `num_views` independent square views with edge uniform in `sizes`,
    each with one mesh of T triangles, T log-uniform in `tri_range`: a displaced geodesic
    icosphere with per-vertex RGB (20 f^2 triangles for the f closest to T) seen from a random
    camera, or a random-triangle soup (per-vertex UV as colour), 50/50; 1x or 4x MSAA (50/50).

    Returns a list of dicts(width, height, samples, kind, vertices, indices, mvp, cull)."""
    rng = np.random.default_rng(seed)
    views = []
    for i in range(num_views):
        size = int(rng.choice(sizes))
        S = int(rng.choice([1, 4]))
        T = int(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]))))
        if rng.uniform() < 0.5:
            f_ = max(1, int(round(math.sqrt(T / 20.0))))
            pos, _uv, idx = geodesic_sphere(f_, 1000 + i)
            col = rng.uniform(0, 1, size=(len(pos), 3)).astype(np.float32)
            verts = np.concatenate([pos, col], 1).astype(np.float32)
            mvp = orbit_camera(rng, rng.uniform(2.2, 4.0), 1.0)
            views.append(dict(width=size, height=size, samples=S, kind="ico", vertices=verts, indices=idx, mvp=mvp,
                              cull=2))
        else:
            verts, idx, mvp = triangle_soup(T, 2000 + i, size, size)
            views.append(dict(width=size, height=size, samples=S, kind="soup", vertices=verts, indices=idx, mvp=mvp,
                              cull=0))
    return views


def c4_scene(seed=4, num_views=64, size=256, subdivisions=5, noise=0.05, tex_size=256):
    """Differentiable workload: an icosphere (subdivision 5: 20,480 triangles) with per-vertex
    RGB colours U[0, 1] and spherical UVs, seen by `num_views` random cameras at distance 3;
    `clean` positions render the target images, `noisy` positions (Gaussian noise of std
    `noise`) are the parameters; float32 RGB value-noise texture of `tex_size`^2.

    Returns dict(clean, noisy, colors, uvs, faces, texture, mvps, width, height)."""
    rng = np.random.default_rng(seed)
    v, f = icosphere(subdivisions)
    clean = v.astype(np.float32)
    noisy = (v + noise * rng.normal(size=v.shape)).astype(np.float32)
    colors = rng.uniform(0.0, 1.0, size=(len(v), 3)).astype(np.float32)
    uvs = np.stack([0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi),
                    0.5 + np.arcsin(np.clip(v[:, 1], -1, 1)) / np.pi], 1).astype(np.float32)
    t8 = value_noise_texture(tex_size, seed)
    texture = np.stack([(t8 >> (8 * c)) & 255 for c in range(3)], -1).astype(np.float32) / 255.0
    mvps = np.stack([orbit_camera(rng, 3.0, 1.0) for _ in range(num_views)]).astype(np.float32)
    return dict(clean=clean, noisy=noisy, colors=colors, uvs=uvs, faces=f.astype(np.int32), texture=texture,
                mvps=mvps, width=size, height=size)


def value_noise_rgba(size, seed, octaves=5, alpha=(0.35, 0.85)):
    """Seeded multi-octave value noise with a noise alpha channel in `alpha`, RGBA8 packed as
    uint32 (size, size).  Each octave's bilinear lattice interpolation (smoothstep weights) is
    separable and evaluated as two matrix products, so large textures are cheap to make."""
    rng = np.random.default_rng(seed)
    acc = np.zeros((4, size, size), np.float32)
    amp, total = 1.0, 0.0
    t = (np.arange(size) + 0.5) / size
    for o in range(octaves):
        cells = 4 * (2 ** o)
        x = t * cells
        i0 = np.floor(x).astype(int)
        f = x - i0
        f = f * f * (3 - 2 * f)
        Wm = np.zeros((size, cells + 1), np.float32)
        Wm[np.arange(size), i0] = 1 - f
        Wm[np.arange(size), i0 + 1] += f
        lat = rng.uniform(0, 1, size=(4, cells + 1, cells + 1)).astype(np.float32)
        lat[:, -1, :] = lat[:, 0, :]
        lat[:, :, -1] = lat[:, :, 0]
        for c in range(4):
            acc[c] += amp * (Wm @ lat[c] @ Wm.T)
        total += amp
        amp *= 0.55
    acc /= total
    acc[3] = alpha[0] + (alpha[1] - alpha[0]) * acc[3]
    b = np.clip(np.round(acc * 255.0), 0, 255).astype(np.uint32)
    return b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24)


def c5_scene(seed=5, instances=40, frequency=112, width=3840, height=2160, blended=0.1, tex_size=4096,
             target_complexity=7.0):
    """Stress workload: `instances` displaced geodesic icospheres of `frequency` (20 f^2 =
    250,880 triangles each at f = 112: 10,035,200 in total) with spherical UVs, random
    positions, orientations and sizes chosen for a front-face depth complexity of about
    `target_complexity` on a `width` x `height` target; a fraction `blended` of the instances are
    alpha-blended and drawn last, back to front.  One shared vertex / index buffer.

    Returns dict(vertices (V,5) [x y z u v], indices (T,3), draws: list of dict(first, count,
    mvp, blend, depth), texture (RGBA8 uint32 with noise alpha), width, height)."""
    rng = np.random.default_rng(seed)
    base_v, base_f = geodesic_mesh(frequency)
    aspect = width / height
    proj = perspective(60.0, aspect, 0.1, 100.0)
    view = look_at((0.0, 0.0, 0.0), (0.0, 0.0, -1.0))
    th = math.tan(math.radians(30.0))
    verts, idx, placed = [], [], []
    off = 0
    for i in range(instances):
        k = rng.normal(size=(6, 3)) * 4.0
        ph = rng.uniform(0, 2 * np.pi, size=6)
        disp = np.sin(base_v @ k.T + ph).mean(axis=1)
        v = base_v * (1.0 + 0.05 * disp)[:, None]
        uv = np.stack([0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi),
                       0.5 + np.arcsin(np.clip(v[:, 1] / np.linalg.norm(v, axis=1), -1, 1)) / np.pi], 1)
        verts.append(np.concatenate([v, uv], 1))
        idx.append(base_f + off)
        off += len(v)
        d = rng.uniform(6.0, 14.0)
        placed.append((d, rng.uniform(-0.8, 0.8) * d * th * aspect, rng.uniform(-0.8, 0.8) * d * th))
    scales = rng.uniform(0.8, 1.2, size=instances)

    def complexity(r):  # mean number of projected discs over a grid of screen points
        ys, xs = np.mgrid[-1:1:108j, -1:1:192j]
        cnt = np.zeros_like(xs)
        for (d, x, y), sc in zip(placed, scales):
            rr = min(r * sc * 1.05, 0.95 * d)  # displaced radius; silhouette half-angle asin(rr / d)
            t_half = rr / math.sqrt(d * d - rr * rr)
            rx, ry = t_half / (th * aspect), t_half / th
            cnt += ((xs - x / (d * th * aspect)) / rx) ** 2 + ((ys - y / (d * th)) / ry) ** 2 <= 1.0
        return cnt.mean()

    lo, hi = 0.1, 20.0  # sphere radius for the target depth complexity (bisection)
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        lo, hi = (mid, hi) if complexity(mid) < target_complexity else (lo, mid)
    radius = 0.5 * (lo + hi)
    draws = []
    for i, (d, x, y) in enumerate(placed):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        a, b, c, w = q
        R = np.array([[1 - 2 * (b * b + c * c), 2 * (a * b - c * w), 2 * (a * c + b * w)],
                      [2 * (a * b + c * w), 1 - 2 * (a * a + c * c), 2 * (b * c - a * w)],
                      [2 * (a * c - b * w), 2 * (b * c + a * w), 1 - 2 * (a * a + b * b)]])
        M = np.eye(4)
        M[:3, :3] = R * radius * scales[i]
        M[:3, 3] = (x, y, -d)
        draws.append(dict(first=3 * i * len(base_f), count=3 * len(base_f),
                          mvp=(proj @ view @ M).astype(np.float32), blend=False, depth=d))
    nblend = int(round(blended * instances))
    order = list(rng.permutation(instances))
    opaque, trans = order[nblend:], order[:nblend]
    trans.sort(key=lambda i: -draws[i]["depth"])  # back to front
    for i in trans:
        draws[i]["blend"] = True
    return dict(vertices=np.concatenate(verts).astype(np.float32), indices=np.concatenate(idx).astype(np.int32),
                draws=[draws[i] for i in opaque + trans], texture=value_noise_rgba(tex_size, seed),
                width=width, height=height, radius=radius)
