// Differentiable shading over a visibility buffer, with analytic silhouette-edge antialiasing,
// and the hand-written adjoints of both.
//
// Forward, per view n and pixel p (centre at NDC ((x + 0.5) / W * 2 - 1, (y + 0.5) / H * 2 - 1),
// the rasterizer's 1x sample position):
//   triangle      T = visibility[n][p] (the rasterizer's view-local triangle id, -1 = none)
//   barycentrics  perspective-correct from the clip positions c_i = MVP_n (pos_i, 1):
//                 a_i = x_i - px w_i, b_i = y_i - py w_i, D = a x b, lambda = D / sum(D)
//   attributes    colour = sum lambda_i col_i, uv = sum lambda_i uv_i
//   texture       bilinear, repeat addressing, texel centres at (i + 0.5) / size
//   shaded        s(p) = colour * texture(uv)   (background: 0)
// Antialiasing, for every horizontally or vertically adjacent pixel pair (p, q) with different
// triangles: the nearer of the two triangles (or the only one) is the occluder T, covering
// pixel `a` of the pair; `b` is the other.  If an edge of T crosses the segment a -> b at
// fraction t, and that edge is a silhouette (no neighbouring triangle across it, or the
// neighbour faces away in this view), the pixel the edge intrudes on is blended:
//   w = t - 1/2;  w >= 0: out(b) += w (s(a) - s(b));  w < 0: out(a) += -w (s(b) - s(a)).
// The image is then continuous in the vertex positions across visibility changes, and t
// carries the position gradient of the silhouette.  The discrete choices of each pair (which
// pixel is covered, which edge) are recorded in `aaCodes` and reused by the backward pass.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/ifrit_gb300.h"

namespace {

struct Tri {
    int v[3];
    float x[3], y[3], w[3];
};

__device__ __forceinline__ void clip_of(const float* m, const float* p, float& x, float& y, float& w) {
    x = m[0] * p[0] + m[1] * p[1] + m[2] * p[2] + m[3];
    y = m[4] * p[0] + m[5] * p[1] + m[6] * p[2] + m[7];
    w = m[12] * p[0] + m[13] * p[1] + m[14] * p[2] + m[15];
}

__device__ __forceinline__ Tri load_tri(const IfritGbDiffPass& P, const float* m, int t) {
    Tri r;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        r.v[i] = min(max(__ldg(P.faces + 3 * t + i), 0), P.numVertices - 1);  // keeps bad indices in bounds
        const float p[3] = {__ldg(P.positions + 3 * r.v[i]), __ldg(P.positions + 3 * r.v[i] + 1),
                            __ldg(P.positions + 3 * r.v[i] + 2)};
        clip_of(m, p, r.x[i], r.y[i], r.w[i]);
    }
    return r;
}

__device__ __forceinline__ void pixel_ndc(const IfritGbDiffPass& P, int x, int y, float& px, float& py) {
    px = ((float)x + 0.5f) / (float)P.width * 2.0f - 1.0f;
    py = ((float)y + 0.5f) / (float)P.height * 2.0f - 1.0f;
}

// p * q - r * s with the rounding error of r * s compensated (Kahan's method: within about
// 1.5 ulp even when the two products nearly cancel).
__device__ __forceinline__ float cross_diff(float p, float q, float r, float s) {
    const float rs = r * s;
    const float err = fmaf(-r, s, rs);
    return fmaf(p, q, -rs) + err;
}

// Perspective-correct barycentrics of NDC point (px, py) on triangle r.
__device__ __forceinline__ void barycentrics(const Tri& r, float px, float py, float a[3], float b[3], float D[3],
                                             float& S, float lam[3]) {
#pragma unroll
    for (int i = 0; i < 3; i++) {  // one rounding each (the product is exact inside the fma)
        a[i] = fmaf(-px, r.w[i], r.x[i]);
        b[i] = fmaf(-py, r.w[i], r.y[i]);
    }
    D[0] = cross_diff(a[1], b[2], a[2], b[1]);
    D[1] = cross_diff(a[2], b[0], a[0], b[2]);
    D[2] = cross_diff(a[0], b[1], a[1], b[0]);
    S = D[0] + D[1] + D[2];
    const float inv = 1.0f / S;
#pragma unroll
    for (int i = 0; i < 3; i++) lam[i] = D[i] * inv;
}

struct TexTap {
    int i0, i1, j0, j1;
    float fx, fy;
};

__device__ __forceinline__ int wrap(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}

__device__ __forceinline__ TexTap tex_tap(const IfritGbDiffPass& P, float u, float v) {
    TexTap t;
    const float s = u * (float)P.texWidth - 0.5f, q = v * (float)P.texHeight - 0.5f;
    const float fs = floorf(s), fq = floorf(q);
    t.fx = s - fs;
    t.fy = q - fq;
    t.i0 = wrap((int)fs, P.texWidth);
    t.i1 = wrap((int)fs + 1, P.texWidth);
    t.j0 = wrap((int)fq, P.texHeight);
    t.j1 = wrap((int)fq + 1, P.texHeight);
    return t;
}

__device__ __forceinline__ float texel(const IfritGbDiffPass& P, int i, int j, int ch) {
    return __ldg(P.texture + ((size_t)j * P.texWidth + i) * 3 + ch);
}

// Shaded colour of triangle t at pixel (x, y) of view n.
__device__ __forceinline__ void shade_pixel(const IfritGbDiffPass& P, const float* m, int t, int x, int y, float out[3]) {
    const Tri r = load_tri(P, m, t);
    float px, py, a[3], b[3], D[3], S, lam[3];
    pixel_ndc(P, x, y, px, py);
    barycentrics(r, px, py, a, b, D, S, lam);
    float col[3] = {0, 0, 0}, uv[2] = {0, 0};
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int c = 0; c < 3; c++) col[c] += lam[i] * __ldg(P.colors + 3 * r.v[i] + c);
        uv[0] += lam[i] * __ldg(P.uvs + 2 * r.v[i]);
        uv[1] += lam[i] * __ldg(P.uvs + 2 * r.v[i] + 1);
    }
    const TexTap k = tex_tap(P, uv[0], uv[1]);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float t00 = texel(P, k.i0, k.j0, c), t10 = texel(P, k.i1, k.j0, c);
        const float t01 = texel(P, k.i0, k.j1, c), t11 = texel(P, k.i1, k.j1, c);
        const float tv = (1.0f - k.fy) * ((1.0f - k.fx) * t00 + k.fx * t10) + k.fy * ((1.0f - k.fx) * t01 + k.fx * t11);
        out[c] = col[c] * tv;
    }
}

__global__ void diff_shade_kernel(IfritGbDiffPass P) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, n = blockIdx.z;
    if (x >= P.width || y >= P.height) return;
    const size_t pix = ((size_t)n * P.height + y) * P.width + x;
    const int t = __ldg(P.visibility + pix);
    float s[3] = {0.0f, 0.0f, 0.0f};
    if (t >= 0 && t < P.numTriangles) shade_pixel(P, P.mvp + 16 * n, t, x, y, s);
    P.shaded[3 * pix] = s[0];
    P.shaded[3 * pix + 1] = s[1];
    P.shaded[3 * pix + 2] = s[2];
}

// ---------------------------------------------------------------------------- antialiasing
// Interpolated clip w (view depth) of triangle t at pixel (x, y).
__device__ __forceinline__ float view_depth(const IfritGbDiffPass& P, const float* m, int t, int x, int y) {
    const Tri r = load_tri(P, m, t);
    float px, py, a[3], b[3], D[3], S, lam[3];
    pixel_ndc(P, x, y, px, py);
    barycentrics(r, px, py, a, b, D, S, lam);
    return lam[0] * r.w[0] + lam[1] * r.w[1] + lam[2] * r.w[2];
}

// Edge function k (opposite vertex k) of the projected triangle at NDC point (px, py), signed
// so that the inside is positive.
__device__ __forceinline__ float edge_fn(const float X[3], const float Y[3], float sgn, int k, float px, float py) {
    const int j = k == 2 ? 0 : k + 1, l = k == 0 ? 2 : k - 1;
    return sgn * ((X[l] - X[j]) * (py - Y[j]) - (Y[l] - Y[j]) * (px - X[j]));
}

__device__ __forceinline__ bool project(const Tri& r, float X[3], float Y[3], float& area) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (!(r.w[i] > 0.0f)) return false;
        X[i] = r.x[i] / r.w[i];
        Y[i] = r.y[i] / r.w[i];
    }
    area = (X[1] - X[0]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[1] - Y[0]);
    return area != 0.0f;
}

// Decision for the pair (p, q) = ((x, y), (x + dx, y + dy)): returns the code
// (a_is_q * 3 + edge) or -1 when the pair is not antialiased.
__device__ int pair_code(const IfritGbDiffPass& P, const float* m, int n, int x, int y, int dx, int dy) {
    const int x2 = x + dx, y2 = y + dy;
    if (x2 >= P.width || y2 >= P.height) return -1;
    const size_t base = (size_t)n * P.height * P.width;
    const int tp = __ldg(P.visibility + base + (size_t)y * P.width + x);
    const int tq = __ldg(P.visibility + base + (size_t)y2 * P.width + x2);
    if (tp == tq) return -1;
    if ((tp >= P.numTriangles) || (tq >= P.numTriangles)) return -1;
    int a_is_q;
    if (tp < 0) a_is_q = 1;
    else if (tq < 0) a_is_q = 0;
    else a_is_q = view_depth(P, m, tq, x2, y2) < view_depth(P, m, tp, x, y) ? 1 : 0;
    const int T = a_is_q ? tq : tp;
    const Tri r = load_tri(P, m, T);
    float X[3], Y[3], area;
    if (!project(r, X, Y, area)) return -1;
    const float sgn = area > 0.0f ? 1.0f : -1.0f;
    float ax, ay, bx, by;
    pixel_ndc(P, a_is_q ? x2 : x, a_is_q ? y2 : y, ax, ay);
    pixel_ndc(P, a_is_q ? x : x2, a_is_q ? y : y2, bx, by);
    int best = -1;
    float best_t = 2.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float ea = edge_fn(X, Y, sgn, k, ax, ay), eb = edge_fn(X, Y, sgn, k, bx, by);
        if (eb < 0.0f && ea > eb) {
            const float t = ea / (ea - eb);
            if (t < best_t) {
                best_t = t;
                best = k;
            }
        }
    }
    if (best < 0) return -1;
    // silhouette test: the triangle across the edge is missing or faces away
    const int nb = __ldg(P.neighbors + 3 * T + best);
    if (nb >= 0 && nb < P.numTriangles) {
        const Tri rn = load_tri(P, m, nb);
        float Xn[3], Yn[3], an;
        if (project(rn, Xn, Yn, an) && (an > 0.0f) == (area > 0.0f)) return -1;
    }
    return a_is_q * 3 + best;
}

// Edge crossing fraction t of a recorded decision, with what the adjoint needs.  The
// difference ea - eb is evaluated directly as the edge function's change between the two pixel
// centres (no cancellation between two nearly equal values).
struct PairGeom {
    int a_x, a_y, b_x, b_y;
    int T, k;
    Tri r;
    float X[3], Y[3], sgn;
    float ax, ay, bx, by, ea, eb, den, t;
};

__device__ __forceinline__ bool pair_geom(const IfritGbDiffPass& P, const float* m, int n, int x, int y, int dx, int dy,
                                          int code, PairGeom& g) {
    const int a_is_q = code >= 3;
    g.k = code % 3;
    g.a_x = a_is_q ? x + dx : x;
    g.a_y = a_is_q ? y + dy : y;
    g.b_x = a_is_q ? x : x + dx;
    g.b_y = a_is_q ? y : y + dy;
    g.T = __ldg(P.visibility + ((size_t)n * P.height + g.a_y) * P.width + g.a_x);
    g.r = load_tri(P, m, g.T);
    float area;
    if (!project(g.r, g.X, g.Y, area)) return false;
    g.sgn = area > 0.0f ? 1.0f : -1.0f;
    pixel_ndc(P, g.a_x, g.a_y, g.ax, g.ay);
    pixel_ndc(P, g.b_x, g.b_y, g.bx, g.by);
    g.ea = edge_fn(g.X, g.Y, g.sgn, g.k, g.ax, g.ay);
    g.eb = edge_fn(g.X, g.Y, g.sgn, g.k, g.bx, g.by);
    const int j = g.k == 2 ? 0 : g.k + 1, l = g.k == 0 ? 2 : g.k - 1;
    g.den = g.sgn * ((g.X[l] - g.X[j]) * (g.ay - g.by) - (g.Y[l] - g.Y[j]) * (g.ax - g.bx));
    if (!(g.den > 0.0f)) return false;
    g.t = fminf(fmaxf(g.ea / g.den, 0.0f), 1.0f);
    return true;
}

__device__ __forceinline__ void load3(const float* p, size_t pix, float v[3]) {
    v[0] = p[3 * pix];
    v[1] = p[3 * pix + 1];
    v[2] = p[3 * pix + 2];
}

// The four pairs touching pixel (x, y): (x-1,y)-(x,y), (x,y)-(x+1,y), (x,y-1)-(x,y), (x,y)-(x,y+1).
// Each is described by its owner pixel (left / upper) and direction.
__device__ __forceinline__ bool pair_of(int i, int x, int y, int& ox, int& oy, int& dx, int& dy, int& dir) {
    switch (i) {
    case 0: ox = x - 1; oy = y; dx = 1; dy = 0; dir = 0; return x > 0;
    case 1: ox = x; oy = y; dx = 1; dy = 0; dir = 0; return true;
    case 2: ox = x; oy = y - 1; dx = 0; dy = 1; dir = 1; return y > 0;
    default: ox = x; oy = y; dx = 0; dy = 1; dir = 1; return true;
    }
}

__global__ void diff_aa_kernel(IfritGbDiffPass P) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, n = blockIdx.z;
    if (x >= P.width || y >= P.height) return;
    const float* m = P.mvp + 16 * n;
    const size_t base = (size_t)n * P.height * P.width;
    const size_t pix = base + (size_t)y * P.width + x;
    float out[3];
    load3(P.shaded, pix, out);
    for (int i = 0; i < 4; i++) {
        int ox, oy, dx, dy, dir;
        if (!pair_of(i, x, y, ox, oy, dx, dy, dir)) continue;
        const int code = pair_code(P, m, n, ox, oy, dx, dy);
        if (ox == x && oy == y) P.aaCodes[2 * pix + dir] = (signed char)code;
        if (code < 0) continue;
        PairGeom g;
        if (!pair_geom(P, m, n, ox, oy, dx, dy, code, g)) continue;
        const float w = g.t - 0.5f;
        const bool to_b = w >= 0.0f;
        const int tx = to_b ? g.b_x : g.a_x, ty = to_b ? g.b_y : g.a_y;
        if (tx != x || ty != y) continue;  // this pair blends the other pixel
        const int sx = to_b ? g.a_x : g.b_x, sy = to_b ? g.a_y : g.b_y;
        float so[3], st[3];
        load3(P.shaded, base + (size_t)sy * P.width + sx, so);
        load3(P.shaded, pix, st);
        const float aw = fabsf(w);
#pragma unroll
        for (int c = 0; c < 3; c++) out[c] += aw * (so[c] - st[c]);
    }
    P.image[3 * pix] = out[0];
    P.image[3 * pix + 1] = out[1];
    P.image[3 * pix + 2] = out[2];
}

// ---------------------------------------------------------------------------- adjoint
// d(clip) -> d(position) through the view's MVP rows x, y, w.
__device__ __forceinline__ void scatter_position(const IfritGbDiffPass& P, const float* m, int v, float gx, float gy,
                                                 float gw) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float g = m[c] * gx + m[4 + c] * gy + m[12 + c] * gw;
        atomicAdd(P.gradPositions + 3 * v + c, g);
    }
}

// Adjoint of t = ea / (ea - eb) with respect to the projected vertices of the edge, then to
// clip coordinates and positions.
__device__ void edge_adjoint(const IfritGbDiffPass& P, const float* m, const PairGeom& g, float gt) {
    const float gea = gt * (-g.eb) / (g.den * g.den), geb = gt * g.ea / (g.den * g.den);
    const int k = g.k, j = k == 2 ? 0 : k + 1, l = k == 0 ? 2 : k - 1;
    // E(P) = (X_l - X_j)(P_y - Y_j) - (Y_l - Y_j)(P_x - X_j), times sgn
    float gX[3] = {0, 0, 0}, gY[3] = {0, 0, 0};
    const float pxs[2] = {g.ax, g.bx}, pys[2] = {g.ay, g.by}, ge[2] = {gea, geb};
#pragma unroll
    for (int s = 0; s < 2; s++) {
        const float e = ge[s] * g.sgn;
        gX[l] += e * (pys[s] - g.Y[j]);
        gX[j] += e * (g.Y[l] - pys[s]);
        gY[l] += e * (-(pxs[s] - g.X[j]));
        gY[j] += e * (pxs[s] - g.X[l]);
    }
    const int vv[2] = {j, l};
#pragma unroll
    for (int s = 0; s < 2; s++) {
        const int i = vv[s];
        const float iw = 1.0f / g.r.w[i];
        const float gx = gX[i] * iw, gy = gY[i] * iw;
        const float gw = -(gX[i] * g.r.x[i] + gY[i] * g.r.y[i]) * iw * iw;
        scatter_position(P, m, g.r.v[i], gx, gy, gw);
    }
}

// Adjoint of shading at pixel (x, y) for triangle t, given dL/ds.
__device__ void shade_adjoint(const IfritGbDiffPass& P, const float* m, int t, int x, int y, const float gs[3]) {
    const Tri r = load_tri(P, m, t);
    float px, py, a[3], b[3], D[3], S, lam[3];
    pixel_ndc(P, x, y, px, py);
    barycentrics(r, px, py, a, b, D, S, lam);
    float ci[3][3], ui[3][2], col[3] = {0, 0, 0}, uv[2] = {0, 0};
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            ci[i][c] = __ldg(P.colors + 3 * r.v[i] + c);
            col[c] += lam[i] * ci[i][c];
        }
        ui[i][0] = __ldg(P.uvs + 2 * r.v[i]);
        ui[i][1] = __ldg(P.uvs + 2 * r.v[i] + 1);
        uv[0] += lam[i] * ui[i][0];
        uv[1] += lam[i] * ui[i][1];
    }
    const TexTap k = tex_tap(P, uv[0], uv[1]);
    float gcol[3], gu = 0.0f, gv = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float t00 = texel(P, k.i0, k.j0, c), t10 = texel(P, k.i1, k.j0, c);
        const float t01 = texel(P, k.i0, k.j1, c), t11 = texel(P, k.i1, k.j1, c);
        const float tv = (1.0f - k.fy) * ((1.0f - k.fx) * t00 + k.fx * t10) + k.fy * ((1.0f - k.fx) * t01 + k.fx * t11);
        const float dtdu = (float)P.texWidth * ((1.0f - k.fy) * (t10 - t00) + k.fy * (t11 - t01));
        const float dtdv = (float)P.texHeight * ((1.0f - k.fx) * (t01 - t00) + k.fx * (t11 - t10));
        gcol[c] = gs[c] * tv;
        const float gtv = gs[c] * col[c];
        gu += gtv * dtdu;
        gv += gtv * dtdv;
    }
    float glam[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        glam[i] = gcol[0] * ci[i][0] + gcol[1] * ci[i][1] + gcol[2] * ci[i][2] + gu * ui[i][0] + gv * ui[i][1];
#pragma unroll
        for (int c = 0; c < 3; c++) atomicAdd(P.gradColors + 3 * r.v[i] + c, lam[i] * gcol[c]);
        atomicAdd(P.gradUvs + 2 * r.v[i], lam[i] * gu);
        atomicAdd(P.gradUvs + 2 * r.v[i] + 1, lam[i] * gv);
    }
    // lambda = D / S
    const float G = glam[0] * lam[0] + glam[1] * lam[1] + glam[2] * lam[2];
    const float inv = 1.0f / S;
    const float gD[3] = {(glam[0] - G) * inv, (glam[1] - G) * inv, (glam[2] - G) * inv};
    const float ga[3] = {-gD[1] * b[2] + gD[2] * b[1], gD[0] * b[2] - gD[2] * b[0], -gD[0] * b[1] + gD[1] * b[0]};
    const float gb[3] = {gD[1] * a[2] - gD[2] * a[1], -gD[0] * a[2] + gD[2] * a[0], gD[0] * a[1] - gD[1] * a[0]};
#pragma unroll
    for (int i = 0; i < 3; i++) scatter_position(P, m, r.v[i], ga[i], gb[i], -px * ga[i] - py * gb[i]);
}

__global__ void diff_backward_kernel(IfritGbDiffPass P) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, n = blockIdx.z;
    if (x >= P.width || y >= P.height) return;
    const float* m = P.mvp + 16 * n;
    const size_t base = (size_t)n * P.height * P.width;
    const size_t pix = base + (size_t)y * P.width + x;
    float gs[3];
    load3(P.gradImage, pix, gs);
    for (int i = 0; i < 4; i++) {
        int ox, oy, dx, dy, dir;
        if (!pair_of(i, x, y, ox, oy, dx, dy, dir)) continue;
        if (ox + dx >= P.width || oy + dy >= P.height) continue;
        const int code = P.aaCodes[2 * (base + (size_t)oy * P.width + ox) + dir];
        if (code < 0) continue;
        PairGeom g;
        if (!pair_geom(P, m, n, ox, oy, dx, dy, code, g)) continue;
        const float w = g.t - 0.5f;
        const bool to_b = w >= 0.0f;
        const int tx = to_b ? g.b_x : g.a_x, ty = to_b ? g.b_y : g.a_y;
        const int sx = to_b ? g.a_x : g.b_x, sy = to_b ? g.a_y : g.b_y;
        const size_t tpix = base + (size_t)ty * P.width + tx, spix = base + (size_t)sy * P.width + sx;
        float gout_t[3];
        load3(P.gradImage, tpix, gout_t);
        const float aw = fabsf(w);
        // out(target) = s(target) + |w| (s(source) - s(target))
        if (tx == x && ty == y) {
#pragma unroll
            for (int c = 0; c < 3; c++) gs[c] -= aw * gout_t[c];
        } else if (sx == x && sy == y) {
#pragma unroll
            for (int c = 0; c < 3; c++) gs[c] += aw * gout_t[c];
        }
        if (ox == x && oy == y) {  // the owner of the pair carries its silhouette gradient
            float ss[3], st[3];
            load3(P.shaded, spix, ss);
            load3(P.shaded, tpix, st);
            float gw = 0.0f;
#pragma unroll
            for (int c = 0; c < 3; c++) gw += gout_t[c] * (ss[c] - st[c]);
            const float gt = to_b ? gw : -gw;  // |w| = w or -w
            if (g.t > 0.0f && g.t < 1.0f) edge_adjoint(P, m, g, gt);
        }
    }
    const int t = __ldg(P.visibility + pix);
    if (t >= 0 && t < P.numTriangles) shade_adjoint(P, m, t, x, y, gs);
}

int check(const IfritGbDiffPass* p) {
    if (!p || p->numViews <= 0 || p->width <= 0 || p->height <= 0 || p->numTriangles < 0 || p->numVertices <= 0)
        return IFTR_ERR_INVALID_ARG;
    if (p->numViews > 65535 || p->texWidth <= 0 || p->texHeight <= 0) return IFTR_ERR_INVALID_ARG;
    if (!p->mvp || !p->positions || !p->colors || !p->uvs || !p->faces || !p->neighbors || !p->texture ||
        !p->visibility || !p->shaded)
        return IFTR_ERR_INVALID_ARG;
    return IFTR_OK;
}

}  // namespace

extern "C" IFTR_API int iftrDiffForward(const IfritGbDiffPass* p, void* cudaStream) {
    int rc = check(p);
    if (rc) return rc;
    if (!p->image || !p->aaCodes) return IFTR_ERR_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(cudaStream);
    dim3 blk(16, 16), grd((p->width + 15) / 16, (p->height + 15) / 16, p->numViews);
    diff_shade_kernel<<<grd, blk, 0, st>>>(*p);
    diff_aa_kernel<<<grd, blk, 0, st>>>(*p);
    return cudaGetLastError() == cudaSuccess ? IFTR_OK : IFTR_ERR_CUDA;
}

extern "C" IFTR_API int iftrDiffBackward(const IfritGbDiffPass* p, void* cudaStream) {
    int rc = check(p);
    if (rc) return rc;
    if (!p->aaCodes || !p->gradImage || !p->gradPositions || !p->gradColors || !p->gradUvs) return IFTR_ERR_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(cudaStream);
    dim3 blk(16, 16), grd((p->width + 15) / 16, (p->height + 15) / 16, p->numViews);
    diff_backward_kernel<<<grd, blk, 0, st>>>(*p);
    return cudaGetLastError() == cudaSuccess ? IFTR_OK : IFTR_ERR_CUDA;
}
