// Device arithmetic of the GB300 triangle pipeline.
//
// Every function here is the sm_103a form of one stage of the soft renderer
// (Aeroraven/Ifrit-v2 projects/softgraphics): vertex transform (TileRasterWorker.cpp:432-476),
// homogeneous clipping (TileRasterWorker.cpp:136-277, TileRasterCoreInvocationCuda.cu:1342-1400),
// culling and setup (TileRasterWorker.cpp:503-727, TileRasterCoreInvocationCuda.cu:1549-1644),
// coverage (TileRasterCoreInvocationCuda.cu:891-982), depth (TileRasterWorker.cpp:2244-2386),
// perspective interpolation with quad derivatives (TileRasterCoreInvocationCuda.cu:2144-2317,
// ShaderBuiltinCuda.cuh:36-94), texture sampling (ShaderBuiltinCuda.cuh:96-272) and blending
// (TileRasterWorker.cpp:2346-2373).
//
// Bit-exactness contract: coverage is integer (16.8 fixed-point vertices, 64-bit edge
// functions, top-left fill rule); every float expression is evaluated in one fixed order with
// IEEE round-to-nearest and no contraction (the library is compiled with --fmad=false, and
// division/sqrt are the IEEE ones), so the CPU checker reproduces every bit.
#pragma once
#include <cstdint>

namespace ifr {

constexpr float kWEps = 1e-5f;
constexpr int kMaxPoly = 10;
constexpr float kSnapLimit = 8000000.0f;
constexpr float kInv255 = 0x1.010102p-8f;

enum { FMT_RGBA8 = 0, FMT_RGBA16F = 1, FMT_RGBA32F = 2, FMT_RGB32F = 3 };
enum { SHADE_GOURAUD = 0, SHADE_TEXTURED = 1, SHADE_PRIMID = 2 };

struct SamplerDev {
    int address_u, address_v, filter, border_white, max_aniso;
    float lod_bias;
};

// One draw of a render pass, as the kernels see it (device pointers).
struct DrawDev {
    int view;  // index of the view (target) this draw renders into
    const float* vertices;
    int stride, num_vertices, attr_offset, attr_count;
    const int* indices;
    int num_triangles, prim_base;
    float mvp[16];
    int cull_mode, front_ccw, depth_func, depth_write;
    int blend_enable, blend_src_color, blend_dst_color, blend_src_alpha, blend_dst_alpha;
    int shading;
    const uint32_t* texels;
    int tex_w, tex_h, tex_levels;
    SamplerDev sampler;
    int lvl_off[16], lvl_w[16], lvl_h[16];  // mip table: texel offset and size of each level
    // scissor test: with scissor_count > 0 a pixel is kept iff it lies in one of the rectangles
    // (inclusive pixel bounds x0, y0, x1, y1); scissor_box is their union's bounds
    int scissor_count;
    int scissor_box[4];
    int scissor[16][4];
    int polygon_mode;  // POLY_FILL / POLY_LINE / POLY_POINT
    int clip_input;    // 1: vertex positions are 4 clip-space floats (a mesh / geometry stage's output), no MVP
};

// Polygon modes (IfritPolygonMode, base/Constants.h:23-28).  LINE: each edge of the culled,
// orientation-normalised triangle is a 1-pixel-wide parallelogram offset +-1/2 pixel along the
// minor axis; POINT: each vertex is a 1-pixel square.  Each part is two sub-triangles
// (sub = 2 * part + half) rasterised with the fill rules; triangles that need clipping are
// dropped in these modes.
enum { POLY_FILL = 0, POLY_LINE = 1, POLY_POINT = 2 };

__device__ __forceinline__ bool scissor_pass(const DrawDev& d, int x, int y) {
    for (int i = 0; i < d.scissor_count; i++)
        if (x >= d.scissor[i][0] && x <= d.scissor[i][2] && y >= d.scissor[i][1] && y <= d.scissor[i][3]) return true;
    return d.scissor_count == 0;
}

// Standard sample positions in 1/256 pixel (the D3D 1/2/4/8/16x patterns): (x, y) of sample k
// of an S-sample pixel.  With S and k compile-time constants (templated sample counts, unrolled
// sample loops) these fold to immediates.
__host__ __device__ constexpr int sample_pos(int S, int k, int axis) {
    const int p1[2] = {128, 128};
    const int p2[4] = {192, 192, 64, 64};
    const int p4[8] = {96, 32, 224, 96, 32, 160, 160, 224};
    const int p8[16] = {144, 80, 112, 176, 208, 144, 80, 48, 48, 208, 16, 112, 176, 240, 240, 16};
    const int p16[32] = {144, 144, 112, 80, 80, 160, 192, 112, 48, 96, 160, 208, 208, 176, 176, 48,
                         96, 224, 128, 16, 64, 32, 32, 192, 0, 128, 240, 64, 224, 240, 16, 0};
    const int i = 2 * k + axis;
    return S == 1 ? p1[i] : S == 2 ? p2[i] : S == 4 ? p4[i] : S == 8 ? p8[i] : p16[i];
}
template <int S>
__device__ __forceinline__ int sample_x(int k) { return sample_pos(S, k, 0); }
template <int S>
__device__ __forceinline__ int sample_y(int k) { return sample_pos(S, k, 1); }

// Sample k's offset on `axis` at run time: every position of the sample patterns is a multiple of 16
// (1/256 pixel), so a pattern packs into 4 bits per sample and axis.
__host__ __device__ constexpr bool sample_patterns_pack() {
    for (int S = 1; S <= 16; S *= 2)
        for (int k = 0; k < S; k++)
            for (int axis = 0; axis < 2; axis++)
                if (sample_pos(S, k, axis) % 16 != 0) return false;
    return true;
}
static_assert(sample_patterns_pack(), "every sample position is a multiple of 1/16 pixel");

template <int S>
__host__ __device__ constexpr unsigned long long packed_sample_axis(int axis) {
    unsigned long long r = 0;
    for (int k = 0; k < S; k++) r |= (unsigned long long)(sample_pos(S, k, axis) / 16) << (4 * k);
    return r;
}
template <int S>
__device__ __forceinline__ int sample_at(int k, int axis) {
    static_assert(S <= 16, "packed patterns of 16 samples at most");
    constexpr unsigned long long px = packed_sample_axis<S>(0), py = packed_sample_axis<S>(1);
    return (int)(((axis ? py : px) >> (4 * k)) & 15u) * 16;
}

// Attributes are evaluated at the pixel centre (1/256-pixel units).
constexpr int kShadeOffset = 128;

// Per-view constants of a pass.
struct PassConst {
    int W, H, S;
    int tile_shift;  // log2 of the screen-tile edge (3: 8x8, 4: 16x16)
    int tiles_x, tiles_y;
    int smin_x, smax_x, smin_y, smax_y;  // bounds of the sample positions
    float W256, H256, gx, gy;
};

struct CVert {
    float p[4];
    float b[3];
};

// A set-up (sub-)triangle: snapped vertices, edge functions, depth plane, pixel bbox.
struct SubTri {
    int32_t X[3], Y[3];
    float z[3], iw[3];
    float bary[3][3];
    int32_t A[3], B[3];
    int64_t C[3], Cb[3];
    float dzdx, dzdy;
    int px0, px1, py0, py1;
    int swapped;  // vertices 1 and 2 were exchanged to make the area positive
};

// Compact set-up of an unclipped triangle, written once per triangle by the counting binner
// and reused by the scattering binner and the tile kernel (64 bytes, four 16-byte vectors).
// Clipped triangles keep only `flags` and `draw` (their sub-triangles are set up again).
struct __align__(16) TriRecord {
    int32_t X0, Y0, X1, Y1;
    int32_t X2, Y2, flags, draw;  // draw: index of the draw the triangle belongs to
    float z0, dzdx, dzdy, iw0;
    float iw1, iw2, pad1, pad2;
};
enum { REC_VALID = 1, REC_SWAPPED = 2, REC_CLIPPED = 4 };

// floor(a / 256): an arithmetic right shift (two's complement)
__device__ __forceinline__ int64_t floordiv256(int64_t a) { return a >> 8; }
__device__ __forceinline__ int64_t ceildiv256(int64_t a) { return -floordiv256(-a); }

__device__ __forceinline__ void xform(const float* m, const float* v, float out[4]) {
    float x = __ldg(v), y = __ldg(v + 1), z = __ldg(v + 2);
#pragma unroll
    for (int r = 0; r < 4; r++) out[r] = m[4 * r + 0] * x + m[4 * r + 1] * y + m[4 * r + 2] * z + m[4 * r + 3];
}

__device__ __forceinline__ float plane_dist(const PassConst& c, int plane, const float* p) {
    switch (plane) {
    case 0: return p[3] - kWEps;
    case 1: return p[2];
    case 2: return p[3] - p[2];
    case 3: return c.gx * p[3] - p[0];
    case 4: return c.gx * p[3] + p[0];
    case 5: return c.gy * p[3] - p[1];
    default: return c.gy * p[3] + p[1];
    }
}

// Sutherland-Hodgman against the 7 planes (w >= eps, 0 <= z <= w, x/y guard band) in fixed order.
static __device__ __noinline__ int clip_polygon(const PassConst& c, CVert* poly) {
    int n = 3;
    CVert tmp[kMaxPoly];
    for (int pl = 0; pl < 7; pl++) {
        bool all_in = true, all_out = true;
        for (int i = 0; i < n; i++) {
            float d = plane_dist(c, pl, poly[i].p);
            if (d >= 0.0f) all_out = false; else all_in = false;
        }
        if (all_out) return 0;
        if (all_in) continue;
        int m = 0;
        for (int i = 0; i < n; i++) {
            const CVert a = poly[i];
            const CVert b = poly[(i + 1) % n];
            float da = plane_dist(c, pl, a.p), db = plane_dist(c, pl, b.p);
            if (da >= 0.0f) tmp[m++] = a;
            if ((da >= 0.0f) != (db >= 0.0f)) {
                float t = da / (da - db);
                CVert q;
#pragma unroll
                for (int k = 0; k < 4; k++) q.p[k] = a.p[k] + t * (b.p[k] - a.p[k]);
#pragma unroll
                for (int k = 0; k < 3; k++) q.b[k] = a.b[k] + t * (b.b[k] - a.b[k]);
                tmp[m++] = q;
            }
        }
        n = m;
        if (n < 3) return 0;
        for (int i = 0; i < n; i++) poly[i] = tmp[i];
    }
    return n;
}

// Pixel range that may hold covered samples (conservative in the sample pattern's extent).
__device__ __forceinline__ bool sub_bbox(const PassConst& c, SubTri& o) {
    int32_t xmin = min(o.X[0], min(o.X[1], o.X[2])), xmax = max(o.X[0], max(o.X[1], o.X[2]));
    int32_t ymin = min(o.Y[0], min(o.Y[1], o.Y[2])), ymax = max(o.Y[0], max(o.Y[1], o.Y[2]));
    int64_t px0 = ceildiv256((int64_t)xmin - c.smax_x), px1 = floordiv256((int64_t)xmax - c.smin_x);
    int64_t py0 = ceildiv256((int64_t)ymin - c.smax_y), py1 = floordiv256((int64_t)ymax - c.smin_y);
    if (px0 < 0) px0 = 0;
    if (py0 < 0) py0 = 0;
    if (px1 > c.W - 1) px1 = c.W - 1;
    if (py1 > c.H - 1) py1 = c.H - 1;
    if (px0 > px1 || py0 > py1) return false;
    o.px0 = (int)px0; o.px1 = (int)px1; o.py0 = (int)py0; o.py1 = (int)py1;
    return true;
}

// Edge functions E_i = A_i x + B_i y + C_i (positive inside) and their top-left biased form.
// Clamps the pixel range of a set-up triangle to the draw's scissor rectangles' union; false when
// nothing is left.
__device__ __forceinline__ bool scissor_clamp(const DrawDev& d, SubTri& s) {
    if (d.scissor_count == 0) return true;
    s.px0 = max(s.px0, d.scissor_box[0]);
    s.py0 = max(s.py0, d.scissor_box[1]);
    s.px1 = min(s.px1, d.scissor_box[2]);
    s.py1 = min(s.py1, d.scissor_box[3]);
    return s.px0 <= s.px1 && s.py0 <= s.py1;
}

__device__ __forceinline__ void sub_edges(SubTri& o) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        int j = (i + 1) % 3, k = (i + 2) % 3;
        o.A[i] = o.Y[j] - o.Y[k];
        o.B[i] = o.X[k] - o.X[j];
        o.C[i] = (int64_t)(o.Y[k] - o.Y[j]) * o.X[j] - (int64_t)(o.X[k] - o.X[j]) * o.Y[j];
        bool topleft = (o.A[i] > 0) || (o.A[i] == 0 && o.B[i] > 0);
        o.Cb[i] = o.C[i] - (topleft ? 0 : 1);
    }
}

// Projection, 16.8 snap, cull, orientation normalisation, edge functions, depth plane and
// the pixel range that may hold covered samples.  Returns false when nothing can be covered.
__device__ __forceinline__ bool setup_sub(const PassConst& c, const DrawDev& d, const CVert& v0, const CVert& v1,
                                          const CVert& v2, SubTri& o) {
    const CVert* v[3] = {&v0, &v1, &v2};
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float iw = 1.0f / v[i]->p[3];
        float xn = v[i]->p[0] * iw, yn = v[i]->p[1] * iw, zn = v[i]->p[2] * iw;
        float fx = (xn * 0.5f + 0.5f) * c.W256;
        float fy = (yn * 0.5f + 0.5f) * c.H256;
        fx = fminf(fmaxf(fx, -kSnapLimit), kSnapLimit);
        fy = fminf(fmaxf(fy, -kSnapLimit), kSnapLimit);
        o.X[i] = __float2int_rn(fx);
        o.Y[i] = __float2int_rn(fy);
        o.z[i] = zn;
        o.iw[i] = iw;
#pragma unroll
        for (int k = 0; k < 3; k++) o.bary[i][k] = v[i]->b[k];
    }
    int64_t a2 = (int64_t)(o.X[1] - o.X[0]) * (o.Y[2] - o.Y[0]) - (int64_t)(o.X[2] - o.X[0]) * (o.Y[1] - o.Y[0]);
    if (a2 == 0) return false;
    bool front = d.front_ccw ? (a2 > 0) : (a2 < 0);
    if (d.cull_mode == 3) return false;
    if (d.cull_mode == 1 && front) return false;
    if (d.cull_mode == 2 && !front) return false;
    o.swapped = 0;
    if (a2 < 0) {
        o.swapped = 1;
        int32_t t;
        float tf;
        t = o.X[1]; o.X[1] = o.X[2]; o.X[2] = t;
        t = o.Y[1]; o.Y[1] = o.Y[2]; o.Y[2] = t;
        tf = o.z[1]; o.z[1] = o.z[2]; o.z[2] = tf;
        tf = o.iw[1]; o.iw[1] = o.iw[2]; o.iw[2] = tf;
#pragma unroll
        for (int k = 0; k < 3; k++) { tf = o.bary[1][k]; o.bary[1][k] = o.bary[2][k]; o.bary[2][k] = tf; }
        a2 = -a2;
    }
    if (!sub_bbox(c, o)) return false;
    sub_edges(o);
    float dX1 = (float)(o.X[1] - o.X[0]), dY1 = (float)(o.Y[1] - o.Y[0]);
    float dX2 = (float)(o.X[2] - o.X[0]), dY2 = (float)(o.Y[2] - o.Y[0]);
    float dz1 = o.z[1] - o.z[0], dz2 = o.z[2] - o.z[0];
    float fa = (float)a2;
    o.dzdx = (dz1 * dY2 - dz2 * dY1) / fa;
    o.dzdy = (dz2 * dX1 - dz1 * dX2) / fa;
    return true;
}

// Fetch + transform the three vertices of triangle t.  Returns false for invalid indices or
// non-finite clip coordinates.  Sets `inside` when no clip plane cuts the triangle.
__device__ __forceinline__ bool fetch_triangle(const PassConst& c, const DrawDev& d, int t, CVert* poly,
                                               bool& inside, bool& rejected) {
    inside = true;
    rejected = false;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        int vid = __ldg(d.indices + 3 * (size_t)t + i);
        if (vid < 0 || vid >= d.num_vertices) return false;
        const float* vp = d.vertices + (size_t)vid * d.stride;
        if (d.clip_input) {
#pragma unroll
            for (int k = 0; k < 4; k++) poly[i].p[k] = __ldg(vp + k);
        } else {
            xform(d.mvp, vp, poly[i].p);
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (!isfinite(poly[i].p[k])) return false;
#pragma unroll
        for (int k = 0; k < 3; k++) poly[i].b[k] = (k == i) ? 1.0f : 0.0f;
    }
#pragma unroll
    for (int pl = 0; pl < 7; pl++) {
        int nin = 0;
#pragma unroll
        for (int i = 0; i < 3; i++) nin += plane_dist(c, pl, poly[i].p) >= 0.0f;
        if (nin == 0) { rejected = true; return false; }
        if (nin != 3) inside = false;
    }
    return true;
}

// Sets up fan triangle `sub` of triangle t (after clipping).  Returns false if it is culled
// or absent.
__device__ __forceinline__ bool setup_triangle_sub(const PassConst& c, const DrawDev& d, int t, int sub, SubTri& o) {
    CVert poly[kMaxPoly];
    bool inside, rejected;
    if (!fetch_triangle(c, d, t, poly, inside, rejected)) return false;
    if (inside) {
        if (sub != 0) return false;
        return setup_sub(c, d, poly[0], poly[1], poly[2], o);
    }
    int n = clip_polygon(c, poly);
    if (sub + 2 >= n) return false;
    return setup_sub(c, d, poly[0], poly[sub + 1], poly[sub + 2], o);
}

__device__ __forceinline__ void record_from_sub(const SubTri& s, TriRecord& r) {
    r.X0 = s.X[0]; r.Y0 = s.Y[0]; r.X1 = s.X[1]; r.Y1 = s.Y[1];
    r.X2 = s.X[2]; r.Y2 = s.Y[2];
    r.flags = REC_VALID | (s.swapped ? REC_SWAPPED : 0);
    r.z0 = s.z[0]; r.dzdx = s.dzdx; r.dzdy = s.dzdy; r.iw0 = s.iw[0];
    r.iw1 = s.iw[1]; r.iw2 = s.iw[2]; r.pad1 = 0.0f; r.pad2 = 0.0f;
}

// Rebuilds the set-up of an unclipped triangle from its record; every field equals what
// setup_sub computed (integers are recomputed exactly, floats are stored values).
__device__ __forceinline__ bool sub_from_record(const PassConst& c, const TriRecord* rp, SubTri& o) {
    const int4 q0 = __ldg(reinterpret_cast<const int4*>(rp));
    const int4 q1 = __ldg(reinterpret_cast<const int4*>(rp) + 1);
    const float4 q2 = __ldg(reinterpret_cast<const float4*>(rp) + 2);
    const float4 q3 = __ldg(reinterpret_cast<const float4*>(rp) + 3);
    o.X[0] = q0.x; o.Y[0] = q0.y; o.X[1] = q0.z; o.Y[1] = q0.w;
    o.X[2] = q1.x; o.Y[2] = q1.y;
    const int flags = q1.z;
    o.swapped = (flags & REC_SWAPPED) != 0;
    o.z[0] = q2.x; o.dzdx = q2.y; o.dzdy = q2.z;
    o.iw[0] = q2.w; o.iw[1] = q3.x; o.iw[2] = q3.y;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) o.bary[i][k] = 0.0f;
    o.bary[0][0] = 1.0f;
    o.bary[1][o.swapped ? 2 : 1] = 1.0f;
    o.bary[2][o.swapped ? 1 : 2] = 1.0f;
    if (!sub_bbox(c, o)) return false;
    sub_edges(o);
    return true;
}

// Set-up of fan triangle `sub` of triangle t, from its record when it is an unclipped one.
// Completes a sub-triangle whose X, Y, z, iw and bary are set: orientation, pixel range, edge
// functions and depth plane (no culling).
__device__ __forceinline__ bool finish_sub(const PassConst& c, SubTri& o) {
    int64_t a2 = (int64_t)(o.X[1] - o.X[0]) * (o.Y[2] - o.Y[0]) - (int64_t)(o.X[2] - o.X[0]) * (o.Y[1] - o.Y[0]);
    if (a2 == 0) return false;
    o.swapped = 0;
    if (a2 < 0) {
        o.swapped = 1;
        int32_t t;
        float tf;
        t = o.X[1]; o.X[1] = o.X[2]; o.X[2] = t;
        t = o.Y[1]; o.Y[1] = o.Y[2]; o.Y[2] = t;
        tf = o.z[1]; o.z[1] = o.z[2]; o.z[2] = tf;
        tf = o.iw[1]; o.iw[1] = o.iw[2]; o.iw[2] = tf;
#pragma unroll
        for (int k = 0; k < 3; k++) { tf = o.bary[1][k]; o.bary[1][k] = o.bary[2][k]; o.bary[2][k] = tf; }
        a2 = -a2;
    }
    if (!sub_bbox(c, o)) return false;
    sub_edges(o);
    float dX1 = (float)(o.X[1] - o.X[0]), dY1 = (float)(o.Y[1] - o.Y[0]);
    float dX2 = (float)(o.X[2] - o.X[0]), dY2 = (float)(o.Y[2] - o.Y[0]);
    float dz1 = o.z[1] - o.z[0], dz2 = o.z[2] - o.z[0];
    float fa = (float)a2;
    o.dzdx = (dz1 * dY2 - dz2 * dY1) / fa;
    o.dzdy = (dz2 * dX1 - dz1 * dX2) / fa;
    return true;
}

// Projection, 16.8 snap, cull and orientation normalisation of a whole unclipped triangle, without
// a pixel range: the base of the LINE / POINT modes.
__device__ __forceinline__ bool project_oriented(const PassConst& c, const DrawDev& d, const CVert* v, SubTri& o) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float iw = 1.0f / v[i].p[3];
        float xn = v[i].p[0] * iw, yn = v[i].p[1] * iw, zn = v[i].p[2] * iw;
        float fx = fminf(fmaxf((xn * 0.5f + 0.5f) * c.W256, -kSnapLimit), kSnapLimit);
        float fy = fminf(fmaxf((yn * 0.5f + 0.5f) * c.H256, -kSnapLimit), kSnapLimit);
        o.X[i] = __float2int_rn(fx);
        o.Y[i] = __float2int_rn(fy);
        o.z[i] = zn;
        o.iw[i] = iw;
#pragma unroll
        for (int k = 0; k < 3; k++) o.bary[i][k] = v[i].b[k];
    }
    int64_t a2 = (int64_t)(o.X[1] - o.X[0]) * (o.Y[2] - o.Y[0]) - (int64_t)(o.X[2] - o.X[0]) * (o.Y[1] - o.Y[0]);
    if (a2 == 0) return false;
    const bool front = d.front_ccw ? (a2 > 0) : (a2 < 0);
    if (d.cull_mode == 3 || (d.cull_mode == 1 && front) || (d.cull_mode == 2 && !front)) return false;
    o.swapped = 0;
    if (a2 < 0) {
        o.swapped = 1;
        int32_t t;
        float tf;
        t = o.X[1]; o.X[1] = o.X[2]; o.X[2] = t;
        t = o.Y[1]; o.Y[1] = o.Y[2]; o.Y[2] = t;
        tf = o.z[1]; o.z[1] = o.z[2]; o.z[2] = tf;
        tf = o.iw[1]; o.iw[1] = o.iw[2]; o.iw[2] = tf;
#pragma unroll
        for (int k = 0; k < 3; k++) { tf = o.bary[1][k]; o.bary[1][k] = o.bary[2][k]; o.bary[2][k] = tf; }
    }
    return true;
}

// Sub-triangle `sub` of a LINE / POINT mode triangle (t: the oriented projected triangle).
__device__ __forceinline__ bool mode_sub(const PassConst& c, int mode, const SubTri& t, int sub, SubTri& o) {
    const int part = sub >> 1, half = sub & 1;
    int32_t cx[4], cy[4];
    int src[4];
    if (mode == POLY_LINE) {
        const int p = part, q = part == 2 ? 0 : part + 1;
        const int32_t dx = t.X[q] - t.X[p], dy = t.Y[q] - t.Y[p];
        if (dx == 0 && dy == 0) return false;
        const bool xmajor = abs(dx) >= abs(dy);
        const int32_t ox = xmajor ? 0 : 128, oy = xmajor ? 128 : 0;
        cx[0] = t.X[p] - ox; cy[0] = t.Y[p] - oy; src[0] = p;
        cx[1] = t.X[q] - ox; cy[1] = t.Y[q] - oy; src[1] = q;
        cx[2] = t.X[q] + ox; cy[2] = t.Y[q] + oy; src[2] = q;
        cx[3] = t.X[p] + ox; cy[3] = t.Y[p] + oy; src[3] = p;
    } else {
        const int p = part;
        cx[0] = t.X[p] - 128; cy[0] = t.Y[p] - 128;
        cx[1] = t.X[p] + 128; cy[1] = t.Y[p] - 128;
        cx[2] = t.X[p] + 128; cy[2] = t.Y[p] + 128;
        cx[3] = t.X[p] - 128; cy[3] = t.Y[p] + 128;
        src[0] = src[1] = src[2] = src[3] = p;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int k = i == 0 ? 0 : (half == 0 ? i : i + 1);  // halves (0, 1, 2) and (0, 2, 3)
        o.X[i] = cx[k];
        o.Y[i] = cy[k];
        o.z[i] = t.z[src[k]];
        o.iw[i] = t.iw[src[k]];
#pragma unroll
        for (int m = 0; m < 3; m++) o.bary[i][m] = t.bary[src[k]][m];
    }
    return finish_sub(c, o);
}

// The oriented projected triangle of a LINE / POINT mode record (its depth-plane fields hold the
// second and third vertices' depths).
__device__ __forceinline__ void tri_from_mode_record(const TriRecord* rp, SubTri& o) {
    const int4 q0 = __ldg(reinterpret_cast<const int4*>(rp));
    const int4 q1 = __ldg(reinterpret_cast<const int4*>(rp) + 1);
    const float4 q2 = __ldg(reinterpret_cast<const float4*>(rp) + 2);
    const float4 q3 = __ldg(reinterpret_cast<const float4*>(rp) + 3);
    o.X[0] = q0.x; o.Y[0] = q0.y; o.X[1] = q0.z; o.Y[1] = q0.w;
    o.X[2] = q1.x; o.Y[2] = q1.y;
    o.swapped = (q1.z & REC_SWAPPED) != 0;
    o.z[0] = q2.x; o.z[1] = q2.y; o.z[2] = q2.z;
    o.iw[0] = q2.w; o.iw[1] = q3.x; o.iw[2] = q3.y;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) o.bary[i][k] = 0.0f;
    o.bary[0][0] = 1.0f;
    o.bary[1][o.swapped ? 2 : 1] = 1.0f;
    o.bary[2][o.swapped ? 1 : 2] = 1.0f;
}

__device__ __forceinline__ void mode_record_from_tri(const SubTri& t, TriRecord& r) {
    r.X0 = t.X[0]; r.Y0 = t.Y[0]; r.X1 = t.X[1]; r.Y1 = t.Y[1];
    r.X2 = t.X[2]; r.Y2 = t.Y[2];
    r.flags = REC_VALID | (t.swapped ? REC_SWAPPED : 0);
    r.z0 = t.z[0]; r.dzdx = t.z[1]; r.dzdy = t.z[2];
    r.iw0 = t.iw[0]; r.iw1 = t.iw[1]; r.iw2 = t.iw[2]; r.pad1 = 0.0f; r.pad2 = 0.0f;
}

// Set-up of LINE / POINT sub-triangle `sub` of binned triangle g (every such triangle has a
// record).  Out of line: keeps the fill path's frame small.
static __device__ __noinline__ bool setup_mode_entry(const PassConst& c, int mode, const TriRecord* records, int g,
                                                     int sub, SubTri* o) {
    if (!(__ldg(&records[g].flags) & REC_VALID)) return false;
    SubTri tri;
    tri_from_mode_record(records + g, tri);
    return mode_sub(c, mode, tri, sub, *o);
}

__device__ __forceinline__ bool setup_entry_sub(const PassConst& c, const DrawDev& d, const TriRecord* records, int g,
                                                int t, int sub, SubTri& o) {
    if (d.polygon_mode != POLY_FILL) return setup_mode_entry(c, d.polygon_mode, records, g, sub, &o);
    if (records && sub == 0) {
        int flags = __ldg(&records[g].flags);
        if (flags & REC_VALID) return sub_from_record(c, records + g, o);
        if (!(flags & REC_CLIPPED)) return false;
    }
    return setup_triangle_sub(c, d, t, sub, o);
}

__device__ __forceinline__ bool covered(const int32_t* A, const int32_t* B, const int64_t* Cb, int32_t x, int32_t y) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 3; i++) ok &= (Cb[i] + (int64_t)A[i] * x + (int64_t)B[i] * y) >= 0;
    return ok;
}

__device__ __forceinline__ float sample_depth(float z0, float dzdx, float dzdy, int32_t X0, int32_t Y0, int32_t x,
                                              int32_t y) {
    return (z0 + dzdx * (float)(x - X0)) + dzdy * (float)(y - Y0);
}

// Depth test by compare op (0 never, 1 less, 2 equal, 3 less or equal, 4 greater, 5 not equal,
// 6 greater or equal, anything else always): bit 0 passes on less, bit 1 on equal, bit 2 on greater;
// unordered operands (NaN) pass only "not equal" and "always".  Selects, no branch per op.
__device__ __forceinline__ bool depth_cmp(int func, float z, float dd) {
    const bool lt = z < dd, eq = z == dd, gt = z > dd;
    const bool pass = ((func & 1) && lt) || ((func & 2) && eq) || ((func & 4) && gt);
    return (unsigned)func >= 7u || pass || (func == 5 && !(lt || eq || gt));
}

// ------------------------------------------------------------------ log2 (own atanh series)
// ln(m) = 2*atanh(s), s = (m-1)/(m+1) (Abramowitz & Stegun 4.1.27), m in [sqrt(1/2), sqrt(2)).
__device__ __forceinline__ float log2_series(float x) {
    if (!(x > 0.0f)) return -__int_as_float(0x7f800000);
    if (x == __int_as_float(0x7f800000)) return 128.0f;
    int e = 0;
    uint32_t b = __float_as_uint(x);
    if ((b >> 23) == 0) {
        x = x * 8388608.0f;
        b = __float_as_uint(x);
        e = -23;
    }
    e += (int)((b >> 23) & 255u) - 127;
    float m = __uint_as_float((b & 0x7fffffu) | 0x3f800000u);
    if (m > 0x1.6a09e6p+0f) {
        m = m * 0.5f;
        e = e + 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = s2 * 0x1.c71c72p-4f + 0x1.24924ap-3f;
    p = p * s2 + 0x1.99999ap-3f;
    p = p * s2 + 0x1.555556p-2f;
    p = p * s2 + 1.0f;
    float lnm = (2.0f * s) * p;
    return (float)e + lnm * 0x1.715476p+0f;
}

// ------------------------------------------------------------------ textures
// Byte k of t as a float (exact).  Building 2^23 + byte with a byte permute and subtracting 2^23
// measured the same on the textured frames.
template <int K>
__device__ __forceinline__ float byte_to_float(uint32_t t) {
    return (float)((t >> (8 * K)) & 255u);
}

__device__ __forceinline__ void unpack_rgba8(uint32_t t, float c[4]) {
    c[0] = byte_to_float<0>(t) * kInv255;
    c[1] = byte_to_float<1>(t) * kInv255;
    c[2] = byte_to_float<2>(t) * kInv255;
    c[3] = byte_to_float<3>(t) * kInv255;
}

__device__ __forceinline__ float lerpf_(float a, float b, float t) { return a + t * (b - a); }

// Repeat (mode 0) and mirrored-repeat (mode 1) wrapping of coordinates beyond the in-line
// shortcuts: fmodf, then into [0, n) or [0, 2n).  Out of line so that the filter's four address
// computations per probe do not each carry a copy of fmodf.
static __device__ __noinline__ float tex_wrap_far(int mode, float v, float nf) {
    const float m = mode == 0 ? nf : nf + nf;
    v = fmodf(v, m);
    if (v < 0.0f) v = v + m;
    return v;
}

// Texel-space wrapping for the address modes other than repeat (mirrored repeat, clamp to
// border, mirror once, clamp to edge); -1 outside a clamp-to-border texture.  Out of line: the
// filter's four address computations per probe inline only the repeat mode.
static __device__ __noinline__ float tex_address_other(int mode, float v, float nf) {
    switch (mode) {
    case 1: {
        float n2 = nf + nf;
        if (v >= 0.0f && v < n2) {
        } else if (v < 0.0f && v > -n2) {
            v = v + n2;
        } else {
            v = tex_wrap_far(1, v, nf);
        }
        v = fminf(v, n2 - v);
        break;
    }
    case 3:
        if (v < 0.0f || v >= nf) return -1.0f;
        break;
    case 4:
        v = fabsf(v);
        v = fminf(v, nf - 1.0f);
        break;
    default:
        v = fmaxf(v, 0.0f);
        v = fminf(v, nf - 1.0f);
        break;
    }
    if (!(v >= 0.0f)) v = 0.0f;
    return v;
}

// Texel-space wrapping per address mode; returns false outside a clamp-to-border texture.
// fmodf is exact, and so are the shortcuts on the ranges where they are taken (Sterbenz:
// v - n is exact for n <= v <= 2n; for |v| < n fmodf returns v itself).
__device__ __forceinline__ bool tex_address(int mode, float& c, float nf) {
    float v = c;
    if (mode != 0) {
        v = tex_address_other(mode, v, nf);
        if (v < 0.0f) return false;
        c = v;
        return true;
    }
    if (v >= 0.0f && v < nf) {
    } else if (v >= nf && v < nf + nf) {
        v = v - nf;
    } else if (v < 0.0f && v > -nf) {
        v = v + nf;
    } else {
        v = tex_wrap_far(0, v, nf);
    }
    if (!(v >= 0.0f)) v = 0.0f;
    c = v;
    return true;
}

// One mip level, with the constants every fetch from it needs.
struct TexLevel {
    const uint32_t* t;
    int w, h;
    float fw, fh;    // size as float (wrap modulus)
    float fw1, fh1;  // size - 1 as float (texel mapping c = uv * (size - 1))
};

struct TexState {
    int addr_u, addr_v, filter, border_white;
};

__device__ __forceinline__ TexLevel tex_level(const DrawDev& d, int level) {
    TexLevel L;
    L.w = d.lvl_w[level];
    L.h = d.lvl_h[level];
    L.t = d.texels + d.lvl_off[level];
    L.fw = (float)L.w;
    L.fh = (float)L.h;
    L.fw1 = (float)(L.w - 1);
    L.fh1 = (float)(L.h - 1);
    return L;
}

__device__ __forceinline__ TexState tex_state(const DrawDev& d) {
    TexState st;
    st.addr_u = d.sampler.address_u;
    st.addr_v = d.sampler.address_v;
    st.filter = d.sampler.filter;
    st.border_white = d.sampler.border_white;
    return st;
}

// Bilinear (or nearest) fetch from one level; texel mapping c = uv * (size - 1) as in
// ShaderBuiltinCuda.cuh:112-113, neighbours clamped to the last texel (:176-179).
__device__ __forceinline__ void tex_bilinear(const TexLevel& L, const TexState& st, float u, float v, float out[4]) {
    float cx = u * L.fw1;
    float cy = v * L.fh1;
    if (!tex_address(st.addr_u, cx, L.fw) || !tex_address(st.addr_v, cy, L.fh)) {
        float b = st.border_white ? 1.0f : 0.0f;
        out[0] = b; out[1] = b; out[2] = b; out[3] = 1.0f;
        return;
    }
    if (st.filter == 0) {
        int x = min((int)(cx + 0.5f), L.w - 1), y = min((int)(cy + 0.5f), L.h - 1);
        unpack_rgba8(__ldg(L.t + y * L.w + x), out);
        return;
    }
    int x0 = (int)cx, y0 = (int)cy;
    float fx = cx - (float)x0, fy = cy - (float)y0;
    x0 = min(x0, L.w - 1);
    y0 = min(y0, L.h - 1);
    const int x1 = min(x0 + 1, L.w - 1), y1 = min(y0 + 1, L.h - 1);
    const uint32_t t00 = __ldg(L.t + y0 * L.w + x0);
    const uint32_t t01 = __ldg(L.t + y0 * L.w + x1);
    const uint32_t t10 = __ldg(L.t + y1 * L.w + x0);
    const uint32_t t11 = __ldg(L.t + y1 * L.w + x1);
    float c00[4], c01[4], c10[4], c11[4];
    unpack_rgba8(t00, c00);
    unpack_rgba8(t01, c01);
    unpack_rgba8(t10, c10);
    unpack_rgba8(t11, c11);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float top = lerpf_(c00[i], c01[i], fx);
        float bot = lerpf_(c10[i], c11[i], fx);
        out[i] = lerpf_(top, bot, fy);
    }
}

struct LodPick {
    int lo, hi;
    float t;
};

__device__ __forceinline__ LodPick pick_lod(const DrawDev& d, float lam) {
    float maxl = (float)(d.tex_levels - 1);
    if (!(lam > 0.0f)) lam = 0.0f;
    if (lam > maxl) lam = maxl;
    LodPick p;
    p.lo = (int)floorf(lam);
    p.t = lam - (float)p.lo;
    p.hi = min(p.lo + 1, d.tex_levels - 1);
    return p;
}

// Trilinear fetch between two prepared levels (one level when `two` is false).
__device__ __forceinline__ void tex_trilinear2(const TexLevel& L0, const TexLevel& L1, const TexState& st, bool two,
                                               float t, float u, float v, float out[4]) {
    tex_bilinear(L0, st, u, v, out);
    if (!two) return;
    float c1[4];
    tex_bilinear(L1, st, u, v, c1);
#pragma unroll
    for (int i = 0; i < 4; i++) out[i] = lerpf_(out[i], c1[i], t);
}

__device__ __forceinline__ float finite_or_zero(float x) { return isfinite(x) ? x : 0.0f; }

// A texture lookup reduced to its probes: n trilinear fetches between levels lo and hi (weight
// t, `two` when the second level contributes) at (u, v) or, anisotropic, along (du, dv); the
// result is the fetch itself (isotropic) or the probes' in-order sum divided by n.
struct TexProbe {
    float u, v, du, dv, t;
    int lo, hi, n;
    bool two, aniso;
};

// Texture sampling with LOD from screen-space derivatives (ShaderBuiltinCuda.cuh:225-272),
// up to the probe loop.
__device__ __forceinline__ void tex_prepare(const DrawDev& d, float u, float v, float dudx, float dvdx, float dudy,
                                            float dvdy, TexProbe& p) {
    u = finite_or_zero(u); v = finite_or_zero(v);
    dudx = finite_or_zero(dudx); dvdx = finite_or_zero(dvdx);
    dudy = finite_or_zero(dudy); dvdy = finite_or_zero(dvdy);
    p.u = u; p.v = v; p.du = 0.0f; p.dv = 0.0f;
    p.n = 1;
    p.aniso = false;
    if (d.sampler.filter == 0) {  // nearest from level 0
        p.lo = p.hi = 0;
        p.t = 0.0f;
        p.two = false;
        return;
    }
    float tw = (float)d.tex_w, th = (float)d.tex_h;
    float xu = dudx * tw, xv = dvdx * th, yu = dudy * tw, yv = dvdy * th;
    float lx2 = xu * xu + xv * xv;
    float ly2 = yu * yu + yv * yv;
    const bool aniso = d.sampler.max_aniso > 1;
    float lx = fmaxf(lx2, ly2);  // isotropic: lambda = log2(max(|d/dx|^2, |d/dy|^2)) / 2
    if (aniso) {                 // anisotropic: lambda = log2(major axis / probes)
        float px = sqrtf(lx2), py = sqrtf(ly2);
        bool major_x = px >= py;
        float pmax = major_x ? px : py, pmin = major_x ? py : px;
        float amax = (float)d.sampler.max_aniso;
        float ratio = pmin > 0.0f ? pmax / pmin : amax;
        ratio = fminf(ratio, amax);
        int n = (int)ceilf(ratio);
        if (n < 1) n = 1;
        p.n = n;
        p.aniso = true;
        lx = pmax / (float)n;
        p.du = major_x ? dudx : dudy;
        p.dv = major_x ? dvdx : dvdy;
    }
    const float l2 = log2_series(lx);  // one copy of the series for both cases
    const float lam = (aniso ? l2 : 0.5f * l2) + d.sampler.lod_bias;
    const LodPick lp = pick_lod(d, lam);
    p.lo = lp.lo;
    p.hi = lp.hi;
    p.t = lp.t;
    p.two = !(lp.hi == lp.lo || lp.t == 0.0f);
}

// Probe i of a prepared lookup.  ROLLED runs the two levels of the trilinear fetch through one
// copy of the bilinear code (the same operations: level lo, then level hi lerped in), for kernels
// bound by instruction fetch.
template <bool ROLLED = false>
__device__ __forceinline__ void tex_probe(const DrawDev& d, const TexProbe& p, int i, float out[4]) {
    const TexState st = tex_state(d);
    float u = p.u, v = p.v;
    if (p.aniso) {
        const float t = (float)(i + 1) / (float)(p.n + 1) - 0.5f;
        u = u + p.du * t;
        v = v + p.dv * t;
    }
    if constexpr (ROLLED) {
        const int nl = p.two ? 2 : 1;
#pragma unroll 1
        for (int l = 0; l < nl; l++) {
            float b[4];
            tex_bilinear(tex_level(d, l == 0 ? p.lo : p.hi), st, u, v, b);
#pragma unroll
            for (int k = 0; k < 4; k++) out[k] = l == 0 ? b[k] : lerpf_(out[k], b[k], p.t);
        }
    } else {
        tex_trilinear2(tex_level(d, p.lo), tex_level(d, p.hi), st, p.two, p.t, u, v, out);
    }
}

// The lookup's result from its probes' in-order sum (isotropic: the single fetch).
__device__ __forceinline__ void tex_finish(const TexProbe& p, const float acc[4], float out[4]) {
    const float fn = (float)p.n;
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = p.aniso ? acc[k] / fn : acc[k];
}

__device__ __forceinline__ void tex_sample(const DrawDev& d, float u, float v, float dudx, float dvdx, float dudy,
                                           float dvdy, float out[4]) {
    TexProbe p;
    tex_prepare(d, u, v, dudx, dvdx, dudy, dvdy, p);
    if (!p.aniso) {
        tex_probe(d, p, 0, out);
        return;
    }
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int i = 0; i < p.n; i++) {
        float cc[4];
        tex_probe(d, p, i, cc);
#pragma unroll
        for (int k = 0; k < 4; k++) acc[k] = acc[k] + cc[k];
    }
    tex_finish(p, acc, out);
}

// ------------------------------------------------------------------ interpolation + shading
// What interpolation needs of a (sub-)triangle.
struct ShadeGeom {
    int32_t A[3], B[3];
    int64_t C[3];
    float iw[3];
    float bary[3][3];
};

__device__ __forceinline__ void shade_geom_from(const SubTri& s, ShadeGeom& g) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        g.A[i] = s.A[i];
        g.B[i] = s.B[i];
        g.C[i] = s.C[i];
        g.iw[i] = s.iw[i];
#pragma unroll
        for (int k = 0; k < 3; k++) g.bary[i][k] = s.bary[i][k];
    }
}

// Perspective-correct interpolation of the draw's attribute at fixed-point position (x, y);
// va/vb/vc hold the attribute of the triangle's three vertices (unused components zero).
__device__ __forceinline__ void interp_attr(const ShadeGeom& s, int attr_count, const float* va, const float* vb,
                                            const float* vc, int32_t x, int32_t y, float out[4]) {
    float p[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float e = (float)(s.C[i] + (int64_t)s.A[i] * x + (int64_t)s.B[i] * y);
        p[i] = e * s.iw[i];
    }
    float sum = (p[0] + p[1]) + p[2];
    float r = 1.0f / sum;
    float b0 = p[0] * r, b1 = p[1] * r, b2 = p[2] * r;
    float W[3];
#pragma unroll
    for (int k = 0; k < 3; k++) W[k] = (b0 * s.bary[0][k] + b1 * s.bary[1][k]) + b2 * s.bary[2][k];
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = k < attr_count ? (W[0] * va[k] + W[1] * vb[k]) + W[2] * vc[k] : 0.0f;
}

__device__ __forceinline__ void load_attr(const float* p, int attr_count, float v[4]) {
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = k < attr_count ? __ldg(p + k) : 0.0f;
}

// Fragment colour of pixel (px, py) for triangle t / fan index `sub` of draw d.  Texture
// LOD uses fine 2x2-quad derivatives: the attribute at the quad's right column minus the
// left column (same row) and bottom row minus top row (same column), each evaluated for this
// primitive exactly as a helper invocation would evaluate it.
// Attributes of the three vertices of triangle t (original vertex order).
__device__ __forceinline__ void fetch_attrs(const DrawDev& d, int t, float a0[4], float a1[4], float a2[4]) {
    load_attr(d.vertices + (size_t)__ldg(d.indices + 3 * (size_t)t + 0) * d.stride + d.attr_offset, d.attr_count, a0);
    load_attr(d.vertices + (size_t)__ldg(d.indices + 3 * (size_t)t + 1) * d.stride + d.attr_offset, d.attr_count, a1);
    load_attr(d.vertices + (size_t)__ldg(d.indices + 3 * (size_t)t + 2) * d.stride + d.attr_offset, d.attr_count, a2);
}

// Vertex attributes of an unclipped triangle stored by the counting binner next to its set-up
// record, so shading does not chase indices and vertex rows (48 bytes: 3 vertices x 4 floats).
struct __align__(16) TriAttr {
    float4 a[3];
};

__device__ __forceinline__ void shade_fragment_attrs(const PassConst& c, const DrawDev& d, const ShadeGeom& s, int t,
                                                     int sub, int px, int py, const float a0[4], const float a1[4],
                                                     const float a2[4], float col[4]);

__device__ __forceinline__ void shade_fragment(const PassConst& c, const DrawDev& d, const ShadeGeom& s, int t, int sub,
                                               int px, int py, float col[4]) {
    float a0[4], a1[4], a2[4];
    if (d.shading == SHADE_PRIMID) {
        a0[0] = a0[1] = a0[2] = a0[3] = 0.0f;
        a1[0] = a1[1] = a1[2] = a1[3] = 0.0f;
        a2[0] = a2[1] = a2[2] = a2[3] = 0.0f;
    } else {
        fetch_attrs(d, t, a0, a1, a2);
    }
    shade_fragment_attrs(c, d, s, t, sub, px, py, a0, a1, a2, col);
}

// Fragment colour from the triangle's vertex attributes.
__device__ __forceinline__ void shade_fragment_attrs(const PassConst& c, const DrawDev& d, const ShadeGeom& s, int t,
                                                     int sub, int px, int py, const float a0[4], const float a1[4],
                                                     const float a2[4], float col[4]) {
    if (d.shading == SHADE_PRIMID) {
        col[0] = (float)(d.prim_base + t); col[1] = (float)sub; col[2] = 0.0f; col[3] = 1.0f;
        return;
    }
    int32_t qx = px * 256 + kShadeOffset, qy = py * 256 + kShadeOffset;
    float a[4];
    interp_attr(s, d.attr_count, a0, a1, a2, qx, qy, a);
    if (d.shading == SHADE_TEXTURED) {
        float ah[4], av[4];  // horizontal and vertical quad partners
        interp_attr(s, d.attr_count, a0, a1, a2, (px ^ 1) * 256 + kShadeOffset, qy, ah);
        interp_attr(s, d.attr_count, a0, a1, a2, qx, (py ^ 1) * 256 + kShadeOffset, av);
        float dudx = (px & 1) ? a[0] - ah[0] : ah[0] - a[0];
        float dvdx = (px & 1) ? a[1] - ah[1] : ah[1] - a[1];
        float dudy = (py & 1) ? a[0] - av[0] : av[0] - a[0];
        float dvdy = (py & 1) ? a[1] - av[1] : av[1] - a[1];
        tex_sample(d, a[0], a[1], dudx, dvdx, dudy, dvdy, col);
        return;
    }
    col[0] = a[0]; col[1] = a[1]; col[2] = a[2];
    col[3] = d.attr_count >= 4 ? a[3] : 1.0f;
}

// As shade_fragment_attrs, with a textured fragment's lookup returned unevaluated in `tp` (the
// result is then true and `col` is not set).
__device__ __forceinline__ bool shade_prepare_attrs(const PassConst& c, const DrawDev& d, const ShadeGeom& s, int t,
                                                    int sub, int px, int py, const float a0[4], const float a1[4],
                                                    const float a2[4], float col[4], TexProbe& tp) {
    if (d.shading == SHADE_PRIMID) {
        col[0] = (float)(d.prim_base + t); col[1] = (float)sub; col[2] = 0.0f; col[3] = 1.0f;
        return false;
    }
    int32_t qx = px * 256 + kShadeOffset, qy = py * 256 + kShadeOffset;
    float a[4];
    interp_attr(s, d.attr_count, a0, a1, a2, qx, qy, a);
    if (d.shading == SHADE_TEXTURED) {
        float ah[4], av[4];  // horizontal and vertical quad partners
        interp_attr(s, d.attr_count, a0, a1, a2, (px ^ 1) * 256 + kShadeOffset, qy, ah);
        interp_attr(s, d.attr_count, a0, a1, a2, qx, (py ^ 1) * 256 + kShadeOffset, av);
        float dudx = (px & 1) ? a[0] - ah[0] : ah[0] - a[0];
        float dvdx = (px & 1) ? a[1] - ah[1] : ah[1] - a[1];
        float dudy = (py & 1) ? a[0] - av[0] : av[0] - a[0];
        float dvdy = (py & 1) ? a[1] - av[1] : av[1] - a[1];
        tex_prepare(d, a[0], a[1], dudx, dvdx, dudy, dvdy, tp);
        return true;
    }
    col[0] = a[0]; col[1] = a[1]; col[2] = a[2];
    col[3] = d.attr_count >= 4 ? a[3] : 1.0f;
    return false;
}

// Blend factor f of channel ch (0 zero, 1 one, 2 / 3 source colour, 4 / 5 destination colour, 6 / 7
// source alpha, 8 / 9 destination alpha, the odd ones as one minus it; anything else zero), by
// selects rather than a branch per factor.
__device__ __forceinline__ float blend_factor(int f, int ch, const float* src, const float* dst) {
    const float x = f <= 3 ? src[ch] : f <= 5 ? dst[ch] : f <= 7 ? src[3] : dst[3];
    const float v = (f & 1) ? 1.0f - x : x;
    return (unsigned)f > 9u || f == 0 ? 0.0f : f == 1 ? 1.0f : v;
}

// Whether any of the draw's four blend factors reads the destination colour (codes 4, 5, 8, 9).
__device__ __forceinline__ bool blend_reads_dst(const DrawDev& d) {
    auto reads = [](int f) { return f == 4 || f == 5 || f == 8 || f == 9; };
    return reads(d.blend_src_color) || reads(d.blend_dst_color) || reads(d.blend_src_alpha) || reads(d.blend_dst_alpha);
}

__device__ __forceinline__ void blend_into(const DrawDev& d, const float* src, float* dst) {
    float out[4];
#pragma unroll
    for (int ch = 0; ch < 4; ch++) {
        int fs = ch < 3 ? d.blend_src_color : d.blend_src_alpha;
        int fd = ch < 3 ? d.blend_dst_color : d.blend_dst_alpha;
        out[ch] = dst[ch] * blend_factor(fd, ch, src, dst) + src[ch] * blend_factor(fs, ch, src, dst);
    }
#pragma unroll
    for (int ch = 0; ch < 4; ch++) dst[ch] = out[ch];
}

}  // namespace ifr
