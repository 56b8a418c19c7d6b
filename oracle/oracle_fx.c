/* Test infrastructure only -- the CPU oracle (checker) for the GB300 rasterizer.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this code.
 *
 * A plain-C restatement of the reference soft renderer's triangle pipeline
 * (Aeroraven/Ifrit-v2, projects/softgraphics), stage by stage, in API order:
 *
 *   vertex transform      TileRasterWorker.cpp:432-476 (VertexShader::execute per vertex)
 *   homogeneous clipping  TileRasterWorker.cpp:136-277, TileRasterCoreInvocationCuda.cu:1342-1400
 *   culling               TileRasterWorker.cpp:301-313, .cu:271-276, .cu:1433-1475
 *   triangle setup        TileRasterWorker.cpp:503-727, .cu:1549-1644
 *   coverage (MSAA)       TileRasterWorker.cpp:787-1223, .cu:891-982 (sample table .cu:208-222)
 *   depth test + write    TileRasterWorker.cpp:2244-2386 (ordered path :1517-1580)
 *   interpolation, ddx/y  TileRasterWorker.cpp:1932-2121, .cu:2144-2317, ShaderBuiltinCuda.cuh:36-94
 *   texture sampling      ShaderBuiltinCuda.cuh:96-272
 *   blend                 TileRasterWorker.cpp:2346-2373 (factor table TileRasterRenderer.cpp:212-333)
 *   MSAA resolve          .cu:2319-2361
 *
 * Deliberate differences from the reference (each applied identically by the GPU path):
 *   - coverage is evaluated on 16.8 fixed-point vertex positions with 64-bit edge
 *     functions and an explicit top-left fill rule (the reference uses float edge
 *     functions with an epsilon bias and no fill rule);
 *   - clipping is against w >= 1e-5, 0 <= z <= w and a guard band (the reference clips
 *     only against w);
 *   - texture LOD uses ddy for the y footprint (the reference reads dx.y there,
 *     ShaderBuiltinCuda.cuh:237), anisotropic taps are centred, and mip levels are clamped;
 *   - blend factors follow their names (the reference swaps SRC_ALPHA/ONE_MINUS_SRC_ALPHA
 *     and DST_ALPHA/ONE_MINUS_DST_ALPHA, TileRasterRenderer.cpp:215-234);
 *   - MSAA resolve averages colour only; depth stays per sample.
 * Every floating-point expression is written in the exact evaluation order the device
 * code uses and the file is compiled with -ffp-contract=off, so results are bit-identical.
 */
#define _POSIX_C_SOURCE 200809L /* pthread barriers under -std=c11 */
#include "oracle_fx.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define OFX_WEPS 1e-5f
#define OFX_MAX_POLY 10
#define OFX_MAX_SUB 8
#define OFX_GUARD_PX 8192
#define OFX_SNAP_LIMIT 8000000.0f

static const float INV255 = 0x1.010102p-8f;

/* ---------------------------------------------------------------- helpers */
static inline float fmin_(float a, float b) { return fminf(a, b); }
static inline float fmax_(float a, float b) { return fmaxf(a, b); }
static inline int imin_(int a, int b) { return a < b ? a : b; }
static inline int imax_(int a, int b) { return a > b ? a : b; }
static inline int64_t floordiv256(int64_t a) { return a >= 0 ? a / 256 : -((-a + 255) / 256); }
static inline int64_t ceildiv256(int64_t a) { return -floordiv256(-a); }
static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* Sample pattern tables (in 1/256 pixel), the standard patterns the reference lists in
 * TileRasterCoreInvocationCuda.cu:208-222, scaled by 256. */
static const int SP1[2] = {128, 128};
static const int SP2[4] = {192, 192, 64, 64};
static const int SP4[8] = {96, 32, 224, 96, 32, 160, 160, 224};
static const int SP8[16] = {144, 80, 112, 176, 208, 144, 80, 48, 48, 208, 16, 112, 176, 240, 240, 16};
static const int SP16[32] = {144, 144, 112, 80, 80, 160, 192, 112, 48, 96, 160, 208, 208, 176, 176, 48,
                             96, 224, 128, 16, 64, 32, 32, 192, 0, 128, 240, 64, 224, 240, 16, 0};

void ofx_sample_positions(int samples, int compat, int* xs, int* ys) {
    const int* t = samples == 1 ? SP1 : samples == 2 ? SP2 : samples == 4 ? SP4 : samples == 8 ? SP8 : SP16;
    for (int k = 0; k < samples; k++) {
        xs[k] = t[2 * k];
        ys[k] = t[2 * k + 1];
    }
    if (compat && samples == 1) { xs[0] = 0; ys[0] = 0; }
}

/* ---------------------------------------------------------------- log2
 * Own log2 from the atanh series ln(m) = 2*atanh(s), s = (m-1)/(m+1)
 * (Abramowitz & Stegun 4.1.27) after splitting x = m * 2^e with m in [sqrt(1/2), sqrt(2)).
 * Only +, *, / and bit operations are used, so CPU and GPU agree to the bit. */
float ofx_log2(float x) {
    if (!(x > 0.0f)) return -INFINITY;
    if (x == INFINITY) return 128.0f;
    int e = 0;
    uint32_t b = f2u(x);
    if ((b >> 23) == 0) { /* subnormal: scale by 2^23 exactly */
        x = x * 8388608.0f;
        b = f2u(x);
        e = -23;
    }
    e += (int)((b >> 23) & 255u) - 127;
    float m = u2f((b & 0x7fffffu) | 0x3f800000u);
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

/* ---------------------------------------------------------------- half */
uint16_t ofx_f32_to_f16(float f) {
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); /* rounds to >= 65520 -> inf */
    if (ax < 0x38800000u) {                                   /* subnormal half or zero */
        if (ax < 0x33000000u) return (uint16_t)sign;         /* < 2^-25 rounds to 0 */
        uint32_t e = ax >> 23;
        uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        uint32_t shift = 126u - e; /* value = m * 2^(e-150); half subnormal unit 2^-24 */
        uint32_t q = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1u);
        uint32_t half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (q & 1u))) q++;
        return (uint16_t)(sign | q);
    }
    uint32_t e = (ax >> 23) - 112u;
    uint32_t m = ax & 0x7fffffu;
    uint32_t q = (e << 10) | (m >> 13);
    uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) q++;
    return (uint16_t)(sign | q);
}

static float f16_to_f32(uint16_t h) {
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 31u, m = h & 1023u;
    if (e == 0) {
        if (m == 0) return u2f(sign);
        float v = (float)m * 0x1p-24f;
        return sign ? -v : v;
    }
    if (e == 31) return u2f(sign | 0x7f800000u | (m << 13));
    return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

/* ---------------------------------------------------------------- textures */
int ofx_mip_chain_texels(int width, int height, int* levels) {
    int total = 0, w = width, h = height, l = 0;
    for (;;) {
        total += w * h;
        l++;
        if (w == 1 && h == 1) break;
        w = (w + 1) >> 1;
        h = (h + 1) >> 1;
    }
    if (levels) *levels = l;
    return total;
}

/* 2x2 box filter with edge clamp, rounded to nearest: each level halves the previous one
 * with the (w+1)>>1 size rule of ShaderBuiltinCuda.cuh:97-105. */
int ofx_build_mips(uint32_t* texels, int width, int height) {
    int w = width, h = height, off = 0, l = 1;
    while (!(w == 1 && h == 1)) {
        int nw = (w + 1) >> 1, nh = (h + 1) >> 1;
        const uint32_t* src = texels + off;
        uint32_t* dst = texels + off + w * h;
        for (int y = 0; y < nh; y++) {
            int y0 = 2 * y, y1 = imin_(2 * y + 1, h - 1);
            for (int x = 0; x < nw; x++) {
                int x0 = 2 * x, x1 = imin_(2 * x + 1, w - 1);
                uint32_t a = src[y0 * w + x0], b = src[y0 * w + x1], c = src[y1 * w + x0], d = src[y1 * w + x1];
                uint32_t out = 0;
                for (int ch = 0; ch < 4; ch++) {
                    uint32_t s = ((a >> (8 * ch)) & 255u) + ((b >> (8 * ch)) & 255u) + ((c >> (8 * ch)) & 255u) +
                                 ((d >> (8 * ch)) & 255u) + 2u;
                    out |= (s >> 2) << (8 * ch);
                }
                dst[y * nw + x] = out;
            }
        }
        off += w * h;
        w = nw;
        h = nh;
        l++;
    }
    return l;
}

static inline void unpack_rgba8(uint32_t t, float c[4]) {
    c[0] = (float)(t & 255u) * INV255;
    c[1] = (float)((t >> 8) & 255u) * INV255;
    c[2] = (float)((t >> 16) & 255u) * INV255;
    c[3] = (float)(t >> 24) * INV255;
}

static inline float lerpf_(float a, float b, float t) { return a + t * (b - a); }

/* Wraps a texel-space coordinate per address mode; returns 0 when the sample is outside a
 * clamp-to-border texture.  After this call 0 <= *c. */
static int address(int mode, float* c, int n) {
    float nf = (float)n;
    float v = *c;
    switch (mode) {
    case 0: /* repeat */
        v = fmodf(v, nf);
        if (v < 0.0f) v = v + nf;
        break;
    case 1: { /* mirrored repeat */
        float n2 = nf + nf;
        v = fmodf(v, n2);
        if (v < 0.0f) v = v + n2;
        v = fmin_(v, n2 - v);
        break;
    }
    case 3: /* clamp to border */
        if (v < 0.0f || v >= nf) return 0;
        break;
    case 4: /* mirror clamp to edge */
        v = fabsf(v);
        v = fmin_(v, nf - 1.0f);
        break;
    default: /* clamp to edge */
        v = fmax_(v, 0.0f);
        v = fmin_(v, nf - 1.0f);
        break;
    }
    if (!(v >= 0.0f)) v = 0.0f;
    *c = v;
    return 1;
}

static void level_info(const ofx_texture* tex, int level, int* w, int* h, int* off) {
    int ww = tex->width, hh = tex->height, o = 0;
    for (int i = 0; i < level; i++) {
        o += ww * hh;
        ww = (ww + 1) >> 1;
        hh = (hh + 1) >> 1;
    }
    *w = ww;
    *h = hh;
    *off = o;
}

/* Bilinear (or nearest) fetch from one mip level; texel mapping c = uv * (size - 1) as in
 * ShaderBuiltinCuda.cuh:112-113, neighbours clamped to the last texel (:176-179). */
static void sample_level(const ofx_texture* tex, const ofx_sampler* s, int level, float u, float v, float out[4]) {
    int w, h, off;
    level_info(tex, level, &w, &h, &off);
    float cx = u * (float)(w - 1);
    float cy = v * (float)(h - 1);
    if (!address(s->address_u, &cx, w) || !address(s->address_v, &cy, h)) {
        float b = s->border_white ? 1.0f : 0.0f;
        out[0] = b; out[1] = b; out[2] = b; out[3] = 1.0f;
        return;
    }
    const uint32_t* t = tex->texels + off;
    if (s->filter == 0) {
        int x = imin_((int)(cx + 0.5f), w - 1), y = imin_((int)(cy + 0.5f), h - 1);
        unpack_rgba8(t[y * w + x], out);
        return;
    }
    int x0 = (int)cx, y0 = (int)cy;
    float fx = cx - (float)x0, fy = cy - (float)y0;
    x0 = imin_(x0, w - 1);
    y0 = imin_(y0, h - 1);
    int x1 = imin_(x0 + 1, w - 1), y1 = imin_(y0 + 1, h - 1);
    float c00[4], c01[4], c10[4], c11[4];
    unpack_rgba8(t[y0 * w + x0], c00);
    unpack_rgba8(t[y0 * w + x1], c01);
    unpack_rgba8(t[y1 * w + x0], c10);
    unpack_rgba8(t[y1 * w + x1], c11);
    for (int i = 0; i < 4; i++) {
        float top = lerpf_(c00[i], c01[i], fx);
        float bot = lerpf_(c10[i], c11[i], fx);
        out[i] = lerpf_(top, bot, fy);
    }
}

static void sample_trilinear(const ofx_texture* tex, const ofx_sampler* s, float u, float v, float lam, float out[4]) {
    float maxl = (float)(tex->levels - 1);
    if (!(lam > 0.0f)) lam = 0.0f;
    if (lam > maxl) lam = maxl;
    int lo = (int)floorf(lam);
    float t = lam - (float)lo;
    int hi = imin_(lo + 1, tex->levels - 1);
    sample_level(tex, s, lo, u, v, out);
    if (hi == lo || t == 0.0f) return;
    float c1[4];
    sample_level(tex, s, hi, u, v, c1);
    for (int i = 0; i < 4; i++) out[i] = lerpf_(out[i], c1[i], t);
}

static inline float finite_or_zero(float x) { return isfinite(x) ? x : 0.0f; }

/* ---------------------------------------------------------------- reference-compatible sampling
 * The reference's sampler as written (ShaderBuiltinCuda.cuh:106-272), with the quirks that the
 * default path above fixes.  It exists only to pin this restatement against the reference's own
 * sampler compiled on the host; the GPU path implements the default path.  Differences from the
 * default path, each reproduced here:
 *   - address modes (:117-157): repeat / mirrored repeat add one period to a negative coordinate
 *     before fmodf; mirror-clamp-to-edge maps c >= size-1 to 0 and c <= 0 to size-1;
 *   - nearest filtering rounds half away from zero and wraps modulo the level size (:159-165),
 *     and is still blended between two levels by the LOD fraction (:214-218);
 *   - the level pair (floor(lod), floor(lod)+1) is not clamped to the chain (:214-217); callers
 *     keep the LOD inside the chain or pad it (texels past the chain read as the last level);
 *   - isotropic LOD: the y footprint uses (du/dy, dv/dx) (the `dx.y` typo, :237), and
 *     lod = max(0, 0.5 log2(max) + bias) (:240);
 *   - anisotropic (:244-272): the footprint axes are the gradients of u and of v,
 *     px = |(du/dx, du/dy)| * width and py = |(dv/dx, dv/dy)| * height (the parameter names there
 *     swap du/dy and dv/dx), the probe direction is (du/dx, du/dy) if px > py else (dv/dx, dv/dy),
 *     n = clamp(ceil(pmax/pmin), 1, maxAniso), lambda = max(0, log2(pmax/n)) before the bias,
 *     and probe i (0-based) sits at i/(n+1) - 1/2 (not centred);
 *   - log2 is the C library's log2f (the reference calls log2). */
static inline float compat_clamp(float x, float mi, float ma) { return (x >= ma) ? ma : ((x <= mi) ? mi : x); }
static inline float compat_mirrorclamp(float x, float mi, float ma) { return (x >= ma) ? mi : ((x <= mi) ? ma : x); }

static int compat_address(int mode, float* c, int n) {
    float v = *c;
    switch (mode) {
    case 0:
        if (v < 0.0f) v = v + (float)n;
        v = fmodf(v, (float)n);
        break;
    case 1:
        if (v < 0.0f) v = v + (float)(2 * n);
        v = fmodf(v, (float)(2 * n));
        v = fmin_(v, (float)(2 * n) - v);
        break;
    case 2: v = compat_clamp(v, 0.0f, (float)n - 1.0f); break;
    case 3:
        if (v >= (float)n || v < 0.0f) return 0;
        break;
    case 4: v = compat_mirrorclamp(v, 0.0f, (float)n - 1.0f); break;
    default: break;
    }
    *c = v;
    return 1;
}

/* One level lookup (textureImplLegacy, :106-182); level sizes continue as 1x1 past the chain. */
static void compat_level(const ofx_texture* tex, const ofx_sampler* s, int level, float u, float v, float out[4]) {
    int w = tex->width, h = tex->height, off = 0;
    for (int i = 0; i < level; i++) {
        off += w * h;
        w = (w + 1) >> 1;
        h = (h + 1) >> 1;
    }
    float cx = u * (float)(w - 1), cy = v * (float)(h - 1);
    if (!compat_address(s->address_u, &cx, w) || !compat_address(s->address_v, &cy, h)) {
        float b = s->border_white ? 1.0f : 0.0f;
        out[0] = b; out[1] = b; out[2] = b; out[3] = 1.0f;
        return;
    }
    const uint32_t* t = tex->texels;
    int last = ofx_mip_chain_texels(tex->width, tex->height, NULL) - 1;
    /* indices outside the chain are out-of-range reads in the reference (a coordinate below
     * one period before 0 in repeat modes, levels past the chain): clamped here */
#define COMPAT_TEXEL(i, dst) unpack_rgba8(t[imax_(0, imin_((i), last))], dst)
    if (s->filter == 0) {
        int x = (int)roundf(cx) % w, y = (int)roundf(cy) % h;
        COMPAT_TEXEL(off + y * w + x, out);
        return;
    }
    int x0 = (int)cx, y0 = (int)cy;
    float fx = cx - (float)x0, fy = cy - (float)y0;
    int x1 = imin_(x0 + 1, w - 1), y1 = imin_(y0 + 1, h - 1);
    float c00[4], c01[4], c10[4], c11[4];
    COMPAT_TEXEL(off + y0 * w + x0, c00);
    COMPAT_TEXEL(off + y0 * w + x1, c01);
    COMPAT_TEXEL(off + y1 * w + x0, c10);
    COMPAT_TEXEL(off + y1 * w + x1, c11);
#undef COMPAT_TEXEL
    for (int i = 0; i < 4; i++) {
        float top = lerpf_(c00[i], c01[i], fx);
        float bot = lerpf_(c10[i], c11[i], fx);
        out[i] = lerpf_(top, bot, fy);
    }
}

/* textureImplLod (:210-218): two levels blended by the LOD fraction, unclamped. */
static void compat_lod(const ofx_texture* tex, const ofx_sampler* s, float u, float v, float lod, float out[4]) {
    int lo = (int)floorf(lod);
    float t = lod - (float)lo;
    float c1[4];
    compat_level(tex, s, lo, u, v, out);
    compat_level(tex, s, lo + 1, u, v, c1);
    for (int i = 0; i < 4; i++) out[i] = lerpf_(out[i], c1[i], t);
}

static void sample_compat(const ofx_texture* tex, const ofx_sampler* s, float u, float v, float dudx, float dvdx,
                          float dudy, float dvdy, float out[4]) {
    const float W = (float)tex->width, H = (float)tex->height;
    if (s->max_aniso <= 1) { /* textureImplAdaptiveLod (:233-243) */
        float xx = dudx * W, xy = dvdx * H, yx = dudy * W, yy = dvdx * H;
        float dx2 = xx * xx + xy * xy, dy2 = yx * yx + yy * yy;
        float d = fmax_(dx2, dy2);
        float lod = fmax_(0.0f, 0.5f * log2f(d) + s->lod_bias);
        compat_lod(tex, s, u, v, lod, out);
        return;
    }
    /* textureImplAnisotropicFilter (:244-272) */
    float px = sqrtf(dudx * dudx + dudy * dudy) * W;
    float py = sqrtf(dvdx * dvdx + dvdy * dvdy) * H;
    float pmax = fmax_(px, py), pmin = fmin_(px, py);
    double r = (double)ceilf(pmax / pmin) + 1e-3;
    double lim = (double)s->max_aniso + 1e-3;
    double m = fmin(r, lim);
    int n = (int)fmax(1.0, m);
    float lambda = fmax_(0.0f, log2f(pmax / (float)n));
    float ddu = px > py ? dudx : dvdx;
    float ddv = px > py ? dudy : dvdy;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int i = 0; i < n; i++) {
        float t = (1.0f * (float)i) / (float)(n + 1) - 0.5f;
        float c[4];
        compat_lod(tex, s, u + ddu * t, v + ddv * t, lambda + s->lod_bias, c);
        for (int k = 0; k < 4; k++) acc[k] = acc[k] + c[k];
    }
    for (int k = 0; k < 4; k++) out[k] = acc[k] / (float)n;
}

/* Texture sampling with LOD from screen-space derivatives (ShaderBuiltinCuda.cuh:225-272). */
void ofx_sample_texture(const ofx_texture* tex, const ofx_sampler* s, float u, float v,
                        float dudx, float dvdx, float dudy, float dvdy, float out[4]) {
    if (s->compat) {
        sample_compat(tex, s, u, v, dudx, dvdx, dudy, dvdy, out);
        return;
    }
    u = finite_or_zero(u); v = finite_or_zero(v);
    dudx = finite_or_zero(dudx); dvdx = finite_or_zero(dvdx);
    dudy = finite_or_zero(dudy); dvdy = finite_or_zero(dvdy);
    if (s->filter == 0) {
        sample_level(tex, s, 0, u, v, out);
        return;
    }
    float tw = (float)tex->width, th = (float)tex->height;
    float xu = dudx * tw, xv = dvdx * th, yu = dudy * tw, yv = dvdy * th;
    float lx2 = xu * xu + xv * xv;
    float ly2 = yu * yu + yv * yv;
    if (s->max_aniso <= 1) {
        float lam = 0.5f * ofx_log2(fmax_(lx2, ly2)) + s->lod_bias;
        sample_trilinear(tex, s, u, v, lam, out);
        return;
    }
    float px = sqrtf(lx2), py = sqrtf(ly2);
    int major_x = px >= py;
    float pmax = major_x ? px : py, pmin = major_x ? py : px;
    float amax = (float)s->max_aniso;
    float ratio = pmin > 0.0f ? pmax / pmin : amax;
    ratio = fmin_(ratio, amax);
    int n = (int)ceilf(ratio);
    if (n < 1) n = 1;
    float lam = ofx_log2(pmax / (float)n) + s->lod_bias;
    float du = major_x ? dudx : dudy, dv = major_x ? dvdx : dvdy;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float inv = (float)(n + 1);
    for (int i = 0; i < n; i++) {
        float t = (float)(i + 1) / inv - 0.5f;
        float c[4];
        sample_trilinear(tex, s, u + du * t, v + dv * t, lam, c);
        for (int k = 0; k < 4; k++) acc[k] = acc[k] + c[k];
    }
    float fn = (float)n;
    for (int k = 0; k < 4; k++) out[k] = acc[k] / fn;
}

/* ---------------------------------------------------------------- geometry */
typedef struct {
    float p[4];
    float b[3];
} cvert;

typedef struct {
    int32_t X[3], Y[3];
    float z[3], iw[3];
    float bary[3][3]; /* original-triangle barycentric of each sub-vertex */
    int32_t A[3], B[3];
    int64_t C[3];     /* unbiased: E_i(v_i) = A2 */
    int64_t Cb[3];    /* fill-rule biased: covered iff Cb + A x + B y >= 0 for all edges */
    float dzdx, dzdy;
    int px0, px1, py0, py1;
    int prim, sub;
} ofx_sub;

typedef struct {
    int W, H, S;
    int r0, r1;  /* rows held by the target buffers: [r0, r1) of the H-row frame */
    int sx[16], sy[16];
    int smin_x, smax_x, smin_y, smax_y;
    int shade_x, shade_y;
    float W256, H256, gx, gy;
} pass_ctx;

static void xform(const float* m, const float* v, float out[4]) {
    float x = v[0], y = v[1], z = v[2];
    for (int r = 0; r < 4; r++) out[r] = m[4 * r + 0] * x + m[4 * r + 1] * y + m[4 * r + 2] * z + m[4 * r + 3];
}

static inline float plane_dist(const pass_ctx* c, int plane, const float* p) {
    switch (plane) {
    case 0: return p[3] - OFX_WEPS;
    case 1: return p[2];
    case 2: return p[3] - p[2];
    case 3: return c->gx * p[3] - p[0];
    case 4: return c->gx * p[3] + p[0];
    case 5: return c->gy * p[3] - p[1];
    default: return c->gy * p[3] + p[1];
    }
}

/* Sutherland-Hodgman against the 7 planes in fixed order; returns polygon size (0 = gone). */
static int clip_polygon(const pass_ctx* c, cvert* poly) {
    int n = 3;
    cvert tmp[OFX_MAX_POLY];
    for (int pl = 0; pl < 7; pl++) {
        int all_in = 1, all_out = 1;
        for (int i = 0; i < n; i++) {
            float d = plane_dist(c, pl, poly[i].p);
            if (d >= 0.0f) all_out = 0; else all_in = 0;
        }
        if (all_out) return 0;
        if (all_in) continue;
        int m = 0;
        for (int i = 0; i < n; i++) {
            const cvert* a = &poly[i];
            const cvert* b = &poly[(i + 1) % n];
            float da = plane_dist(c, pl, a->p), db = plane_dist(c, pl, b->p);
            if (da >= 0.0f) tmp[m++] = *a;
            if ((da >= 0.0f) != (db >= 0.0f)) {
                float t = da / (da - db);
                cvert q;
                for (int k = 0; k < 4; k++) q.p[k] = a->p[k] + t * (b->p[k] - a->p[k]);
                for (int k = 0; k < 3; k++) q.b[k] = a->b[k] + t * (b->b[k] - a->b[k]);
                tmp[m++] = q;
            }
        }
        n = m;
        if (n < 3) return 0;
        memcpy(poly, tmp, sizeof(cvert) * n);
    }
    return n;
}

/* Projects, snaps, culls and sets up one fan triangle; returns 1 if it may cover samples. */
static int setup_sub(const pass_ctx* c, const ofx_draw* d, const cvert* v0, const cvert* v1, const cvert* v2,
                     int prim, int sub, ofx_sub* o) {
    const cvert* v[3] = {v0, v1, v2};
    for (int i = 0; i < 3; i++) {
        float iw = 1.0f / v[i]->p[3];
        float xn = v[i]->p[0] * iw, yn = v[i]->p[1] * iw, zn = v[i]->p[2] * iw;
        float fx = (xn * 0.5f + 0.5f) * c->W256;
        float fy = (yn * 0.5f + 0.5f) * c->H256;
        fx = fmin_(fmax_(fx, -OFX_SNAP_LIMIT), OFX_SNAP_LIMIT);
        fy = fmin_(fmax_(fy, -OFX_SNAP_LIMIT), OFX_SNAP_LIMIT);
        o->X[i] = (int32_t)rintf(fx);
        o->Y[i] = (int32_t)rintf(fy);
        o->z[i] = zn;
        o->iw[i] = iw;
        for (int k = 0; k < 3; k++) o->bary[i][k] = v[i]->b[k];
    }
    int64_t a2 = (int64_t)(o->X[1] - o->X[0]) * (o->Y[2] - o->Y[0]) - (int64_t)(o->X[2] - o->X[0]) * (o->Y[1] - o->Y[0]);
    if (a2 == 0) return 0;
    int front = d->front_ccw ? (a2 > 0) : (a2 < 0);
    if (d->cull_mode == 3) return 0;
    if (d->cull_mode == 1 && front) return 0;
    if (d->cull_mode == 2 && !front) return 0;
    if (a2 < 0) { /* orientation normalisation: swap vertices 1 and 2 */
        int32_t t32;
        float tf;
        t32 = o->X[1]; o->X[1] = o->X[2]; o->X[2] = t32;
        t32 = o->Y[1]; o->Y[1] = o->Y[2]; o->Y[2] = t32;
        tf = o->z[1]; o->z[1] = o->z[2]; o->z[2] = tf;
        tf = o->iw[1]; o->iw[1] = o->iw[2]; o->iw[2] = tf;
        for (int k = 0; k < 3; k++) { tf = o->bary[1][k]; o->bary[1][k] = o->bary[2][k]; o->bary[2][k] = tf; }
        a2 = -a2;
    }
    int32_t xmin = imin_(o->X[0], imin_(o->X[1], o->X[2])), xmax = imax_(o->X[0], imax_(o->X[1], o->X[2]));
    int32_t ymin = imin_(o->Y[0], imin_(o->Y[1], o->Y[2])), ymax = imax_(o->Y[0], imax_(o->Y[1], o->Y[2]));
    int64_t px0 = ceildiv256((int64_t)xmin - c->smax_x), px1 = floordiv256((int64_t)xmax - c->smin_x);
    int64_t py0 = ceildiv256((int64_t)ymin - c->smax_y), py1 = floordiv256((int64_t)ymax - c->smin_y);
    if (px0 < 0) px0 = 0;
    if (py0 < 0) py0 = 0;
    if (px1 > c->W - 1) px1 = c->W - 1;
    if (py1 > c->H - 1) py1 = c->H - 1;
    if (px0 > px1 || py0 > py1) return 0;
    o->px0 = (int)px0; o->px1 = (int)px1; o->py0 = (int)py0; o->py1 = (int)py1;
    for (int i = 0; i < 3; i++) {
        int j = (i + 1) % 3, k = (i + 2) % 3;
        o->A[i] = o->Y[j] - o->Y[k];
        o->B[i] = o->X[k] - o->X[j];
        o->C[i] = (int64_t)(o->Y[k] - o->Y[j]) * o->X[j] - (int64_t)(o->X[k] - o->X[j]) * o->Y[j];
        int topleft = (o->A[i] > 0) || (o->A[i] == 0 && o->B[i] > 0);
        o->Cb[i] = o->C[i] - (topleft ? 0 : 1);
    }
    float dX1 = (float)(o->X[1] - o->X[0]), dY1 = (float)(o->Y[1] - o->Y[0]);
    float dX2 = (float)(o->X[2] - o->X[0]), dY2 = (float)(o->Y[2] - o->Y[0]);
    float dz1 = o->z[1] - o->z[0], dz2 = o->z[2] - o->z[0];
    float fa = (float)a2;
    o->dzdx = (dz1 * dY2 - dz2 * dY1) / fa;
    o->dzdy = (dz2 * dX1 - dz1 * dX2) / fa;
    o->prim = prim;
    o->sub = sub;
    return 1;
}

/* Full per-triangle front end: fetch, transform, clip, fan; returns sub-triangle count. */
/* Completes a sub-triangle whose X, Y, z, iw and bary are set: orientation, pixel range, edge
 * functions and depth plane (no culling). */
static int finish_sub(const pass_ctx* c, int prim, int sub, ofx_sub* o) {
    int64_t a2 = (int64_t)(o->X[1] - o->X[0]) * (o->Y[2] - o->Y[0]) - (int64_t)(o->X[2] - o->X[0]) * (o->Y[1] - o->Y[0]);
    if (a2 == 0) return 0;
    if (a2 < 0) {
        int32_t t32;
        float tf;
        t32 = o->X[1]; o->X[1] = o->X[2]; o->X[2] = t32;
        t32 = o->Y[1]; o->Y[1] = o->Y[2]; o->Y[2] = t32;
        tf = o->z[1]; o->z[1] = o->z[2]; o->z[2] = tf;
        tf = o->iw[1]; o->iw[1] = o->iw[2]; o->iw[2] = tf;
        for (int k = 0; k < 3; k++) { tf = o->bary[1][k]; o->bary[1][k] = o->bary[2][k]; o->bary[2][k] = tf; }
        a2 = -a2;
    }
    int32_t xmin = imin_(o->X[0], imin_(o->X[1], o->X[2])), xmax = imax_(o->X[0], imax_(o->X[1], o->X[2]));
    int32_t ymin = imin_(o->Y[0], imin_(o->Y[1], o->Y[2])), ymax = imax_(o->Y[0], imax_(o->Y[1], o->Y[2]));
    int64_t px0 = ceildiv256((int64_t)xmin - c->smax_x), px1 = floordiv256((int64_t)xmax - c->smin_x);
    int64_t py0 = ceildiv256((int64_t)ymin - c->smax_y), py1 = floordiv256((int64_t)ymax - c->smin_y);
    if (px0 < 0) px0 = 0;
    if (py0 < 0) py0 = 0;
    if (px1 > c->W - 1) px1 = c->W - 1;
    if (py1 > c->H - 1) py1 = c->H - 1;
    if (px0 > px1 || py0 > py1) return 0;
    o->px0 = (int)px0; o->px1 = (int)px1; o->py0 = (int)py0; o->py1 = (int)py1;
    for (int i = 0; i < 3; i++) {
        int j = (i + 1) % 3, k = (i + 2) % 3;
        o->A[i] = o->Y[j] - o->Y[k];
        o->B[i] = o->X[k] - o->X[j];
        o->C[i] = (int64_t)(o->Y[k] - o->Y[j]) * o->X[j] - (int64_t)(o->X[k] - o->X[j]) * o->Y[j];
        int topleft = (o->A[i] > 0) || (o->A[i] == 0 && o->B[i] > 0);
        o->Cb[i] = o->C[i] - (topleft ? 0 : 1);
    }
    float dX1 = (float)(o->X[1] - o->X[0]), dY1 = (float)(o->Y[1] - o->Y[0]);
    float dX2 = (float)(o->X[2] - o->X[0]), dY2 = (float)(o->Y[2] - o->Y[0]);
    float dz1 = o->z[1] - o->z[0], dz2 = o->z[2] - o->z[0];
    float fa = (float)a2;
    o->dzdx = (dz1 * dY2 - dz2 * dY1) / fa;
    o->dzdy = (dz2 * dX1 - dz1 * dX2) / fa;
    o->prim = prim;
    o->sub = sub;
    return 1;
}

/* Line / point polygon modes: the sub-triangles of triangle t (see ofx_draw::polygon_mode). */
static int mode_subs(const pass_ctx* c, const ofx_draw* d, int t, const cvert* poly, ofx_sub* subs) {
    for (int pl = 0; pl < 7; pl++)
        for (int i = 0; i < 3; i++)
            if (plane_dist(c, pl, poly[i].p) < 0.0f) return 0; /* needs clipping: dropped */
    /* projection, snap, cull and orientation of the whole triangle */
    ofx_sub tri;
    for (int i = 0; i < 3; i++) {
        float iw = 1.0f / poly[i].p[3];
        float xn = poly[i].p[0] * iw, yn = poly[i].p[1] * iw, zn = poly[i].p[2] * iw;
        float fx = fmin_(fmax_((xn * 0.5f + 0.5f) * c->W256, -OFX_SNAP_LIMIT), OFX_SNAP_LIMIT);
        float fy = fmin_(fmax_((yn * 0.5f + 0.5f) * c->H256, -OFX_SNAP_LIMIT), OFX_SNAP_LIMIT);
        tri.X[i] = (int32_t)rintf(fx);
        tri.Y[i] = (int32_t)rintf(fy);
        tri.z[i] = zn;
        tri.iw[i] = iw;
        for (int k = 0; k < 3; k++) tri.bary[i][k] = poly[i].b[k];
    }
    int64_t a2 = (int64_t)(tri.X[1] - tri.X[0]) * (tri.Y[2] - tri.Y[0]) - (int64_t)(tri.X[2] - tri.X[0]) * (tri.Y[1] - tri.Y[0]);
    if (a2 == 0) return 0;
    int front = d->front_ccw ? (a2 > 0) : (a2 < 0);
    if (d->cull_mode == 3 || (d->cull_mode == 1 && front) || (d->cull_mode == 2 && !front)) return 0;
    int ord[3] = {0, 1, 2};
    if (a2 < 0) { ord[1] = 2; ord[2] = 1; }
    int cnt = 0;
    for (int part = 0; part < 3; part++) {
        int32_t cx[4], cy[4];
        int src[4];
        if (d->polygon_mode == 1) { /* edge part -> part + 1 of the oriented triangle */
            int p = ord[part], q = ord[(part + 1) % 3];
            int32_t dx = tri.X[q] - tri.X[p], dy = tri.Y[q] - tri.Y[p];
            if (dx == 0 && dy == 0) continue;
            int xmajor = (dx < 0 ? -dx : dx) >= (dy < 0 ? -dy : dy);
            int32_t ox = xmajor ? 0 : 128, oy = xmajor ? 128 : 0;
            cx[0] = tri.X[p] - ox; cy[0] = tri.Y[p] - oy; src[0] = p;
            cx[1] = tri.X[q] - ox; cy[1] = tri.Y[q] - oy; src[1] = q;
            cx[2] = tri.X[q] + ox; cy[2] = tri.Y[q] + oy; src[2] = q;
            cx[3] = tri.X[p] + ox; cy[3] = tri.Y[p] + oy; src[3] = p;
        } else { /* vertex part of the oriented triangle */
            int p = ord[part];
            cx[0] = tri.X[p] - 128; cy[0] = tri.Y[p] - 128;
            cx[1] = tri.X[p] + 128; cy[1] = tri.Y[p] - 128;
            cx[2] = tri.X[p] + 128; cy[2] = tri.Y[p] + 128;
            cx[3] = tri.X[p] - 128; cy[3] = tri.Y[p] + 128;
            src[0] = src[1] = src[2] = src[3] = p;
        }
        static const int halves[2][3] = {{0, 1, 2}, {0, 2, 3}};
        for (int h = 0; h < 2; h++) {
            ofx_sub* o = &subs[cnt];
            for (int i = 0; i < 3; i++) {
                int k = halves[h][i];
                o->X[i] = cx[k];
                o->Y[i] = cy[k];
                o->z[i] = tri.z[src[k]];
                o->iw[i] = tri.iw[src[k]];
                for (int m = 0; m < 3; m++) o->bary[i][m] = tri.bary[src[k]][m];
            }
            if (finish_sub(c, d->prim_base + t, 2 * part + h, o)) cnt++;
        }
    }
    return cnt;
}

static int triangle_subs(const pass_ctx* c, const ofx_draw* d, int t, ofx_sub* subs) {
    cvert poly[OFX_MAX_POLY];
    for (int i = 0; i < 3; i++) {
        int vid = d->indices[3 * t + i];
        if (vid < 0 || vid >= d->num_vertices) return 0;
        xform(d->mvp, d->vertices + (size_t)vid * d->vertex_stride, poly[i].p);
        for (int k = 0; k < 4; k++)
            if (!isfinite(poly[i].p[k])) return 0;
        for (int k = 0; k < 3; k++) poly[i].b[k] = (k == i) ? 1.0f : 0.0f;
    }
    if (d->polygon_mode != 0) return mode_subs(c, d, t, poly, subs);
    int n = clip_polygon(c, poly);
    int cnt = 0;
    for (int i = 1; i + 1 < n; i++)
        if (setup_sub(c, d, &poly[0], &poly[i], &poly[i + 1], d->prim_base + t, i - 1, &subs[cnt])) cnt++;
    return cnt;
}

static inline int covered(const ofx_sub* s, int64_t x, int64_t y) {
    for (int i = 0; i < 3; i++)
        if (s->Cb[i] + (int64_t)s->A[i] * x + (int64_t)s->B[i] * y < 0) return 0;
    return 1;
}

static inline float sample_depth(const ofx_sub* s, int32_t x, int32_t y) {
    return (s->z[0] + s->dzdx * (float)(x - s->X[0])) + s->dzdy * (float)(y - s->Y[0]);
}

static inline int depth_cmp(int func, float z, float d) {
    switch (func) {
    case 0: return 0;
    case 1: return z < d;
    case 2: return z == d;
    case 3: return z <= d;
    case 4: return z > d;
    case 5: return z != d;
    case 6: return z >= d;
    default: return 1;
    }
}

/* Perspective-correct interpolation of the bound attribute at fixed-point position (x, y). */
static void interp_attr(const ofx_sub* s, const ofx_draw* d, int t, int32_t x, int32_t y, float out[4]) {
    float p[3];
    for (int i = 0; i < 3; i++) {
        float e = (float)(s->C[i] + (int64_t)s->A[i] * x + (int64_t)s->B[i] * y);
        p[i] = e * s->iw[i];
    }
    float sum = (p[0] + p[1]) + p[2];
    float r = 1.0f / sum;
    float b[3] = {p[0] * r, p[1] * r, p[2] * r};
    float W[3];
    for (int k = 0; k < 3; k++) W[k] = (b[0] * s->bary[0][k] + b[1] * s->bary[1][k]) + b[2] * s->bary[2][k];
    const float* a[3];
    for (int j = 0; j < 3; j++) a[j] = d->vertices + (size_t)d->indices[3 * t + j] * d->vertex_stride + d->attr_offset;
    for (int k = 0; k < 4; k++) out[k] = 0.0f;
    for (int k = 0; k < d->attr_count; k++) out[k] = (W[0] * a[0][k] + W[1] * a[1][k]) + W[2] * a[2][k];
}

/* Fragment shading of pixel (px, py) for sub-triangle s of draw d (triangle t). */
static void shade(const pass_ctx* c, const ofx_draw* d, const ofx_sub* s, int t, int px, int py, float col[4]) {
    int32_t qx = px * 256 + c->shade_x, qy = py * 256 + c->shade_y;
    if (d->shading == OFX_SHADE_PRIMID) {
        col[0] = (float)s->prim; col[1] = (float)s->sub; col[2] = 0.0f; col[3] = 1.0f;
        return;
    }
    float a[4];
    interp_attr(s, d, t, qx, qy, a);
    if (d->shading == OFX_SHADE_TEXTURED) {
        int xl = px & ~1, yt = py & ~1;
        float al[4], ar[4], at[4], ab[4];
        interp_attr(s, d, t, xl * 256 + c->shade_x, qy, al);
        interp_attr(s, d, t, (xl + 1) * 256 + c->shade_x, qy, ar);
        interp_attr(s, d, t, qx, yt * 256 + c->shade_y, at);
        interp_attr(s, d, t, qx, (yt + 1) * 256 + c->shade_y, ab);
        float dudx = ar[0] - al[0], dvdx = ar[1] - al[1];
        float dudy = ab[0] - at[0], dvdy = ab[1] - at[1];
        ofx_sample_texture(&d->tex, &d->sampler, a[0], a[1], dudx, dvdx, dudy, dvdy, col);
        return;
    }
    col[0] = a[0]; col[1] = a[1]; col[2] = a[2];
    col[3] = d->attr_count >= 4 ? a[3] : 1.0f;
}

static inline float blend_factor(int f, int ch, const float* src, const float* dst) {
    switch (f) {
    case 0: return 0.0f;
    case 1: return 1.0f;
    case 2: return src[ch];
    case 3: return 1.0f - src[ch];
    case 4: return dst[ch];
    case 5: return 1.0f - dst[ch];
    case 6: return src[3];
    case 7: return 1.0f - src[3];
    case 8: return dst[3];
    case 9: return 1.0f - dst[3];
    default: return 0.0f;
    }
}

/* The reference's coefficient vector per factor (TileRasterRenderer.cpp:212-333). */
static void compat_coefs(int f, float k[4]) {
    k[0] = k[1] = k[2] = k[3] = 0.0f;
    switch (f) {
    case 1: k[0] = 1.0f; break;                   /* ONE */
    case 8: k[2] = 1.0f; break;                   /* DST_ALPHA */
    case 6: k[1] = 1.0f; break;                   /* SRC_ALPHA */
    case 9: k[0] = 1.0f; k[2] = -1.0f; break;     /* ONE_MINUS_DST_ALPHA */
    case 7: k[0] = 1.0f; k[1] = -1.0f; break;     /* ONE_MINUS_SRC_ALPHA */
    default: k[3] = 1.0f; break;                  /* ZERO (and unsupported factors) */
    }
}

static inline float compat_factor(int f, const float* src, const float* dst) {
    float k[4];
    compat_coefs(f, k);
    return (k[0] + k[1] * (1.0f - src[3]) + k[2] * (1.0f - dst[3])) * (1.0f - k[3]);
}

static void blend(const ofx_draw* d, const float* src, float* dst) {
    float out[4];
    if (d->blend_compat) { /* TileRasterWorker.cpp:2350-2366 */
        float sx = compat_factor(d->blend_src_color, src, dst), dx = compat_factor(d->blend_dst_color, src, dst);
        float sa = compat_factor(d->blend_src_alpha, src, dst), da = compat_factor(d->blend_dst_alpha, src, dst);
        for (int ch = 0; ch < 3; ch++) out[ch] = dst[ch] * dx + src[ch] * sx;
        out[3] = dst[3] * da + src[3] * sa;
        for (int ch = 0; ch < 4; ch++) dst[ch] = out[ch];
        return;
    }
    for (int ch = 0; ch < 4; ch++) {
        int fs = ch < 3 ? d->blend_src_color : d->blend_src_alpha;
        int fd = ch < 3 ? d->blend_dst_color : d->blend_dst_alpha;
        out[ch] = dst[ch] * blend_factor(fd, ch, src, dst) + src[ch] * blend_factor(fs, ch, src, dst);
    }
    for (int ch = 0; ch < 4; ch++) dst[ch] = out[ch];
}

/* ---------------------------------------------------------------- pass
 * Two phases per chunk of OFX_CHUNK triangles (in submission order): every thread sets up its
 * slice of the chunk once (clip, snap, cull, edge functions), then every thread rasterises the
 * whole chunk's sub-triangles, in submission order, into its own band of rows (depth test and
 * write immediately, as the reference's in-order path).  The draws before the first blended one
 * are shaded deferred, as the reference's tag-buffer path (TileRasterWorker.cpp:1932-2121): each
 * sample remembers the last fragment that passed it, and each (pixel, fragment) pair that
 * survives is shaded once when the prefix ends -- the same colour forward shading leaves there,
 * since unblended fragments overwrite.  From the first blended draw on, every passing fragment
 * is shaded in order (a blend reads the colour under it). */
#define OFX_CHUNK 16384

typedef struct {
    ofx_sub s;
    int draw, tri, slot; /* slot: index of s in triangle_subs()'s output */
} setup_rec;

typedef struct {
    const ofx_draw* draws;
    int ndraws;
    ofx_target* t;
    const pass_ctx* c;
    float* scol;        /* per-sample colour for the whole frame */
    int64_t* win;       /* deferred passes: per-sample last passing fragment, -1 = none */
    int id, nthreads;
    int y0, y1;         /* this thread's band of rows */
    pthread_barrier_t* bar;
    setup_rec** lists;  /* per-thread set-up records of the current chunk */
    int* counts;
} pass_job;

/* Scissor test of pixel (x, y) for draw d (TileRasterCoreInvocationCuda.cu:1950-1962). */
static int scissor_pass(const ofx_draw* d, int x, int y) {
    if (!d->scissor_enable || d->scissor_count <= 0) return 1;
    for (int i = 0; i < d->scissor_count && i < 16; i++) {
        const float* r = d->scissor[i];
        const float fx = (float)x, fy = (float)y;
        if (fx >= r[0] && fx <= r[0] + r[2] && fy >= r[1] && fy <= r[1] + r[3]) return 1;
    }
    return 0;
}

static inline int64_t pack_frag(int draw, int tri, int slot) {
    return ((int64_t)draw << 36) | ((int64_t)tri << 4) | (int64_t)slot;
}

static void raster_rec(pass_job* j, const setup_rec* r) {
    const pass_ctx* c = j->c;
    ofx_target* tg = j->t;
    const ofx_draw* d = &j->draws[r->draw];
    const ofx_sub* s = &r->s;
    const int S = c->S;
    const int func = d->depth_test ? d->depth_func : 7;
    const int ya = imax_(s->py0, j->y0), yb = imin_(s->py1, j->y1 - 1);
    for (int py = ya; py <= yb; py++) {
        for (int px = s->px0; px <= s->px1; px++) {
            if (!scissor_pass(d, px, py)) continue;
            size_t base = ((size_t)(py - c->r0) * c->W + px) * S;
            unsigned passmask = 0;
            for (int k = 0; k < S; k++) {
                int32_t sx = px * 256 + c->sx[k], sy = py * 256 + c->sy[k];
                if (!covered(s, sx, sy)) continue;
                float z = sample_depth(s, sx, sy);
                if (!depth_cmp(func, z, tg->depth[base + k])) continue;
                if (d->depth_write) tg->depth[base + k] = z;
                if (tg->vis) tg->vis[base + k] = s->prim;
                passmask |= 1u << k;
            }
            if (!passmask) continue;
            if (j->win) {
                int64_t f = pack_frag(r->draw, r->tri, r->slot);
                for (int k = 0; k < S; k++)
                    if (passmask & (1u << k)) j->win[base + k] = f;
                continue;
            }
            float col[4];
            shade(c, d, s, r->tri, px, py, col);
            for (int k = 0; k < S; k++) {
                if (!(passmask & (1u << k))) continue;
                float* dst = j->scol + (base + k) * 4;
                if (d->blend_enable) blend(d, col, dst);
                else memcpy(dst, col, sizeof(float) * 4);
            }
        }
    }
}

/* Deferred shading of this thread's band: one shade per (pixel, surviving fragment). */
static void shade_band(pass_job* j) {
    const pass_ctx* c = j->c;
    const int S = c->S;
    ofx_sub subs[OFX_MAX_SUB];
    int64_t cached = -1;
    int ncached = 0;
    for (int py = j->y0; py < j->y1; py++) {
        for (int px = 0; px < c->W; px++) {
            size_t base = ((size_t)(py - c->r0) * c->W + px) * S;
            unsigned done = 0;
            for (int k = 0; k < S; k++) {
                int64_t f = j->win[base + k];
                if (f < 0 || (done & (1u << k))) continue;
                int draw = (int)(f >> 36), tri = (int)((f >> 4) & 0xffffffffll), slot = (int)(f & 15);
                const ofx_draw* d = &j->draws[draw];
                if ((f & ~(int64_t)15) != cached) {
                    ncached = triangle_subs(c, d, tri, subs);
                    cached = f & ~(int64_t)15;
                }
                if (slot >= ncached) continue; /* cannot happen: set-up is deterministic */
                float col[4];
                shade(c, d, &subs[slot], tri, px, py, col);
                for (int q = k; q < S; q++) {
                    if (j->win[base + q] != f) continue;
                    memcpy(j->scol + (base + q) * 4, col, sizeof(float) * 4);
                    done |= 1u << q;
                }
            }
        }
    }
}

static void* run_pass(void* arg) {
    pass_job* j = (pass_job*)arg;
    ofx_sub subs[OFX_MAX_SUB];
    for (int di = 0; di < j->ndraws; di++) {
        const ofx_draw* d = &j->draws[di];
        if (j->win && d->blend_enable) { /* the deferred prefix ends: shade it, then go forward */
            shade_band(j);
            j->win = NULL;
        }
        for (int t0 = 0; t0 < d->num_triangles; t0 += OFX_CHUNK) {
            int t1 = imin_(t0 + OFX_CHUNK, d->num_triangles);
            int a = t0 + (int)((int64_t)(t1 - t0) * j->id / j->nthreads);
            int b = t0 + (int)((int64_t)(t1 - t0) * (j->id + 1) / j->nthreads);
            setup_rec* out = j->lists[j->id];
            int n = 0;
            for (int t = a; t < b; t++) {
                int ns = triangle_subs(j->c, d, t, subs);
                for (int si = 0; si < ns; si++) {
                    if (subs[si].py1 < j->c->r0 || subs[si].py0 >= j->c->r1) continue;
                    out[n].s = subs[si];
                    out[n].draw = di;
                    out[n].tri = t;
                    out[n].slot = si;
                    n++;
                }
            }
            j->counts[j->id] = n;
            pthread_barrier_wait(j->bar);
            for (int th = 0; th < j->nthreads; th++)
                for (int i = 0; i < j->counts[th]; i++) raster_rec(j, &j->lists[th][i]);
            pthread_barrier_wait(j->bar);
        }
    }
    if (j->win) shade_band(j);
    return NULL;
}

/* ---------------------------------------------------------------- reference line / point rules
 * polygon_rules == 1: the reference CUDA renderer's own line and point pipelines
 * (TileRasterCoreInvocationCuda.cu:2780-3334), which do not go through triangle coverage:
 *   points (:2782-2822): every index of the draw is a point: clip = MVP * position; skipped if
 *     w < 1e-8; NDC x, y, z = clip / w; x, y mapped by v * 0.5 + 0.5 and skipped outside [0, 1];
 *     pixel (int)(x * (W - 1)), (int)(y * (H - 1)) (truncation);
 *   lines (:2974-3055, 3062-3115): the three edges (v0 v1), (v1 v2), (v2 v0) of every triangle,
 *     no culling; an edge with both w < 0 is dropped, one endpoint with w < 0 moves to the point
 *     where w = 1 (t = (w_other - 1) / (w_other - w), lerp from the other endpoint); the same NDC
 *     mapping; an edge is dropped when its first endpoint leaves [0, 1]^2 or its second endpoint has
 *     x < 0 or y < 0 (the second endpoint's upper bounds are not tested, :3010: fragments past the
 *     frame's right or top edge are dropped here, as they never reach a pixel of the frame there);
 *     pixels from a Bresenham walk between the truncated endpoints (float error term against 1/2,
 *     x-major when |dx| > |dy|);
 *   fragments (:2855-2920, 3167-3280): per pixel, the candidate with the smallest z wins (a point's
 *     NDC z; a line fragment's z interpolated by the fraction of the pixel along the edge's major
 *     axis in pixel units, (p - a W) / (b W - a W)); ties go to the earlier point / edge in
 *     submission order (the reference leaves them to atomic arrival order); the winner is kept if
 *     its z is below the depth in the buffer (strict, whatever the depth function), and writes
 *     depth and colour.  Colour: the vertex attribute of a point; for a line fragment the two
 *     endpoints' attributes interpolated perspective-correctly with the endpoints' w.  The
 *     interpolation lerp is a + (b - a) t (ShaderOpsCuda.cuh:98-109).
 *   Single-sample targets only; visibility holds the triangle the point or edge belongs to. */
typedef struct {
    uint64_t key;  /* ordered depth bits << 32 | candidate order; ~0 = none */
} ref_cand;

static inline uint64_t depth_key(float z, uint32_t order) {
    uint32_t u = f2u(z + 0.0f);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((uint64_t)u << 32) | order;
}

static inline float key_depth(uint64_t k) {
    uint32_t u = (uint32_t)(k >> 32);
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return u2f(u);
}

static inline void ref_offer(uint64_t* keys, const pass_ctx* c, int px, int py, float z, uint32_t order) {
    if (px < 0 || py < c->r0 || px >= c->W || py >= c->r1 || z != z) return;
    uint64_t k = depth_key(z, order);
    size_t i = (size_t)(py - c->r0) * c->W + px;
    if (k < keys[i]) keys[i] = k;
}

/* The edge from vertex a to vertex b of triangle t after the w < 0 clip and the NDC mapping;
 * returns 0 when the edge is dropped.  out: x, y in [0, 1] units, z = NDC z, w. */
static int ref_edge(const ofx_draw* d, int t, int e, float p1[4], float p2[4]) {
    const int ia = d->indices[3 * t + e], ib = d->indices[3 * t + (e + 1) % 3];
    if (ia < 0 || ia >= d->num_vertices || ib < 0 || ib >= d->num_vertices) return 0;
    float v1[4], v2[4];
    xform(d->mvp, d->vertices + (size_t)ia * d->vertex_stride, v1);
    xform(d->mvp, d->vertices + (size_t)ib * d->vertex_stride, v2);
    if (v1[3] < 0.0f && v2[3] < 0.0f) return 0;
    if (v1[3] < 0.0f) {
        float t1 = (-1.0f + v2[3]) / (v2[3] - v1[3]);
        for (int k = 0; k < 4; k++) v1[k] = v2[k] + (v1[k] - v2[k]) * t1;
    }
    if (v2[3] < 0.0f) {
        float t2 = (-1.0f + v1[3]) / (v1[3] - v2[3]);
        for (int k = 0; k < 4; k++) v2[k] = v1[k] + (v2[k] - v1[k]) * t2;
    }
    for (int k = 0; k < 3; k++) { v1[k] = v1[k] / v1[3]; v2[k] = v2[k] / v2[3]; }
    v1[0] = v1[0] * 0.5f + 0.5f; v1[1] = v1[1] * 0.5f + 0.5f;
    v2[0] = v2[0] * 0.5f + 0.5f; v2[1] = v2[1] * 0.5f + 0.5f;
    if (v1[0] < 0.0f || v1[1] < 0.0f || v1[0] > 1.0f || v1[1] > 1.0f) return 0;
    if (v2[0] < 0.0f || v2[1] < 0.0f) return 0;
    memcpy(p1, v1, 16);
    memcpy(p2, v2, 16);
    return 1;
}

/* Fraction of pixel (px, py) along the edge, along its major axis in pixel units. */
static inline float ref_percent(const pass_ctx* c, const float* p1, const float* p2, int px, int py) {
    float ax = p1[0] * (float)c->W, ay = p1[1] * (float)c->H, bx = p2[0] * (float)c->W, by = p2[1] * (float)c->H;
    if (fabsf(bx - ax) >= fabsf(by - ay)) return ((float)px - ax) / (bx - ax);
    return ((float)py - ay) / (by - ay);
}

static void ref_line_fragments(uint64_t* keys, const pass_ctx* c, const float* p1, const float* p2, uint32_t order) {
    int x1 = (int)(p1[0] * (float)(c->W - 1)), y1 = (int)(p1[1] * (float)(c->H - 1));
    int x2 = (int)(p2[0] * (float)(c->W - 1)), y2 = (int)(p2[1] * (float)(c->H - 1));
    int dx = abs(x1 - x2), dy = abs(y1 - y2);
    if (dx > dy) {
        if (x2 < x1) { int q = x1; x1 = x2; x2 = q; q = y1; y1 = y2; y2 = q; }
        float slope = fabsf(1.0f * (float)(y2 - y1) / (float)(x2 - x1));
        int step = (y2 - y1) > 0 ? 1 : -1;
        float err = 0.0f;
        int cx = x1, cy = y1;
        for (int i = 0; i <= x2 - x1; i++) {
            if (cx < c->W && cy < c->H) {
                float f = ref_percent(c, p1, p2, cx, cy);
                ref_offer(keys, c, cx, cy, p1[2] + (p2[2] - p1[2]) * f, order);
            }
            err = err + slope;
            if (err > 0.5f) { cy += step; err = err - 1.0f; }
            cx++;
        }
    } else {
        if (y2 < y1) { int q = x1; x1 = x2; x2 = q; q = y1; y1 = y2; y2 = q; }
        float slope = fabsf(1.0f * (float)(x2 - x1) / (float)(y2 - y1));
        int step = (x2 - x1) > 0 ? 1 : -1;
        float err = 0.0f;
        int cx = x1, cy = y1;
        for (int i = 0; i <= y2 - y1; i++) {
            if (cx < c->W && cy < c->H) {
                float f = ref_percent(c, p1, p2, cx, cy);
                ref_offer(keys, c, cx, cy, p1[2] + (p2[2] - p1[2]) * f, order);
            }
            err = err + slope;
            if (err > 0.5f) { cx += step; err = err - 1.0f; }
            cy++;
        }
    }
}

static void ref_attr(const ofx_draw* d, int vid, float out[4]) {
    const float* a = d->vertices + (size_t)vid * d->vertex_stride + d->attr_offset;
    for (int k = 0; k < 4; k++) out[k] = k < d->attr_count ? a[k] : 0.0f;
}

/* One draw under the reference's line / point rules into the (single-sample) pass state. */
static int ref_rules_draw(const pass_ctx* c, const ofx_draw* d, ofx_target* tg, float* scol) {
    size_t npix = (size_t)c->W * (size_t)(c->r1 - c->r0);
    uint64_t* keys = (uint64_t*)malloc(npix * sizeof(uint64_t));
    if (!keys) return 3;
    for (size_t i = 0; i < npix; i++) keys[i] = ~(uint64_t)0;
    if (d->polygon_mode == 2) {
        for (int i = 0; i < 3 * d->num_triangles; i++) {
            int vid = d->indices[i];
            if (vid < 0 || vid >= d->num_vertices) continue;
            float v[4];
            xform(d->mvp, d->vertices + (size_t)vid * d->vertex_stride, v);
            if (v[3] < 1e-8f) continue;
            float x = v[0] / v[3], y = v[1] / v[3], z = v[2] / v[3];
            x = x * 0.5f + 0.5f;
            y = y * 0.5f + 0.5f;
            if (x < 0.0f || x > 1.0f || y < 0.0f || y > 1.0f) continue;
            ref_offer(keys, c, (int)(x * (float)(c->W - 1)), (int)(y * (float)(c->H - 1)), z, (uint32_t)i);
        }
    } else {
        for (int t = 0; t < d->num_triangles; t++)
            for (int e = 0; e < 3; e++) {
                float p1[4], p2[4];
                if (ref_edge(d, t, e, p1, p2)) ref_line_fragments(keys, c, p1, p2, (uint32_t)(3 * t + e));
            }
    }
    for (int py = c->r0; py < c->r1; py++)
        for (int px = 0; px < c->W; px++) {
            size_t i = (size_t)(py - c->r0) * c->W + px;
            uint64_t k = keys[i];
            if (k == ~(uint64_t)0) continue;
            float z = key_depth(k);
            if (!(z < tg->depth[i])) continue;
            uint32_t order = (uint32_t)k;
            int t = (int)(order / 3u), e = (int)(order % 3u);
            float col[4];
            if (d->shading == OFX_SHADE_PRIMID) {
                col[0] = (float)(d->prim_base + t); col[1] = (float)e; col[2] = 0.0f; col[3] = 1.0f;
            } else if (d->polygon_mode == 2) {
                ref_attr(d, d->indices[order], col);
                if (d->attr_count < 4) col[3] = 1.0f;
            } else {
                float p1[4], p2[4], a1[4], a2[4];
                ref_edge(d, t, e, p1, p2);
                float f = ref_percent(c, p1, p2, px, py);
                float z1 = p1[3], z2 = p2[3];
                float zt = z1 * z2 / (z2 + f * (z1 - z2));
                ref_attr(d, d->indices[3 * t + e], a1);
                ref_attr(d, d->indices[3 * t + (e + 1) % 3], a2);
                for (int q = 0; q < 4; q++) {
                    float u1 = a1[q] / z1, u2 = a2[q] / z2;
                    col[q] = (f * (u2 - u1) + u1) * zt;
                }
                if (d->attr_count < 4) col[3] = 1.0f;
            }
            tg->depth[i] = z;
            if (tg->vis) tg->vis[i] = d->prim_base + (d->polygon_mode == 2 ? (int)(order / 3u) : t);
            memcpy(scol + i * 4, col, 16);
        }
    free(keys);
    return 0;
}

static void decode_color(const ofx_target* t, size_t pix, float c[4]) {
    switch (t->format) {
    case OFX_FMT_RGBA8: unpack_rgba8(((const uint32_t*)t->color)[pix], c); break;
    case OFX_FMT_RGBA16F: {
        uint64_t v = ((const uint64_t*)t->color)[pix];
        for (int i = 0; i < 4; i++) c[i] = f16_to_f32((uint16_t)(v >> (16 * i)));
        break;
    }
    case OFX_FMT_RGBA32F: memcpy(c, (const float*)t->color + pix * 4, 16); break;
    default:
        memcpy(c, (const float*)t->color + pix * 3, 12);
        c[3] = 1.0f;
        break;
    }
}

static void encode_color(ofx_target* t, size_t pix, const float c[4]) {
    switch (t->format) {
    case OFX_FMT_RGBA8: {
        uint32_t v = 0;
        for (int i = 0; i < 4; i++) {
            float x = fmin_(fmax_(c[i], 0.0f), 1.0f);
            v |= ((uint32_t)rintf(x * 255.0f)) << (8 * i);
        }
        ((uint32_t*)t->color)[pix] = v;
        break;
    }
    case OFX_FMT_RGBA16F: {
        uint64_t v = 0;
        for (int i = 0; i < 4; i++) v |= (uint64_t)ofx_f32_to_f16(c[i]) << (16 * i);
        ((uint64_t*)t->color)[pix] = v;
        break;
    }
    case OFX_FMT_RGBA32F: memcpy((float*)t->color + pix * 4, c, 16); break;
    default: memcpy((float*)t->color + pix * 3, c, 12); break;
    }
}

int ofx_render_pass(const ofx_draw* draws, int ndraws, ofx_target* t, int clear,
                    const float* clear_color, float clear_depth, int nthreads) {
    int S = t->samples;
    if (!(S == 1 || S == 2 || S == 4 || S == 8 || S == 16)) return 1;
    if (t->width <= 0 || t->height <= 0 || t->width > 16384 || t->height > 16384) return 2;
    pass_ctx c;
    c.W = t->width; c.H = t->height; c.S = S;
    c.r0 = t->rows > 0 ? t->row0 : 0;
    c.r1 = t->rows > 0 ? t->row0 + t->rows : t->height;
    if (c.r0 < 0 || c.r1 > c.H || c.r0 >= c.r1) return 4;
    ofx_sample_positions(S, t->sample_compat, c.sx, c.sy);
    c.smin_x = c.smax_x = c.sx[0];
    c.smin_y = c.smax_y = c.sy[0];
    for (int k = 1; k < S; k++) {
        c.smin_x = imin_(c.smin_x, c.sx[k]); c.smax_x = imax_(c.smax_x, c.sx[k]);
        c.smin_y = imin_(c.smin_y, c.sy[k]); c.smax_y = imax_(c.smax_y, c.sy[k]);
    }
    c.shade_x = t->sample_compat ? 0 : 128;
    c.shade_y = t->sample_compat ? 0 : 128;
    c.W256 = (float)c.W * 256.0f;
    c.H256 = (float)c.H * 256.0f;
    c.gx = (float)(1.0 + 2.0 * OFX_GUARD_PX / (double)c.W);
    c.gy = (float)(1.0 + 2.0 * OFX_GUARD_PX / (double)c.H);

    size_t npix = (size_t)c.W * (size_t)(c.r1 - c.r0);
    float* scol = (float*)malloc(npix * S * 4 * sizeof(float));
    if (!scol) return 3;
    for (size_t p = 0; p < npix; p++) {
        float bg[4];
        if (clear) memcpy(bg, clear_color, 16);
        else decode_color(t, p, bg);
        for (int k = 0; k < S; k++) {
            memcpy(scol + (p * S + k) * 4, bg, 16);
            if (clear) t->depth[p * S + k] = clear_depth;
            if (t->vis) t->vis[p * S + k] = -1;
        }
    }
    for (int i = 0; i < ndraws; i++)
        if (draws[i].polygon_rules && draws[i].polygon_mode != 0) {
            int rc = (ndraws == 1 && S == 1) ? ref_rules_draw(&c, &draws[0], t, scol) : 5;
            if (rc) { free(scol); return rc; }
            ndraws = 0;  /* drawn; resolve below */
        }
    if (nthreads < 1) nthreads = 1;
    if (nthreads > c.r1 - c.r0) nthreads = c.r1 - c.r0;
    if (nthreads > 256) nthreads = 256;
    /* the draws before the first blended one are shaded deferred */
    int deferred = ndraws > 0 && !draws[0].blend_enable;
    int64_t* win = NULL;
    if (deferred) {
        win = (int64_t*)malloc(npix * S * sizeof(int64_t));
        if (!win) { free(scol); return 3; }
        for (size_t i = 0; i < npix * S; i++) win[i] = -1;
    }
    pass_job jobs[256];
    pthread_t th[256];
    setup_rec* lists[256];
    int counts[256];
    const int per_thread = (OFX_CHUNK + nthreads - 1) / nthreads * OFX_MAX_SUB;
    int rc = 0;
    for (int i = 0; i < nthreads; i++) {
        lists[i] = (setup_rec*)malloc(sizeof(setup_rec) * (size_t)per_thread);
        if (!lists[i]) rc = 3;
    }
    pthread_barrier_t bar;
    if (!rc && pthread_barrier_init(&bar, NULL, (unsigned)nthreads) != 0) rc = 3;
    if (!rc) {
        for (int i = 0; i < nthreads; i++) {
            jobs[i].draws = draws; jobs[i].ndraws = ndraws; jobs[i].t = t; jobs[i].c = &c; jobs[i].scol = scol;
            jobs[i].win = win; jobs[i].id = i; jobs[i].nthreads = nthreads; jobs[i].bar = &bar;
            jobs[i].lists = lists; jobs[i].counts = counts;
            jobs[i].y0 = c.r0 + (int)((int64_t)(c.r1 - c.r0) * i / nthreads);
            jobs[i].y1 = c.r0 + (int)((int64_t)(c.r1 - c.r0) * (i + 1) / nthreads);
        }
        if (nthreads == 1) run_pass(&jobs[0]);
        else {
            for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, run_pass, &jobs[i]);
            for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
        }
        pthread_barrier_destroy(&bar);
    }
    for (int i = 0; i < nthreads; i++) free(lists[i]);
    free(win);
    if (rc) { free(scol); return rc; }
    float invS = 1.0f / (float)S;
    for (size_t p = 0; p < npix; p++) {
        float acc[4];
        memcpy(acc, scol + p * S * 4, 16);
        for (int k = 1; k < S; k++)
            for (int i = 0; i < 4; i++) acc[i] = acc[i] + scol[(p * S + k) * 4 + i];
        for (int i = 0; i < 4; i++) acc[i] = acc[i] * invS;
        encode_color(t, p, acc);
    }
    free(scol);
    return 0;
}
