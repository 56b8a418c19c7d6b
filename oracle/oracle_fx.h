/* Test infrastructure only -- never linked into the product.
 *
 * oracle_fx: a plain-C, single-pass, in-API-order CPU restatement of the soft-renderer
 * triangle pipeline (Ifrit-v2 projects/softgraphics), with the fixed-point coverage
 * contract the sm_103a kernels implement.  It processes every triangle in submission
 * order and every covered sample with an immediate depth test, exactly like the
 * reference's ordered CPU path (TileRasterWorker.cpp:1517-1580), and is the checker the
 * GPU path is compared against bit-for-bit (visibility ids, per-sample depth) and to
 * within one RGBA8 step (colour).  It is pinned against the reference CPU renderer itself
 * (oracle/_ref) in its reference-compatibility mode.
 */
#ifndef ORACLE_FX_H
#define ORACLE_FX_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OFX_FMT_RGBA8 = 0, OFX_FMT_RGBA16F = 1, OFX_FMT_RGBA32F = 2, OFX_FMT_RGB32F = 3 };
enum { OFX_SHADE_GOURAUD = 0, OFX_SHADE_TEXTURED = 1, OFX_SHADE_PRIMID = 2 };

typedef struct {
    int address_u, address_v;   /* IfritSamplerAddressMode numbering */
    int filter;                 /* 0 nearest, 1 linear (trilinear across mips) */
    int border_white;
    int max_aniso;              /* 1 disables anisotropic filtering */
    float lod_bias;
    int compat;                 /* 1: the reference's sampler as written (pinning only; see oracle_fx.c) */
} ofx_sampler;

typedef struct {
    const uint32_t* texels;     /* RGBA8 texels, full mip chain packed level after level */
    int width, height, levels;
} ofx_texture;

typedef struct {
    /* geometry (host arrays) */
    const float* vertices;      /* AoS float vertices */
    int vertex_stride;          /* floats per vertex */
    int num_vertices;
    int attr_offset;            /* first float of the interpolated attribute */
    int attr_count;             /* 0..4 floats */
    const int* indices;         /* 3 per triangle */
    int num_triangles;
    int prim_base;              /* primitive id of triangle 0 */
    float mvp[16];              /* row-major: clip = M * (x, y, z, 1) */
    /* fixed-function state */
    int cull_mode;              /* 0 none, 1 front, 2 back, 3 front+back */
    int front_ccw;              /* 1: counter-clockwise (positive fixed-point area) is front */
    int depth_test;             /* 0 behaves as ALWAYS */
    int depth_func;             /* IfritCompareOp numbering */
    int depth_write;
    int blend_enable;
    int blend_src_color, blend_dst_color, blend_src_alpha, blend_dst_alpha; /* IfritBlendFactor */
    int shading;                /* OFX_SHADE_* */
    ofx_texture tex;
    ofx_sampler sampler;
    /* scissor test (TileRasterRendererCuda.h:101-102, TileRasterCoreInvocationCuda.cu:1950-1962):
     * with scissor_enable and scissor_count > 0 a pixel (x, y) is kept iff for one rectangle
     * (sx, sy, sw, sh): x >= sx, x <= sx + sw, y >= sy, y <= sy + sh (float compares) */
    int scissor_enable;
    int scissor_count;
    float scissor[16][4];       /* x, y, w, h */
    /* polygon mode (IfritPolygonMode, base/Constants.h:23-28): 0 fill, 1 line, 2 point.  Line:
     * each edge of the (culled, orientation-normalised) triangle is a 1-pixel-wide parallelogram,
     * offset +-1/2 pixel along the minor axis; point: each vertex is a 1-pixel square.  Each is
     * two sub-triangles (sub = 2 * edge or vertex + half) through the fill-mode rules; triangles
     * that need clipping are dropped in these modes. */
    int polygon_mode;
    /* 1: blend factors from the reference's coefficient table as written
     * (TileRasterRenderer.cpp:212-333, applied as TileRasterWorker.cpp:2346-2366): a factor is
     * (k0 + k1 (1 - src.a) + k2 (1 - dst.a)) (1 - k3), which swaps SRC_ALPHA with
     * ONE_MINUS_SRC_ALPHA and DST_ALPHA with ONE_MINUS_DST_ALPHA; only the six factors the
     * reference supports (ZERO, ONE, SRC_ALPHA, ONE_MINUS_SRC_ALPHA, DST_ALPHA,
     * ONE_MINUS_DST_ALPHA).  Pinning only; the GPU path blends by the factors' names. */
    int blend_compat;
    /* polygon_mode 1 / 2 with polygon_rules = 1: the reference's own line and point pipelines
     * (Bresenham lines over triangle edges, truncated points per index; see oracle_fx.c) instead
     * of the fill-rule parts above; only as the single draw of a pass on a 1-sample target. */
    int polygon_rules;
} ofx_draw;

typedef struct {
    int width, height, samples; /* samples in {1,2,4,8,16} */
    int format;                 /* OFX_FMT_* */
    int sample_compat;          /* 1: 1x sample and shading point at the pixel corner */
    void* color;                /* resolved colour, format-dependent, row-major */
    float* depth;               /* per-sample depth [H][W][S] */
    int* vis;                   /* per-sample visible primitive id [H][W][S], -1 = none */
    int row0, rows;             /* rows > 0: the buffers hold only rows [row0, row0 + rows) of the
                                   height-row frame (a horizontal band rendered alone) */
} ofx_target;

/* Renders one pass of `ndraws` draws into `t`.  clear != 0 clears colour to clear_color
 * and depth to clear_depth first; otherwise per-sample colour starts from the decoded
 * resolved colour and depth from t->depth.  nthreads > 1 splits the frame into row bands.
 * Returns 0 on success, nonzero on invalid arguments. */
int ofx_render_pass(const ofx_draw* draws, int ndraws, ofx_target* t, int clear,
                    const float* clear_color, float clear_depth, int nthreads);

/* Builds the RGBA8 mip chain in place: level 0 must be filled; returns level count. */
int ofx_build_mips(uint32_t* texels, int width, int height);
int ofx_mip_chain_texels(int width, int height, int* levels);

/* Exposed arithmetic kernels for unit tests. */
float ofx_log2(float x);
void ofx_sample_texture(const ofx_texture* tex, const ofx_sampler* s, float u, float v,
                        float dudx, float dvdx, float dudy, float dvdy, float out[4]);
uint16_t ofx_f32_to_f16(float f);
void ofx_sample_positions(int samples, int compat, int* xs, int* ys);

#ifdef __cplusplus
}
#endif
#endif
