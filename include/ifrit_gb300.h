/*
 * ifrit_gb300.h -- C-ABI of the GB300 (sm_103a) software triangle rasterizer.
 *
 * Drop-in boundary for Ifrit-v2's soft renderer (projects/softgraphics).  Entry points keep
 * the reference's exported names and argument meaning (iftr*, ifcr*, ifbuf*); every call is
 * noexcept and returns an int status (IFTR_OK = 0) where the reference returned void.
 * Objects created here are opaque handles.  Framebuffers, images, vertex buffers and
 * varying descriptors are caller-owned and bound by pointer (non-owning), as in the
 * reference (TileRasterContext.h:62-69); the renderer owns its device memory.
 *
 * References (Aeroraven/Ifrit-v2):
 *   TRE = include/ifrit/softgraphics/engine/export/TileRasterRendererExport.h
 *   ECE = include/ifrit/softgraphics/engine/export/EngineCommonExport.h
 *   CE  = include/ifrit/softgraphics/core/export/CommonExport.h
 *   BME = include/ifrit/softgraphics/engine/export/BufferManagerExport.h
 *   TRC = include/ifrit/softgraphics/engine/tilerastercuda/TileRasterRendererCuda.h
 */
#ifndef IFRIT_GB300_H
#define IFRIT_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define IFTR_API __declspec(dllexport)
#else
#define IFTR_API __attribute__((visibility("default")))
#endif

/* ---- status codes */
enum {
    IFTR_OK = 0,
    IFTR_ERR_INVALID_ARG = 1,
    IFTR_ERR_UNSUPPORTED = 2,   /* e.g. host function-pointer shaders */
    IFTR_ERR_CUDA = 3,
    IFTR_ERR_OVERFLOW = 4,      /* a scratch capacity was exceeded; see iftrReserve */
    IFTR_ERR_NO_DEVICE = 5,
    IFTR_ERR_STATE = 6,         /* missing binding (framebuffer, vertex/index buffer, shader) */
    IFTR_ERR_LIMIT = 7          /* an ordered pass had more than 8192 entries in one 16x16 tile */
};

/* ---- enums (same numbering as the reference, base/Constants.h:23-96, TypeDescriptor.h:26-40) */
enum { IF_POLYGON_MODE_FILL = 0, IF_POLYGON_MODE_LINE = 1, IF_POLYGON_MODE_POINT = 2 };
enum { IFTP_FLOAT1 = 1, IFTP_FLOAT2 = 2, IFTP_FLOAT3 = 3, IFTP_FLOAT4 = 4 };
enum { IF_CULL_MODE_NONE = 0, IF_CULL_MODE_FRONT = 1, IF_CULL_MODE_BACK = 2, IF_CULL_MODE_FRONT_AND_BACK = 3 };
enum {
    IF_COMPARE_OP_NEVER = 0, IF_COMPARE_OP_LESS = 1, IF_COMPARE_OP_EQUAL = 2, IF_COMPARE_OP_LESS_OR_EQUAL = 3,
    IF_COMPARE_OP_GREATER = 4, IF_COMPARE_OP_NOT_EQUAL = 5, IF_COMPARE_OP_GREATER_OR_EQUAL = 6,
    IF_COMPARE_OP_ALWAYS = 7
};
enum {
    IF_BLEND_FACTOR_ZERO = 0, IF_BLEND_FACTOR_ONE = 1, IF_BLEND_FACTOR_SRC_COLOR = 2,
    IF_BLEND_FACTOR_ONE_MINUS_SRC_COLOR = 3, IF_BLEND_FACTOR_DST_COLOR = 4, IF_BLEND_FACTOR_ONE_MINUS_DST_COLOR = 5,
    IF_BLEND_FACTOR_SRC_ALPHA = 6, IF_BLEND_FACTOR_ONE_MINUS_SRC_ALPHA = 7, IF_BLEND_FACTOR_DST_ALPHA = 8,
    IF_BLEND_FACTOR_ONE_MINUS_DST_ALPHA = 9
};
enum {
    IF_SAMPLER_ADDRESS_MODE_REPEAT = 0, IF_SAMPLER_ADDRESS_MODE_MIRRORED_REPEAT = 1,
    IF_SAMPLER_ADDRESS_MODE_CLAMP_TO_EDGE = 2, IF_SAMPLER_ADDRESS_MODE_CLAMP_TO_BORDER = 3,
    IF_SAMPLER_ADDRESS_MODE_MIRROR_CLAMP_TO_EDGE = 4
};
enum { IF_FILTER_NEAREST = 0, IF_FILTER_LINEAR = 1 };
/* colour attachment formats held on the device */
enum { IFTR_FORMAT_RGBA8 = 0, IFTR_FORMAT_RGBA16F = 1, IFTR_FORMAT_RGBA32F = 2, IFTR_FORMAT_RGB32F = 3 };
/* built-in shading models (device shaders; see iftrBindFragmentShaderBuiltin) */
enum { IFTR_FS_GOURAUD = 0, IFTR_FS_TEXTURED = 1, IFTR_FS_PRIMITIVE_ID = 2 };
enum { IFTR_VS_MVP_TRANSFORM = 0 };

/* IfritColorAttachmentBlendState (base/Structures.h:91-98) */
typedef struct {
    int blendEnable;
    int srcColorBlendFactor, dstColorBlendFactor, srcAlphaBlendFactor, dstAlphaBlendFactor;
} IfritGbBlendState;

/* IfritSamplerT (base/Structures.h:52-61) */
typedef struct {
    int filterMode, addressModeU, addressModeV, addressModeW, borderColor;
    int anisotropyEnable;
    float maxAnisotropy;
    float lodBias;
} IfritGbSampler;

typedef struct {
    uint64_t triangles_in;        /* triangles submitted in the last pass */
    uint64_t tile_pairs;          /* (triangle, tile) overlaps binned in the last pass */
    uint64_t pair_capacity;       /* current scratch capacity in pairs */
    int retries;                  /* overflow re-runs of the last synchronous draw */
    int deferred_tiles;           /* ordered tiles whose fragments the last pass shaded in the fragment kernels */
    uint64_t deferred_fragments;  /* those tiles' fragments */
} IfritGbStats;

typedef struct IfritGbRenderer IfritGbRenderer;
typedef struct IfritGbFrameBuffer IfritGbFrameBuffer;
typedef struct IfritGbVertexBuffer IfritGbVertexBuffer;
typedef struct IfritGbVaryingDescriptor IfritGbVaryingDescriptor;
typedef struct IfritGbImageF32 IfritGbImageF32;

/* ---- renderer instance (TRE:33-78, TRC:81-115) */
IFTR_API IfritGbRenderer* iftrCreateInstance(void);                                  /* TRE:33 */
IFTR_API int iftrDestroyInstance(IfritGbRenderer* h);                                /* TRE:35 */
IFTR_API int iftrInit(IfritGbRenderer* h);                                           /* TRE:71 */
IFTR_API int iftrBindFrameBuffer(IfritGbRenderer* h, IfritGbFrameBuffer* fb);        /* TRE:37 */
IFTR_API int iftrBindVertexBuffer(IfritGbRenderer* h, const IfritGbVertexBuffer* vb); /* TRE:40 */
IFTR_API int iftrBindIndexBuffer(IfritGbRenderer* h, void* indexBuffer);             /* TRE:43, ifbuf buffer */
/* Host function-pointer and C++-object shaders cannot execute on the device: these return
 * IFTR_ERR_UNSUPPORTED (TRE:45, TRE:49, TRE:75, TRE:77).  Use the built-in device shaders. */
IFTR_API int iftrBindVertexShaderFunc(IfritGbRenderer* h, void* func, IfritGbVaryingDescriptor* vsOut);
IFTR_API int iftrBindFragmentShaderFunc(IfritGbRenderer* h, void* func);
IFTR_API int iftrBindVertexShader(IfritGbRenderer* h, void* pVertexShader);
IFTR_API int iftrBindFragmentShader(IfritGbRenderer* h, void* pFragmentShader);
/* Built-in device shaders replacing the bound shader objects of TileRasterRenderer::
 * bindVertexShader / bindFragmentShader (TileRasterRenderer.h:96-99): the vertex shader is
 * clip = MVP * (attribute 0 xyz, 1) with attribute 1 as the interpolated varying; the MVP is
 * uniform binding 0, set 0 (16 floats, row-major). */
IFTR_API int iftrBindVertexShaderBuiltin(IfritGbRenderer* h, int kind, const IfritGbVaryingDescriptor* vsOut);
IFTR_API int iftrBindFragmentShaderBuiltin(IfritGbRenderer* h, int model);
IFTR_API int iftrBindUniformBuffer(IfritGbRenderer* h, int binding, int set, void* buffer); /* TileRasterRenderer.h:100 */
IFTR_API int iftrSetBlendFunc(IfritGbRenderer* h, const IfritGbBlendState* state);   /* TRE:52 */
IFTR_API int iftrSetDepthFunc(IfritGbRenderer* h, int compareOp);                   /* TRE:55 */
IFTR_API int iftrOptsetForceDeterministic(IfritGbRenderer* h, int opt);             /* TRE:58; always deterministic */
IFTR_API int iftrOptSetDepthTestEnable(IfritGbRenderer* h, int opt);                /* TRE:61 */
IFTR_API int iftrDrawLegacy(IfritGbRenderer* h, int numIndices, int clearFramebuffer); /* TRE:64, synchronous */
IFTR_API int iftrClear(IfritGbRenderer* h);                                          /* TRE:67 */
/* Multi-draw render pass (no counterpart call in the reference, whose drawElements is one draw
 * per pass): draws recorded between Begin and End snapshot the state current at each
 * iftrPassDraw (MVP, shading, blend, depth, cull, texture, geometry) and run as one pass, so
 * MSAA samples of all draws resolve together on chip.  Geometry bound from host objects must
 * not change inside a pass.  Passes that blend, use NOT_EQUAL with depth writes or mix depth
 * states run the ordered path (triangles applied per sample in submission order). */
IFTR_API int iftrBeginPass(IfritGbRenderer* h, int clearFramebuffer);
IFTR_API int iftrPassDraw(IfritGbRenderer* h, int firstIndex, int numIndices);
IFTR_API int iftrEndPass(IfritGbRenderer* h);
/* CUDA-renderer state (TRC:91-111) */
IFTR_API int iftrSetCullMode(IfritGbRenderer* h, int cullMode);                      /* TRC:107 */
IFTR_API int iftrSetFrontFace(IfritGbRenderer* h, int counterClockwise);
IFTR_API int iftrSetMsaaSamples(IfritGbRenderer* h, int samples);                    /* TRC:103, 1/2/4/8/16 */
IFTR_API int iftrSetClearValues(IfritGbRenderer* h, const float* rgba, float depth); /* TRC:108 */
IFTR_API int iftrSetDepthWriteEnable(IfritGbRenderer* h, int enable);
/* Scissor rectangles (x, y, w, h), at most 16, and the scissor test switch (TRC:101-102): with the
 * test on and at least one rectangle, a pixel (x, y) is drawn iff x >= rx, x <= rx + rw, y >= ry
 * and y <= ry + rh for one rectangle (bounds inclusive, as the reference's test). */
IFTR_API int iftrSetScissors(IfritGbRenderer* h, const float* rects, int count);
/* Polygon mode (TRC:106 setRasterizerPolygonMode): FILL; LINE draws each edge of a (culled)
 * triangle as a 1-pixel-wide parallelogram offset +-1/2 pixel along the edge's minor axis; POINT
 * draws each vertex as a 1-pixel square.  Both go through the fill rules (MSAA, depth, shading);
 * triangles that need clipping are dropped in these modes. */
IFTR_API int iftrSetRasterizerPolygonMode(IfritGbRenderer* h, int mode);
/* Rules of the LINE and POINT polygon modes (no entry point in the reference; its CUDA renderer
 * has only these rules for those modes, TileRasterCoreInvocationCuda.cu:2780-3334).
 * FILL_PARTS (default): the parallelograms / squares above.  REFERENCE: the reference's own line
 * and point pipelines: POINT draws every index of the draw as the pixel (int)(x (W-1)),
 * (int)(y (H-1)) of its NDC position mapped to [0, 1] (w < 1e-8 and positions outside [0, 1]
 * skipped); LINE draws the three edges of every triangle (no culling) with Bresenham between
 * truncated endpoints after moving an endpoint with w < 0 to w = 1; per pixel the nearest candidate
 * wins (ties: the earlier point or edge in submission order) and is kept if its depth is below the
 * buffer's (strict, whatever the depth function); colour is the point's vertex attribute or the
 * edge's endpoint attributes interpolated perspective-correctly.  REFERENCE needs a single-sample
 * target, GOURAUD or PRIMITIVE_ID shading and a single-draw pass (iftrDrawLegacy / iftrDrawAsync);
 * otherwise the draw returns IFTR_ERR_UNSUPPORTED.  Visibility holds the triangle the point or edge
 * belongs to. */
enum { IFTR_POLYGON_RULES_FILL_PARTS = 0, IFTR_POLYGON_RULES_REFERENCE = 1 };
IFTR_API int iftrSetPolygonRules(IfritGbRenderer* h, int rules);
/* Fragments of ordered (blended) draws (no counterpart in the reference): the ordered stage
 * resolves coverage and depth tile by tile in submission order and hands each tile's passing
 * fragments to a shading kernel that keeps every thread busy and a blending kernel that applies
 * them per pixel in order.  The image is the same either way.  fragments = -1 (default): buffer
 * for one fragment per pixel, grown after a pass that needed more; 0: the ordered stage shades
 * its fragments itself; n > 0: a buffer of exactly n fragments.  Tiles whose fragments do not fit
 * (or with more than 6 fragments on one pixel) are finished by the ordered stage itself. */
IFTR_API int iftrSetOrderedFragmentCapacity(IfritGbRenderer* h, long long fragments);
/* Raster path of order-independent passes (no counterpart in the reference).  TILED (default):
 * triangles binned into 16x16 tiles, resolved per tile in shared memory.  ATOMIC: no binning;
 * each triangle's thread resolves its samples into per-sample 64-bit (depth, primitive) keys in
 * device memory with atomicMin (the same keys, so the same image), then the shade stage runs.
 * On the 1M-triangle 1080p benchmark frame it is far slower than the tiles (one thread walks a
 * large triangle's whole bbox); it exists for comparison and for scenes of uniformly tiny
 * triangles.  Passes that need submission order always use the tiles. */
enum { IFTR_RASTER_TILED = 0, IFTR_RASTER_ATOMIC = 1 };
IFTR_API int iftrSetRasterPath(IfritGbRenderer* h, int path);
IFTR_API int iftrSetScissorTestEnable(IfritGbRenderer* h, int enable);
/* Outputs of a mesh (or geometry) shading stage drawn as one pass (the boundary of the reference's
 * MeshShadingStage / GeneralGeometryStage, TileRasterCoreInvocationCuda.cu:355-561, whose shader
 * objects produce per-work-group vertices and triangle lists that are compacted and fed to
 * triangle set-up).  Device arrays: work group g holds numVertices[g] <= maxVertices vertices at
 * positions[(g * maxVertices + i) * 4] (clip-space x, y, z, w; no MVP is applied) with one float4
 * varying at attributes[(g * maxVertices + i) * 4] (attrCount components used, NULL when 0), and
 * numIndices[g] <= maxIndices (a multiple of 3) group-local vertex indices at
 * indices[g * maxIndices + k].  Groups are compacted in group order (triangle ids follow it) and
 * drawn with the current state, synchronously like iftrDrawLegacy.  A geometry stage's output is
 * the same with one group per input primitive.  Counts out of range return
 * IFTR_ERR_INVALID_ARG; an index outside its group's vertices drops the triangle. */
IFTR_API int iftrDrawMeshOutputs(IfritGbRenderer* h, int numGroups, const float* positions, const float* attributes,
                                 int attrCount, const int* indices, const int* numVertices, const int* numIndices,
                                 int maxVertices, int maxIndices, int clear);
IFTR_API int iftrCreateTexture(IfritGbRenderer* h, int slot, int width, int height, int mipLevels); /* TRC:91, RGBA8 */
IFTR_API int iftrCopyHostBufferToImage(IfritGbRenderer* h, const void* rgba8, int slot); /* TRC:96, level 0 */
IFTR_API int iftrGenerateMipmap(IfritGbRenderer* h, int slot, int filter);           /* TRC:93 */
IFTR_API int iftrCreateSampler(IfritGbRenderer* h, int slot, const IfritGbSampler* sampler); /* TRC:92 */
IFTR_API int iftrBindTexture(IfritGbRenderer* h, int textureSlot, int samplerSlot);
/* ---- device-resident extensions (no host copies) */
IFTR_API int iftrSetStream(IfritGbRenderer* h, void* cudaStream);
IFTR_API int iftrDrawAsync(IfritGbRenderer* h, int numIndices, int clearFramebuffer);
IFTR_API int iftrFinish(IfritGbRenderer* h);
IFTR_API int iftrBindVertexBufferDevice(IfritGbRenderer* h, const float* vertices, int strideFloats, int numVertices,
                                        int attrOffsetFloats, int attrCount);
IFTR_API int iftrBindIndexBufferDevice(IfritGbRenderer* h, const int* indices, int numIndices);
IFTR_API int iftrSetUniformMatrix(IfritGbRenderer* h, const float* mvpRowMajor);
IFTR_API int iftrSetVisibilityOutput(IfritGbRenderer* h, int enable);
IFTR_API int iftrReserve(IfritGbRenderer* h, size_t tilePairs);
IFTR_API int iftrGetDeviceAttachments(IfritGbRenderer* h, void** color, float** depth, int** visibility);
IFTR_API int iftrReadbackColor(IfritGbRenderer* h, void* dst, size_t bytes);
IFTR_API int iftrReadbackDepth(IfritGbRenderer* h, float* dst, size_t count);
IFTR_API int iftrReadbackVisibility(IfritGbRenderer* h, int* dst, size_t count);
IFTR_API int iftrGetStats(IfritGbRenderer* h, IfritGbStats* out);
/* Per-stage device timing of the last pass, from CUDA events on the renderer's stream:
 * ms[0] counting binner, ms[1] list-offset scan, ms[2] scattering binner, ms[3] tile raster
 * (coverage + depth test; passes without an order-independent part: the in-order stage),
 * ms[4] tile shading + resolve, ms[5] in-order stage after shading (blended passes).  Enable
 * before the draw; read after iftrFinish/iftrDrawLegacy. */
IFTR_API int iftrSetStageTiming(IfritGbRenderer* h, int enable);
IFTR_API int iftrGetStageTimes(IfritGbRenderer* h, float* ms, int n);
IFTR_API const char* iftrGetErrorString(int status);

/* ---- allocation-free pass (no counterpart in the reference)
 * For callers that cannot allocate device memory at draw time: plugins inside a host
 * application that owns all GPU memory, real-time loops with an allocation budget of zero,
 * and code that records its work into an already-built memory plan.  iftrDrawNoAlloc renders
 * one pass from device buffers the caller owns into device outputs the caller owns.  All
 * intermediate data (binning lists, set-up records, per-sample winners, status words) lives in
 * one file-scope device array inside the library, of IFTR_NOALLOC_SCRATCH_BYTES, which every
 * GPU that loads the library holds until the process exits.  The call makes no cudaMalloc,
 * cudaFree or other allocating call.  Every call looks up the array's device address on the
 * current device (a lookup that allocates nothing); the first call on a device may also load the
 * library's device code there, so make it before any stream capture.
 * The array is shared by every call and keeps the last call's contents: calls that overlap on
 * the GPU (different streams or threads) race and must be serialised by the caller.  The call
 * is synchronous on `cudaStream` (it reads a status word back) and returns
 * IFTR_ERR_INVALID_ARG for sizes above the limits below (and for a width or height above
 * 16384, as every other entry point) and IFTR_ERR_OVERFLOW if the scene produces more
 * (triangle, tile) overlaps than the list capacity.  After IFTR_ERR_OVERFLOW the colour, depth
 * and visibility outputs are undefined (the pass has cleared and partly written them); the
 * next call starts afresh. */
#define IFTR_NOALLOC_MAX_TRIANGLES (1 << 16)   /* numIndices / 3 */
#define IFTR_NOALLOC_MAX_SAMPLES (1 << 21)     /* width * height * samples */
#define IFTR_NOALLOC_MAX_TILE_PAIRS (1 << 19)  /* (triangle, 16x16 tile) overlaps */
#define IFTR_NOALLOC_MAX_TILES 8192            /* ceil(width/16) * ceil(height/16) */
#define IFTR_NOALLOC_SCRATCH_BYTES (15u << 20)
typedef struct {
    const float* vertices;          /* device, AoS floats; position = floats 0..2 */
    int strideFloats, numVertices, attrOffsetFloats, attrCount;
    const int* indices;             /* device, 3 per triangle */
    int numIndices;
    float mvp[16];                  /* row-major, clip = mvp * (x, y, z, 1) */
    int width, height, samples;     /* samples: 1, 2, 4, 8 or 16 */
    int colorFormat;                /* IFTR_FORMAT_* */
    void* color;                    /* device, resolved colour */
    float* depth;                   /* device, per-sample depth [H][W][S] */
    int* visibility;                /* device, per-sample primitive id, or NULL */
    int clear;
    float clearColor[4];
    float clearDepth;
    int depthFunc, depthTest, depthWrite, cullMode, frontCounterClockwise;
    int shadingModel;               /* IFTR_FS_* */
    const uint32_t* texels;         /* device RGBA8 mip chain (IFTR_FS_TEXTURED), level after level */
    int texWidth, texHeight, texLevels;
    IfritGbSampler sampler;
} IfritGbNoAllocPass;
IFTR_API int iftrDrawNoAlloc(const IfritGbNoAllocPass* pass, void* cudaStream);

/* ---- batched views (no counterpart in the reference, which renders one view per drawElements)
 * Many independent views of uneven size, sample count and triangle count rendered as one pass:
 * one binning launch over all views' triangles and one persistent launch per tile stage and
 * (samples, path, tile size) group, pulling tiles from per-group work queues.  Inputs and
 * outputs are caller-owned device buffers; each view has its own target and clear values, each
 * draw names its view and carries its own state.  Within a view, draws keep their array order
 * (it decides depth ties and blending order).  The first call with a given description sizes
 * the scratch (synchronously), optionally autotunes the launch parameters, and captures the
 * pass into a CUDA graph; later calls with a byte-identical description replay that graph
 * asynchronously on the renderer's stream.  iftrFinish returns the status (IFTR_ERR_OVERFLOW or
 * IFTR_ERR_LIMIT if a replay exceeded the sized scratch, after growing it; the next call then
 * re-sizes and re-captures). */
typedef struct {
    int width, height, samples;     /* samples: 1, 2, 4, 8 or 16 */
    int colorFormat;                /* IFTR_FORMAT_* */
    void* color;                    /* device, resolved colour */
    float* depth;                   /* device, per-sample depth [H][W][S] */
    int* visibility;                /* device, per-sample primitive id, or NULL */
    int clear;
    float clearColor[4];
    float clearDepth;
} IfritGbBatchView;
typedef struct {
    int view;                       /* index into the view array */
    const float* vertices;          /* device, AoS floats; position = floats 0..2 */
    int strideFloats, numVertices, attrOffsetFloats, attrCount;
    const int* indices;             /* device, 3 per triangle */
    int numIndices;
    float mvp[16];                  /* row-major */
    int depthFunc, depthTest, depthWrite, cullMode, frontCounterClockwise;
    int shadingModel;               /* IFTR_FS_* */
    IfritGbBlendState blend;
    const uint32_t* texels;         /* device RGBA8 mip chain (IFTR_FS_TEXTURED) */
    int texWidth, texHeight, texLevels;
    IfritGbSampler sampler;
} IfritGbBatchDraw;
#define IFTR_MAX_BATCH_VIEWS 4096
#define IFTR_MAX_BATCH_DRAWS 65536
IFTR_API int iftrDrawBatch(IfritGbRenderer* h, const IfritGbBatchView* views, int numViews,
                           const IfritGbBatchDraw* draws, int numDraws);
/* Launch parameters of batched passes.  autotune = 1 (default): the first call of a new batch
 * description times each candidate (tile edge 8 or 16 for 1x/4x views, persistent CTAs per SM
 * at full or half occupancy) and keeps the fastest; autotune = 0 uses tileSize (8 or 16; views
 * whose sample count has no 8x8 kernels use 16) and ctasPerSm (0: full occupancy). */
IFTR_API int iftrSetBatchTuning(IfritGbRenderer* h, int autotune, int tileSize, int ctasPerSm);
IFTR_API int iftrGetBatchTuning(IfritGbRenderer* h, int* tileSize, int* ctasPerSm);

/* ---- differentiable shading (no counterpart in the reference)
 * Shading and silhouette antialiasing of many views of one triangle mesh over visibility
 * buffers produced by iftrDrawBatch (1x, one triangle id per pixel), and the adjoint of both.
 * Forward: perspective-correct barycentrics from the triangle id, colour * bilinear texture(uv)
 * per pixel (`shaded`), then every horizontally or vertically adjacent pixel pair across a
 * silhouette edge of the nearer triangle is blended by how far the edge reaches past the pixel
 * boundary (`image`; decisions in `aaCodes`).  Backward: gradients of a loss with respect to
 * per-vertex positions, colours and UVs, given dL/dimage; they are added to the gradient
 * buffers (zero them first).  Both calls are asynchronous on `cudaStream`. */
typedef struct {
    int numViews, width, height;
    const float* mvp;               /* device [numViews][16], row-major */
    const float* positions;         /* device [numVertices][3] */
    const float* colors;            /* device [numVertices][3] */
    const float* uvs;               /* device [numVertices][2] */
    const int* faces;               /* device [numTriangles][3] */
    const int* neighbors;           /* device [numTriangles][3]: triangle across the edge opposite vertex k, or -1 */
    int numVertices, numTriangles;
    const float* texture;           /* device [texHeight][texWidth][3], repeat addressing, bilinear */
    int texWidth, texHeight;
    const int* visibility;          /* device [numViews][height][width]: triangle id or -1 */
    float* shaded;                  /* device [numViews][height][width][3], before antialiasing */
    float* image;                   /* device [numViews][height][width][3], forward output */
    signed char* aaCodes;           /* device [numViews][height][width][2], antialiasing decisions */
    const float* gradImage;         /* device [numViews][height][width][3], dL/dimage (backward) */
    float* gradPositions;           /* device [numVertices][3] (backward, accumulated) */
    float* gradColors;              /* device [numVertices][3] (backward, accumulated) */
    float* gradUvs;                 /* device [numVertices][2] (backward, accumulated) */
} IfritGbDiffPass;
IFTR_API int iftrDiffForward(const IfritGbDiffPass* pass, void* cudaStream);
IFTR_API int iftrDiffBackward(const IfritGbDiffPass* pass, void* cudaStream);

/* ---- framebuffers and images (ECE:31-40, CE:25-31) */
IFTR_API IfritGbFrameBuffer* iftrCreateFrameBuffer(void);                            /* ECE:31 */
IFTR_API int iftrDestroyFrameBuffer(IfritGbFrameBuffer* fb);                         /* ECE:33 */
IFTR_API int iftrSetFrameBufferColorAttachmentFP32(IfritGbFrameBuffer* fb, IfritGbImageF32* const* images,
                                                   size_t nums);                     /* ECE:35 */
IFTR_API int iftrSetFrameBufferDepthAttachmentFP32(IfritGbFrameBuffer* fb, IfritGbImageF32* image); /* ECE:38 */
/* Device-format colour attachment of the given size (no host image; read back explicitly). */
IFTR_API int iftrSetFrameBufferColorAttachmentDevice(IfritGbFrameBuffer* fb, int format, int width, int height);
IFTR_API IfritGbImageF32* ifcrCreateImageFP32(size_t width, size_t height, size_t channel); /* CE:25 */
IFTR_API int ifcrDestroyImageFP32(IfritGbImageF32* image);                          /* CE:27 */
IFTR_API float* ifcrGetImageRawDataFP32(IfritGbImageF32* image);                     /* CE:29 */

/* ---- varying descriptors and vertex buffers (ECE:43-69) */
IFTR_API IfritGbVaryingDescriptor* iftrCreateVaryingDescriptor(void);                /* ECE:43 */
IFTR_API int iftrDestroyVaryingDescriptor(IfritGbVaryingDescriptor* vd);             /* ECE:45 */
IFTR_API int iftrWriteVaryingDescriptor(IfritGbVaryingDescriptor* vd, const int* desc, size_t num); /* ECE:47 */
IFTR_API IfritGbVertexBuffer* iftrCreateVertexBuffer(void);                          /* ECE:53 */
IFTR_API int iftrDestroyVertexBuffer(IfritGbVertexBuffer* vb);                       /* ECE:55 */
IFTR_API int iftrSetVertexBufferLayout(IfritGbVertexBuffer* vb, const int* desc, size_t num); /* ECE:57 */
IFTR_API int iftrSetVertexBufferSize(IfritGbVertexBuffer* vb, size_t num);           /* ECE:61 */
IFTR_API int iftrAllocateVertexBuffer(IfritGbVertexBuffer* vb);                      /* ECE:64 */
IFTR_API int iftrSetVertexBufferValueFloat4(IfritGbVertexBuffer* vb, int index, int attr, void* value); /* ECE:66 */
IFTR_API int iftrSetVertexBufferData(IfritGbVertexBuffer* vb, const void* src, size_t bytes);
/* Raw (page-locked when a device is present) storage of the vertex buffer, as
 * VertexBuffer::GetBufferUnsafe (VertexBuffer.h:75); after writing through it call
 * iftrSetVertexBufferDirty so the next draw uploads it. */
IFTR_API void* iftrGetVertexBufferRawData(IfritGbVertexBuffer* vb);
IFTR_API int iftrSetVertexBufferDirty(IfritGbVertexBuffer* vb);

/* ---- buffer manager (BME:24-35) */
IFTR_API void* ifbufCreateBufferManager(void);                                       /* BME:24 */
IFTR_API int ifbufDestroyBufferManager(void* manager);                               /* BME:26 */
IFTR_API void* ifbufCreateBuffer(void* manager, size_t bufSize);                     /* BME:28 */
IFTR_API int ifbufDestroyBuffer(void* buffer);                                       /* BME:30 */
IFTR_API int ifbufBufferData(void* buffer, const void* data, size_t offset, size_t size); /* BME:32 */
/* Raw storage of a buffer (TrivialBufferManager::mapBufferMemory, BufferManager.h:73) and
 * its dirty mark for writes made through it. */
IFTR_API void* ifbufGetBufferRawData(void* buffer);
IFTR_API int ifbufSetBufferDirty(void* buffer);

#ifdef __cplusplus
}
#endif
#endif /* IFRIT_GB300_H */
