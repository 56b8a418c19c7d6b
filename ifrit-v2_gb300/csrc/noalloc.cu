// Allocation-free pass entry point (iftrDrawNoAlloc).
//
// For callers that cannot allocate device memory while drawing (a plugin inside a host
// application that owns every GPU allocation, a real-time loop with a zero allocation budget,
// work recorded into a pre-planned memory layout): the caller passes device inputs and
// outputs; every intermediate buffer of the pass lives in one file-scope device array below,
// of IFTR_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the library until exit.  The
// pipeline kernels are the same ones the renderer uses; only where their scratch lives differs.
//
// The array is shared by all calls and keeps the previous call's contents, so everything that
// must start at zero is cleared here on every call, and calls that overlap on the GPU race
// (the caller serialises them).  Nothing in this file calls cudaMalloc, cudaFree or any other
// allocating routine.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/ifrit_gb300.h"
#include "raster_kernels.cuh"

namespace {

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

constexpr size_t kOffStatus = 0;
constexpr size_t kOffDraw = kOffStatus + align256(ifr::ST_WORDS * sizeof(uint32_t));
constexpr size_t kOffDrawStart = kOffDraw + align256(sizeof(ifr::DrawDev));
constexpr size_t kOffTileCount = kOffDrawStart + align256(2 * sizeof(int));
constexpr size_t kOffTileOffset = kOffTileCount + align256((size_t)IFTR_NOALLOC_MAX_TILES * 4);
constexpr size_t kOffTileCursor = kOffTileOffset + align256((size_t)(IFTR_NOALLOC_MAX_TILES + 1) * 4);
constexpr size_t kOffPairs = kOffTileCursor + align256((size_t)IFTR_NOALLOC_MAX_TILES * 4);
constexpr size_t kOffRecords = kOffPairs + align256((size_t)IFTR_NOALLOC_MAX_TILE_PAIRS * 4);
constexpr size_t kOffEntries = kOffRecords + align256((size_t)IFTR_NOALLOC_MAX_TRIANGLES * sizeof(ifr::TriRecord));
constexpr size_t kScratchEnd = kOffEntries + align256((size_t)IFTR_NOALLOC_MAX_SAMPLES * 4);
static_assert(kScratchEnd <= IFTR_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds IFTR_NOALLOC_SCRATCH_BYTES");

static __device__ __align__(256) unsigned char g_noalloc_scratch[IFTR_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device; the
// array's host-side name is only a stand-in and must never be passed to a kernel).
cudaError_t scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

void sample_pattern(int S, int* xs, int* ys) {
    static const int P1[2] = {128, 128};
    static const int P2[4] = {192, 192, 64, 64};
    static const int P4[8] = {96, 32, 224, 96, 32, 160, 160, 224};
    static const int P8[16] = {144, 80, 112, 176, 208, 144, 80, 48, 48, 208, 16, 112, 176, 240, 240, 16};
    static const int P16[32] = {144, 144, 112, 80, 80, 160, 192, 112, 48, 96, 160, 208, 208, 176, 176, 48,
                                96, 224, 128, 16, 64, 32, 32, 192, 0, 128, 240, 64, 224, 240, 16, 0};
    const int* t = S == 1 ? P1 : S == 2 ? P2 : S == 4 ? P4 : S == 8 ? P8 : P16;
    for (int k = 0; k < S; k++) { xs[k] = t[2 * k]; ys[k] = t[2 * k + 1]; }
}

}  // namespace

extern "C" IFTR_API int iftrDrawNoAlloc(const IfritGbNoAllocPass* p, void* cudaStream) {
    if (!p) return IFTR_ERR_INVALID_ARG;
    const int S = p->samples;
    if (!(S == 1 || S == 2 || S == 4 || S == 8 || S == 16)) return IFTR_ERR_INVALID_ARG;
    if (p->width <= 0 || p->height <= 0 || p->numIndices < 0 || p->numIndices % 3 != 0) return IFTR_ERR_INVALID_ARG;
    const int tiles_x = (p->width + ifr::kTileSize - 1) / ifr::kTileSize;
    const int tiles_y = (p->height + ifr::kTileSize - 1) / ifr::kTileSize;
    const size_t T = (size_t)tiles_x * tiles_y;
    if ((size_t)p->numIndices / 3 > IFTR_NOALLOC_MAX_TRIANGLES || T > IFTR_NOALLOC_MAX_TILES ||
        (size_t)p->width * p->height * S > IFTR_NOALLOC_MAX_SAMPLES)
        return IFTR_ERR_INVALID_ARG;
    if (!p->color || !p->depth || (p->numIndices > 0 && (!p->vertices || !p->indices))) return IFTR_ERR_INVALID_ARG;
    if (p->colorFormat < 0 || p->colorFormat > 3 || p->shadingModel < 0 || p->shadingModel > 2) return IFTR_ERR_INVALID_ARG;
    if (p->strideFloats < 3 || p->attrCount < 0 || p->attrCount > 4 || p->attrOffsetFloats + p->attrCount > p->strideFloats)
        return IFTR_ERR_INVALID_ARG;
    if (p->depthFunc < 0 || p->depthFunc > 7 || p->cullMode < 0 || p->cullMode > 3) return IFTR_ERR_INVALID_ARG;
    if (p->shadingModel == IFTR_FS_TEXTURED && (!p->texels || p->texWidth <= 0 || p->texHeight <= 0 ||
                                                p->texLevels <= 0 || p->texLevels > 16))
        return IFTR_ERR_INVALID_ARG;
    const int func = p->depthTest ? p->depthFunc : IF_COMPARE_OP_ALWAYS;
    if (p->depthWrite && func == IF_COMPARE_OP_NOT_EQUAL) return IFTR_ERR_UNSUPPORTED;

    unsigned char* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return IFTR_ERR_CUDA;
    cudaStream_t stream = static_cast<cudaStream_t>(cudaStream);

    ifr::DrawDev d;
    std::memset(&d, 0, sizeof(d));
    d.vertices = p->vertices;
    d.stride = p->strideFloats;
    d.num_vertices = p->numVertices;
    d.attr_offset = p->attrOffsetFloats;
    d.attr_count = p->attrCount;
    d.indices = p->indices;
    d.num_triangles = p->numIndices / 3;
    d.prim_base = 0;
    std::memcpy(d.mvp, p->mvp, sizeof(d.mvp));
    d.cull_mode = p->cullMode;
    d.front_ccw = p->frontCounterClockwise != 0;
    d.depth_func = func;
    d.depth_write = p->depthWrite != 0;
    d.shading = p->shadingModel;
    d.texels = p->texels;
    d.tex_w = p->texWidth;
    d.tex_h = p->texHeight;
    d.tex_levels = p->texLevels;
    d.sampler.address_u = p->sampler.addressModeU;
    d.sampler.address_v = p->sampler.addressModeV;
    d.sampler.filter = p->sampler.filterMode;
    d.sampler.border_white = p->sampler.borderColor;
    d.sampler.max_aniso = p->sampler.anisotropyEnable ? (p->sampler.maxAnisotropy >= 1.0f ? (int)p->sampler.maxAnisotropy : 1) : 1;
    d.sampler.lod_bias = p->sampler.lodBias;
    int w = p->texWidth, h = p->texHeight, off = 0;
    for (int l = 0; l < 16; l++) {
        d.lvl_off[l] = off;
        d.lvl_w[l] = w;
        d.lvl_h[l] = h;
        off += w * h;
        w = w > 1 ? (w + 1) >> 1 : 1;
        h = h > 1 ? (h + 1) >> 1 : 1;
    }
    const int draw_start[2] = {0, d.num_triangles};

    ifr::PassArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c.W = p->width;
    a.c.H = p->height;
    a.c.S = S;
    a.c.tiles_x = tiles_x;
    a.c.tiles_y = tiles_y;
    sample_pattern(S, a.c.sx, a.c.sy);
    a.c.smin_x = a.c.smax_x = a.c.sx[0];
    a.c.smin_y = a.c.smax_y = a.c.sy[0];
    for (int k = 1; k < S; k++) {
        a.c.smin_x = a.c.sx[k] < a.c.smin_x ? a.c.sx[k] : a.c.smin_x;
        a.c.smax_x = a.c.sx[k] > a.c.smax_x ? a.c.sx[k] : a.c.smax_x;
        a.c.smin_y = a.c.sy[k] < a.c.smin_y ? a.c.sy[k] : a.c.smin_y;
        a.c.smax_y = a.c.sy[k] > a.c.smax_y ? a.c.sy[k] : a.c.smax_y;
    }
    a.c.shade_x = 128;
    a.c.shade_y = 128;
    a.c.W256 = (float)p->width * 256.0f;
    a.c.H256 = (float)p->height * 256.0f;
    a.c.gx = (float)(1.0 + 2.0 * 8192.0 / (double)p->width);
    a.c.gy = (float)(1.0 + 2.0 * 8192.0 / (double)p->height);
    a.draws = reinterpret_cast<const ifr::DrawDev*>(base + kOffDraw);
    a.draw_start = reinterpret_cast<const int*>(base + kOffDrawStart);
    a.ndraws = 1;
    a.total_tris = d.num_triangles;
    a.format = p->colorFormat;
    a.color = p->color;
    a.depth = p->depth;
    a.vis = p->visibility;
    a.entries = reinterpret_cast<int*>(base + kOffEntries);
    a.clear = p->clear != 0;
    std::memcpy(a.clear_color, p->clearColor, sizeof(a.clear_color));
    a.clear_depth = p->clearDepth;
    a.depth_func = func;
    a.depth_write = d.depth_write;
    a.tile_count = reinterpret_cast<uint32_t*>(base + kOffTileCount);
    a.tile_offset = reinterpret_cast<uint32_t*>(base + kOffTileOffset);
    a.tile_cursor = reinterpret_cast<uint32_t*>(base + kOffTileCursor);
    a.pairs = reinterpret_cast<uint32_t*>(base + kOffPairs);
    a.pair_capacity = IFTR_NOALLOC_MAX_TILE_PAIRS;
    a.records = reinterpret_cast<ifr::TriRecord*>(base + kOffRecords);
    a.status = reinterpret_cast<uint32_t*>(base + kOffStatus);

    // zero what the pass expects to start at zero (status words and per-tile counts)
    if (cudaMemsetAsync(base + kOffStatus, 0, ifr::ST_WORDS * sizeof(uint32_t), stream) != cudaSuccess ||
        cudaMemsetAsync(base + kOffTileCount, 0, T * 4, stream) != cudaSuccess ||
        cudaMemcpyAsync(base + kOffDraw, &d, sizeof(d), cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(base + kOffDrawStart, draw_start, sizeof(draw_start), cudaMemcpyHostToDevice, stream) != cudaSuccess)
        return IFTR_ERR_CUDA;
    if (ifr::launch_pass(a, stream, nullptr) != cudaSuccess) return IFTR_ERR_CUDA;
    uint32_t status[ifr::ST_WORDS] = {0, 0, 0, 0};
    if (cudaMemcpyAsync(status, base + kOffStatus, sizeof(status), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
        return IFTR_ERR_CUDA;
    return status[ifr::ST_OVERFLOW] ? IFTR_ERR_OVERFLOW : IFTR_OK;
}
