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

#include "../../include/ifrit_gb300.h"
#include "pass_plan.h"
#include "raster_kernels.cuh"

namespace {

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

constexpr size_t kOffStatus = 0;
constexpr size_t kOffDraw = kOffStatus + align256(ifr::ST_WORDS * sizeof(uint32_t));
constexpr size_t kOffDrawStart = kOffDraw + align256(sizeof(ifr::DrawDev));
constexpr size_t kOffView = kOffDrawStart + align256(2 * sizeof(int));
constexpr size_t kOffViewTiles = kOffView + align256(sizeof(ifr::ViewArgs));
constexpr size_t kOffQueues = kOffViewTiles + align256(2 * sizeof(int));
constexpr size_t kOffTileCount = kOffQueues + align256(3 * ifr::kMaxGroups * sizeof(uint32_t));
constexpr size_t kOffTileOffset = kOffTileCount + align256((size_t)IFTR_NOALLOC_MAX_TILES * 4);
constexpr size_t kOffTileCursor = kOffTileOffset + align256((size_t)(IFTR_NOALLOC_MAX_TILES + 1) * 4);
constexpr size_t kOffBlockSums = kOffTileCursor + align256((size_t)IFTR_NOALLOC_MAX_TILES * 4);
constexpr size_t kOffPairs = kOffBlockSums + align256((size_t)ifr::scan_blocks(IFTR_NOALLOC_MAX_TILES) * 4);
constexpr size_t kOffRecords = kOffPairs + align256((size_t)IFTR_NOALLOC_MAX_TILE_PAIRS * 4);
constexpr size_t kOffEntries =
    kOffRecords + align256((size_t)IFTR_NOALLOC_MAX_TRIANGLES * (sizeof(ifr::TriRecord) + sizeof(uint2)));  // + bin words
constexpr size_t kScratchEnd = kOffEntries + align256((size_t)IFTR_NOALLOC_MAX_SAMPLES * 4);
static_assert(kScratchEnd <= IFTR_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds IFTR_NOALLOC_SCRATCH_BYTES");

static __device__ __align__(256) unsigned char g_noalloc_scratch[IFTR_NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array on the current device.  The array's host-side name is
// only a stand-in and must never be passed to a kernel.  The address is looked up on every call
// (the lookup allocates nothing), so it stays right if the context is torn down and the module
// reloaded at another address.
cudaError_t scratch_address(unsigned char** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *out = static_cast<unsigned char*>(p);
    return cudaSuccess;
}

}  // namespace

extern "C" IFTR_API int iftrDrawNoAlloc(const IfritGbNoAllocPass* p, void* cudaStream) {
    if (!p) return IFTR_ERR_INVALID_ARG;
    const int S = p->samples;
    if (!(S == 1 || S == 2 || S == 4 || S == 8 || S == 16)) return IFTR_ERR_INVALID_ARG;
    if (p->width <= 0 || p->height <= 0 || p->width > 16384 || p->height > 16384 || p->numIndices < 0 ||
        p->numIndices % 3 != 0)
        return IFTR_ERR_INVALID_ARG;
    const size_t T = (size_t)ifr::tiles_of(p->width, p->height, 16);
    if ((size_t)p->numIndices / 3 > IFTR_NOALLOC_MAX_TRIANGLES || T > IFTR_NOALLOC_MAX_TILES ||
        (size_t)p->width * p->height * S > IFTR_NOALLOC_MAX_SAMPLES)
        return IFTR_ERR_INVALID_ARG;
    if (!p->color || !p->depth || (p->numIndices > 0 && (!p->vertices || !p->indices))) return IFTR_ERR_INVALID_ARG;
    if (!ifr::targets_aligned(p->color, p->colorFormat, p->depth, p->visibility, S) || (uintptr_t)p->vertices % 4 ||
        (uintptr_t)p->indices % 4 || (uintptr_t)p->texels % 4)
        return IFTR_ERR_INVALID_ARG;
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
    if (p->shadingModel == IFTR_FS_TEXTURED) ifr::fill_texture(d, p->texels, p->texWidth, p->texHeight, p->texLevels, p->sampler);
    const int draw_start[2] = {0, d.num_triangles};

    ifr::ViewArgs v;
    std::memset(&v, 0, sizeof(v));
    ifr::fill_pass_const(v.c, p->width, p->height, S, 16);
    v.format = p->colorFormat;
    v.color = p->color;
    v.depth = p->depth;
    v.vis = p->visibility;
    v.entries = reinterpret_cast<int*>(base + kOffEntries);
    v.clear = p->clear != 0;
    std::memcpy(v.clear_color, p->clearColor, sizeof(v.clear_color));
    v.clear_depth = p->clearDepth;
    ifr::set_view_depth_state(v, &d, 1);
    int view_tiles[2] = {0, 0};
    ifr::LaunchPlan plan;
    int total_tiles = 0;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return IFTR_ERR_CUDA;
    if (!ifr::plan_groups(&v, 1, view_tiles, sms, 0, plan, total_tiles)) return IFTR_ERR_INVALID_ARG;

    ifr::PassArgs a;
    std::memset(&a, 0, sizeof(a));
    a.draws = reinterpret_cast<const ifr::DrawDev*>(base + kOffDraw);
    a.draw_start = reinterpret_cast<const int*>(base + kOffDrawStart);
    a.ndraws = 1;
    a.total_tris = d.num_triangles;
    a.views = reinterpret_cast<const ifr::ViewArgs*>(base + kOffView);
    a.view_tile_start = reinterpret_cast<const int*>(base + kOffViewTiles);
    a.nviews = 1;
    a.total_tiles = total_tiles;
    a.tile_count = reinterpret_cast<uint32_t*>(base + kOffTileCount);
    a.tile_offset = reinterpret_cast<uint32_t*>(base + kOffTileOffset);
    a.tile_cursor = reinterpret_cast<uint32_t*>(base + kOffTileCursor);
    a.block_sums = reinterpret_cast<uint32_t*>(base + kOffBlockSums);
    a.pairs = reinterpret_cast<uint32_t*>(base + kOffPairs);
    a.pair_capacity = IFTR_NOALLOC_MAX_TILE_PAIRS;
    a.records = reinterpret_cast<ifr::TriRecord*>(base + kOffRecords);
    a.status = reinterpret_cast<uint32_t*>(base + kOffStatus);
    a.queues = reinterpret_cast<uint32_t*>(base + kOffQueues);

    // zero what the pass expects to start at zero (status words and per-tile counts)
    if (cudaMemsetAsync(base + kOffStatus, 0, ifr::ST_WORDS * sizeof(uint32_t), stream) != cudaSuccess ||
        cudaMemsetAsync(base + kOffTileCount, 0, T * 4, stream) != cudaSuccess ||
        cudaMemcpyAsync(base + kOffDraw, &d, sizeof(d), cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(base + kOffDrawStart, draw_start, sizeof(draw_start), cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(base + kOffView, &v, sizeof(v), cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(base + kOffViewTiles, view_tiles, sizeof(view_tiles), cudaMemcpyHostToDevice, stream) != cudaSuccess)
        return IFTR_ERR_CUDA;
    if (ifr::launch_pass(a, plan, stream, nullptr) != cudaSuccess) return IFTR_ERR_CUDA;
    uint32_t status[ifr::ST_WORDS] = {};
    if (cudaMemcpyAsync(status, base + kOffStatus, sizeof(status), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
        return IFTR_ERR_CUDA;
    if (status[ifr::ST_STICKY] & 4u) return IFTR_ERR_CUDA;  // a bulk copy into shared memory did not complete
    return status[ifr::ST_OVERFLOW] ? IFTR_ERR_OVERFLOW : IFTR_OK;
}
