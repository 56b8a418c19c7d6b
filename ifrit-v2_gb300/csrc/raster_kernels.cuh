// Kernel-side pass description shared by raster_kernels.cu and the host runtime.
#pragma once
#include <cstdint>
#include "raster_math.cuh"

namespace ifr {

constexpr int kTileShift = 4;  // 16x16-pixel screen tiles
constexpr int kTileSize = 1 << kTileShift;
constexpr int kTileThreads = kTileSize * kTileSize;
constexpr int kMaxDraws = 256;

enum StatusWord { ST_OVERFLOW = 0, ST_PAIRS = 1, ST_ORDERED_LIMIT = 2, ST_WORDS = 4 };
constexpr int kOrderedCap = 8192;  // entries per tile an ordered (in-API-order) pass can sort

struct PassArgs {
    PassConst c;
    const DrawDev* draws;    // device array [ndraws]
    const int* draw_start;   // device array [ndraws + 1], prefix of triangle counts
    int ndraws;
    int total_tris;
    // targets
    int format;
    void* color;             // resolved colour (format-dependent)
    float* depth;            // per-sample depth [H][W][S]
    int* vis;                // per-sample primitive id [H][W][S] or nullptr
    int* entries;            // scratch: per-sample winning entry [H][W][S] (raster -> shade)
    int clear;
    float clear_color[4];
    float clear_depth;
    int depth_func;          // pass-uniform depth function (deferred path)
    int depth_write;
    int ordered;             // 1: triangles applied to each sample in API order (blending, NOT_EQUAL,
                             //    or draws with different depth state)
    // binning
    uint32_t* tile_count;    // [T], zero between passes
    uint32_t* tile_offset;   // [T + 1]
    uint32_t* tile_cursor;   // [T]
    uint32_t* pairs;         // (global triangle << 3 | fan index), capacity entries
    TriRecord* records;      // [total_tris] compact set-ups written by the counting binner
    uint32_t pair_capacity;
    uint32_t* status;        // StatusWord
};

}  // namespace ifr

// Host-callable launchers (defined in raster_kernels.cu).
namespace ifr {
// ev: optional array of 6 events recorded before binning, after counting, after the scan,
// after scattering, after the raster kernel and after the shade kernel (per-stage timing).
cudaError_t launch_pass(const PassArgs& a, cudaStream_t stream, cudaEvent_t* ev);
cudaError_t launch_mip_level(const uint32_t* src, int sw, int sh, uint32_t* dst, int dw, int dh, cudaStream_t stream);
}  // namespace ifr
