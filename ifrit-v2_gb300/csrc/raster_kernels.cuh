// Kernel-side pass description shared by raster_kernels.cu and the host runtime.
//
// A pass renders one or more views (each its own target, size and sample count); a single
// frame is a pass with one view.  Triangles of all views are binned together into the
// concatenation of every view's screen tiles; the tile stages then run as persistent CTAs
// that pull tiles from a queue per launch group (views of equal sample count and path).
#pragma once
#include <cstdint>
#include "raster_math.cuh"

namespace ifr {

constexpr int kMaxDraws = 256;
constexpr int kMaxViews = 4096;

// Status words of a pass.  Words below ST_PASS_WORDS describe the latest pass and are cleared
// when it starts; ST_STICKY (bit 0: some pass overflowed its pair list, bit 1: some ordered tile
// exceeded kOrderedCap, bit 2: a bulk copy into shared memory was not seen complete within the
// wait limit), ST_MAX_PAIRS and ST_MAX_FRAGS accumulate until the host reads and clears them.
enum StatusWord {
    ST_OVERFLOW = 0,
    ST_PAIRS = 1,
    ST_ORDERED_LIMIT = 2,
    ST_FRAGS = 3,       // deferred ordered fragments allocated (may run past the capacity)
    ST_FRAG_FAIL = 4,   // 0xFFFFFFFF - offset of the first allocation that did not fit; 0: none
    ST_FWD_TILES = 5,   // ordered tiles whose fragments were deferred
    ST_REDO = 6,        // ordered tiles left for the in-stage form (a pixel with too many fragments, buffer full)
    ST_FRAG_NEXT = 7,   // next deferred fragment the fragment shading kernel hands out
    ST_PASS_WORDS = 8,
    ST_STICKY = 8,
    ST_MAX_PAIRS = 9,
    ST_MAX_FRAGS = 10,  // largest fragment demand of a pass that did not fit (grows the buffer)
    ST_WORDS = 12
};
constexpr int kOrderedCap = 8192;  // entries per tile an ordered (in-API-order) pass can sort

// One view (render target) of a pass.
struct ViewArgs {
    PassConst c;
    int tile_start;          // global index of the view's first tile
    int first_tri;           // global index of the view's first triangle (its primitive id 0)
    int format;
    void* color;             // resolved colour (format-dependent)
    float* depth;            // per-sample depth [H][W][S]
    int* vis;                // per-sample primitive id [H][W][S] or nullptr
    int* entries;            // scratch: per-sample winning entry [H][W][S] (raster -> shade)
    int clear;
    float clear_color[4];
    float clear_depth;
    int depth_func;          // view-uniform depth function (deferred path)
    int depth_write;
    int ordered;             // 1: triangles applied to each sample in API order (blending, NOT_EQUAL,
                             //    or draws with different depth state)
    int ordered_prefix;      // ordered views: triangles of the leading draws that need no ordering
                             //    (opaque, the first draw's depth state); they go through the
                             //    order-independent raster stage and the rest is applied on top
    int ordered_cull;        // ordered views: 1 when the prefix writes depth under LESS / LEQUAL and
                             //    no later draw can raise a depth, so that an ordered entry lying
                             //    behind a tile's farthest prefix depth cannot pass anywhere there
    unsigned long long* keys;  // atomic visibility path: per-sample 64-bit keys [H][W][S], else nullptr
    float4* sample_colors;   // ordered views: per-sample colour of the order-independent prefix,
                             //    handed from the shade stage to the ordered stage, tile-major
                             //    [tiles][S][256] (16x16 tiles, lanes in tile_pixel order)
};

struct PassArgs {
    const DrawDev* draws;    // device array [ndraws]
    const int* draw_start;   // device array [ndraws + 1], prefix of triangle counts
    int ndraws;
    int total_tris;
    const ViewArgs* views;   // device array [nviews]
    const int* view_tile_start;  // device array [nviews + 1]
    int nviews;
    int total_tiles;
    // binning
    uint32_t* tile_count;    // [total_tiles], zero between passes
    uint32_t* tile_offset;   // [total_tiles + 1]
    uint32_t* tile_cursor;   // [total_tiles]
    uint32_t* block_sums;    // [scan_blocks(total_tiles)] scan partials
    uint32_t* pairs;         // (global triangle << 3 | fan index), capacity entries
    TriRecord* records;      // [total_tris] compact set-ups written by the counting binner
    TriAttr* attrs;          // [total_tris] vertex attributes of unclipped triangles, or nullptr
    uint32_t pair_capacity;
    uint32_t* status;        // StatusWord
    uint32_t* queues;        // persistent tile counters, 3 per launch group (raster, shade, ordered)
};

// Deferred shading of ordered fragments, passed to the ordered stage and the fragment kernels only
// (frags == nullptr: the ordered stage shades its own fragments).
struct FragArgs {
    uint4* frags;            // [frag_capacity] entry, px | py << 16, sample mask, draw
    float4* frag_cols;       // [frag_capacity] colour of each fragment
    uint32_t frag_capacity;
    uint4* fwd_tiles;        // [total_tiles] deferred tiles: global tile, first fragment, view, hand-off flag
    uint16_t* fwd_pix_end;   // [total_tiles][256] end of each pixel's fragments, from the tile's first
    uint32_t* redo_tiles;    // [total_tiles] tiles the deferring stage left to the in-stage form
};

constexpr int kMaxGroups = 16;  // launch groups of a pass: (samples, path, tile size) combinations

// A contiguous range of views sharing sample count and path, with its tiles.
struct GroupArgs {
    int view_begin, view_end;
    int tile_begin, tile_end;
    int queue;               // index of the group's counters in PassArgs::queues
};

// Launch plan of a pass (host side).
struct LaunchPlan {
    int ngroups;
    GroupArgs groups[kMaxGroups];
    int samples[kMaxGroups];
    int tile_size[kMaxGroups];  // 8 or 16
    int ordered[kMaxGroups];
    int hybrid[kMaxGroups];     // ordered group with an order-independent prefix: raster, then ordered
    int ctas[kMaxGroups];       // persistent CTAs of the group's first stage (raster or ordered)
    int ctas_shade[kMaxGroups]; // persistent CTAs of the group's shade stage
    int ctas_fwd[kMaxGroups];   // hybrid groups: persistent CTAs of the ordered stage after shading
    int atomic;                 // one deferred view resolved by the atomic visibility path (no binning)
    int atomic_pixels;          // its W * H
    int defer_group;            // the only ordered group, whose fragments may be shaded by their own
                                //    kernels (when FragArgs::frags is set); -1: none
    int ctas_frag_shade;        // CTAs of the deferred fragment shading and blending kernels
    int ctas_frag_blend;
    int ctas_fwd_defer;         // CTAs of the defer group's ordered stage in its deferring form
};

}  // namespace ifr

// Host-callable launchers (defined in raster_kernels.cu).
namespace ifr {
// Entries of PassArgs::block_sums a pass over `tiles` tiles needs.
constexpr int scan_blocks(int tiles) { return (tiles + 4095) / 4096 + 1; }
// ev: optional array of kStageEvents events recorded before binning, after counting, after the
// scan, after scattering, after the raster stage, after the shade stage and after the ordered
// stage (per-stage timing).
constexpr int kStageEvents = 7;
// A second stream and two events on which the ordered stage's in-stage form finishes the tiles
// the deferring form left (the redo list) while the deferred fragments are shaded and blended on
// the pass's stream: the two touch disjoint tiles.
struct SideStream {
    cudaStream_t stream;
    cudaEvent_t fork, join;
};
// fa: buffers of the deferred ordered fragments, or nullptr; side: optional, without it the redo
// kernel runs in stream order before the fragment kernels.
cudaError_t launch_pass(const PassArgs& a, const LaunchPlan& plan, cudaStream_t stream, cudaEvent_t* ev,
                        const FragArgs* fa = nullptr, const SideStream* side = nullptr);
// Reference line / point rules (iftrSetPolygonRules): one single-sample draw; `keys` holds W*H
// 64-bit entries of scratch.
cudaError_t launch_reference_rules(const DrawDev& d, const ViewArgs& v, unsigned long long* keys, cudaStream_t stream);
cudaError_t launch_mip_level(const uint32_t* src, int sw, int sh, uint32_t* dst, int dw, int dh, cudaStream_t stream);
// Mesh-stage outputs: per-group vertex / index offsets (totals: vertices, indices, bad-count flag),
// then the compaction into [x y z w a0 a1 a2 a3] rows and rebased indices.
cudaError_t launch_mesh_offsets(const int* nv, const int* ni, int groups, int max_v, int max_i, int* off_v, int* off_i,
                                long long* totals, cudaStream_t stream);
cudaError_t launch_mesh_compact(const float* pos, const float* attr, const int* idx, const int* nv, const int* ni,
                                const int* off_v, const int* off_i, int groups, int max_v, int max_i, float* out_v,
                                int* out_i, cudaStream_t stream);
// Maximum resident CTAs per SM of a tile kernel for (samples, tile size, ordered); stage 0 is
// the raster (or ordered) kernel, stage 1 the shade kernel.
int tile_kernel_occupancy(int samples, int tile_size, int ordered, int stage);
// Resident CTAs per SM of the deferred fragment shading (stage 0) and blending (stage 1) kernels
// and of the ordered stage's deferring form (stage 2).
int frag_kernel_occupancy(int samples, int stage);
}  // namespace ifr
