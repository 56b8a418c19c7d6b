// Host runtime of the GB300 rasterizer behind the C-ABI in include/ifrit_gb300.h.
//
// Mirrors the reference's host API shape (TileRasterRenderer / TileRasterRendererCuda and the
// iftr*/ifcr*/ifbuf* exports): caller-owned framebuffer, vertex buffer and image objects are
// bound by pointer; the renderer owns the device copies and all scratch.  Device state stays
// resident across draws: host vertex/index data are uploaded only when their contents
// change, attachments are reallocated only when the framebuffer geometry changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/ifrit_gb300.h"
#include "pass_plan.h"
#include "raster_kernels.cuh"

using ifr::DrawDev;
using ifr::PassArgs;

// ----------------------------------------------------------------------------- host objects
// Host bytes, page-locked when a CUDA device is present so uploads run at full link speed.
struct HostBytes {
    uint8_t* p = nullptr;
    size_t n = 0;
    bool pinned = false;
    HostBytes() = default;
    HostBytes(const HostBytes&) = delete;
    HostBytes& operator=(const HostBytes&) = delete;
    ~HostBytes() { release(); }
    bool assign(size_t bytes) {
        release();
        if (bytes == 0) return true;
        if (cudaHostAlloc(reinterpret_cast<void**>(&p), bytes, cudaHostAllocPortable) == cudaSuccess) {
            pinned = true;
        } else {
            cudaGetLastError();
            p = static_cast<uint8_t*>(std::malloc(bytes));
            pinned = false;
            if (!p) return false;
        }
        std::memset(p, 0, bytes);
        n = bytes;
        return true;
    }
    void release() {
        if (p) {
            if (pinned) cudaFreeHost(p); else std::free(p);
        }
        p = nullptr;
        n = 0;
        pinned = false;
    }
    size_t size() const { return n; }
    uint8_t* data() { return p; }
    const uint8_t* data() const { return p; }
};

struct IfritGbImageF32 {
    size_t w = 0, h = 0, c = 0;
    std::vector<float> data;
};

struct IfritGbFrameBuffer {
    std::vector<IfritGbImageF32*> color;
    IfritGbImageF32* depth = nullptr;
    int dev_format = -1;  // >= 0: device-format colour attachment of dev_w x dev_h
    int dev_w = 0, dev_h = 0;
};

struct IfritGbVertexBuffer {
    std::vector<int> layout;
    std::vector<int> offsets;
    int elem_size = 0;
    size_t count = 0;
    HostBytes data;
    uint64_t generation = 1;
};

struct IfritGbVaryingDescriptor {
    std::vector<int> desc;
};

namespace {

struct HostBuffer {
    HostBytes data;
    uint64_t generation = 1;
};

struct BufferManager {
    std::vector<HostBuffer*> buffers;
};

int type_components(int t) { return (t >= IFTP_FLOAT1 && t <= IFTP_FLOAT4) ? t : (t >= 5 && t <= 12 ? ((t - 5) % 4) + 1 : 0); }

// Growable device allocation.
struct DevMem {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

struct Texture {
    DevMem mem;
    int w = 0, h = 0, levels = 0;
};

uint64_t g_id_counter = 1;

// Device scratch and pinned descriptor staging of a pass.  Buffers grow on demand; each growth
// bumps `generation`, which invalidates CUDA graphs captured with the old addresses.
struct PassScratch {
    DevMem tile_count, tile_offset, tile_cursor, block_sums, pairs, records, attrs, status, desc, queues, entries,
        sample_colors, frags, frag_cols, fwd_tiles, fwd_pix_end, redo_tiles;
    // the pass descriptors share one block (one upload per pass): draws | draw starts | views | view
    // tile starts, each at a 256-byte offset sized for cap_draws / cap_views
    size_t cap_draws = 0, cap_views = 0, off_draw_start = 0, off_views = 0, off_view_tiles = 0;
    size_t tiles_alloc = 0;
    uint32_t pair_capacity = 0;
    uint32_t frag_capacity = 0;  // deferred ordered fragments the buffers hold
    size_t frag_want = 0;        // capacity the next pass with ordered tiles reserves
    uint64_t generation = 1;
    uint32_t* h_status = nullptr;  // pinned copy of the status words, written by each pass
    HostBytes staging;             // pinned descriptors: draws | draw starts | views | view tile starts
    cudaEvent_t staged = nullptr;  // recorded after the last descriptor upload
    bool staged_pending = false;
    void release() {
        for (DevMem* m : {&tile_count, &tile_offset, &tile_cursor, &block_sums, &pairs, &records, &attrs, &status, &desc,
                          &queues, &entries, &sample_colors, &frags, &frag_cols, &fwd_tiles, &fwd_pix_end, &redo_tiles})
            m->release();
        if (h_status) cudaFreeHost(h_status);
        h_status = nullptr;
        staging.release();
        if (staged) cudaEventDestroy(staged);
        staged = nullptr;
    }
};

// A batched pass prepared from one description (views + draws), with its captured graph.
struct BatchState {
    PassScratch scratch;
    std::vector<uint8_t> key;  // description bytes and tuning settings of the captured graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t captured_generation = 0;
    cudaStream_t capture_stream = nullptr;
    int autotune = 1, tile_size = 16, ctas_per_sm = 0;  // settings
    int tuned_tile = 16, tuned_ctas = 0;                // last choice
    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        key.clear();
    }
};

}  // namespace

struct IfritGbRenderer {
    bool inited = false;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    ifr::SideStream side{};  // created with the first pass that defers ordered fragments
    int sms = 0;
    // bindings
    IfritGbFrameBuffer* fb = nullptr;
    const IfritGbVertexBuffer* vb = nullptr;
    HostBuffer* ib = nullptr;
    HostBuffer* uniform_mvp = nullptr;
    const float* ext_vertices = nullptr;
    int ext_stride = 0, ext_nverts = 0, ext_attr_off = 0, ext_attr_cnt = 0;
    const int* ext_indices = nullptr;
    int ext_nidx = 0;
    float mvp[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    int fs_model = IFTR_FS_GOURAUD;
    // fixed-function state
    int cull_mode = IF_CULL_MODE_BACK;
    int front_ccw = 1;
    int depth_func = IF_COMPARE_OP_LESS;
    int depth_test = 1;
    int depth_write = 1;
    IfritGbBlendState blend{0, IF_BLEND_FACTOR_ONE, IF_BLEND_FACTOR_ZERO, IF_BLEND_FACTOR_ONE, IF_BLEND_FACTOR_ZERO};
    int samples = 1;
    float clear_color[4] = {0, 0, 0, 0};
    float clear_depth = 1.0f;
    bool vis_output = false;
    int polygon_mode = 0;  // IF_POLYGON_MODE_*
    int polygon_rules = IFTR_POLYGON_RULES_FILL_PARTS;
    int raster_path = IFTR_RASTER_TILED;
    long long frag_capacity_setting = -1;  // deferred ordered fragments: -1 automatic, 0 off, n fixed
    bool scissor_enable = false;
    std::vector<float> scissors;  // (x, y, w, h) per rectangle, at most 16
    // device state
    DevMem d_vertices, d_indices, d_color, d_depth, d_vis, d_entries, d_sample_colors, d_keys;
    DevMem d_mesh_meta, d_mesh_vertices, d_mesh_indices;  // compacted mesh-stage outputs
    const void* up_vb_key = nullptr;
    uint64_t up_vb_gen = 0;
    const void* up_ib_key = nullptr;
    uint64_t up_ib_gen = 0;
    int att_w = 0, att_h = 0, att_s = 0, att_fmt = -1;
    PassScratch pass;  // scratch of the plain (single-view) passes
    BatchState batch;
    Texture tex[16];
    IfritGbSampler samplers[16];
    int bound_tex = 0, bound_sampler = 0;
    IfritGbStats stats{};
    bool timing = false;
    cudaEvent_t ev[ifr::kStageEvents] = {};
    float stage_ms[ifr::kStageEvents - 1] = {};
    std::string last_error;
    int pending = 0;        // plain passes whose status has not been checked
    int pending_batch = 0;  // batched passes whose status has not been checked
    bool in_pass = false;
    int pass_clear = 0;
    std::vector<DrawDev> pass_draws;
};

namespace {

int cuda_fail(IfritGbRenderer* h, cudaError_t e) {
    if (e == cudaSuccess) return IFTR_OK;
    if (h) h->last_error = cudaGetErrorString(e);
    return IFTR_ERR_CUDA;
}

#define IFTR_CUDA(h, expr)                          \
    do {                                            \
        cudaError_t _e = (expr);                    \
        if (_e != cudaSuccess) return cuda_fail(h, _e); \
    } while (0)

size_t color_bytes(int fmt) {
    switch (fmt) {
    case IFTR_FORMAT_RGBA8: return 4;
    case IFTR_FORMAT_RGBA16F: return 8;
    case IFTR_FORMAT_RGBA32F: return 16;
    default: return 12;
    }
}

// Framebuffer geometry and device colour format.
bool fb_geometry(const IfritGbFrameBuffer* fb, int& W, int& H, int& fmt) {
    if (!fb) return false;
    if (fb->dev_format >= 0) {
        W = fb->dev_w; H = fb->dev_h; fmt = fb->dev_format;
        return W > 0 && H > 0;
    }
    if (!fb->color.empty() && fb->color[0]) {
        W = (int)fb->color[0]->w; H = (int)fb->color[0]->h; fmt = IFTR_FORMAT_RGBA32F;
        return W > 0 && H > 0 && fb->color[0]->c == 4;
    }
    return false;
}

int ensure_attachments(IfritGbRenderer* h, int W, int H, int S, int fmt) {
    if (h->att_w == W && h->att_h == H && h->att_s == S && h->att_fmt == fmt && (!h->vis_output || h->d_vis.p)) return IFTR_OK;
    size_t npix = (size_t)W * H;
    IFTR_CUDA(h, h->d_color.reserve(npix * color_bytes(fmt)));
    IFTR_CUDA(h, h->d_depth.reserve(npix * S * sizeof(float)));
    IFTR_CUDA(h, h->d_entries.reserve(npix * S * sizeof(int)));
    if (h->vis_output) IFTR_CUDA(h, h->d_vis.reserve(npix * S * sizeof(int)));
    bool fresh = !(h->att_w == W && h->att_h == H && h->att_s == S && h->att_fmt == fmt);
    h->att_w = W; h->att_h = H; h->att_s = S; h->att_fmt = fmt;
    if (fresh) {
        IFTR_CUDA(h, cudaMemsetAsync(h->d_color.p, 0, npix * color_bytes(fmt), h->stream));
        // depth starts at the clear value
        std::vector<float> dv(npix * S, h->clear_depth);
        IFTR_CUDA(h, cudaMemcpyAsync(h->d_depth.p, dv.data(), dv.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
        IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return IFTR_OK;
}

int scratch_init(IfritGbRenderer* h, PassScratch& s) {
    if (s.h_status) return IFTR_OK;
    IFTR_CUDA(h, cudaMallocHost(&s.h_status, ifr::ST_WORDS * sizeof(uint32_t)));
    std::memset(s.h_status, 0, ifr::ST_WORDS * sizeof(uint32_t));
    IFTR_CUDA(h, s.status.reserve(ifr::ST_WORDS * sizeof(uint32_t)));
    IFTR_CUDA(h, cudaMemsetAsync(s.status.p, 0, ifr::ST_WORDS * sizeof(uint32_t), h->stream));
    IFTR_CUDA(h, s.queues.reserve(3 * ifr::kMaxGroups * sizeof(uint32_t)));
    IFTR_CUDA(h, cudaEventCreateWithFlags(&s.staged, cudaEventDisableTiming));
    return IFTR_OK;
}

int ensure_pairs(IfritGbRenderer* h, PassScratch& s, size_t want) {
    if (want <= s.pair_capacity) return IFTR_OK;
    if (want > 0x7fffffffu) return IFTR_ERR_OVERFLOW;
    IFTR_CUDA(h, s.pairs.reserve(want * 4));
    s.pair_capacity = (uint32_t)want;
    s.generation++;
    return IFTR_OK;
}

// Grows the scratch of a pass over `tiles` screen tiles and `tris` triangles; `entries` is the
// per-sample winner scratch in ints (0: the views bring their own).
int scratch_reserve(IfritGbRenderer* h, PassScratch& s, size_t tiles, size_t tris, size_t ndraws, size_t nviews,
                    size_t entries) {
    int rc = scratch_init(h, s);
    if (rc) return rc;
    const uint64_t gen0 = s.generation;
    auto grow = [&](DevMem& m, size_t bytes) -> cudaError_t {
        if (bytes <= m.bytes) return cudaSuccess;
        s.generation++;
        return m.reserve(bytes + bytes / 4);
    };
    if (tiles > s.tiles_alloc) {
        const size_t n = tiles + tiles / 4;
        IFTR_CUDA(h, s.tile_count.reserve(n * 4));
        IFTR_CUDA(h, s.tile_offset.reserve((n + 1) * 4));
        IFTR_CUDA(h, s.tile_cursor.reserve(n * 4));
        IFTR_CUDA(h, s.block_sums.reserve((size_t)ifr::scan_blocks((int)n) * 4));
        IFTR_CUDA(h, cudaMemsetAsync(s.tile_count.p, 0, n * 4, h->stream));  // counts start at zero
        s.tiles_alloc = n;
        s.generation++;
    }
    // the records, then one 8-byte bin word per triangle (written by the counting pass)
    IFTR_CUDA(h, grow(s.records, std::max<size_t>(1, tris) * (sizeof(ifr::TriRecord) + sizeof(uint2))));
    IFTR_CUDA(h, grow(s.attrs, std::max<size_t>(1, tris) * sizeof(ifr::TriAttr)));
    if (ndraws > s.cap_draws || nviews > s.cap_views || !s.desc.p) {
        s.cap_draws = std::max(s.cap_draws, std::max<size_t>(1, ndraws + ndraws / 4));
        s.cap_views = std::max(s.cap_views, std::max<size_t>(1, nviews + nviews / 4));
        auto a256 = [](size_t x) { return (x + 255) / 256 * 256; };
        s.off_draw_start = a256(s.cap_draws * sizeof(DrawDev));
        s.off_views = s.off_draw_start + a256((s.cap_draws + 1) * sizeof(int));
        s.off_view_tiles = s.off_views + a256(s.cap_views * sizeof(ifr::ViewArgs));
        s.generation++;
        IFTR_CUDA(h, s.desc.reserve(s.off_view_tiles + a256((s.cap_views + 1) * sizeof(int))));
    }
    if (entries) IFTR_CUDA(h, grow(s.entries, entries * sizeof(int)));
    if (s.pair_capacity == 0) {
        rc = ensure_pairs(h, s, std::max<size_t>(1u << 20, tris * 4));
        if (rc) return rc;
    }
    (void)gen0;
    return IFTR_OK;
}

// Copies the pass descriptors to the device through pinned staging (reused once the previous
// upload has executed), in one copy: the staging buffer has the device block's layout.
int upload_descriptors(IfritGbRenderer* h, PassScratch& s, const std::vector<DrawDev>& draws,
                       const std::vector<int>& draw_start, const std::vector<ifr::ViewArgs>& views,
                       const std::vector<int>& view_tiles) {
    const size_t b0 = draws.size() * sizeof(DrawDev), b1 = draw_start.size() * sizeof(int);
    const size_t b2 = views.size() * sizeof(ifr::ViewArgs), b3 = view_tiles.size() * sizeof(int);
    if (draws.size() > s.cap_draws || views.size() > s.cap_views) return IFTR_ERR_INVALID_ARG;  // reserved first
    if (s.staged_pending) {
        IFTR_CUDA(h, cudaEventSynchronize(s.staged));
        s.staged_pending = false;
    }
    const size_t total = s.off_view_tiles + b3;
    if (s.staging.size() < total && !s.staging.assign(total)) return IFTR_ERR_CUDA;
    uint8_t* p = s.staging.data();
    std::memcpy(p, draws.data(), b0);
    std::memcpy(p + s.off_draw_start, draw_start.data(), b1);
    std::memcpy(p + s.off_views, views.data(), b2);
    std::memcpy(p + s.off_view_tiles, view_tiles.data(), b3);
    IFTR_CUDA(h, cudaMemcpyAsync(s.desc.p, p, total, cudaMemcpyHostToDevice, h->stream));
    IFTR_CUDA(h, cudaEventRecord(s.staged, h->stream));
    s.staged_pending = true;
    return IFTR_OK;
}

PassArgs make_args(const PassScratch& s, int ndraws, int total_tris, int nviews, int total_tiles) {
    PassArgs a;
    std::memset(&a, 0, sizeof(a));
    a.draws = s.desc.as<DrawDev>();
    a.draw_start = reinterpret_cast<const int*>(s.desc.as<uint8_t>() + s.off_draw_start);
    a.ndraws = ndraws;
    a.total_tris = total_tris;
    a.views = reinterpret_cast<const ifr::ViewArgs*>(s.desc.as<uint8_t>() + s.off_views);
    a.view_tile_start = reinterpret_cast<const int*>(s.desc.as<uint8_t>() + s.off_view_tiles);
    a.nviews = nviews;
    a.total_tiles = total_tiles;
    a.tile_count = s.tile_count.as<uint32_t>();
    a.tile_offset = s.tile_offset.as<uint32_t>();
    a.tile_cursor = s.tile_cursor.as<uint32_t>();
    a.block_sums = s.block_sums.as<uint32_t>();
    a.pairs = s.pairs.as<uint32_t>();
    a.records = s.records.as<ifr::TriRecord>();
    a.attrs = s.attrs.as<ifr::TriAttr>();
    a.pair_capacity = s.pair_capacity;
    a.status = s.status.as<uint32_t>();
    a.queues = s.queues.as<uint32_t>();
    return a;
}

// Buffers of the deferred ordered fragments: per-tile bookkeeping for `tiles` tiles and at least
// `pixels` fragments (more when an earlier pass needed more).
int reserve_fragments(IfritGbRenderer* h, PassScratch& s, size_t tiles, size_t pixels) {
    IFTR_CUDA(h, s.fwd_tiles.reserve(std::max<size_t>(1, tiles) * sizeof(uint4)));
    IFTR_CUDA(h, s.fwd_pix_end.reserve(std::max<size_t>(1, tiles) * 256 * sizeof(uint16_t)));
    IFTR_CUDA(h, s.redo_tiles.reserve(std::max<size_t>(1, tiles) * sizeof(uint32_t)));
    size_t want = h->frag_capacity_setting > 0 ? (size_t)h->frag_capacity_setting
                                               : std::max(s.frag_want, std::max<size_t>(1u << 20, pixels));
    // below 2^32 with room for the fragment shading kernel's counter, which runs past the count by
    // up to 32 per warp
    want = std::min<size_t>(want, 0xFFF00000u);
    IFTR_CUDA(h, s.frags.reserve(want * sizeof(uint4)));
    IFTR_CUDA(h, s.frag_cols.reserve(want * sizeof(float4)));
    s.frag_capacity = (uint32_t)want;
    return IFTR_OK;
}

ifr::FragArgs fragment_args(const PassScratch& s) {
    ifr::FragArgs f;
    f.frags = s.frags.as<uint4>();
    f.frag_cols = s.frag_cols.as<float4>();
    f.frag_capacity = s.frag_capacity;
    f.fwd_tiles = s.fwd_tiles.as<uint4>();
    f.fwd_pix_end = s.fwd_pix_end.as<uint16_t>();
    f.redo_tiles = s.redo_tiles.as<uint32_t>();
    return f;
}

// Stream work of one pass: clear the per-pass status words, run the pipeline, copy the status
// back to pinned memory.  Contains no host synchronisation (it is also captured into graphs).
cudaError_t launch_with_status(PassScratch& s, const PassArgs& a, const ifr::LaunchPlan& plan, cudaStream_t st,
                               cudaEvent_t* ev, const ifr::FragArgs* fa = nullptr,
                               const ifr::SideStream* side = nullptr) {
    cudaError_t e = cudaMemsetAsync(s.status.p, 0, ifr::ST_PASS_WORDS * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = ifr::launch_pass(a, plan, st, ev, fa, side);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.h_status, s.status.p, ifr::ST_WORDS * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    return e;
}

// Reads the sticky status of a scratch after the stream was synchronised, grows the pair list
// if a pass overflowed, and clears the sticky words.
int consume_status(IfritGbRenderer* h, PassScratch& s) {
    const uint32_t sticky = s.h_status[ifr::ST_STICKY];
    const uint32_t max_pairs = s.h_status[ifr::ST_MAX_PAIRS];
    const uint32_t max_frags = s.h_status[ifr::ST_MAX_FRAGS];
    h->stats.tile_pairs = s.h_status[ifr::ST_PAIRS];
    const uint32_t frag_fail = s.h_status[ifr::ST_FRAG_FAIL];
    h->stats.deferred_fragments = frag_fail ? 0xFFFFFFFFu - frag_fail : s.h_status[ifr::ST_FRAGS];
    h->stats.deferred_tiles = (int)s.h_status[ifr::ST_FWD_TILES];
    if (sticky || max_pairs || max_frags) {
        IFTR_CUDA(h, cudaMemsetAsync(s.status.as<uint32_t>() + ifr::ST_STICKY, 0,
                                     (ifr::ST_WORDS - ifr::ST_STICKY) * sizeof(uint32_t), h->stream));
        s.h_status[ifr::ST_STICKY] = 0;
        s.h_status[ifr::ST_MAX_PAIRS] = 0;
        s.h_status[ifr::ST_MAX_FRAGS] = 0;
    }
    // ordered tiles that found the fragment buffer full were finished by the ordered stage itself
    // (same image); the next pass reserves room for them
    if (max_frags > s.frag_capacity) s.frag_want = std::max(s.frag_want, (size_t)max_frags + max_frags / 4);
    if (sticky & 1u) {
        size_t want = (size_t)max_pairs + max_pairs / 4 + 1024;
        int rc = ensure_pairs(h, s, want);
        return rc ? rc : IFTR_ERR_OVERFLOW;
    }
    if (sticky & 2u) return IFTR_ERR_LIMIT;
    if (sticky & 4u) return IFTR_ERR_CUDA;  // a bulk copy into shared memory did not complete in time
    return IFTR_OK;
}

// Resolves the vertex/index sources of a draw; uploads host data when it changed.
int prepare_geometry(IfritGbRenderer* h, int numIndices, DrawDev& d) {
    if (h->ext_vertices) {
        d.vertices = h->ext_vertices;
        d.stride = h->ext_stride;
        d.num_vertices = h->ext_nverts;
        d.attr_offset = h->ext_attr_off;
        d.attr_count = h->ext_attr_cnt;
    } else {
        const IfritGbVertexBuffer* vb = h->vb;
        if (!vb || vb->layout.empty() || vb->elem_size % 4 != 0) return IFTR_ERR_STATE;
        size_t bytes = vb->data.size();
        if (h->up_vb_key != vb || h->up_vb_gen != vb->generation) {
            IFTR_CUDA(h, h->d_vertices.reserve(std::max<size_t>(bytes, 16)));
            IFTR_CUDA(h, cudaMemcpyAsync(h->d_vertices.p, vb->data.data(), bytes, cudaMemcpyHostToDevice, h->stream));
            h->up_vb_key = vb;
            h->up_vb_gen = vb->generation;
        }
        d.vertices = h->d_vertices.as<float>();
        d.stride = vb->elem_size / 4;
        d.num_vertices = (int)vb->count;
        if (vb->layout.size() > 1) {
            d.attr_offset = vb->offsets[1] / 4;
            d.attr_count = std::min(4, type_components(vb->layout[1]));
        } else {
            d.attr_offset = 0;
            d.attr_count = 0;
        }
    }
    if (h->ext_indices) {
        if (numIndices > h->ext_nidx) return IFTR_ERR_INVALID_ARG;
        d.indices = h->ext_indices;
    } else {
        if (!h->ib) return IFTR_ERR_STATE;
        size_t bytes = h->ib->data.size();
        if ((size_t)numIndices * 4 > bytes) return IFTR_ERR_INVALID_ARG;
        if (h->up_ib_key != h->ib || h->up_ib_gen != h->ib->generation) {
            IFTR_CUDA(h, h->d_indices.reserve(std::max<size_t>(bytes, 16)));
            IFTR_CUDA(h, cudaMemcpyAsync(h->d_indices.p, h->ib->data.data(), bytes, cudaMemcpyHostToDevice, h->stream));
            h->up_ib_key = h->ib;
            h->up_ib_gen = h->ib->generation;
        }
        d.indices = h->d_indices.as<int>();
    }
    d.num_triangles = numIndices / 3;
    return IFTR_OK;
}

void fill_state(IfritGbRenderer* h, DrawDev& d) {
    const float* m = h->mvp;
    if (h->uniform_mvp && h->uniform_mvp->data.size() >= 64) m = reinterpret_cast<const float*>(h->uniform_mvp->data.data());
    std::memcpy(d.mvp, m, sizeof(d.mvp));
    d.prim_base = 0;
    d.cull_mode = h->cull_mode;
    d.front_ccw = h->front_ccw;
    d.depth_func = h->depth_test ? h->depth_func : IF_COMPARE_OP_ALWAYS;
    d.depth_write = h->depth_write;
    ifr::fill_blend(d, h->blend);
    d.shading = h->fs_model;
    ifr::fill_scissor(d, h->scissor_enable, h->scissors.data(), (int)h->scissors.size() / 4);
    d.polygon_mode = h->polygon_mode;
    const Texture& t = h->tex[h->bound_tex];
    ifr::fill_texture(d, t.mem.as<uint32_t>(), t.w, t.h, t.levels, h->samplers[h->bound_sampler]);
}

int ensure_init(IfritGbRenderer* h) {
    if (h->inited) return IFTR_OK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return IFTR_ERR_NO_DEVICE;
    if (!h->stream) {
        IFTR_CUDA(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    int dev = 0;
    IFTR_CUDA(h, cudaGetDevice(&dev));
    IFTR_CUDA(h, cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev));
    int rc = scratch_init(h, h->pass);
    if (rc) return rc;
    for (auto& s : h->samplers) {
        s = IfritGbSampler{IF_FILTER_LINEAR, IF_SAMPLER_ADDRESS_MODE_REPEAT, IF_SAMPLER_ADDRESS_MODE_REPEAT,
                           IF_SAMPLER_ADDRESS_MODE_REPEAT, 0, 0, 1.0f, 0.0f};
    }
    h->inited = true;
    return IFTR_OK;
}

// Snapshot of the current state as one draw of `numIndices` indices starting at `firstIndex`.
int prepare_draw(IfritGbRenderer* h, int firstIndex, int numIndices, DrawDev& d) {
    if (numIndices < 0 || numIndices % 3 != 0 || firstIndex < 0 || firstIndex % 3 != 0) return IFTR_ERR_INVALID_ARG;
    std::memset(&d, 0, sizeof(d));
    if (numIndices > 0) {
        int rc = prepare_geometry(h, firstIndex + numIndices, d);
        if (rc) return rc;
        d.indices += firstIndex;
    }
    d.num_triangles = numIndices / 3;
    fill_state(h, d);
    if (d.shading == IFTR_FS_TEXTURED && (!d.texels || d.tex_levels <= 0)) return IFTR_ERR_STATE;
    return IFTR_OK;
}

// Enqueues one pass of draws into the bound framebuffer on the renderer's stream.
int enqueue_pass(IfritGbRenderer* h, std::vector<DrawDev>& draws, int clear) {
    int rc = ensure_init(h);
    if (rc) return rc;
    if (draws.empty() || draws.size() > (size_t)ifr::kMaxDraws) return IFTR_ERR_INVALID_ARG;
    int W, H, fmt;
    if (!fb_geometry(h->fb, W, H, fmt)) return IFTR_ERR_STATE;
    if (W > 16384 || H > 16384) return IFTR_ERR_INVALID_ARG;
    int S = h->samples;
    rc = ensure_attachments(h, W, H, S, fmt);
    if (rc) return rc;
    // global triangle ids: draw i covers [start_i, start_{i+1})
    std::vector<int> draw_start(draws.size() + 1);
    int64_t total = 0;
    for (size_t i = 0; i < draws.size(); i++) {
        DrawDev& d = draws[i];
        d.view = 0;
        d.prim_base = (int)total;
        draw_start[i] = (int)total;
        total += d.num_triangles;
        if (total >= (int64_t)1 << 28) return IFTR_ERR_INVALID_ARG;  // entry = triangle << 3 | fan index
    }
    draw_start[draws.size()] = (int)total;
    std::vector<ifr::ViewArgs> views(1);
    ifr::ViewArgs& v = views[0];
    std::memset(&v, 0, sizeof(v));
    ifr::fill_pass_const(v.c, W, H, S, 16);
    v.format = fmt;
    v.color = h->d_color.p;
    v.depth = h->d_depth.as<float>();
    v.vis = h->vis_output ? h->d_vis.as<int>() : nullptr;
    v.entries = h->d_entries.as<int>();
    v.clear = clear;
    bool reference_rules = false;
    for (const DrawDev& d : draws)
        if (d.polygon_mode != IF_POLYGON_MODE_FILL && h->polygon_rules == IFTR_POLYGON_RULES_REFERENCE)
            reference_rules = true;
    if (reference_rules) {  // the reference's own line / point pipelines: a separate path
        const DrawDev& d = draws[0];
        if (draws.size() != 1 || S != 1 || (d.shading != IFTR_FS_GOURAUD && d.shading != IFTR_FS_PRIMITIVE_ID))
            return IFTR_ERR_UNSUPPORTED;
        std::memcpy(v.clear_color, h->clear_color, sizeof(v.clear_color));
        v.clear_depth = h->clear_depth;
        IFTR_CUDA(h, h->d_keys.reserve((size_t)W * H * sizeof(unsigned long long)));
        IFTR_CUDA(h, cudaMemsetAsync(h->pass.status.p, 0, ifr::ST_PASS_WORDS * sizeof(uint32_t), h->stream));
        IFTR_CUDA(h, ifr::launch_reference_rules(d, v, h->d_keys.as<unsigned long long>(), h->stream));
        IFTR_CUDA(h, cudaMemcpyAsync(h->pass.h_status, h->pass.status.p, ifr::ST_WORDS * sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, h->stream));
        h->stats.triangles_in = (uint64_t)total;
        h->pending = 1;
        return IFTR_OK;
    }
    std::memcpy(v.clear_color, h->clear_color, sizeof(v.clear_color));
    v.clear_depth = h->clear_depth;
    ifr::set_view_depth_state(v, draws.data(), (int)draws.size());
    if (v.ordered) {  // per-sample colours handed from the shade stage to the ordered stage
        IFTR_CUDA(h, h->d_sample_colors.reserve((size_t)ifr::tiles_of(W, H, 16) * 256 * S * sizeof(float4)));
        v.sample_colors = h->d_sample_colors.as<float4>();
    }
    if (h->raster_path == IFTR_RASTER_ATOMIC && !v.ordered) {  // per-sample keys in global memory
        IFTR_CUDA(h, h->d_keys.reserve((size_t)W * H * S * sizeof(unsigned long long)));
        v.keys = h->d_keys.as<unsigned long long>();
    }
    std::vector<int> view_tiles(2);
    ifr::LaunchPlan plan;
    int T = 0;
    if (!ifr::plan_groups(views.data(), 1, view_tiles.data(), h->sms, 0, plan, T)) return IFTR_ERR_INVALID_ARG;
    if (v.keys) {
        plan.atomic = 1;
        plan.atomic_pixels = W * H;
    }
    rc = scratch_reserve(h, h->pass, (size_t)T, (size_t)total, draws.size(), 1, 0);
    if (rc) return rc;
    rc = upload_descriptors(h, h->pass, draws, draw_start, views, view_tiles);
    if (rc) return rc;
    PassArgs a = make_args(h->pass, (int)draws.size(), (int)total, 1, T);
    ifr::FragArgs fa;
    const bool defer = plan.defer_group >= 0 && h->frag_capacity_setting != 0;
    if (defer) {
        rc = reserve_fragments(h, h->pass, (size_t)T, (size_t)W * H);
        if (rc) return rc;
        fa = fragment_args(h->pass);
        if (!h->side.fork) IFTR_CUDA(h, cudaEventCreateWithFlags(&h->side.fork, cudaEventDisableTiming));
        if (!h->side.join) IFTR_CUDA(h, cudaEventCreateWithFlags(&h->side.join, cudaEventDisableTiming));
        if (!h->side.stream) IFTR_CUDA(h, cudaStreamCreateWithFlags(&h->side.stream, cudaStreamNonBlocking));
    }
    IFTR_CUDA(h, launch_with_status(h->pass, a, plan, h->stream, h->timing ? h->ev : nullptr, defer ? &fa : nullptr,
                                    defer ? &h->side : nullptr));
    h->stats.triangles_in = (uint64_t)total;
    h->pending = 1;
    return IFTR_OK;
}

// Enqueues a single-draw pass with the current state.
int enqueue_draw(IfritGbRenderer* h, int numIndices, int clear) {
    int rc = ensure_init(h);
    if (rc) return rc;
    std::vector<DrawDev> one(1);
    rc = prepare_draw(h, 0, numIndices, one[0]);
    if (rc) return rc;
    return enqueue_pass(h, one, clear);
}

int check_pending(IfritGbRenderer* h) {
    if (!h->pending && !h->pending_batch) return IFTR_OK;
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    int rc = IFTR_OK;
    if (h->pending) {
        h->pending = 0;
        if (h->timing)
            for (int i = 0; i + 1 < ifr::kStageEvents; i++) cudaEventElapsedTime(&h->stage_ms[i], h->ev[i], h->ev[i + 1]);
        rc = consume_status(h, h->pass);
        h->stats.pair_capacity = h->pass.pair_capacity;
    }
    if (h->pending_batch) {
        h->pending_batch = 0;
        int rb = consume_status(h, h->batch.scratch);
        if (rb == IFTR_ERR_OVERFLOW) h->batch.drop_graph();  // re-size and re-capture on the next call
        if (!rc) rc = rb;
    }
    return rc;
}

int copy_back_host_images(IfritGbRenderer* h) {
    IfritGbFrameBuffer* fb = h->fb;
    if (!fb || fb->dev_format >= 0) return IFTR_OK;
    size_t npix = (size_t)h->att_w * h->att_h;
    if (!fb->color.empty() && fb->color[0])
        IFTR_CUDA(h, cudaMemcpyAsync(fb->color[0]->data.data(), h->d_color.p, npix * 16, cudaMemcpyDeviceToHost, h->stream));
    if (fb->depth && fb->depth->w == (size_t)h->att_w && fb->depth->h == (size_t)h->att_h) {
        int S = h->att_s;
        if (S == 1) {
            IFTR_CUDA(h, cudaMemcpyAsync(fb->depth->data.data(), h->d_depth.p, npix * 4, cudaMemcpyDeviceToHost, h->stream));
            IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
        } else {  // host FP32 depth image holds the per-pixel mean, as the reference resolve does
            std::vector<float> tmp(npix * S);
            IFTR_CUDA(h, cudaMemcpyAsync(tmp.data(), h->d_depth.p, tmp.size() * 4, cudaMemcpyDeviceToHost, h->stream));
            IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
            for (size_t p = 0; p < npix; p++) {
                float acc = tmp[p * S];
                for (int k = 1; k < S; k++) acc += tmp[p * S + k];
                fb->depth->data[p * fb->depth->c] = acc / (float)S;
            }
        }
    }
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    return IFTR_OK;
}

// ----------------------------------------------------------------------------- batched views
int validate_batch(const IfritGbBatchView* views, int nv, const IfritGbBatchDraw* draws, int nd) {
    if (!views || nv <= 0 || nv > IFTR_MAX_BATCH_VIEWS || nd < 0 || nd > IFTR_MAX_BATCH_DRAWS || (nd > 0 && !draws))
        return IFTR_ERR_INVALID_ARG;
    for (int i = 0; i < nv; i++) {
        const IfritGbBatchView& v = views[i];
        if (v.width <= 0 || v.height <= 0 || v.width > 16384 || v.height > 16384 || !ifr::valid_samples(v.samples))
            return IFTR_ERR_INVALID_ARG;
        if (v.colorFormat < 0 || v.colorFormat > 3 || !v.color || !v.depth) return IFTR_ERR_INVALID_ARG;
        if (!ifr::targets_aligned(v.color, v.colorFormat, v.depth, v.visibility, v.samples)) return IFTR_ERR_INVALID_ARG;
    }
    int64_t total = 0;
    for (int i = 0; i < nd; i++) {
        const IfritGbBatchDraw& d = draws[i];
        if (d.view < 0 || d.view >= nv || d.numIndices < 0 || d.numIndices % 3 != 0) return IFTR_ERR_INVALID_ARG;
        if (d.numIndices > 0 && (!d.vertices || !d.indices)) return IFTR_ERR_INVALID_ARG;
        if ((uintptr_t)d.vertices % 4 || (uintptr_t)d.indices % 4 || (uintptr_t)d.texels % 4) return IFTR_ERR_INVALID_ARG;
        if (d.strideFloats < 3 || d.attrCount < 0 || d.attrCount > 4 || d.attrOffsetFloats < 0 ||
            d.attrOffsetFloats + d.attrCount > d.strideFloats)
            return IFTR_ERR_INVALID_ARG;
        if (d.depthFunc < 0 || d.depthFunc > 7 || d.cullMode < 0 || d.cullMode > 3 || d.shadingModel < IFTR_FS_GOURAUD ||
            d.shadingModel > IFTR_FS_PRIMITIVE_ID)
            return IFTR_ERR_INVALID_ARG;
        for (int f : {d.blend.srcColorBlendFactor, d.blend.dstColorBlendFactor, d.blend.srcAlphaBlendFactor,
                      d.blend.dstAlphaBlendFactor})
            if (d.blend.blendEnable && (f < 0 || f > 9)) return IFTR_ERR_INVALID_ARG;
        if (d.shadingModel == IFTR_FS_TEXTURED &&
            (!d.texels || d.texWidth <= 0 || d.texHeight <= 0 || d.texLevels <= 0 || d.texLevels > 16))
            return IFTR_ERR_INVALID_ARG;
        total += d.numIndices / 3;
    }
    if (total >= (int64_t)1 << 28) return IFTR_ERR_INVALID_ARG;  // entry = triangle << 3 | fan index
    return IFTR_OK;
}

// Descriptor bytes of a batch call (struct padding left out) plus the tuning settings; a call
// whose key equals the captured one replays the graph.
std::vector<uint8_t> batch_key(const BatchState& b, const IfritGbBatchView* views, int nv, const IfritGbBatchDraw* draws,
                               int nd) {
    constexpr size_t d0 = offsetof(IfritGbBatchDraw, vertices);
    constexpr size_t d1 = offsetof(IfritGbBatchDraw, sampler) + sizeof(IfritGbSampler);
    const int settings[5] = {b.autotune, b.tile_size, b.ctas_per_sm, nv, nd};
    std::vector<uint8_t> key(sizeof(settings) + (size_t)nv * sizeof(IfritGbBatchView) + (size_t)nd * (4 + d1 - d0));
    uint8_t* p = key.data();
    std::memcpy(p, settings, sizeof(settings));
    p += sizeof(settings);
    std::memcpy(p, views, (size_t)nv * sizeof(IfritGbBatchView));
    p += (size_t)nv * sizeof(IfritGbBatchView);
    for (int i = 0; i < nd; i++) {
        std::memcpy(p, &draws[i].view, 4);
        std::memcpy(p + 4, reinterpret_cast<const uint8_t*>(&draws[i]) + d0, d1 - d0);
        p += 4 + d1 - d0;
    }
    return key;
}

// Host descriptors of a batch for one choice of tile size and persistent CTAs.  Views are
// reordered so that each launch group is contiguous; the draws of each view follow in array
// order, so global triangle ids keep every view's submission order.
struct BatchBuild {
    std::vector<DrawDev> draws;
    std::vector<int> draw_start;
    std::vector<ifr::ViewArgs> views;
    std::vector<size_t> entry_offset;  // per internal view, ints into the entries scratch
    std::vector<size_t> color_offset;  // per internal view, float4s into the sample colour scratch (or ~0)
    size_t sample_colors = 0;
    std::vector<int> view_tiles;
    ifr::LaunchPlan plan;
    int total_tiles = 0;
    int64_t total_tris = 0;
    size_t entries = 0;
};

int build_batch(IfritGbRenderer* h, const IfritGbBatchView* views, int nv, const IfritGbBatchDraw* draws, int nd,
                int tile_size, int ctas_per_sm, BatchBuild& out) {
    std::vector<std::vector<int>> per_view(nv);
    for (int i = 0; i < nd; i++) per_view[draws[i].view].push_back(i);
    std::vector<DrawDev> dd(nd);
    for (int i = 0; i < nd; i++) {
        const IfritGbBatchDraw& s = draws[i];
        DrawDev& d = dd[i];
        std::memset(&d, 0, sizeof(d));
        d.vertices = s.vertices;
        d.stride = s.strideFloats;
        d.num_vertices = s.numVertices;
        d.attr_offset = s.attrOffsetFloats;
        d.attr_count = s.attrCount;
        d.indices = s.indices;
        d.num_triangles = s.numIndices / 3;
        std::memcpy(d.mvp, s.mvp, sizeof(d.mvp));
        d.cull_mode = s.cullMode;
        d.front_ccw = s.frontCounterClockwise != 0;
        d.depth_func = s.depthTest ? s.depthFunc : IF_COMPARE_OP_ALWAYS;
        d.depth_write = s.depthWrite != 0;
        d.shading = s.shadingModel;
        ifr::fill_blend(d, s.blend);
        if (s.shadingModel == IFTR_FS_TEXTURED) ifr::fill_texture(d, s.texels, s.texWidth, s.texHeight, s.texLevels, s.sampler);
    }
    std::vector<ifr::ViewArgs> uv(nv);
    std::vector<DrawDev> tmp;
    for (int i = 0; i < nv; i++) {
        const IfritGbBatchView& s = views[i];
        ifr::ViewArgs& v = uv[i];
        std::memset(&v, 0, sizeof(v));
        tmp.clear();
        for (int di : per_view[i]) tmp.push_back(dd[di]);
        ifr::set_view_depth_state(v, tmp.data(), (int)tmp.size());
        const int TS = ifr::tile_size_supported(s.samples, tile_size, v.ordered != 0) ? tile_size : 16;
        ifr::fill_pass_const(v.c, s.width, s.height, s.samples, TS);
        v.format = s.colorFormat;
        v.color = s.color;
        v.depth = s.depth;
        v.vis = s.visibility;
        v.clear = s.clear != 0;
        std::memcpy(v.clear_color, s.clearColor, sizeof(v.clear_color));
        v.clear_depth = s.clearDepth;
    }
    std::vector<int> order(nv);
    for (int i = 0; i < nv; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return ifr::group_key(uv[x]) < ifr::group_key(uv[y]); });
    out.draws.clear();
    out.draw_start.clear();
    out.views.clear();
    out.entry_offset.clear();
    out.color_offset.clear();
    int64_t tri = 0;
    size_t ent = 0, cols = 0;
    for (int k = 0; k < nv; k++) {
        const int vi = order[k];
        ifr::ViewArgs v = uv[vi];
        v.first_tri = (int)tri;
        int prim = 0;
        for (int di : per_view[vi]) {
            DrawDev d = dd[di];
            d.view = k;
            d.prim_base = prim;
            out.draw_start.push_back((int)tri);
            out.draws.push_back(d);
            prim += d.num_triangles;
            tri += d.num_triangles;
        }
        out.entry_offset.push_back(ent);
        // every view gets winner scratch (a launch group that runs the raster stage writes it for
        // all its views), each starting on a 256-byte boundary (the tile kernels move it as int4)
        ent += ((size_t)v.c.W * v.c.H * v.c.S + 63) / 64 * 64;
        out.color_offset.push_back(v.ordered ? cols : ~(size_t)0);
        if (v.ordered) cols += (size_t)v.c.tiles_x * v.c.tiles_y * 256 * v.c.S;  // ordered views use 16x16 tiles
        out.views.push_back(v);
    }
    out.draw_start.push_back((int)tri);
    out.total_tris = tri;
    out.entries = std::max<size_t>(ent, 1);
    out.sample_colors = cols;
    out.view_tiles.assign(nv + 1, 0);
    if (!ifr::plan_groups(out.views.data(), nv, out.view_tiles.data(), h->sms, ctas_per_sm, out.plan, out.total_tiles))
        return IFTR_ERR_INVALID_ARG;
    return IFTR_OK;
}

// Grows the batch scratch for `bb`, points its views at the entries scratch and uploads the
// descriptors.
int stage_batch(IfritGbRenderer* h, BatchBuild& bb) {
    PassScratch& s = h->batch.scratch;
    int rc = scratch_reserve(h, s, (size_t)bb.total_tiles, (size_t)bb.total_tris, bb.draws.size(), bb.views.size(), bb.entries);
    if (rc) return rc;
    if (bb.sample_colors * sizeof(float4) > s.sample_colors.bytes) {
        s.generation++;  // captured graphs hold the old address
        IFTR_CUDA(h, s.sample_colors.reserve(bb.sample_colors * sizeof(float4)));
    }
    for (size_t k = 0; k < bb.views.size(); k++) {
        bb.views[k].entries = s.entries.as<int>() + bb.entry_offset[k];
        bb.views[k].sample_colors =
            bb.color_offset[k] == ~(size_t)0 ? nullptr : s.sample_colors.as<float4>() + bb.color_offset[k];
    }
    if (bb.draws.empty()) bb.draws.resize(1);  // keeps the upload well-formed; ndraws stays 0
    return upload_descriptors(h, s, bb.draws, bb.draw_start, bb.views, bb.view_tiles);
}

PassArgs batch_args(IfritGbRenderer* h, const BatchBuild& bb, int nd) {
    return make_args(h->batch.scratch, nd, (int)bb.total_tris, (int)bb.views.size(), bb.total_tiles);
}

// Saved colour and depth of the views that do not clear, so that sizing and tuning runs (which
// execute the pass more than once) leave those targets as the one real run sees them.
struct TargetBackup {
    DevMem mem;
    std::vector<std::pair<void*, size_t>> spans;  // (target, bytes), packed in order
    int save(IfritGbRenderer* h, const IfritGbBatchView* views, int nv) {
        size_t total = 0;
        spans.clear();
        for (int i = 0; i < nv; i++) {
            if (views[i].clear) continue;
            const size_t npix = (size_t)views[i].width * views[i].height;
            spans.push_back({views[i].color, npix * color_bytes(views[i].colorFormat)});
            spans.push_back({views[i].depth, npix * views[i].samples * sizeof(float)});
            if (views[i].visibility) spans.push_back({views[i].visibility, npix * views[i].samples * sizeof(int)});
        }
        for (auto& sp : spans) total += sp.second;
        if (!total) return IFTR_OK;
        IFTR_CUDA(h, mem.reserve(total));
        size_t off = 0;
        for (auto& sp : spans) {
            IFTR_CUDA(h, cudaMemcpyAsync(mem.as<uint8_t>() + off, sp.first, sp.second, cudaMemcpyDeviceToDevice, h->stream));
            off += sp.second;
        }
        return IFTR_OK;
    }
    int restore(IfritGbRenderer* h) {
        size_t off = 0;
        for (auto& sp : spans) {
            IFTR_CUDA(h, cudaMemcpyAsync(sp.first, mem.as<uint8_t>() + off, sp.second, cudaMemcpyDeviceToDevice, h->stream));
            off += sp.second;
        }
        return IFTR_OK;
    }
};

// Runs the staged batch once, synchronously, growing the pair list until it fits.
int run_sized(IfritGbRenderer* h, BatchBuild& bb, int nd, TargetBackup& backup, bool& ran) {
    for (int attempt = 0; attempt < 4; attempt++) {
        int rc = stage_batch(h, bb);
        if (rc) return rc;
        if (ran) {
            rc = backup.restore(h);
            if (rc) return rc;
        }
        PassArgs a = batch_args(h, bb, nd);
        IFTR_CUDA(h, launch_with_status(h->batch.scratch, a, bb.plan, h->stream, nullptr));
        IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
        ran = true;
        rc = consume_status(h, h->batch.scratch);
        if (rc != IFTR_ERR_OVERFLOW) return rc;
    }
    return IFTR_ERR_OVERFLOW;
}

// Sizes the scratch, picks the launch parameters and captures the pass into a graph.
int prepare_batch(IfritGbRenderer* h, const IfritGbBatchView* views, int nv, const IfritGbBatchDraw* draws, int nd) {
    BatchState& b = h->batch;
    b.drop_graph();
    std::vector<std::pair<int, int>> cands;
    if (b.autotune) {
        bool any8 = false;
        for (int i = 0; i < nv; i++) any8 |= ifr::tile_size_supported(views[i].samples, 8, false);
        cands = {{16, 0}, {16, -2}};
        if (any8) {
            cands.push_back({8, 0});
            cands.push_back({8, -2});
        }
    } else {
        cands = {{b.tile_size, b.ctas_per_sm}};
    }
    TargetBackup backup;
    int rc = backup.save(h, views, nv);
    if (rc) return rc;
    bool ran = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cands.size() > 1) {
        IFTR_CUDA(h, cudaEventCreate(&e0));
        IFTR_CUDA(h, cudaEventCreate(&e1));
    }
    float best_ms = 1e30f;
    int best = -1;
    std::vector<ifr::LaunchPlan> seen;
    for (size_t ci = 0; ci < cands.size() && !rc; ci++) {
        BatchBuild bb;
        rc = build_batch(h, views, nv, draws, nd, cands[ci].first, cands[ci].second, bb);
        if (rc) break;
        bool dup = false;
        for (const auto& p : seen) dup |= std::memcmp(&p, &bb.plan, sizeof(p)) == 0;
        if (dup) continue;
        seen.push_back(bb.plan);
        rc = run_sized(h, bb, nd, backup, ran);
        if (rc) break;
        if (cands.size() == 1) {
            best = (int)ci;
            break;
        }
        PassArgs a = batch_args(h, bb, nd);
        cudaEventRecord(e0, h->stream);
        for (int r = 0; r < 2 && !rc; r++) rc = cuda_fail(h, launch_with_status(b.scratch, a, bb.plan, h->stream, nullptr));
        cudaEventRecord(e1, h->stream);
        if (rc) break;
        IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        rc = consume_status(h, b.scratch);
        if (rc == IFTR_ERR_OVERFLOW) {  // cannot happen after a sized run; skip the candidate
            rc = IFTR_OK;
            continue;
        }
        if (!rc && ms < best_ms) {
            best_ms = ms;
            best = (int)ci;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc) return rc;
    if (best < 0) return IFTR_ERR_OVERFLOW;
    b.tuned_tile = cands[best].first;
    b.tuned_ctas = cands[best].second;
    BatchBuild bb;
    rc = build_batch(h, views, nv, draws, nd, b.tuned_tile, b.tuned_ctas, bb);
    if (rc) return rc;
    rc = stage_batch(h, bb);
    if (rc) return rc;
    if (ran) {
        rc = backup.restore(h);
        if (rc) return rc;
    }
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    backup.mem.release();
    // capture on the renderer's private stream (the caller's stream may be the legacy stream)
    if (!b.capture_stream) IFTR_CUDA(h, cudaStreamCreateWithFlags(&b.capture_stream, cudaStreamNonBlocking));
    PassArgs a = batch_args(h, bb, nd);
    IFTR_CUDA(h, cudaStreamBeginCapture(b.capture_stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_with_status(b.scratch, a, bb.plan, b.capture_stream, nullptr);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b.capture_stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(h, e != cudaSuccess ? e : e2);
    }
    b.graph = g;
    IFTR_CUDA(h, cudaGraphInstantiate(&b.exec, g, 0));
    b.captured_generation = b.scratch.generation;
    h->stats.triangles_in = (uint64_t)bb.total_tris;
    return IFTR_OK;
}

}  // namespace

// ============================================================================ C-ABI
extern "C" {

IFTR_API IfritGbRenderer* iftrCreateInstance(void) { return new (std::nothrow) IfritGbRenderer(); }

IFTR_API int iftrDestroyInstance(IfritGbRenderer* h) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (h->inited) {
        cudaStreamSynchronize(h->stream);
        for (DevMem* m : {&h->d_vertices, &h->d_indices, &h->d_color, &h->d_depth, &h->d_vis, &h->d_entries,
                          &h->d_sample_colors, &h->d_keys, &h->d_mesh_meta, &h->d_mesh_vertices, &h->d_mesh_indices})
            m->release();
        h->pass.release();
        h->batch.drop_graph();
        h->batch.scratch.release();
        if (h->batch.capture_stream) cudaStreamDestroy(h->batch.capture_stream);
        for (auto& t : h->tex) t.mem.release();
        for (cudaEvent_t e : h->ev)
            if (e) cudaEventDestroy(e);
        if (h->side.stream) {
            cudaStreamSynchronize(h->side.stream);
            cudaStreamDestroy(h->side.stream);
        }
        if (h->side.fork) cudaEventDestroy(h->side.fork);
        if (h->side.join) cudaEventDestroy(h->side.join);
        if (h->own_stream) cudaStreamDestroy(h->stream);
    }
    delete h;
    return IFTR_OK;
}

IFTR_API int iftrInit(IfritGbRenderer* h) { return h ? ensure_init(h) : IFTR_ERR_INVALID_ARG; }

IFTR_API int iftrBindFrameBuffer(IfritGbRenderer* h, IfritGbFrameBuffer* fb) {
    if (!h || !fb) return IFTR_ERR_INVALID_ARG;
    h->fb = fb;
    return IFTR_OK;
}

IFTR_API int iftrBindVertexBuffer(IfritGbRenderer* h, const IfritGbVertexBuffer* vb) {
    if (!h || !vb) return IFTR_ERR_INVALID_ARG;
    h->vb = vb;
    h->ext_vertices = nullptr;
    return IFTR_OK;
}

IFTR_API int iftrBindIndexBuffer(IfritGbRenderer* h, void* indexBuffer) {
    if (!h || !indexBuffer) return IFTR_ERR_INVALID_ARG;
    h->ib = static_cast<HostBuffer*>(indexBuffer);
    h->ext_indices = nullptr;
    return IFTR_OK;
}

IFTR_API int iftrBindVertexShaderFunc(IfritGbRenderer*, void*, IfritGbVaryingDescriptor*) { return IFTR_ERR_UNSUPPORTED; }
IFTR_API int iftrBindFragmentShaderFunc(IfritGbRenderer*, void*) { return IFTR_ERR_UNSUPPORTED; }
IFTR_API int iftrBindVertexShader(IfritGbRenderer*, void*) { return IFTR_ERR_UNSUPPORTED; }
IFTR_API int iftrBindFragmentShader(IfritGbRenderer*, void*) { return IFTR_ERR_UNSUPPORTED; }

IFTR_API int iftrBindVertexShaderBuiltin(IfritGbRenderer* h, int kind, const IfritGbVaryingDescriptor* vd) {
    if (!h || kind != IFTR_VS_MVP_TRANSFORM) return IFTR_ERR_INVALID_ARG;
    if (vd && vd->desc.size() > 1) return IFTR_ERR_UNSUPPORTED;
    return IFTR_OK;
}

IFTR_API int iftrBindFragmentShaderBuiltin(IfritGbRenderer* h, int model) {
    if (!h || model < IFTR_FS_GOURAUD || model > IFTR_FS_PRIMITIVE_ID) return IFTR_ERR_INVALID_ARG;
    h->fs_model = model;
    return IFTR_OK;
}

IFTR_API int iftrBindUniformBuffer(IfritGbRenderer* h, int binding, int set, void* buffer) {
    if (!h || !buffer) return IFTR_ERR_INVALID_ARG;
    if (binding != 0 || set != 0) return IFTR_ERR_UNSUPPORTED;
    h->uniform_mvp = static_cast<HostBuffer*>(buffer);
    return IFTR_OK;
}

IFTR_API int iftrSetUniformMatrix(IfritGbRenderer* h, const float* m) {
    if (!h || !m) return IFTR_ERR_INVALID_ARG;
    std::memcpy(h->mvp, m, sizeof(h->mvp));
    h->uniform_mvp = nullptr;
    return IFTR_OK;
}

IFTR_API int iftrSetBlendFunc(IfritGbRenderer* h, const IfritGbBlendState* s) {
    if (!h || !s) return IFTR_ERR_INVALID_ARG;
    for (int f : {s->srcColorBlendFactor, s->dstColorBlendFactor, s->srcAlphaBlendFactor, s->dstAlphaBlendFactor})
        if (f < 0 || f > 9) return IFTR_ERR_INVALID_ARG;
    h->blend = *s;
    return IFTR_OK;
}

IFTR_API int iftrSetDepthFunc(IfritGbRenderer* h, int op) {
    if (!h || op < 0 || op > 7) return IFTR_ERR_INVALID_ARG;
    h->depth_func = op;
    return IFTR_OK;
}

IFTR_API int iftrOptsetForceDeterministic(IfritGbRenderer* h, int) { return h ? IFTR_OK : IFTR_ERR_INVALID_ARG; }

IFTR_API int iftrOptSetDepthTestEnable(IfritGbRenderer* h, int opt) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    h->depth_test = opt != 0;
    return IFTR_OK;
}

IFTR_API int iftrSetDepthWriteEnable(IfritGbRenderer* h, int enable) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    h->depth_write = enable != 0;
    return IFTR_OK;
}

IFTR_API int iftrDrawBatch(IfritGbRenderer* h, const IfritGbBatchView* views, int numViews, const IfritGbBatchDraw* draws,
                           int numDraws) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (h->in_pass) return IFTR_ERR_STATE;
    int rc = validate_batch(views, numViews, draws, numDraws);
    if (rc) return rc;
    rc = ensure_init(h);
    if (rc) return rc;
    BatchState& b = h->batch;
    std::vector<uint8_t> key = batch_key(b, views, numViews, draws, numDraws);
    if (!(b.exec && b.captured_generation == b.scratch.generation && key == b.key)) {
        rc = prepare_batch(h, views, numViews, draws, numDraws);
        if (rc) {
            b.drop_graph();
            return rc;
        }
        b.key = std::move(key);
    }
    IFTR_CUDA(h, cudaGraphLaunch(b.exec, h->stream));
    h->pending_batch = 1;
    return IFTR_OK;
}

IFTR_API int iftrSetBatchTuning(IfritGbRenderer* h, int autotune, int tileSize, int ctasPerSm) {
    if (!h || (tileSize != 8 && tileSize != 16) || ctasPerSm < -8 || ctasPerSm > 64) return IFTR_ERR_INVALID_ARG;
    h->batch.autotune = autotune != 0;
    h->batch.tile_size = tileSize;
    h->batch.ctas_per_sm = ctasPerSm;
    return IFTR_OK;
}

IFTR_API int iftrGetBatchTuning(IfritGbRenderer* h, int* tileSize, int* ctasPerSm) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (tileSize) *tileSize = h->batch.tuned_tile;
    if (ctasPerSm) *ctasPerSm = h->batch.tuned_ctas;
    return IFTR_OK;
}

IFTR_API int iftrDrawAsync(IfritGbRenderer* h, int numIndices, int clear) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    return enqueue_draw(h, numIndices, clear);
}

IFTR_API int iftrFinish(IfritGbRenderer* h) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (!h->inited) return IFTR_OK;
    return check_pending(h);
}

// Renders one prepared pass synchronously; a pass whose tile lists overflowed is drawn again with
// the grown scratch (clearing passes only).
int draw_sync(IfritGbRenderer* h, std::vector<DrawDev>& draws, int clear) {
    h->stats.retries = 0;
    for (int attempt = 0; attempt < 4; attempt++) {
        int rc = enqueue_pass(h, draws, clear);
        if (rc) return rc;
        rc = check_pending(h);
        if (rc == IFTR_ERR_OVERFLOW) {
            h->stats.retries++;
            if (!clear) return rc;  // the pass may have partially updated depth; caller decides
            continue;
        }
        if (rc) return rc;
        return copy_back_host_images(h);
    }
    return IFTR_ERR_OVERFLOW;
}

IFTR_API int iftrDrawLegacy(IfritGbRenderer* h, int numIndices, int clear) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (h->in_pass) return iftrPassDraw(h, 0, numIndices);
    int rc = ensure_init(h);
    if (rc) return rc;
    std::vector<DrawDev> one(1);
    rc = prepare_draw(h, 0, numIndices, one[0]);
    if (rc) return rc;
    return draw_sync(h, one, clear);
}

IFTR_API int iftrDrawMeshOutputs(IfritGbRenderer* h, int numGroups, const float* positions, const float* attributes,
                                 int attrCount, const int* indices, const int* numVertices, const int* numIndices,
                                 int maxVertices, int maxIndices, int clear) {
    if (!h || numGroups < 0 || maxVertices <= 0 || maxIndices <= 0 || attrCount < 0 || attrCount > 4 ||
        (numGroups > 0 && (!positions || !indices || !numVertices || !numIndices)) || (attrCount > 0 && !attributes))
        return IFTR_ERR_INVALID_ARG;
    if (h->in_pass) return IFTR_ERR_STATE;
    int rc = ensure_init(h);
    if (rc) return rc;
    long long totals[3] = {0, 0, 0};
    if (numGroups > 0) {
        const size_t meta = ((size_t)2 * numGroups * sizeof(int) + 15) / 16 * 16;
        IFTR_CUDA(h, h->d_mesh_meta.reserve(meta + 3 * sizeof(long long)));
        int* off_v = h->d_mesh_meta.as<int>();
        int* off_i = off_v + numGroups;
        long long* d_totals = reinterpret_cast<long long*>(h->d_mesh_meta.as<uint8_t>() + meta);
        IFTR_CUDA(h, ifr::launch_mesh_offsets(numVertices, numIndices, numGroups, maxVertices, maxIndices, off_v, off_i,
                                              d_totals, h->stream));
        IFTR_CUDA(h, cudaMemcpyAsync(totals, d_totals, sizeof(totals), cudaMemcpyDeviceToHost, h->stream));
        IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
        if (totals[2] || totals[0] > (1 << 27) || totals[1] > (1LL << 30)) return IFTR_ERR_INVALID_ARG;
        IFTR_CUDA(h, h->d_mesh_vertices.reserve(std::max<size_t>(16, (size_t)totals[0] * 8 * sizeof(float))));
        IFTR_CUDA(h, h->d_mesh_indices.reserve(std::max<size_t>(16, (size_t)totals[1] * sizeof(int))));
        IFTR_CUDA(h, ifr::launch_mesh_compact(positions, attrCount > 0 ? attributes : nullptr, indices, numVertices,
                                              numIndices, off_v, off_i, numGroups, maxVertices, maxIndices,
                                              h->d_mesh_vertices.as<float>(), h->d_mesh_indices.as<int>(), h->stream));
    }
    std::vector<DrawDev> one(1);
    DrawDev& d = one[0];
    std::memset(&d, 0, sizeof(d));
    d.vertices = h->d_mesh_vertices.as<float>();
    d.stride = 8;
    d.num_vertices = (int)totals[0];
    d.attr_offset = 4;
    d.attr_count = attrCount;
    d.indices = h->d_mesh_indices.as<int>();
    d.num_triangles = (int)(totals[1] / 3);
    fill_state(h, d);
    d.clip_input = 1;
    if (d.shading == IFTR_FS_TEXTURED && (!d.texels || d.tex_levels <= 0)) return IFTR_ERR_STATE;
    return draw_sync(h, one, clear);
}

IFTR_API int iftrBeginPass(IfritGbRenderer* h, int clear) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (h->in_pass) return IFTR_ERR_STATE;
    int rc = ensure_init(h);
    if (rc) return rc;
    h->in_pass = true;
    h->pass_clear = clear;
    h->pass_draws.clear();
    return IFTR_OK;
}

IFTR_API int iftrPassDraw(IfritGbRenderer* h, int firstIndex, int numIndices) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (!h->in_pass) return IFTR_ERR_STATE;
    if (h->pass_draws.size() >= (size_t)ifr::kMaxDraws) return IFTR_ERR_INVALID_ARG;
    DrawDev d;
    int rc = prepare_draw(h, firstIndex, numIndices, d);
    if (rc) return rc;
    h->pass_draws.push_back(d);
    return IFTR_OK;
}

IFTR_API int iftrEndPass(IfritGbRenderer* h) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (!h->in_pass) return IFTR_ERR_STATE;
    h->in_pass = false;
    if (h->pass_draws.empty()) return h->pass_clear ? iftrClear(h) : IFTR_OK;
    h->stats.retries = 0;
    for (int attempt = 0; attempt < 4; attempt++) {
        std::vector<DrawDev> draws = h->pass_draws;
        int rc = enqueue_pass(h, draws, h->pass_clear);
        if (rc) return rc;
        rc = check_pending(h);
        if (rc == IFTR_ERR_OVERFLOW) {
            h->stats.retries++;
            if (!h->pass_clear) return rc;
            continue;
        }
        if (rc) return rc;
        return copy_back_host_images(h);
    }
    return IFTR_ERR_OVERFLOW;
}

IFTR_API int iftrClear(IfritGbRenderer* h) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    int rc = enqueue_draw(h, 0, 1);
    if (rc) return rc;
    rc = check_pending(h);
    return rc ? rc : copy_back_host_images(h);
}

IFTR_API int iftrSetScissors(IfritGbRenderer* h, const float* rects, int count) {
    if (!h || count < 0 || count > 16 || (count > 0 && !rects)) return IFTR_ERR_INVALID_ARG;
    h->scissors.assign(rects, rects + 4 * count);
    return IFTR_OK;
}

IFTR_API int iftrSetRasterPath(IfritGbRenderer* h, int path) {
    if (!h || (path != IFTR_RASTER_TILED && path != IFTR_RASTER_ATOMIC)) return IFTR_ERR_INVALID_ARG;
    h->raster_path = path;
    return IFTR_OK;
}

IFTR_API int iftrSetRasterizerPolygonMode(IfritGbRenderer* h, int mode) {
    if (!h || mode < IF_POLYGON_MODE_FILL || mode > IF_POLYGON_MODE_POINT) return IFTR_ERR_INVALID_ARG;
    h->polygon_mode = mode;
    return IFTR_OK;
}

IFTR_API int iftrSetOrderedFragmentCapacity(IfritGbRenderer* h, long long fragments) {
    if (!h || fragments < -1 || fragments > 0xFFFFFFF0LL) return IFTR_ERR_INVALID_ARG;
    if (h->in_pass) return IFTR_ERR_STATE;
    h->frag_capacity_setting = fragments;
    return IFTR_OK;
}

IFTR_API int iftrSetPolygonRules(IfritGbRenderer* h, int rules) {
    if (!h || (rules != IFTR_POLYGON_RULES_FILL_PARTS && rules != IFTR_POLYGON_RULES_REFERENCE))
        return IFTR_ERR_INVALID_ARG;
    h->polygon_rules = rules;
    return IFTR_OK;
}

IFTR_API int iftrSetScissorTestEnable(IfritGbRenderer* h, int enable) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    h->scissor_enable = enable != 0;
    return IFTR_OK;
}

IFTR_API int iftrSetCullMode(IfritGbRenderer* h, int m) {
    if (!h || m < 0 || m > 3) return IFTR_ERR_INVALID_ARG;
    h->cull_mode = m;
    return IFTR_OK;
}

IFTR_API int iftrSetFrontFace(IfritGbRenderer* h, int ccw) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    h->front_ccw = ccw != 0;
    return IFTR_OK;
}

IFTR_API int iftrSetMsaaSamples(IfritGbRenderer* h, int s) {
    if (!h || !(s == 1 || s == 2 || s == 4 || s == 8 || s == 16)) return IFTR_ERR_INVALID_ARG;
    h->samples = s;
    return IFTR_OK;
}

IFTR_API int iftrSetClearValues(IfritGbRenderer* h, const float* rgba, float depth) {
    if (!h || !rgba) return IFTR_ERR_INVALID_ARG;
    std::memcpy(h->clear_color, rgba, sizeof(h->clear_color));
    h->clear_depth = depth;
    return IFTR_OK;
}

IFTR_API int iftrCreateTexture(IfritGbRenderer* h, int slot, int width, int height, int mipLevels) {
    if (!h || slot < 0 || slot >= 16 || width <= 0 || height <= 0 || width > 16384 || height > 16384) return IFTR_ERR_INVALID_ARG;
    int rc = ensure_init(h);
    if (rc) return rc;
    int full = 0, w = width, hh = height;
    size_t total = 0;
    for (;;) {
        total += (size_t)w * hh;
        full++;
        if (w == 1 && hh == 1) break;
        w = (w + 1) >> 1;
        hh = (hh + 1) >> 1;
    }
    int levels = (mipLevels <= 0 || mipLevels > full) ? full : mipLevels;
    Texture& t = h->tex[slot];
    IFTR_CUDA(h, t.mem.reserve(total * 4));
    IFTR_CUDA(h, cudaMemsetAsync(t.mem.p, 0, total * 4, h->stream));
    t.w = width;
    t.h = height;
    t.levels = levels;
    return IFTR_OK;
}

IFTR_API int iftrCopyHostBufferToImage(IfritGbRenderer* h, const void* rgba8, int slot) {
    if (!h || !rgba8 || slot < 0 || slot >= 16 || !h->tex[slot].mem.p) return IFTR_ERR_INVALID_ARG;
    Texture& t = h->tex[slot];
    IFTR_CUDA(h, cudaMemcpyAsync(t.mem.p, rgba8, (size_t)t.w * t.h * 4, cudaMemcpyHostToDevice, h->stream));
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    return IFTR_OK;
}

IFTR_API int iftrGenerateMipmap(IfritGbRenderer* h, int slot, int filter) {
    if (!h || slot < 0 || slot >= 16 || !h->tex[slot].mem.p) return IFTR_ERR_INVALID_ARG;
    (void)filter;  // 2x2 box filter (the reference blits bilinearly at exactly half size)
    Texture& t = h->tex[slot];
    int w = t.w, hh = t.h;
    uint32_t* base = t.mem.as<uint32_t>();
    size_t off = 0;
    for (int l = 1; l < t.levels; l++) {
        int nw = (w + 1) >> 1, nh = (hh + 1) >> 1;
        IFTR_CUDA(h, ifr::launch_mip_level(base + off, w, hh, base + off + (size_t)w * hh, nw, nh, h->stream));
        off += (size_t)w * hh;
        w = nw;
        hh = nh;
    }
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    return IFTR_OK;
}

IFTR_API int iftrCreateSampler(IfritGbRenderer* h, int slot, const IfritGbSampler* s) {
    if (!h || !s || slot < 0 || slot >= 16) return IFTR_ERR_INVALID_ARG;
    int rc = ensure_init(h);
    if (rc) return rc;
    h->samplers[slot] = *s;
    return IFTR_OK;
}

IFTR_API int iftrBindTexture(IfritGbRenderer* h, int tslot, int sslot) {
    if (!h || tslot < 0 || tslot >= 16 || sslot < 0 || sslot >= 16) return IFTR_ERR_INVALID_ARG;
    h->bound_tex = tslot;
    h->bound_sampler = sslot;
    return IFTR_OK;
}

IFTR_API int iftrSetStream(IfritGbRenderer* h, void* stream) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (h->inited) cudaStreamSynchronize(h->stream);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    h->stream = static_cast<cudaStream_t>(stream);
    h->own_stream = false;
    return IFTR_OK;
}

IFTR_API int iftrBindVertexBufferDevice(IfritGbRenderer* h, const float* v, int stride, int n, int off, int cnt) {
    if (!h || !v || stride < 3 || n < 0 || off < 0 || cnt < 0 || cnt > 4 || off + cnt > stride) return IFTR_ERR_INVALID_ARG;
    h->ext_vertices = v;
    h->ext_stride = stride;
    h->ext_nverts = n;
    h->ext_attr_off = off;
    h->ext_attr_cnt = cnt;
    return IFTR_OK;
}

IFTR_API int iftrBindIndexBufferDevice(IfritGbRenderer* h, const int* idx, int n) {
    if (!h || !idx || n < 0) return IFTR_ERR_INVALID_ARG;
    h->ext_indices = idx;
    h->ext_nidx = n;
    return IFTR_OK;
}

IFTR_API int iftrSetVisibilityOutput(IfritGbRenderer* h, int enable) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    h->vis_output = enable != 0;
    return IFTR_OK;
}

IFTR_API int iftrReserve(IfritGbRenderer* h, size_t pairs) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    int rc = ensure_init(h);
    return rc ? rc : ensure_pairs(h, h->pass, pairs);
}

IFTR_API int iftrGetDeviceAttachments(IfritGbRenderer* h, void** color, float** depth, int** vis) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (color) *color = h->d_color.p;
    if (depth) *depth = h->d_depth.as<float>();
    if (vis) *vis = h->vis_output ? h->d_vis.as<int>() : nullptr;
    return IFTR_OK;
}

IFTR_API int iftrReadbackColor(IfritGbRenderer* h, void* dst, size_t bytes) {
    if (!h || !dst || h->att_fmt < 0) return IFTR_ERR_INVALID_ARG;
    size_t need = (size_t)h->att_w * h->att_h * color_bytes(h->att_fmt);
    if (bytes < need) return IFTR_ERR_INVALID_ARG;
    IFTR_CUDA(h, cudaMemcpyAsync(dst, h->d_color.p, need, cudaMemcpyDeviceToHost, h->stream));
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    return IFTR_OK;
}

IFTR_API int iftrReadbackDepth(IfritGbRenderer* h, float* dst, size_t count) {
    if (!h || !dst || h->att_fmt < 0) return IFTR_ERR_INVALID_ARG;
    size_t need = (size_t)h->att_w * h->att_h * h->att_s;
    if (count < need) return IFTR_ERR_INVALID_ARG;
    IFTR_CUDA(h, cudaMemcpyAsync(dst, h->d_depth.p, need * 4, cudaMemcpyDeviceToHost, h->stream));
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    return IFTR_OK;
}

IFTR_API int iftrReadbackVisibility(IfritGbRenderer* h, int* dst, size_t count) {
    if (!h || !dst || h->att_fmt < 0 || !h->vis_output || !h->d_vis.p) return IFTR_ERR_STATE;
    size_t need = (size_t)h->att_w * h->att_h * h->att_s;
    if (count < need) return IFTR_ERR_INVALID_ARG;
    IFTR_CUDA(h, cudaMemcpyAsync(dst, h->d_vis.p, need * 4, cudaMemcpyDeviceToHost, h->stream));
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    return IFTR_OK;
}

IFTR_API int iftrGetStats(IfritGbRenderer* h, IfritGbStats* out) {
    if (!h || !out) return IFTR_ERR_INVALID_ARG;
    *out = h->stats;
    return IFTR_OK;
}

IFTR_API int iftrSetStageTiming(IfritGbRenderer* h, int enable) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    int rc = ensure_init(h);
    if (rc) return rc;
    if (enable && !h->ev[0])
        for (auto& e : h->ev) IFTR_CUDA(h, cudaEventCreate(&e));
    h->timing = enable != 0;
    return IFTR_OK;
}

IFTR_API int iftrGetStageTimes(IfritGbRenderer* h, float* ms, int n) {
    if (!h || !ms || n < 0) return IFTR_ERR_INVALID_ARG;
    for (int i = 0; i < n && i + 1 < ifr::kStageEvents; i++) ms[i] = h->stage_ms[i];
    return IFTR_OK;
}

IFTR_API const char* iftrGetErrorString(int status) {
    switch (status) {
    case IFTR_OK: return "ok";
    case IFTR_ERR_INVALID_ARG: return "invalid argument";
    case IFTR_ERR_UNSUPPORTED: return "unsupported";
    case IFTR_ERR_CUDA: return "CUDA error";
    case IFTR_ERR_OVERFLOW: return "scratch capacity exceeded";
    case IFTR_ERR_NO_DEVICE: return "no CUDA device";
    case IFTR_ERR_STATE: return "missing binding";
    default: return "unknown status";
    }
}

// ---- framebuffers / images
IFTR_API IfritGbFrameBuffer* iftrCreateFrameBuffer(void) { return new (std::nothrow) IfritGbFrameBuffer(); }
IFTR_API int iftrDestroyFrameBuffer(IfritGbFrameBuffer* fb) {
    if (!fb) return IFTR_ERR_INVALID_ARG;
    delete fb;
    return IFTR_OK;
}
IFTR_API int iftrSetFrameBufferColorAttachmentFP32(IfritGbFrameBuffer* fb, IfritGbImageF32* const* images, size_t n) {
    if (!fb || (n && !images)) return IFTR_ERR_INVALID_ARG;
    fb->color.assign(images, images + n);
    fb->dev_format = -1;
    return IFTR_OK;
}
IFTR_API int iftrSetFrameBufferDepthAttachmentFP32(IfritGbFrameBuffer* fb, IfritGbImageF32* image) {
    if (!fb) return IFTR_ERR_INVALID_ARG;
    fb->depth = image;
    return IFTR_OK;
}
IFTR_API int iftrSetFrameBufferColorAttachmentDevice(IfritGbFrameBuffer* fb, int format, int w, int h) {
    if (!fb || format < 0 || format > 3 || w <= 0 || h <= 0 || w > 16384 || h > 16384) return IFTR_ERR_INVALID_ARG;
    fb->dev_format = format;
    fb->dev_w = w;
    fb->dev_h = h;
    return IFTR_OK;
}
IFTR_API IfritGbImageF32* ifcrCreateImageFP32(size_t w, size_t h, size_t c) {
    IfritGbImageF32* img = new (std::nothrow) IfritGbImageF32();
    if (!img) return nullptr;
    img->w = w; img->h = h; img->c = c;
    try { img->data.assign(w * h * c, 0.0f); } catch (...) { delete img; return nullptr; }
    return img;
}
IFTR_API int ifcrDestroyImageFP32(IfritGbImageF32* img) {
    if (!img) return IFTR_ERR_INVALID_ARG;
    delete img;
    return IFTR_OK;
}
IFTR_API float* ifcrGetImageRawDataFP32(IfritGbImageF32* img) { return img ? img->data.data() : nullptr; }

// ---- varying descriptors / vertex buffers
IFTR_API IfritGbVaryingDescriptor* iftrCreateVaryingDescriptor(void) { return new (std::nothrow) IfritGbVaryingDescriptor(); }
IFTR_API int iftrDestroyVaryingDescriptor(IfritGbVaryingDescriptor* vd) {
    if (!vd) return IFTR_ERR_INVALID_ARG;
    delete vd;
    return IFTR_OK;
}
IFTR_API int iftrWriteVaryingDescriptor(IfritGbVaryingDescriptor* vd, const int* desc, size_t n) {
    if (!vd || (n && !desc)) return IFTR_ERR_INVALID_ARG;
    vd->desc.assign(desc, desc + n);
    return IFTR_OK;
}
IFTR_API IfritGbVertexBuffer* iftrCreateVertexBuffer(void) { return new (std::nothrow) IfritGbVertexBuffer(); }
IFTR_API int iftrDestroyVertexBuffer(IfritGbVertexBuffer* vb) {
    if (!vb) return IFTR_ERR_INVALID_ARG;
    delete vb;
    return IFTR_OK;
}
IFTR_API int iftrSetVertexBufferLayout(IfritGbVertexBuffer* vb, const int* desc, size_t n) {
    if (!vb || !desc || n == 0) return IFTR_ERR_INVALID_ARG;
    if (type_components(desc[0]) < 3) return IFTR_ERR_UNSUPPORTED;  // attribute 0 is the position
    vb->layout.assign(desc, desc + n);
    vb->offsets.clear();
    int off = 0;
    for (int t : vb->layout) {
        int comps = type_components(t);
        if (comps == 0) return IFTR_ERR_INVALID_ARG;
        vb->offsets.push_back(off);
        off += 4 * comps;
    }
    vb->elem_size = off;
    vb->generation = ++g_id_counter;
    return IFTR_OK;
}
IFTR_API int iftrSetVertexBufferSize(IfritGbVertexBuffer* vb, size_t n) {
    if (!vb) return IFTR_ERR_INVALID_ARG;
    vb->count = n;
    return IFTR_OK;
}
IFTR_API int iftrAllocateVertexBuffer(IfritGbVertexBuffer* vb) {
    if (!vb || vb->elem_size == 0) return IFTR_ERR_STATE;
    if (!vb->data.assign(vb->count * vb->elem_size)) return IFTR_ERR_INVALID_ARG;
    vb->generation = ++g_id_counter;
    return IFTR_OK;
}
IFTR_API int iftrSetVertexBufferValueFloat4(IfritGbVertexBuffer* vb, int index, int attr, void* value) {
    if (!vb || !value || index < 0 || (size_t)index >= vb->count || attr < 0 || (size_t)attr >= vb->layout.size())
        return IFTR_ERR_INVALID_ARG;
    int comps = type_components(vb->layout[attr]);
    std::memcpy(vb->data.data() + (size_t)index * vb->elem_size + vb->offsets[attr], value, 4 * comps);
    vb->generation = ++g_id_counter;
    return IFTR_OK;
}
IFTR_API int iftrSetVertexBufferData(IfritGbVertexBuffer* vb, const void* src, size_t bytes) {
    if (!vb || !src || bytes != vb->data.size()) return IFTR_ERR_INVALID_ARG;
    std::memcpy(vb->data.data(), src, bytes);
    vb->generation = ++g_id_counter;
    return IFTR_OK;
}

IFTR_API void* iftrGetVertexBufferRawData(IfritGbVertexBuffer* vb) { return vb ? vb->data.data() : nullptr; }
IFTR_API int iftrSetVertexBufferDirty(IfritGbVertexBuffer* vb) {
    if (!vb) return IFTR_ERR_INVALID_ARG;
    vb->generation = ++g_id_counter;
    return IFTR_OK;
}

// ---- buffer manager
IFTR_API void* ifbufCreateBufferManager(void) { return new (std::nothrow) BufferManager(); }
IFTR_API int ifbufDestroyBufferManager(void* m) {
    if (!m) return IFTR_ERR_INVALID_ARG;
    BufferManager* bm = static_cast<BufferManager*>(m);
    for (HostBuffer* b : bm->buffers) delete b;
    delete bm;
    return IFTR_OK;
}
IFTR_API void* ifbufCreateBuffer(void* m, size_t size) {
    if (!m) return nullptr;
    HostBuffer* b = new (std::nothrow) HostBuffer();
    if (!b) return nullptr;
    if (!b->data.assign(size)) { delete b; return nullptr; }
    b->generation = ++g_id_counter;
    static_cast<BufferManager*>(m)->buffers.push_back(b);
    return b;
}
IFTR_API int ifbufDestroyBuffer(void* buf) {
    // buffers are owned by their manager (TrivialBufferManager semantics); release the bytes
    if (!buf) return IFTR_ERR_INVALID_ARG;
    HostBuffer* b = static_cast<HostBuffer*>(buf);
    b->data.release();
    b->generation = ++g_id_counter;
    return IFTR_OK;
}
IFTR_API int ifbufBufferData(void* buf, const void* data, size_t offset, size_t size) {
    if (!buf || (size && !data)) return IFTR_ERR_INVALID_ARG;
    HostBuffer* b = static_cast<HostBuffer*>(buf);
    if (offset + size > b->data.size()) return IFTR_ERR_INVALID_ARG;
    std::memcpy(b->data.data() + offset, data, size);
    b->generation = ++g_id_counter;
    return IFTR_OK;
}

IFTR_API void* ifbufGetBufferRawData(void* buf) { return buf ? static_cast<HostBuffer*>(buf)->data.data() : nullptr; }
IFTR_API int ifbufSetBufferDirty(void* buf) {
    if (!buf) return IFTR_ERR_INVALID_ARG;
    static_cast<HostBuffer*>(buf)->generation = ++g_id_counter;
    return IFTR_OK;
}

}  // extern "C"
