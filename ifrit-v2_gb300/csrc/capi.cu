// Host runtime of the GB300 rasterizer behind the C-ABI in include/ifrit_gb300.h.
//
// Mirrors the reference's host API shape (TileRasterRenderer / TileRasterRendererCuda and the
// iftr*/ifcr*/ifbuf* exports): caller-owned framebuffer, vertex buffer and image objects are
// bound by pointer; the renderer owns the device copies and all scratch.  Device state stays
// resident across draws: host vertex/index data are uploaded only when their contents
// change, attachments are reallocated only when the framebuffer geometry changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/ifrit_gb300.h"
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

}  // namespace

struct IfritGbRenderer {
    bool inited = false;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
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
    // device state
    DevMem d_vertices, d_indices, d_color, d_depth, d_vis, d_entries;
    const void* up_vb_key = nullptr;
    uint64_t up_vb_gen = 0;
    const void* up_ib_key = nullptr;
    uint64_t up_ib_gen = 0;
    int att_w = 0, att_h = 0, att_s = 0, att_fmt = -1;
    DevMem d_tile_count, d_tile_offset, d_tile_cursor, d_pairs, d_status, d_draws, d_draw_start, d_records;
    int tiles_alloc = 0;
    uint32_t pair_capacity = 0;
    uint32_t* h_status = nullptr;  // pinned
    DrawDev* h_draws = nullptr;    // pinned staging
    int* h_draw_start = nullptr;   // pinned staging
    Texture tex[16];
    IfritGbSampler samplers[16];
    int bound_tex = 0, bound_sampler = 0;
    IfritGbStats stats{};
    bool timing = false;
    cudaEvent_t ev[6] = {};
    float stage_ms[5] = {0, 0, 0, 0, 0};
    std::string last_error;
    int pending = 0;  // an async pass whose status has not been checked
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
        std::vector<float> init(1, h->clear_depth);
        // depth starts at the clear value
        std::vector<float> dv(npix * S, h->clear_depth);
        IFTR_CUDA(h, cudaMemcpyAsync(h->d_depth.p, dv.data(), dv.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
        IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    int tx = (W + ifr::kTileSize - 1) / ifr::kTileSize, ty = (H + ifr::kTileSize - 1) / ifr::kTileSize;
    int T = tx * ty;
    if (T > h->tiles_alloc) {
        IFTR_CUDA(h, h->d_tile_count.reserve((size_t)T * 4));
        IFTR_CUDA(h, h->d_tile_offset.reserve((size_t)(T + 1) * 4));
        IFTR_CUDA(h, h->d_tile_cursor.reserve((size_t)T * 4));
        IFTR_CUDA(h, cudaMemsetAsync(h->d_tile_count.p, 0, (size_t)T * 4, h->stream));
        h->tiles_alloc = T;
    }
    return IFTR_OK;
}

int ensure_pairs(IfritGbRenderer* h, size_t want) {
    if (want <= h->pair_capacity) return IFTR_OK;
    if (want > 0x7fffffffu) return IFTR_ERR_OVERFLOW;
    IFTR_CUDA(h, h->d_pairs.reserve(want * 4));
    h->pair_capacity = (uint32_t)want;
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
    d.blend_enable = h->blend.blendEnable;
    d.blend_src_color = h->blend.srcColorBlendFactor;
    d.blend_dst_color = h->blend.dstColorBlendFactor;
    d.blend_src_alpha = h->blend.srcAlphaBlendFactor;
    d.blend_dst_alpha = h->blend.dstAlphaBlendFactor;
    d.shading = h->fs_model;
    const Texture& t = h->tex[h->bound_tex];
    d.texels = t.mem.as<uint32_t>();
    d.tex_w = t.w;
    d.tex_h = t.h;
    d.tex_levels = t.levels;
    const IfritGbSampler& s = h->samplers[h->bound_sampler];
    d.sampler.address_u = s.addressModeU;
    d.sampler.address_v = s.addressModeV;
    d.sampler.filter = s.filterMode;
    d.sampler.border_white = s.borderColor;
    d.sampler.max_aniso = s.anisotropyEnable ? std::max(1, (int)s.maxAnisotropy) : 1;
    d.sampler.lod_bias = s.lodBias;
    int w = t.w, hh = t.h, off = 0;
    for (int l = 0; l < 16; l++) {
        d.lvl_off[l] = off;
        d.lvl_w[l] = w;
        d.lvl_h[l] = hh;
        off += w * hh;
        w = (w + 1) >> 1;
        hh = (hh + 1) >> 1;
        if (w < 1) w = 1;
        if (hh < 1) hh = 1;
    }
}

void sample_table(int S, int* xs, int* ys) {
    static const int SP1[2] = {128, 128};
    static const int SP2[4] = {192, 192, 64, 64};
    static const int SP4[8] = {96, 32, 224, 96, 32, 160, 160, 224};
    static const int SP8[16] = {144, 80, 112, 176, 208, 144, 80, 48, 48, 208, 16, 112, 176, 240, 240, 16};
    static const int SP16[32] = {144, 144, 112, 80, 80, 160, 192, 112, 48, 96, 160, 208, 208, 176, 176, 48,
                                 96, 224, 128, 16, 64, 32, 32, 192, 0, 128, 240, 64, 224, 240, 16, 0};
    const int* t = S == 1 ? SP1 : S == 2 ? SP2 : S == 4 ? SP4 : S == 8 ? SP8 : SP16;
    for (int k = 0; k < S; k++) { xs[k] = t[2 * k]; ys[k] = t[2 * k + 1]; }
}

void fill_pass_const(ifr::PassConst& c, int W, int H, int S) {
    std::memset(&c, 0, sizeof(c));
    c.W = W; c.H = H; c.S = S;
    c.tiles_x = (W + ifr::kTileSize - 1) / ifr::kTileSize;
    c.tiles_y = (H + ifr::kTileSize - 1) / ifr::kTileSize;
    sample_table(S, c.sx, c.sy);
    c.smin_x = c.smax_x = c.sx[0];
    c.smin_y = c.smax_y = c.sy[0];
    for (int k = 1; k < S; k++) {
        c.smin_x = std::min(c.smin_x, c.sx[k]); c.smax_x = std::max(c.smax_x, c.sx[k]);
        c.smin_y = std::min(c.smin_y, c.sy[k]); c.smax_y = std::max(c.smax_y, c.sy[k]);
    }
    c.shade_x = 128;
    c.shade_y = 128;
    c.W256 = (float)W * 256.0f;
    c.H256 = (float)H * 256.0f;
    c.gx = (float)(1.0 + 2.0 * 8192.0 / (double)W);
    c.gy = (float)(1.0 + 2.0 * 8192.0 / (double)H);
}

int ensure_init(IfritGbRenderer* h) {
    if (h->inited) return IFTR_OK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return IFTR_ERR_NO_DEVICE;
    if (!h->stream) {
        IFTR_CUDA(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    IFTR_CUDA(h, cudaMallocHost(&h->h_status, ifr::ST_WORDS * sizeof(uint32_t)));
    IFTR_CUDA(h, cudaMallocHost(&h->h_draws, ifr::kMaxDraws * sizeof(DrawDev)));
    IFTR_CUDA(h, cudaMallocHost(&h->h_draw_start, (ifr::kMaxDraws + 1) * sizeof(int)));
    IFTR_CUDA(h, h->d_status.reserve(ifr::ST_WORDS * sizeof(uint32_t)));
    IFTR_CUDA(h, h->d_draws.reserve(ifr::kMaxDraws * sizeof(DrawDev)));
    IFTR_CUDA(h, h->d_draw_start.reserve((ifr::kMaxDraws + 1) * sizeof(int)));
    std::memset(h->h_status, 0, ifr::ST_WORDS * sizeof(uint32_t));
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

// Enqueues one pass of draws on the renderer's stream.
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
    int64_t total = 0;
    bool ordered = false;
    for (size_t i = 0; i < draws.size(); i++) {
        DrawDev& d = draws[i];
        d.prim_base = (int)total;
        h->h_draw_start[i] = (int)total;
        total += d.num_triangles;
        if (d.blend_enable || (d.depth_write && d.depth_func == IF_COMPARE_OP_NOT_EQUAL) ||
            d.depth_func != draws[0].depth_func || d.depth_write != draws[0].depth_write)
            ordered = true;
        h->h_draws[i] = d;
    }
    if (total >= (int64_t)1 << 28) return IFTR_ERR_INVALID_ARG;  // entry = triangle << 3 | fan index
    h->h_draw_start[draws.size()] = (int)total;
    IFTR_CUDA(h, cudaMemcpyAsync(h->d_draws.p, h->h_draws, draws.size() * sizeof(DrawDev), cudaMemcpyHostToDevice, h->stream));
    IFTR_CUDA(h, cudaMemcpyAsync(h->d_draw_start.p, h->h_draw_start, (draws.size() + 1) * sizeof(int),
                                 cudaMemcpyHostToDevice, h->stream));
    if (h->pair_capacity == 0) {
        rc = ensure_pairs(h, std::max<size_t>(1u << 20, (size_t)total * 4));
        if (rc) return rc;
    }
    IFTR_CUDA(h, h->d_records.reserve(std::max<size_t>(1, (size_t)total) * sizeof(ifr::TriRecord)));
    IFTR_CUDA(h, cudaMemsetAsync(h->d_status.p, 0, ifr::ST_WORDS * sizeof(uint32_t), h->stream));
    PassArgs a;
    std::memset(&a, 0, sizeof(a));
    fill_pass_const(a.c, W, H, S);
    a.draws = h->d_draws.as<DrawDev>();
    a.draw_start = h->d_draw_start.as<int>();
    a.ndraws = (int)draws.size();
    a.total_tris = (int)total;
    a.format = fmt;
    a.color = h->d_color.p;
    a.depth = h->d_depth.as<float>();
    a.vis = h->vis_output ? h->d_vis.as<int>() : nullptr;
    a.entries = h->d_entries.as<int>();
    a.clear = clear;
    std::memcpy(a.clear_color, h->clear_color, sizeof(a.clear_color));
    a.clear_depth = h->clear_depth;
    a.depth_func = draws[0].depth_func;
    a.depth_write = draws[0].depth_write;
    a.ordered = ordered ? 1 : 0;
    a.tile_count = h->d_tile_count.as<uint32_t>();
    a.tile_offset = h->d_tile_offset.as<uint32_t>();
    a.tile_cursor = h->d_tile_cursor.as<uint32_t>();
    a.pairs = h->d_pairs.as<uint32_t>();
    a.records = h->d_records.as<ifr::TriRecord>();
    a.pair_capacity = h->pair_capacity;
    a.status = h->d_status.as<uint32_t>();
    IFTR_CUDA(h, ifr::launch_pass(a, h->stream, h->timing ? h->ev : nullptr));
    IFTR_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status.p, ifr::ST_WORDS * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
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
    if (!h->pending) return IFTR_OK;
    IFTR_CUDA(h, cudaStreamSynchronize(h->stream));
    h->pending = 0;
    if (h->timing)
        for (int i = 0; i < 5; i++) cudaEventElapsedTime(&h->stage_ms[i], h->ev[i], h->ev[i + 1]);
    h->stats.tile_pairs = h->h_status[ifr::ST_PAIRS];
    h->stats.pair_capacity = h->pair_capacity;
    if (h->h_status[ifr::ST_OVERFLOW]) {
        size_t want = (size_t)h->h_status[ifr::ST_PAIRS] + h->h_status[ifr::ST_PAIRS] / 4 + 1024;
        int rc = ensure_pairs(h, want);
        return rc ? rc : IFTR_ERR_OVERFLOW;
    }
    if (h->h_status[ifr::ST_ORDERED_LIMIT]) return IFTR_ERR_LIMIT;
    return IFTR_OK;
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

}  // namespace

// ============================================================================ C-ABI
extern "C" {

IFTR_API IfritGbRenderer* iftrCreateInstance(void) { return new (std::nothrow) IfritGbRenderer(); }

IFTR_API int iftrDestroyInstance(IfritGbRenderer* h) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (h->inited) {
        cudaStreamSynchronize(h->stream);
        for (DevMem* m : {&h->d_vertices, &h->d_indices, &h->d_color, &h->d_depth, &h->d_vis, &h->d_entries, &h->d_tile_count,
                          &h->d_tile_offset, &h->d_tile_cursor, &h->d_pairs, &h->d_status, &h->d_draws, &h->d_draw_start,
                          &h->d_records})
            m->release();
        for (auto& t : h->tex) t.mem.release();
        for (cudaEvent_t e : h->ev)
            if (e) cudaEventDestroy(e);
        cudaFreeHost(h->h_status);
        cudaFreeHost(h->h_draws);
        cudaFreeHost(h->h_draw_start);
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

IFTR_API int iftrDrawAsync(IfritGbRenderer* h, int numIndices, int clear) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    return enqueue_draw(h, numIndices, clear);
}

IFTR_API int iftrFinish(IfritGbRenderer* h) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (!h->inited) return IFTR_OK;
    return check_pending(h);
}

IFTR_API int iftrDrawLegacy(IfritGbRenderer* h, int numIndices, int clear) {
    if (!h) return IFTR_ERR_INVALID_ARG;
    if (h->in_pass) return iftrPassDraw(h, 0, numIndices);
    h->stats.retries = 0;
    for (int attempt = 0; attempt < 4; attempt++) {
        int rc = enqueue_draw(h, numIndices, clear);
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
    return rc ? rc : ensure_pairs(h, pairs);
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
    for (int i = 0; i < n && i < 5; i++) ms[i] = h->stage_ms[i];
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
