// Host-side planning of a pass, shared by the renderer runtime (capi.cu) and the
// allocation-free entry point (noalloc.cu): per-view constants, the tile ranges of the views
// and the launch groups of the tile stages.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/ifrit_gb300.h"
#include "raster_kernels.cuh"

namespace ifr {

inline void fill_blend(DrawDev& d, const IfritGbBlendState& b) {
    d.blend_enable = b.blendEnable != 0;
    d.blend_src_color = b.srcColorBlendFactor;
    d.blend_dst_color = b.dstColorBlendFactor;
    d.blend_src_alpha = b.srcAlphaBlendFactor;
    d.blend_dst_alpha = b.dstAlphaBlendFactor;
}

// Scissor rectangles (x, y, w, h) of a draw as inclusive pixel bounds: pixel x passes the
// reference's test x >= sx && x <= sx + sw (float compares, TileRasterCoreInvocationCuda.cu:1950-1962)
// exactly when ceil(sx) <= x <= floor(sx + sw).  Disabled, or enabled with no rectangle: no test.
inline int clamp_pixel_bound(float v) { return v < -1.0e9f ? -1000000000 : v > 1.0e9f ? 1000000000 : (int)v; }

inline void fill_scissor(DrawDev& d, bool enable, const float* rects, int count) {
    d.scissor_count = enable ? std::min(count, 16) : 0;
    int box[4] = {1000000000, 1000000000, -1000000000, -1000000000};
    for (int i = 0; i < d.scissor_count; i++) {
        const float* r = rects + 4 * i;
        const float x1 = r[0] + r[2], y1 = r[1] + r[3];
        int* q = d.scissor[i];
        q[0] = clamp_pixel_bound(std::ceil(r[0]));
        q[1] = clamp_pixel_bound(std::ceil(r[1]));
        q[2] = clamp_pixel_bound(std::floor(x1));
        q[3] = clamp_pixel_bound(std::floor(y1));
        if (q[0] > q[2] || q[1] > q[3]) continue;  // passes no pixel
        box[0] = std::min(box[0], q[0]);
        box[1] = std::min(box[1], q[1]);
        box[2] = std::max(box[2], q[2]);
        box[3] = std::max(box[3], q[3]);
    }
    for (int k = 0; k < 4; k++) d.scissor_box[k] = box[k];
}

// Texture and sampler of a draw; the mip chain is stored level after level, each level
// ((w + 1) >> 1) x ((h + 1) >> 1) of the previous one.
inline void fill_texture(DrawDev& d, const uint32_t* texels, int w, int h, int levels, const IfritGbSampler& s) {
    d.texels = texels;
    d.tex_w = w;
    d.tex_h = h;
    d.tex_levels = levels;
    d.sampler.address_u = s.addressModeU;
    d.sampler.address_v = s.addressModeV;
    d.sampler.filter = s.filterMode;
    d.sampler.border_white = s.borderColor;
    d.sampler.max_aniso = s.anisotropyEnable ? (s.maxAnisotropy >= 1.0f ? (int)s.maxAnisotropy : 1) : 1;
    d.sampler.lod_bias = s.lodBias;
    int off = 0;
    for (int l = 0; l < 16; l++) {
        d.lvl_off[l] = off;
        d.lvl_w[l] = w;
        d.lvl_h[l] = h;
        off += w * h;
        w = w > 1 ? (w + 1) >> 1 : 1;
        h = h > 1 ? (h + 1) >> 1 : 1;
    }
}

// Depth state and path of a view from its draws: the deferred path needs one depth function
// and write mask for the whole view and no blending or NOT_EQUAL writes; anything else runs the
// ordered path, whose leading draws that satisfy those conditions (the order-independent prefix)
// still go through the deferred raster stage.
inline bool order_independent(const DrawDev& d, const DrawDev& first) {
    return !d.blend_enable && !(d.depth_write && d.depth_func == IF_COMPARE_OP_NOT_EQUAL) &&
           d.depth_func == first.depth_func && d.depth_write == first.depth_write;
}

inline void set_view_depth_state(ViewArgs& v, const DrawDev* draws, int n) {
    v.depth_func = n > 0 ? draws[0].depth_func : IF_COMPARE_OP_LESS;
    v.depth_write = n > 0 ? draws[0].depth_write : 1;
    v.ordered = 0;
    v.ordered_prefix = 0;
    int i = 0;
    while (i < n && order_independent(draws[i], draws[0])) v.ordered_prefix += draws[i++].num_triangles;
    if (i < n) v.ordered = 1;
    // Occlusion culling of ordered entries per tile: depths only ever decrease after a prefix that
    // writes under LESS / LEQUAL when every later draw either writes nothing or writes under LESS,
    // LEQUAL, EQUAL or NEVER.
    v.ordered_cull = 0;
    if (v.ordered && v.ordered_prefix > 0 && v.depth_write &&
        (v.depth_func == IF_COMPARE_OP_LESS || v.depth_func == IF_COMPARE_OP_LESS_OR_EQUAL)) {
        v.ordered_cull = 1;
        for (int j = i; j < n; j++) {
            const int f = draws[j].depth_func;
            if (draws[j].depth_write && f != IF_COMPARE_OP_LESS && f != IF_COMPARE_OP_LESS_OR_EQUAL &&
                f != IF_COMPARE_OP_EQUAL && f != IF_COMPARE_OP_NEVER)
                v.ordered_cull = 0;
        }
    }
}

inline bool valid_samples(int S) { return S == 1 || S == 2 || S == 4 || S == 8 || S == 16; }

// Screen-tile edges the tile kernels are built for: 16 for every sample count, 8 for 1x and 4x
// deferred views (the ordered path always runs 16x16 tiles).
inline bool tile_size_supported(int S, int TS, bool ordered) {
    if (TS == 16) return true;
    return TS == 8 && !ordered && (S == 1 || S == 4);
}

inline int tiles_of(int W, int H, int TS) { return ((W + TS - 1) / TS) * ((H + TS - 1) / TS); }

// Alignment the tile kernels' vector accesses need on a view's targets: 16-byte float4 depth
// stores when the sample count is a multiple of 4, 8/16-byte colour stores for RGBA16F/RGBA32F.
inline bool targets_aligned(const void* color, int fmt, const void* depth, const void* vis, int S) {
    const uintptr_t ca = fmt == IFTR_FORMAT_RGBA32F ? 16 : fmt == IFTR_FORMAT_RGBA16F ? 8 : 4;
    const uintptr_t da = S % 4 == 0 ? 16 : 4;
    return (uintptr_t)color % ca == 0 && (uintptr_t)depth % da == 0 && (uintptr_t)vis % 4 == 0;
}

inline void fill_pass_const(PassConst& c, int W, int H, int S, int TS) {
    std::memset(&c, 0, sizeof(c));
    c.W = W;
    c.H = H;
    c.S = S;
    c.tile_shift = TS == 8 ? 3 : 4;
    c.tiles_x = (W + TS - 1) / TS;
    c.tiles_y = (H + TS - 1) / TS;
    c.smin_x = c.smax_x = sample_pos(S, 0, 0);
    c.smin_y = c.smax_y = sample_pos(S, 0, 1);
    for (int k = 1; k < S; k++) {
        c.smin_x = std::min(c.smin_x, sample_pos(S, k, 0));
        c.smax_x = std::max(c.smax_x, sample_pos(S, k, 0));
        c.smin_y = std::min(c.smin_y, sample_pos(S, k, 1));
        c.smax_y = std::max(c.smax_y, sample_pos(S, k, 1));
    }
    c.W256 = (float)W * 256.0f;
    c.H256 = (float)H * 256.0f;
    // guard band: clip space is clipped to +-(1 + 2 * 8192 / size) so snapped coordinates fit
    c.gx = (float)(1.0 + 2.0 * 8192.0 / (double)W);
    c.gy = (float)(1.0 + 2.0 * 8192.0 / (double)H);
}

// Launch-group key of a view: views of one group share the tile kernels' template arguments.
inline int group_key(const ViewArgs& v) { return v.c.S * 4 + (v.ordered ? 2 : 0) + (v.c.tile_shift == 3 ? 1 : 0); }

// Assigns each view its tile range and splits the views into launch groups of equal sample
// count, path and tile size.  `v` must already be ordered so that each group is contiguous.
// Persistent CTAs per SM: `ctas_per_sm` > 0 as given (at most the occupancy), 0 the kernels'
// full occupancy, -k the full occupancy divided by k.  Returns false if the views need more
// launch groups than a plan holds or a view's tile size is not built.
inline bool plan_groups(ViewArgs* v, int n, int* view_tile_start, int sms, int ctas_per_sm, LaunchPlan& plan,
                        int& total_tiles) {
    std::memset(&plan, 0, sizeof(plan));
    int t = 0;
    for (int i = 0; i < n; i++) {
        const int TS = 1 << v[i].c.tile_shift;
        if (!tile_size_supported(v[i].c.S, TS, v[i].ordered != 0)) return false;
        v[i].tile_start = t;
        view_tile_start[i] = t;
        t += v[i].c.tiles_x * v[i].c.tiles_y;
        if (i == 0 || group_key(v[i]) != group_key(v[i - 1])) {
            if (plan.ngroups == kMaxGroups) return false;
            GroupArgs& g = plan.groups[plan.ngroups];
            g.view_begin = i;
            g.tile_begin = v[i].tile_start;
            g.queue = plan.ngroups;
            plan.samples[plan.ngroups] = v[i].c.S;
            plan.tile_size[plan.ngroups] = TS;
            plan.ordered[plan.ngroups] = v[i].ordered ? 1 : 0;
            plan.ngroups++;
        }
        if (v[i].ordered && v[i].ordered_prefix > 0) plan.hybrid[plan.ngroups - 1] = 1;
        GroupArgs& g = plan.groups[plan.ngroups - 1];
        g.view_end = i + 1;
        g.tile_end = t;
    }
    view_tile_start[n] = t;
    total_tiles = t;
    plan.defer_group = -1;
    for (int k = 0; k < plan.ngroups; k++)
        if (plan.ordered[k]) plan.defer_group = plan.defer_group == -1 ? k : -2;
    if (plan.defer_group >= 0) {
        const int S = plan.samples[plan.defer_group];
        const GroupArgs& dg = plan.groups[plan.defer_group];
        plan.ctas_frag_shade = sms * frag_kernel_occupancy(S, 0);
        plan.ctas_frag_blend = sms * frag_kernel_occupancy(S, 1);
        plan.ctas_fwd_defer = std::max(1, std::min(dg.tile_end - dg.tile_begin, sms * frag_kernel_occupancy(S, 2)));
    } else {
        plan.defer_group = -1;
    }
    for (int k = 0; k < plan.ngroups; k++) {
        const int tiles = plan.groups[k].tile_end - plan.groups[k].tile_begin;
        const int S = plan.samples[k], TS = plan.tile_size[k];
        // stage kernels: raster, shade (deferred); raster, shade, ordered (hybrid); ordered (ordered)
        const int occ_raster = tile_kernel_occupancy(S, TS, 0, 0), occ_shade = tile_kernel_occupancy(S, TS, 0, 1);
        const int occ_ordered = plan.ordered[k] ? tile_kernel_occupancy(S, TS, 1, 0) : 1;
        const int occ[3] = {plan.ordered[k] && !plan.hybrid[k] ? occ_ordered : occ_raster, occ_shade, occ_ordered};
        int* out[3] = {plan.ctas, plan.ctas_shade, plan.ctas_fwd};
        for (int stage = 0; stage < 3; stage++) {
            const int per_sm = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ[stage])
                               : ctas_per_sm < 0 ? std::max(1, occ[stage] / -ctas_per_sm)
                                                 : occ[stage];
            out[stage][k] = std::max(1, std::min(tiles, sms * per_sm));
        }
    }
    return true;
}

}  // namespace ifr
