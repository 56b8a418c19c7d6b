// sm_103a kernels of one render pass.
//
//   bin_kernel<false>   per triangle: fetch + transform + clip + set up, count (tile, triangle)
//                       overlaps per 16x16 tile  (reference: first/second binners,
//                       TileRasterCoreInvocationCuda.cu:721-1339, CPU executeBinner
//                       TileRasterWorker.cpp:314-397)
//   scan_kernel         exclusive scan of the per-tile counts -> list offsets; resets counts
//   bin_kernel<true>    same front end, scatters (triangle, fan index) into the tile lists
//   tile_kernel<S>      one CTA per tile, one thread per pixel holding S samples in
//                       registers: coverage + early depth test for every listed triangle
//                       (pixelTaggingExecKernel, .cu:1900-2142), then deferred shading of the
//                       visible primitives with quad derivatives (pixelShadingExecKernel,
//                       .cu:2144-2317), on-chip MSAA resolve (.cu:2319-2361), and one store of
//                       depth / visibility / colour per pixel.
//
// Visibility is order independent: a sample keeps the primitive that wins under the pass's
// depth function with ties broken by API order (earlier wins for LESS/GREATER, later for
// LEQUAL/GEQUAL/EQUAL/ALWAYS), which is exactly what processing triangles in submission
// order produces.  So the tile lists need no sorting and the result is deterministic.
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include "raster_kernels.cuh"

namespace ifr {

__device__ __forceinline__ int find_draw(const PassArgs& a, int g) {
    int lo = 0, hi = a.ndraws - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(a.draw_start + mid) <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void bin_sub(const PassArgs& a, const SubTri& s, uint32_t entry, bool scatter) {
    int tx0 = s.px0 >> kTileShift, tx1 = s.px1 >> kTileShift;
    int ty0 = s.py0 >> kTileShift, ty1 = s.py1 >> kTileShift;
    for (int ty = ty0; ty <= ty1; ty++)
        for (int tx = tx0; tx <= tx1; tx++) {
            int tile = ty * a.c.tiles_x + tx;
            if (scatter) {
                uint32_t pos = atomicAdd(a.tile_cursor + tile, 1u);
                if (pos < a.pair_capacity) a.pairs[pos] = entry;
            } else {
                atomicAdd(a.tile_count + tile, 1u);
            }
        }
}

// Counting pass: full front end per triangle; unclipped triangles leave a compact record.
__global__ void __launch_bounds__(256) bin_count_kernel(PassArgs a) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.total_tris) return;
    int di = find_draw(a, g);
    const DrawDev& d = a.draws[di];
    int t = g - __ldg(a.draw_start + di);
    CVert poly[kMaxPoly];
    bool inside, rejected;
    TriRecord* rec = a.records + g;
    if (!fetch_triangle(a.c, d, t, poly, inside, rejected)) {
        rec->flags = 0;
        return;
    }
    if (inside) {
        SubTri s;
        if (!setup_sub(a.c, d, poly[0], poly[1], poly[2], s)) {
            rec->flags = 0;
            return;
        }
        TriRecord r;
        record_from_sub(s, r);
        const int4* src = reinterpret_cast<const int4*>(&r);
        int4* dst = reinterpret_cast<int4*>(rec);
        dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2]; dst[3] = src[3];
        bin_sub(a, s, (uint32_t)g << 3, false);
        return;
    }
    rec->flags = REC_CLIPPED;
    int n = clip_polygon(a.c, poly);
    for (int i = 1; i + 1 < n; i++) {
        SubTri s;
        if (setup_sub(a.c, d, poly[0], poly[i], poly[i + 1], s)) bin_sub(a, s, ((uint32_t)g << 3) | (uint32_t)(i - 1), false);
    }
}

// Scattering pass: same overlaps as the counting pass, read back from the records (clipped
// triangles run the front end again).
__global__ void __launch_bounds__(256) bin_scatter_kernel(PassArgs a) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.total_tris) return;
    if (a.status[ST_OVERFLOW]) return;
    const int flags = __ldg(&a.records[g].flags);
    if (flags & REC_VALID) {
        SubTri s;
        if (sub_from_record(a.c, a.records + g, s)) bin_sub(a, s, (uint32_t)g << 3, true);
        return;
    }
    if (!(flags & REC_CLIPPED)) return;
    int di = find_draw(a, g);
    const DrawDev& d = a.draws[di];
    int t = g - __ldg(a.draw_start + di);
    CVert poly[kMaxPoly];
    bool inside, rejected;
    if (!fetch_triangle(a.c, d, t, poly, inside, rejected)) return;
    int n = clip_polygon(a.c, poly);
    for (int i = 1; i + 1 < n; i++) {
        SubTri s;
        if (setup_sub(a.c, d, poly[0], poly[i], poly[i + 1], s)) bin_sub(a, s, ((uint32_t)g << 3) | (uint32_t)(i - 1), true);
    }
}

__global__ void __launch_bounds__(1024) scan_kernel(PassArgs a, int T) {
    __shared__ uint32_t part[1024];
    int tid = threadIdx.x;
    int per = (T + 1023) / 1024;
    int b = min(tid * per, T), e = min(b + per, T);
    uint32_t sum = 0;
    for (int i = b; i < e; i++) sum += a.tile_count[i];
    part[tid] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = tid >= off ? part[tid - off] : 0u;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    uint32_t run = part[tid] - sum;
    for (int i = b; i < e; i++) {
        uint32_t c = a.tile_count[i];
        a.tile_offset[i] = run;
        a.tile_cursor[i] = run;
        a.tile_count[i] = 0u;
        run += c;
    }
    if (tid == 1023) {
        a.tile_offset[T] = part[1023];
        a.status[ST_PAIRS] = part[1023];
        if (part[1023] > a.pair_capacity) a.status[ST_OVERFLOW] = 1u;
    }
}

// Initial depth of sample k of pixel (x, y) for the explicit-compare key modes.
__device__ __forceinline__ float d0_of(const PassArgs& a, int x, int y, int k) {
    return a.clear ? a.clear_depth : a.depth[((size_t)y * a.c.W + x) * a.c.S + k];
}

__device__ __forceinline__ void decode_color(const PassArgs& a, size_t pix, float c[4]) {
    switch (a.format) {
    case FMT_RGBA8: unpack_rgba8(static_cast<const uint32_t*>(a.color)[pix], c); break;
    case FMT_RGBA16F: {
        uint2 v = static_cast<const uint2*>(a.color)[pix];
        c[0] = __half2float(__ushort_as_half((unsigned short)(v.x & 0xffffu)));
        c[1] = __half2float(__ushort_as_half((unsigned short)(v.x >> 16)));
        c[2] = __half2float(__ushort_as_half((unsigned short)(v.y & 0xffffu)));
        c[3] = __half2float(__ushort_as_half((unsigned short)(v.y >> 16)));
        break;
    }
    case FMT_RGBA32F: {
        float4 v = static_cast<const float4*>(a.color)[pix];
        c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
        break;
    }
    default: {
        const float* p = static_cast<const float*>(a.color) + pix * 3;
        c[0] = p[0]; c[1] = p[1]; c[2] = p[2]; c[3] = 1.0f;
        break;
    }
    }
}

__device__ __forceinline__ void encode_color(const PassArgs& a, size_t pix, const float c[4]) {
    switch (a.format) {
    case FMT_RGBA8: {
        uint32_t v = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            float x = fminf(fmaxf(c[i], 0.0f), 1.0f);
            v |= __float2uint_rn(x * 255.0f) << (8 * i);
        }
        static_cast<uint32_t*>(a.color)[pix] = v;
        break;
    }
    case FMT_RGBA16F: {
        uint2 v;
        v.x = (uint32_t)__half_as_ushort(__float2half_rn(c[0])) | ((uint32_t)__half_as_ushort(__float2half_rn(c[1])) << 16);
        v.y = (uint32_t)__half_as_ushort(__float2half_rn(c[2])) | ((uint32_t)__half_as_ushort(__float2half_rn(c[3])) << 16);
        static_cast<uint2*>(a.color)[pix] = v;
        break;
    }
    case FMT_RGBA32F: static_cast<float4*>(a.color)[pix] = make_float4(c[0], c[1], c[2], c[3]); break;
    default: {
        float* p = static_cast<float*>(a.color) + pix * 3;
        p[0] = c[0]; p[1] = c[1]; p[2] = c[2];
        break;
    }
    }
}

// ---------------------------------------------------------------------------- tile kernel
// Visibility keys.  Every sample holds one 64-bit key in shared memory; a fragment that
// passes the depth test lowers it with atomicMin, so the final key is the same whatever the
// order fragments arrive in:
//   high word: depth order  (LESS/LEQUAL: z ascending, GREATER/GEQUAL: descending; 0 for the
//              functions whose pass test is an explicit compare against the initial depth)
//   low word:  entry order  (entry = global triangle << 3 | fan index; "earliest wins" modes
//              store entry + 1 with the background at 0, "latest wins" modes store
//              0xFFFFFFFE - entry with the background at 0xFFFFFFFF)
// Ties therefore resolve exactly as submission-order processing does: LESS/GREATER keep the
// earlier primitive, LEQUAL/GEQUAL/EQUAL/ALWAYS (and any test without depth writes) the later.
enum KeyMode { KM_EARLIEST = 0, KM_LATEST = 1 };

__device__ __forceinline__ uint32_t depth_order(float z) {
    uint32_t u = __float_as_uint(z);
    if (u == 0x80000000u) u = 0u;  // -0 and +0 compare equal
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

struct KeyRule {
    int func;       // depth function
    int write;      // depth writes enabled
    int explicit_;  // pass decided by compare against the initial depth; depth word = 0
    int invert;     // GREATER/GEQUAL: descending depth order
    int mode;       // KM_EARLIEST / KM_LATEST
};

__device__ __forceinline__ KeyRule key_rule(int func, int write) {
    KeyRule r;
    r.func = func;
    r.write = write;
    r.explicit_ = !write || func == 2 || func == 7 || func == 0;
    r.invert = func == 4 || func == 6;
    r.mode = (write && (func == 1 || func == 4)) ? KM_EARLIEST : KM_LATEST;
    return r;
}

__device__ __forceinline__ unsigned long long background_key(const KeyRule& r, float d0) {
    uint32_t hi = 0u;
    if (!r.explicit_) hi = r.invert ? ~depth_order(d0) : depth_order(d0);
    uint32_t lo = r.mode == KM_EARLIEST ? 0u : 0xFFFFFFFFu;
    return ((unsigned long long)hi << 32) | lo;
}

__device__ __forceinline__ int key_entry(const KeyRule& r, unsigned long long key) {
    uint32_t lo = (uint32_t)key;
    if (r.mode == KM_EARLIEST) return lo == 0u ? -1 : (int)(lo - 1u);
    return lo == 0xFFFFFFFFu ? -1 : (int)(0xFFFFFFFEu - lo);
}

struct RecordPlane {
    float z0, dzdx, dzdy;
    int32_t X0, Y0;
};

__device__ __forceinline__ void shade_entry_geom(const PassArgs& a, int e, const ShadeGeom& g, int px, int py, float* col) {
    int gi = e >> 3, sub = e & 7;
    int di = find_draw(a, gi);
    shade_fragment(a.c, a.draws[di], g, gi - __ldg(a.draw_start + di), sub, px, py, col);
}

// Set-up of entry e (global triangle << 3 | fan index) for shading: geometry + depth plane.
__device__ __noinline__ void setup_entry(const PassArgs& a, int e, ShadeGeom* g, RecordPlane* pl) {
    int gi = e >> 3, sub = e & 7;
    int di = find_draw(a, gi);
    SubTri s;
    setup_entry_sub(a.c, a.draws[di], a.records, gi, gi - __ldg(a.draw_start + di), sub, s);
    shade_geom_from(s, *g);
    pl->z0 = s.z[0];
    pl->dzdx = s.dzdx;
    pl->dzdy = s.dzdy;
    pl->X0 = s.X[0];
    pl->Y0 = s.Y[0];
}

// Raster set-up of entry e for the batch phase (out of line: one copy of the clip path).
__device__ __noinline__ bool setup_raster_entry(const PassArgs& a, uint32_t e, SubTri* s) {
    int g = (int)(e >> 3), sub = (int)(e & 7u);
    int di = find_draw(a, g);
    return setup_entry_sub(a.c, a.draws[di], a.records, g, g - __ldg(a.draw_start + di), sub, *s);
}

// Set-up and shading of an entry that did not fit the tile's set-up cache (rare; out of line).
__device__ __noinline__ void shade_uncached(const PassArgs& a, int e, int px, int py, float* col, RecordPlane* pl) {
    ShadeGeom g;
    setup_entry(a, e, &g, pl);
    shade_entry_geom(a, e, g, px, py, col);
}

struct TileRecords {
    int32_t A[3][kTileThreads], B[3][kTileThreads];
    long long Cb[3][kTileThreads];
    float z0[kTileThreads], dzdx[kTileThreads], dzdy[kTileThreads];
    int32_t X0[kTileThreads], Y0[kTileThreads];
    int32_t org[kTileThreads];    // tile-local x0 | y0 << 8 of the clipped bbox
    int32_t width[kTileThreads];  // clipped bbox width in pixels
    float rwidth[kTileThreads];   // 1 / width
    int32_t key[kTileThreads];    // entry
    uint32_t start[kTileThreads + 1];  // exclusive prefix of pixel counts
};


// Raster stage: one CTA per 16x16 tile.  The tile's list is consumed in batches of up to 256
// set-ups; every (triangle, pixel) pair of a batch is spread over the CTA, and each covered
// sample that passes the depth test lowers its key.  The winning entry of every sample
// (or -1) is written for the shading stage.
template <int S>
__global__ void __launch_bounds__(kTileThreads) raster_kernel(PassArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileRecords& rec = *reinterpret_cast<TileRecords*>(smem_raw);
    unsigned long long* skey = reinterpret_cast<unsigned long long*>(smem_raw + sizeof(TileRecords));
    __shared__ uint32_t warp_sum[kTileThreads / 32];

    const int tile = blockIdx.x;
    const int tx = tile % a.c.tiles_x, ty = tile / a.c.tiles_x;
    const int tx0 = tx * kTileSize, ty0 = ty * kTileSize;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int lx = ((tid >> 2) & 7) * 2 + (tid & 1);
    const int ly = (tid >> 5) * 2 + ((tid >> 1) & 1);
    const int px = tx0 + lx, py = ty0 + ly;
    const bool inpix = px < a.c.W && py < a.c.H;
    const size_t pix = (size_t)py * a.c.W + px;
    const KeyRule rule = key_rule(a.depth_func, a.depth_write);

#pragma unroll
    for (int k = 0; k < S; k++) {
        float d0 = a.clear ? a.clear_depth : (inpix ? a.depth[pix * S + k] : 0.0f);
        skey[(ly * kTileSize + lx) * S + k] = background_key(rule, d0);
    }
    const bool has_list = a.total_tris > 0 && a.status[ST_OVERFLOW] == 0 && rule.func != 0;
    const uint32_t beg = has_list ? a.tile_offset[tile] : 0u;
    const uint32_t end = has_list ? a.tile_offset[tile + 1] : 0u;
    const int xmax = min(a.c.W, tx0 + kTileSize) - 1, ymax = min(a.c.H, ty0 + kTileSize) - 1;

    for (uint32_t base = beg; base < end; base += kTileThreads) {
        const int nb = (int)min((uint32_t)kTileThreads, end - base);
        uint32_t cnt = 0;
        if (tid < nb) {
            uint32_t e = __ldg(a.pairs + base + tid);
            SubTri s;
            if (setup_raster_entry(a, e, &s)) {
                int x0 = max(s.px0, tx0), x1 = min(s.px1, xmax);
                int y0 = max(s.py0, ty0), y1 = min(s.py1, ymax);
                if (x0 <= x1 && y0 <= y1) {
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        rec.A[i][tid] = s.A[i];
                        rec.B[i][tid] = s.B[i];
                        rec.Cb[i][tid] = s.Cb[i];
                    }
                    rec.z0[tid] = s.z[0];
                    rec.dzdx[tid] = s.dzdx;
                    rec.dzdy[tid] = s.dzdy;
                    rec.X0[tid] = s.X[0];
                    rec.Y0[tid] = s.Y[0];
                    int w = x1 - x0 + 1;
                    rec.org[tid] = (x0 - tx0) | ((y0 - ty0) << 8);
                    rec.width[tid] = w;
                    rec.rwidth[tid] = 1.0f / (float)w;
                    cnt = (uint32_t)(w * (y1 - y0 + 1));
                }
            }
            rec.key[tid] = (int)e;
        }
        // block-wide exclusive scan of the per-record pixel counts
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_sum[wid] = incl;
        __syncthreads();
        uint32_t wbase = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kTileThreads / 32; w++) {
            uint32_t v = warp_sum[w];
            if (w < wid) wbase += v;
            total += v;
        }
        rec.start[tid] = wbase + incl - cnt;
        if (tid == 0) rec.start[kTileThreads] = total;
        __syncthreads();
        for (uint32_t p = tid; p < total; p += kTileThreads) {
            int lo = 0, hi = nb - 1;
            while (lo < hi) {  // last record with start <= p
                int mid = (lo + hi + 1) >> 1;
                if (rec.start[mid] <= p) lo = mid; else hi = mid - 1;
            }
            const int r = lo;
            const int local = (int)(p - rec.start[r]);
            const int w = rec.width[r];
            const int oy = (int)(((float)local + 0.5f) * rec.rwidth[r]);
            const int ox = local - oy * w;
            const int org = rec.org[r];
            const int qx = (org & 255) + ox, qy = (org >> 8) + oy;
            const int gx = tx0 + qx, gy = ty0 + qy;
            int32_t A[3] = {rec.A[0][r], rec.A[1][r], rec.A[2][r]};
            int32_t B[3] = {rec.B[0][r], rec.B[1][r], rec.B[2][r]};
            int64_t Cb[3] = {rec.Cb[0][r], rec.Cb[1][r], rec.Cb[2][r]};
            const float z0 = rec.z0[r], gzx = rec.dzdx[r], gzy = rec.dzdy[r];
            const int32_t X0 = rec.X0[r], Y0 = rec.Y0[r];
            const uint32_t e = (uint32_t)rec.key[r];
            const uint32_t lo_word = rule.mode == KM_EARLIEST ? e + 1u : 0xFFFFFFFEu - e;
            unsigned long long* kp = skey + (qy * kTileSize + qx) * S;
            // (float)(sx - X0) == fbx + sample offset exactly: every term is an integer below
            // 2^24 in magnitude (guard-band bound), so no conversion per sample is needed.
            const float fbx = (float)(gx * 256 - X0), fby = (float)(gy * 256 - Y0);
#pragma unroll
            for (int k = 0; k < S; k++) {
                const int32_t sx = gx * 256 + a.c.sx[k], sy = gy * 256 + a.c.sy[k];
                if (!covered(A, B, Cb, sx, sy)) continue;
                const float z = (z0 + gzx * (fbx + (float)a.c.sx[k])) + gzy * (fby + (float)a.c.sy[k]);
                uint32_t hi_word;
                if (rule.explicit_) {
                    if (!depth_cmp(rule.func, z, d0_of(a, gx, gy, k))) continue;
                    hi_word = 0u;
                } else {
                    hi_word = rule.invert ? ~depth_order(z) : depth_order(z);
                }
                const unsigned long long kv = ((unsigned long long)hi_word << 32) | lo_word;
                if (kv < kp[k]) atomicMin(kp + k, kv);
            }
        }
        __syncthreads();
    }
    if (!inpix) return;
    int out[S];
#pragma unroll
    for (int k = 0; k < S; k++) out[k] = key_entry(rule, skey[(ly * kTileSize + lx) * S + k]);
    int* ep = a.entries + pix * S;
    if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) reinterpret_cast<int4*>(ep)[k / 4] = make_int4(out[k], out[k + 1], out[k + 2], out[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < S; k++) ep[k] = out[k];
    }
}

// Shading stage: one CTA per tile, one thread per pixel.  Each pixel lists its distinct
// visible entries in sample order; the warp shades list slot i of all its lanes together
// (set-up straight from the binner's record, quad derivatives, texture filtering), then the
// samples are resolved on chip and depth, visibility and the resolved colour stored once.
template <int S>
__global__ void __launch_bounds__(kTileThreads, 2) shade_kernel(PassArgs a) {
    __shared__ DrawDev sdraw;
    __shared__ float4 scol[4][kTileThreads];  // colours of each thread's (up to 4) distinct entries

    const int tile = blockIdx.x;
    const int tx = tile % a.c.tiles_x, ty = tile / a.c.tiles_x;
    const int tid = threadIdx.x;
    const int lx = ((tid >> 2) & 7) * 2 + (tid & 1);
    const int ly = (tid >> 5) * 2 + ((tid >> 1) & 1);
    const int px = tx * kTileSize + lx, py = ty * kTileSize + ly;
    const bool inpix = px < a.c.W && py < a.c.H;
    const size_t pix = (size_t)py * a.c.W + px;
    const KeyRule rule = key_rule(a.depth_func, a.depth_write);
    if (a.ndraws == 1) {  // stage the draw descriptor on chip (read by every shading step)
        const int* src = reinterpret_cast<const int*>(a.draws);
        int* dst = reinterpret_cast<int*>(&sdraw);
        for (int i = tid; i < (int)(sizeof(DrawDev) / 4); i += kTileThreads) dst[i] = src[i];
    }
    int ent[S];
    if (inpix) {
        const int* ep = a.entries + pix * S;
        if constexpr (S % 4 == 0) {
#pragma unroll
            for (int k = 0; k < S; k += 4) {
                int4 v = reinterpret_cast<const int4*>(ep)[k / 4];
                ent[k] = v.x; ent[k + 1] = v.y; ent[k + 2] = v.z; ent[k + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < S; k++) ent[k] = ep[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < S; k++) ent[k] = -1;
    }
    __syncthreads();
    const DrawDev& d0 = a.ndraws == 1 ? sdraw : a.draws[0];

    // distinct visible entries of this pixel, in sample order; sample k uses list slot which[k]
    constexpr int U = S < 4 ? S : 4;  // slots shaded together across the warp
    int uniq[U], which[S];
    int nu = 0;
#pragma unroll
    for (int k = 0; k < S; k++) {
        which[k] = -1;
        if (ent[k] < 0) continue;
        int found = -1;
#pragma unroll
        for (int j = 0; j < k; j++)
            if (which[j] >= 0 && ent[j] == ent[k]) found = which[j];
        if (found < 0) {
            found = nu;
#pragma unroll
            for (int j = 0; j < U; j++)
                if (j == nu) uniq[j] = ent[k];
            nu++;
        }
        which[k] = found;
    }
    int nmax = min(nu, U);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
    float dep[S];
#pragma unroll
    for (int k = 0; k < S; k++) dep[k] = 0.0f;
    for (int i = 0; i < nmax; i++) {
        int e = -1;
#pragma unroll
        for (int j = 0; j < U; j++)
            if (j == i) e = uniq[j];
        if (i < nu) {
            const int g = e >> 3, sub = e & 7;
            const int di = a.ndraws == 1 ? 0 : find_draw(a, g);
            const DrawDev& d = a.ndraws == 1 ? d0 : a.draws[di];
            const int t = g - (a.ndraws == 1 ? 0 : __ldg(a.draw_start + di));
            SubTri st;
            setup_entry_sub(a.c, d, a.records, g, t, sub, st);
            ShadeGeom geo;
            shade_geom_from(st, geo);
            float c[4];
            shade_fragment(a.c, d, geo, t, sub, px, py, c);
            scol[i][tid] = make_float4(c[0], c[1], c[2], c[3]);
#pragma unroll
            for (int k = 0; k < S; k++)
                if (which[k] == i)
                    dep[k] = sample_depth(st.z[0], st.dzdx, st.dzdy, st.X[0], st.Y[0], px * 256 + a.c.sx[k],
                                          py * 256 + a.c.sy[k]);
        }
    }
    if (!inpix) return;
    float bg[4];
    if (a.clear) {
        bg[0] = a.clear_color[0]; bg[1] = a.clear_color[1]; bg[2] = a.clear_color[2]; bg[3] = a.clear_color[3];
    } else {
        decode_color(a, pix, bg);
    }
    float acc[4];
#pragma unroll
    for (int k = 0; k < S; k++) {
        float c[4];
        const float d0v = a.clear ? a.clear_depth : a.depth[pix * S + k];
        if (which[k] < 0) {
            c[0] = bg[0]; c[1] = bg[1]; c[2] = bg[2]; c[3] = bg[3];
            dep[k] = d0v;
        } else {
            if (which[k] < U) {
                float4 v = scol[which[k]][tid];
                c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
            } else {  // more than U distinct primitives in one pixel: shade this one here
                RecordPlane pl;
                shade_uncached(a, ent[k], px, py, c, &pl);
                dep[k] = sample_depth(pl.z0, pl.dzdx, pl.dzdy, pl.X0, pl.Y0, px * 256 + a.c.sx[k], py * 256 + a.c.sy[k]);
            }
            if (!rule.write) dep[k] = d0v;
        }
        if (k == 0) {
            acc[0] = c[0]; acc[1] = c[1]; acc[2] = c[2]; acc[3] = c[3];
        } else {
            acc[0] = acc[0] + c[0]; acc[1] = acc[1] + c[1]; acc[2] = acc[2] + c[2]; acc[3] = acc[3] + c[3];
        }
    }
    const float invS = 1.0f / (float)S;
    acc[0] = acc[0] * invS; acc[1] = acc[1] * invS; acc[2] = acc[2] * invS; acc[3] = acc[3] * invS;
    encode_color(a, pix, acc);

    float* dp = a.depth + pix * S;
    if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) reinterpret_cast<float4*>(dp)[k / 4] = make_float4(dep[k], dep[k + 1], dep[k + 2], dep[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < S; k++) dp[k] = dep[k];
    }
    if (a.vis) {
        int* vp = a.vis + pix * S;
#pragma unroll
        for (int k = 0; k < S; k++) vp[k] = ent[k] < 0 ? -1 : (ent[k] >> 3);
    }
}

// Ordered stage (forward path), one CTA per tile.  Used when results depend on submission
// order: blending, NOT_EQUAL with depth writes, or draws of one pass with different depth
// state.  The tile's entries are sorted into API order in shared memory, then every pixel
// applies them one after another exactly as the reference's ordered CPU path does
// (TileRasterWorker.cpp:1517-1580): per-sample depth test and write, one shading per pixel
// and triangle when any sample passes, per-sample blend (TileRasterWorker.cpp:2346-2373,
// pixelShadingAlphaBlendKernel .cu:1648-1897), then the on-chip resolve.
struct FwdRecords {
    int32_t A[3][kTileThreads], B[3][kTileThreads];
    long long Cb[3][kTileThreads];
    float z0[kTileThreads], dzdx[kTileThreads], dzdy[kTileThreads];
    int32_t X0[kTileThreads], Y0[kTileThreads];
    int32_t bx[kTileThreads], by[kTileThreads];  // px0 | px1 << 16, py0 | py1 << 16
    int32_t key[kTileThreads];
    int32_t draw[kTileThreads];
};

template <int S>
__global__ void __launch_bounds__(kTileThreads) forward_kernel(PassArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FwdRecords& rec = *reinterpret_cast<FwdRecords*>(smem_raw);
    float4* scol = reinterpret_cast<float4*>(smem_raw + sizeof(FwdRecords));                  // [S][256]
    uint32_t* list = reinterpret_cast<uint32_t*>(smem_raw + sizeof(FwdRecords) + sizeof(float4) * S * kTileThreads);

    const int tile = blockIdx.x;
    const int tx = tile % a.c.tiles_x, ty = tile / a.c.tiles_x;
    const int tid = threadIdx.x;
    const int lx = ((tid >> 2) & 7) * 2 + (tid & 1);
    const int ly = (tid >> 5) * 2 + ((tid >> 1) & 1);
    const int px = tx * kTileSize + lx, py = ty * kTileSize + ly;
    const bool inpix = px < a.c.W && py < a.c.H;
    const size_t pix = (size_t)py * a.c.W + px;

    float dep[S];
    int vid[S];
    {
        float bg[4];
        if (a.clear) {
            bg[0] = a.clear_color[0]; bg[1] = a.clear_color[1]; bg[2] = a.clear_color[2]; bg[3] = a.clear_color[3];
        } else if (inpix) {
            decode_color(a, pix, bg);
        } else {
            bg[0] = bg[1] = bg[2] = bg[3] = 0.0f;
        }
#pragma unroll
        for (int k = 0; k < S; k++) {
            dep[k] = a.clear ? a.clear_depth : (inpix ? a.depth[pix * S + k] : 0.0f);
            vid[k] = -1;
            scol[k * kTileThreads + tid] = make_float4(bg[0], bg[1], bg[2], bg[3]);
        }
    }
    const bool has_list = a.total_tris > 0 && a.status[ST_OVERFLOW] == 0;
    const uint32_t beg = has_list ? a.tile_offset[tile] : 0u;
    const uint32_t end = has_list ? a.tile_offset[tile + 1] : 0u;
    int n = (int)(end - beg);
    if (n > kOrderedCap) {  // cannot order this tile on chip: report and leave it cleared
        if (tid == 0) atomicOr(a.status + ST_ORDERED_LIMIT, 1u);
        n = 0;
    }
    // load and sort the tile's entries into submission order (bitonic, padded to 2^k)
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = tid; i < P; i += kTileThreads) list[i] = i < n ? __ldg(a.pairs + beg + i) : 0xFFFFFFFFu;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < P; i += kTileThreads) {
                int ixj = i ^ j;
                if (ixj > i) {
                    uint32_t x = list[i], y = list[ixj];
                    bool up = (i & k) == 0;
                    if ((x > y) == up) {
                        list[i] = y;
                        list[ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
    }

    for (int base = 0; base < n; base += kTileThreads) {
        const int nb = min(kTileThreads, n - base);
        if (tid < nb) {
            uint32_t e = list[base + tid];
            int g = (int)(e >> 3), sub = (int)(e & 7u);
            int di = find_draw(a, g);
            SubTri s;
            if (setup_entry_sub(a.c, a.draws[di], a.records, g, g - __ldg(a.draw_start + di), sub, s)) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    rec.A[i][tid] = s.A[i];
                    rec.B[i][tid] = s.B[i];
                    rec.Cb[i][tid] = s.Cb[i];
                }
                rec.z0[tid] = s.z[0];
                rec.dzdx[tid] = s.dzdx;
                rec.dzdy[tid] = s.dzdy;
                rec.X0[tid] = s.X[0];
                rec.Y0[tid] = s.Y[0];
                rec.bx[tid] = s.px0 | (s.px1 << 16);
                rec.by[tid] = s.py0 | (s.py1 << 16);
            } else {
                rec.bx[tid] = 1;
                rec.by[tid] = 1;
            }
            rec.key[tid] = (int)e;
            rec.draw[tid] = di;
        }
        __syncthreads();
        if (inpix) {
            for (int r = 0; r < nb; r++) {
                const int bx = rec.bx[r], by = rec.by[r];
                if (px < (bx & 0xffff) || px > (bx >> 16) || py < (by & 0xffff) || py > (by >> 16)) continue;
                const int32_t A[3] = {rec.A[0][r], rec.A[1][r], rec.A[2][r]};
                const int32_t B[3] = {rec.B[0][r], rec.B[1][r], rec.B[2][r]};
                const int64_t Cb[3] = {rec.Cb[0][r], rec.Cb[1][r], rec.Cb[2][r]};
                const DrawDev& d = a.draws[rec.draw[r]];
                const int func = d.depth_func, write = d.depth_write;
                const int e = rec.key[r];
                unsigned mask = 0;
#pragma unroll
                for (int k = 0; k < S; k++) {
                    const int32_t sx = px * 256 + a.c.sx[k], sy = py * 256 + a.c.sy[k];
                    if (!covered(A, B, Cb, sx, sy)) continue;
                    const float z = sample_depth(rec.z0[r], rec.dzdx[r], rec.dzdy[r], rec.X0[r], rec.Y0[r], sx, sy);
                    if (!depth_cmp(func, z, dep[k])) continue;
                    if (write) dep[k] = z;
                    vid[k] = e >> 3;
                    mask |= 1u << k;
                }
                if (!mask) continue;
                float c[4];
                RecordPlane pl;
                shade_uncached(a, e, px, py, c, &pl);
#pragma unroll
                for (int k = 0; k < S; k++) {
                    if (!(mask & (1u << k))) continue;
                    float4& sc = scol[k * kTileThreads + tid];
                    if (d.blend_enable) {
                        float dst[4] = {sc.x, sc.y, sc.z, sc.w};
                        blend_into(d, c, dst);
                        sc = make_float4(dst[0], dst[1], dst[2], dst[3]);
                    } else {
                        sc = make_float4(c[0], c[1], c[2], c[3]);
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!inpix) return;
    float acc[4];
#pragma unroll
    for (int k = 0; k < S; k++) {
        const float4 v = scol[k * kTileThreads + tid];
        if (k == 0) {
            acc[0] = v.x; acc[1] = v.y; acc[2] = v.z; acc[3] = v.w;
        } else {
            acc[0] = acc[0] + v.x; acc[1] = acc[1] + v.y; acc[2] = acc[2] + v.z; acc[3] = acc[3] + v.w;
        }
    }
    const float invS = 1.0f / (float)S;
    acc[0] = acc[0] * invS; acc[1] = acc[1] * invS; acc[2] = acc[2] * invS; acc[3] = acc[3] * invS;
    encode_color(a, pix, acc);
    float* dp = a.depth + pix * S;
#pragma unroll
    for (int k = 0; k < S; k++) dp[k] = dep[k];
    if (a.vis) {
        int* vp = a.vis + pix * S;
#pragma unroll
        for (int k = 0; k < S; k++) vp[k] = vid[k];
    }
}

template <int S>
size_t forward_smem_bytes() {
    return sizeof(FwdRecords) + sizeof(float4) * S * kTileThreads + sizeof(uint32_t) * kOrderedCap;
}

template <int S>
size_t raster_smem_bytes() {
    return sizeof(TileRecords) + (size_t)kTileThreads * S * sizeof(unsigned long long);
}


__global__ void mip_kernel(const uint32_t* __restrict__ src, int sw, int sh, uint32_t* __restrict__ dst, int dw, int dh) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    int x0 = 2 * x, x1 = min(2 * x + 1, sw - 1), y0 = 2 * y, y1 = min(2 * y + 1, sh - 1);
    uint32_t p = src[y0 * sw + x0], q = src[y0 * sw + x1], r = src[y1 * sw + x0], s = src[y1 * sw + x1];
    uint32_t out = 0;
#pragma unroll
    for (int ch = 0; ch < 4; ch++) {
        uint32_t v = ((p >> (8 * ch)) & 255u) + ((q >> (8 * ch)) & 255u) + ((r >> (8 * ch)) & 255u) +
                     ((s >> (8 * ch)) & 255u) + 2u;
        out |= (v >> 2) << (8 * ch);
    }
    dst[y * dw + x] = out;
}

cudaError_t launch_mip_level(const uint32_t* src, int sw, int sh, uint32_t* dst, int dw, int dh, cudaStream_t stream) {
    dim3 blk(16, 16), grd((dw + 15) / 16, (dh + 15) / 16);
    mip_kernel<<<grd, blk, 0, stream>>>(src, sw, sh, dst, dw, dh);
    return cudaGetLastError();
}

template <int S>
cudaError_t launch_tile(const PassArgs& a, int T, cudaStream_t stream, cudaEvent_t mid) {
    if (a.ordered) {
        static bool fconfigured = false;
        const size_t fbytes = forward_smem_bytes<S>();
        if (!fconfigured) {
            cudaError_t e = cudaFuncSetAttribute(forward_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fbytes);
            if (e != cudaSuccess) return e;
            fconfigured = true;
        }
        forward_kernel<S><<<T, kTileThreads, fbytes, stream>>>(a);
        if (mid) cudaEventRecord(mid, stream);
        return cudaSuccess;
    }
    static bool configured = false;
    const size_t rbytes = raster_smem_bytes<S>();
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(raster_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rbytes);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    raster_kernel<S><<<T, kTileThreads, rbytes, stream>>>(a);
    if (mid) cudaEventRecord(mid, stream);
    shade_kernel<S><<<T, kTileThreads, 0, stream>>>(a);
    return cudaSuccess;
}

cudaError_t launch_pass(const PassArgs& a, cudaStream_t stream, cudaEvent_t* ev) {
    const int T = a.c.tiles_x * a.c.tiles_y;
    if (ev) cudaEventRecord(ev[0], stream);
    if (a.total_tris > 0) {
        int blocks = (a.total_tris + 255) / 256;
        bin_count_kernel<<<blocks, 256, 0, stream>>>(a);
        if (ev) cudaEventRecord(ev[1], stream);
        scan_kernel<<<1, 1024, 0, stream>>>(a, T);
        if (ev) cudaEventRecord(ev[2], stream);
        bin_scatter_kernel<<<blocks, 256, 0, stream>>>(a);
        if (ev) cudaEventRecord(ev[3], stream);
    } else if (ev) {
        cudaEventRecord(ev[1], stream);
        cudaEventRecord(ev[2], stream);
        cudaEventRecord(ev[3], stream);
    }
    cudaError_t err = cudaSuccess;
    cudaEvent_t mid = ev ? ev[4] : nullptr;
    switch (a.c.S) {
    case 1: err = launch_tile<1>(a, T, stream, mid); break;
    case 2: err = launch_tile<2>(a, T, stream, mid); break;
    case 4: err = launch_tile<4>(a, T, stream, mid); break;
    case 8: err = launch_tile<8>(a, T, stream, mid); break;
    case 16: err = launch_tile<16>(a, T, stream, mid); break;
    default: err = cudaErrorInvalidValue;
    }
    if (ev) cudaEventRecord(ev[5], stream);
    return err != cudaSuccess ? err : cudaGetLastError();
}

}  // namespace ifr
