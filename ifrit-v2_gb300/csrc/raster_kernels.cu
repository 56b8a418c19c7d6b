// sm_103a kernels of one render pass (one or many views).
//
//   bin_count_kernel    per triangle: fetch + transform + clip + set up, count (tile, triangle)
//                       overlaps per screen tile of the triangle's view (reference: first and
//                       second binners, TileRasterCoreInvocationCuda.cu:721-1339; CPU
//                       executeBinner TileRasterWorker.cpp:314-397); unclipped triangles
//                       leave a compact 64-byte set-up record
//   scan_*_kernel       exclusive scan of the per-tile counts -> list offsets; resets counts
//   bin_scatter_kernel  same overlaps (from the records), scatters entries into tile lists
//   raster_kernel       persistent CTAs over a tile queue, one CTA per tile at a time: coverage
//                       + early depth test of every listed triangle with order-independent
//                       64-bit keys in shared memory (pixelTaggingExecKernel, .cu:1900-2142)
//   shade_kernel        persistent CTAs: deferred shading of the visible primitives with quad
//                       derivatives (pixelShadingExecKernel, .cu:2144-2317), on-chip MSAA
//                       resolve (.cu:2319-2361), one store of depth / visibility / colour
//   forward_kernel      ordered path: entries sorted into API order, per-sample depth test,
//                       shading and blend in order (.cu:1648-1897, TileRasterWorker.cpp:1517-1580)
//
// Visibility in the deferred path is order independent: a sample keeps the primitive that
// wins under the view's depth function with ties broken by API order (earlier wins for
// LESS/GREATER, later for LEQUAL/GEQUAL/EQUAL/ALWAYS), which is exactly what processing
// triangles in submission order produces.  So tile lists need no sorting there and the
// result is deterministic.
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cstring>

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

// Draw of triangle g for a full warp of consecutive triangles: lane 0 searches, and lanes past
// the end of its draw search on their own.
__device__ __forceinline__ int find_draw_warp(const PassArgs& a, int g) {
    int lead = 0;
    if ((threadIdx.x & 31) == 0) lead = find_draw(a, g);
    lead = __shfl_sync(0xffffffffu, lead, 0);
    return (g >= __ldg(a.draw_start + lead) && g < __ldg(a.draw_start + lead + 1)) ? lead : find_draw(a, g);
}

// Draw of a binned triangle (its record holds it).
__device__ __forceinline__ int record_draw(const PassArgs& a, int g) { return __ldg(&a.records[g].draw); }

__device__ __forceinline__ void bin_sub(const PassArgs& a, const ViewArgs& v, const DrawDev& d, SubTri s,
                                        uint32_t entry, bool scatter) {
    if (!scissor_clamp(d, s)) return;
    const int sh = v.c.tile_shift;
    int tx0 = s.px0 >> sh, tx1 = s.px1 >> sh;
    int ty0 = s.py0 >> sh, ty1 = s.py1 >> sh;
    for (int ty = ty0; ty <= ty1; ty++)
        for (int tx = tx0; tx <= tx1; tx++) {
            int tile = v.tile_start + ty * v.c.tiles_x + tx;
            if (scatter) {
                uint32_t pos = atomicAdd(a.tile_cursor + tile, 1u);
                if (pos < a.pair_capacity) a.pairs[pos] = entry;
            } else {
                atomicAdd(a.tile_count + tile, 1u);
            }
        }
}

// Front end of triangle g (draw di), shared by the counting binner and the atomic visibility
// path: fetch, transform, clip and set-up; writes the triangle's record (and vertex attributes)
// and hands every visible (sub-)triangle to emit(view, draw, sub-triangle, entry).
// What the counting pass leaves the scattering pass for a triangle (see bin_words).
enum BinKind { BIN_NONE = 0, BIN_RANGE = 1, BIN_CLIPPED = 2, BIN_MODE = 3 };

template <class Emit>
__device__ __forceinline__ void front_end(const PassArgs& a, int g, int di, const Emit& emit) {
    const DrawDev& d = a.draws[di];
    const ViewArgs& v = a.views[d.view];
    int t = g - __ldg(a.draw_start + di);
    CVert poly[3];  // registers: only the rare clipping path below goes through memory
    bool inside, rejected;
    TriRecord* rec = a.records + g;
    // culled triangles leave their record untouched: only binned entries' records are read
    if (!fetch_triangle(v.c, d, t, poly, inside, rejected)) return;
    if (d.polygon_mode != POLY_FILL) {  // LINE / POINT: record the projected triangle, emit its parts
        SubTri tri;
        if (!inside || !project_oriented(v.c, d, poly, tri)) return;
        emit.mark(BIN_MODE);
        TriRecord r;
        mode_record_from_tri(tri, r);
        r.draw = di;
        if (a.attrs && d.shading != SHADE_PRIMID && d.attr_count > 0) {
            float a0[4], a1[4], a2[4];
            fetch_attrs(d, t, a0, a1, a2);
            float4* dst = a.attrs[g].a;
            dst[0] = make_float4(a0[0], a0[1], a0[2], a0[3]);
            dst[1] = make_float4(a1[0], a1[1], a1[2], a1[3]);
            dst[2] = make_float4(a2[0], a2[1], a2[2], a2[3]);
        }
        const int4* src = reinterpret_cast<const int4*>(&r);
        int4* dst = reinterpret_cast<int4*>(rec);
        dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2]; dst[3] = src[3];
        for (int sub = 0; sub < 6; sub++) {
            SubTri s;
            if (mode_sub(v.c, d.polygon_mode, tri, sub, s)) emit(v, d, s, ((uint32_t)g << 3) | (uint32_t)sub);
        }
        return;
    }
    if (inside) {
        SubTri s;
        if (!setup_sub(v.c, d, poly[0], poly[1], poly[2], s)) return;
        TriRecord r;
        record_from_sub(s, r);
        r.draw = di;
        if (a.attrs && d.shading != SHADE_PRIMID && d.attr_count > 0) {
            float a0[4], a1[4], a2[4];
            fetch_attrs(d, t, a0, a1, a2);
            float4* dst = a.attrs[g].a;
            dst[0] = make_float4(a0[0], a0[1], a0[2], a0[3]);
            dst[1] = make_float4(a1[0], a1[1], a1[2], a1[3]);
            dst[2] = make_float4(a2[0], a2[1], a2[2], a2[3]);
        }
        const int4* src = reinterpret_cast<const int4*>(&r);
        int4* dst = reinterpret_cast<int4*>(rec);
        dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2]; dst[3] = src[3];
        emit(v, d, s, (uint32_t)g << 3);
        return;
    }
    emit.mark(BIN_CLIPPED);
    rec->flags = REC_CLIPPED;
    rec->draw = di;
    CVert clip[kMaxPoly];
    clip[0] = poly[0];
    clip[1] = poly[1];
    clip[2] = poly[2];
    int n = clip_polygon(v.c, clip);
    for (int i = 1; i + 1 < n; i++) {
        SubTri s;
        if (setup_sub(v.c, d, clip[0], clip[i], clip[i + 1], s)) emit(v, d, s, ((uint32_t)g << 3) | (uint32_t)(i - 1));
    }
}

// The tile range a lane hands to its warp: ranges over more than kWarpTiles tiles are walked by
// the whole warp one at a time (big); smaller ones (small) go through warp-aggregated atomics.
constexpr int kWarpTiles = 4;
struct WarpTiles {
    bool big, small;
    int kind;  // BIN_MODE / BIN_CLIPPED: the scattering pass re-emits the triangle's parts itself
    int tx0, tx1, ty0, ty1, tbase, tiles_x;
    uint32_t entry;  // list entry of a small range
};

// Bin word of every triangle of the pass (8 bytes, after the records in the same allocation), written
// by the counting pass so that the scattering pass need not read the records back:
//   x = tx0 | tx1 << 16, y = ty0 | ty1 << 14 | kind << 28 (the tile range, for BIN_RANGE); tile
//   coordinates stay below 2^11 (targets of at most 16384 pixels, tiles of at least 8).
__device__ __forceinline__ uint2* bin_words(const PassArgs& a) { return reinterpret_cast<uint2*>(a.records + a.total_tris); }

struct CountEmit {
    const PassArgs& a;
    WarpTiles& w;
    __device__ void mark(int kind) const { w.kind = kind; }
    __device__ void operator()(const ViewArgs& v, const DrawDev& d, const SubTri& s, uint32_t entry) const {
        SubTri c = s;
        if (w.big || w.small) {  // a second fan triangle of a clipped triangle (rare): direct atomics
            bin_sub(a, v, d, s, entry, false);
            return;
        }
        if (!scissor_clamp(d, c)) return;
        const int sh = v.c.tile_shift;
        w.tx0 = c.px0 >> sh; w.tx1 = c.px1 >> sh;
        w.ty0 = c.py0 >> sh; w.ty1 = c.py1 >> sh;
        w.tbase = v.tile_start;
        w.tiles_x = v.c.tiles_x;
        w.entry = entry;
        if ((w.tx1 - w.tx0 + 1) * (w.ty1 - w.ty0 + 1) > kWarpTiles) w.big = true;
        else w.small = true;
    }
};

// Warp-aggregated list slots for the lanes' small tile ranges (the scattering pass, whose atomics
// return the slot the store waits for; the counting pass needs no result and issues one
// fire-and-forget reduction per tile instead): for every tile slot k of the ranges, the lanes naming
// the same tile (__match_any_sync) make one atomicAdd of their count, issued by the lowest of them,
// and each lane's list slot is the returned base plus its rank among those lanes.  Lanes of a warp hold consecutive triangles, which in a mesh are
// neighbours and mostly share tiles.  List order within a tile carries no meaning (the
// order-independent stages key by entry, the ordered stage sorts).
__device__ __forceinline__ void warp_small_tiles(const PassArgs& a, const WarpTiles& w, bool scatter) {
    const unsigned lane = threadIdx.x & 31u;
    const int wd = w.small ? w.tx1 - w.tx0 + 1 : 1;
    const int n = w.small ? wd * (w.ty1 - w.ty0 + 1) : 0;
    const int nmax = __reduce_max_sync(0xffffffffu, n);
    for (int k = 0; k < nmax; k++) {
        const bool has = k < n;
        const uint32_t tile = has ? (uint32_t)(w.tbase + (w.ty0 + k / wd) * w.tiles_x + w.tx0 + k % wd) : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, tile);
        if (!has) continue;
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd((scatter ? a.tile_cursor : a.tile_count) + tile, (uint32_t)__popc(peers));
        if (scatter) {
            base = __shfl_sync(peers, base, leader);
            const uint32_t pos = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
            if (pos < a.pair_capacity) a.pairs[pos] = w.entry;
        }
    }
}

// The warp adds the counts (or, scattering, takes the list slots) of its lanes' large tile ranges,
// one range at a time.
__device__ __forceinline__ void warp_tiles(const PassArgs& a, const WarpTiles& w, int g, bool scatter) {
    const int lane = threadIdx.x & 31;
    unsigned m = __ballot_sync(0xffffffffu, w.big);
    while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const int sx0 = __shfl_sync(0xffffffffu, w.tx0, src), sx1 = __shfl_sync(0xffffffffu, w.tx1, src);
        const int sy0 = __shfl_sync(0xffffffffu, w.ty0, src), sy1 = __shfl_sync(0xffffffffu, w.ty1, src);
        const int sbase = __shfl_sync(0xffffffffu, w.tbase, src), stx = __shfl_sync(0xffffffffu, w.tiles_x, src);
        const uint32_t entry = (uint32_t)(g - lane + src) << 3;
        const int wd = sx1 - sx0 + 1, n = wd * (sy1 - sy0 + 1);
        for (int i = lane; i < n; i += 32) {
            const int tile = sbase + (sy0 + i / wd) * stx + sx0 + i % wd;
            if (scatter) {
                const uint32_t pos = atomicAdd(a.tile_cursor + tile, 1u);
                if (pos < a.pair_capacity) a.pairs[pos] = entry;
            } else {
                atomicAdd(a.tile_count + tile, 1u);
            }
        }
    }
}

// ---- bulk copies into shared memory (TMA, cp.async.bulk) with an mbarrier
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arms the barrier's current phase for `bytes` of bulk-copy data and copies [src, src + bytes)
// (both 16-byte aligned, bytes a multiple of 16) into shared memory at dst.  One thread.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// A CTA's bulk-copy barrier: phases used so far (the same in every thread), whether bulk copies
// are still in use, and whether one was left in flight after a wait gave up.
struct BulkState {
    uint64_t* bar;
    uint32_t phase;
    bool ok, pending;
};

// Waits for the barrier phase of the given parity, giving up after kBulkWaitLimit polls.
constexpr int kBulkWaitLimit = 1 << 20;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < kBulkWaitLimit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Counting pass: full front end per triangle; unclipped triangles leave a compact record.  (Bulk
// copies of each block's index slice into shared memory measured slower on this HBM-bound pass,
// whether waited for at once or prefetched a block ahead by persistent CTAs.)
__global__ void __launch_bounds__(256) bin_count_kernel(PassArgs a) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int di = find_draw_warp(a, min(g, a.total_tris - 1));
    WarpTiles w;
    w.big = w.small = false;
    w.kind = BIN_NONE;
    if (g < a.total_tris) {
        front_end(a, g, di, CountEmit{a, w});
        uint2 b = make_uint2(0u, (uint32_t)w.kind << 28);
        if (w.kind == BIN_NONE && (w.small || w.big))
            b = make_uint2((uint32_t)w.tx0 | ((uint32_t)w.tx1 << 16),
                           (uint32_t)w.ty0 | ((uint32_t)w.ty1 << 14) | ((uint32_t)BIN_RANGE << 28));
        bin_words(a)[g] = b;
    }
    if (w.small)  // counts need no result back: one fire-and-forget reduction per tile
        for (int ty = w.ty0; ty <= w.ty1; ty++)
            for (int tx = w.tx0; tx <= w.tx1; tx++) atomicAdd(a.tile_count + w.tbase + ty * w.tiles_x + tx, 1u);
    warp_tiles(a, w, g, false);
}

// Scattering pass: same overlaps as the counting pass, from its bin words (clipped triangles run the
// front end again, LINE / POINT parts come from their records).  Every list slot comes from an
// atomicAdd whose result the store waits for, so a triangle over many tiles would serialise hundreds of
// round trips in one thread: the tile ranges of unclipped triangles over more than kWarpTiles tiles are
// walked by the whole warp instead, and the smaller ones take their slots through warp-aggregated
// atomics.  Eight CTAs per SM (32 registers): the kernel waits on its slot atomics, and more warps hide
// them.
__global__ void __launch_bounds__(256, 8) bin_scatter_kernel(PassArgs a) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int di = find_draw_warp(a, min(g, a.total_tris - 1));
    WarpTiles w;
    w.big = w.small = false;
    if (g < a.total_tris && !a.status[ST_OVERFLOW]) {
        const uint2 b = bin_words(a)[g];
        const int kind = (int)(b.y >> 28);
        if (kind != BIN_NONE) {
            const DrawDev& d = a.draws[di];
            const ViewArgs& v = a.views[d.view];
            if (kind == BIN_RANGE) {  // the counting pass's tile range
                w.tx0 = (int)(b.x & 0xffffu); w.tx1 = (int)(b.x >> 16);
                w.ty0 = (int)(b.y & 0x3fffu); w.ty1 = (int)((b.y >> 14) & 0x3fffu);
                w.tbase = v.tile_start;
                w.tiles_x = v.c.tiles_x;
                w.entry = (uint32_t)g << 3;
                w.big = (w.tx1 - w.tx0 + 1) * (w.ty1 - w.ty0 + 1) > kWarpTiles;
                w.small = !w.big;
            } else if (kind == BIN_MODE) {
                SubTri tri;
                tri_from_mode_record(a.records + g, tri);
                for (int sub = 0; sub < 6; sub++) {
                    SubTri s;
                    if (mode_sub(v.c, d.polygon_mode, tri, sub, s))
                        bin_sub(a, v, d, s, ((uint32_t)g << 3) | (uint32_t)sub, true);
                }
            } else {  // clipped: the front end again
                const int t = g - __ldg(a.draw_start + di);
                CVert poly[kMaxPoly];
                bool inside, rejected;
                if (fetch_triangle(v.c, d, t, poly, inside, rejected)) {
                    const int n = clip_polygon(v.c, poly);
                    for (int i = 1; i + 1 < n; i++) {
                        SubTri s;
                        if (setup_sub(v.c, d, poly[0], poly[i], poly[i + 1], s))
                            bin_sub(a, v, d, s, ((uint32_t)g << 3) | (uint32_t)(i - 1), true);
                    }
                }
            }
        }
    }
    warp_small_tiles(a, w, true);
    warp_tiles(a, w, g, true);
}

// List offsets: exclusive scan of the per-tile counts in three launches (per-CTA scans of
// kScanTile tiles, a scan of the CTA totals, then the CTA offsets added back).  Also sets the
// scatter cursors, clears the counts for the next pass and checks the list capacity.
constexpr int kScanThreads = 1024;
constexpr int kScanTile = 4 * kScanThreads;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t* wsum, uint32_t& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t q = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += q;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = wsum[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t q = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += q;
        }
        wsum[lane] = wi - w;  // exclusive prefix of the warp totals
        if (lane == 31) wsum[32] = wi;
    }
    __syncthreads();
    total = wsum[32];
    return wsum[wid] + incl - x;
}

__global__ void __launch_bounds__(kScanThreads) scan_local_kernel(PassArgs a, int T) {
    __shared__ uint32_t wsum[33];
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    uint32_t c[4];
#pragma unroll
    for (int i = 0; i < 4; i++) c[i] = base + i < T ? a.tile_count[base + i] : 0u;
    uint32_t total;
    uint32_t run = block_exclusive_scan(c[0] + c[1] + c[2] + c[3], wsum, total);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        if (base + i < T) a.tile_offset[base + i] = run;
        run += c[i];
    }
    if (threadIdx.x == 0) a.block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(PassArgs a, int T, int nb) {
    __shared__ uint32_t wsum[33];
    const int per = (nb + kScanThreads - 1) / kScanThreads;
    const int b = min((int)threadIdx.x * per, nb), e = min(b + per, nb);
    uint32_t sum = 0;
    for (int i = b; i < e; i++) sum += a.block_sums[i];
    uint32_t total;
    uint32_t run = block_exclusive_scan(sum, wsum, total);
    for (int i = b; i < e; i++) {
        const uint32_t x = a.block_sums[i];
        a.block_sums[i] = run;
        run += x;
    }
    if (threadIdx.x == 0) {
        a.tile_offset[T] = total;
        a.status[ST_PAIRS] = total;
        atomicMax(a.status + ST_MAX_PAIRS, total);
        if (total > a.pair_capacity) {
            a.status[ST_OVERFLOW] = 1u;
            atomicOr(a.status + ST_STICKY, 1u);
        }
    }
}

// Up to kScanSingle tiles: the whole scan in one launch.  Warp w owns tiles [1024 w, 1024 w + 1024),
// read and written coalesced as 32 rows of 32 (tile 1024 w + 32 i + lane in row i); rows are
// scanned across the lanes in order, then the warp totals across the block.
constexpr int kScanRows = 32;
constexpr int kScanSingle = kScanRows * kScanThreads;

__global__ void __launch_bounds__(kScanThreads) scan_single_kernel(PassArgs a, int T) {
    __shared__ uint32_t wsum[33];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int first = wid * 32 * kScanRows + lane;
    uint32_t ex[kScanRows];
    uint32_t run = 0;
#pragma unroll
    for (int i = 0; i < kScanRows; i++) {
        const int t = first + 32 * i;
        ex[i] = t < T ? a.tile_count[t] : 0u;
    }
#pragma unroll
    for (int i = 0; i < kScanRows; i++) {
        const uint32_t x = ex[i];
        uint32_t incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t q = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += q;
        }
        ex[i] = run + incl - x;
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) wsum[wid] = run;
    __syncthreads();
    if (wid == 0) {
        const uint32_t w = wsum[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t q = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += q;
        }
        wsum[lane] = wi - w;
        if (lane == 31) wsum[32] = wi;
    }
    __syncthreads();
    const uint32_t add = wsum[wid], total = wsum[32];
#pragma unroll
    for (int i = 0; i < kScanRows; i++) {
        const int t = first + 32 * i;
        if (t < T) {
            a.tile_offset[t] = add + ex[i];
            a.tile_cursor[t] = add + ex[i];
            a.tile_count[t] = 0u;
        }
    }
    if (threadIdx.x == 0) {
        a.tile_offset[T] = total;
        a.status[ST_PAIRS] = total;
        atomicMax(a.status + ST_MAX_PAIRS, total);
        if (total > a.pair_capacity) {
            a.status[ST_OVERFLOW] = 1u;
            atomicOr(a.status + ST_STICKY, 1u);
        }
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(PassArgs a, int T) {
    const uint32_t add = a.block_sums[blockIdx.x];
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int t = base + i;
        if (t < T) {
            const uint32_t off = a.tile_offset[t] + add;
            a.tile_offset[t] = off;
            a.tile_cursor[t] = off;
            a.tile_count[t] = 0u;
        }
    }
}

// Initial depth of sample k of pixel (x, y) for the explicit-compare key modes.
__device__ __forceinline__ float d0_of(const ViewArgs& v, int x, int y, int k) {
    return v.clear ? v.clear_depth : v.depth[((size_t)y * v.c.W + x) * v.c.S + k];
}

__device__ __forceinline__ void decode_color(const ViewArgs& v, size_t pix, float c[4]) {
    switch (v.format) {
    case FMT_RGBA8: unpack_rgba8(static_cast<const uint32_t*>(v.color)[pix], c); break;
    case FMT_RGBA16F: {
        uint2 q = static_cast<const uint2*>(v.color)[pix];
        c[0] = __half2float(__ushort_as_half((unsigned short)(q.x & 0xffffu)));
        c[1] = __half2float(__ushort_as_half((unsigned short)(q.x >> 16)));
        c[2] = __half2float(__ushort_as_half((unsigned short)(q.y & 0xffffu)));
        c[3] = __half2float(__ushort_as_half((unsigned short)(q.y >> 16)));
        break;
    }
    case FMT_RGBA32F: {
        float4 q = static_cast<const float4*>(v.color)[pix];
        c[0] = q.x; c[1] = q.y; c[2] = q.z; c[3] = q.w;
        break;
    }
    default: {
        const float* p = static_cast<const float*>(v.color) + pix * 3;
        c[0] = p[0]; c[1] = p[1]; c[2] = p[2]; c[3] = 1.0f;
        break;
    }
    }
}

__device__ __forceinline__ void encode_color(const ViewArgs& v, size_t pix, const float c[4]) {
    switch (v.format) {
    case FMT_RGBA8: {
        uint32_t q = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            float x = fminf(fmaxf(c[i], 0.0f), 1.0f);
            q |= __float2uint_rn(x * 255.0f) << (8 * i);
        }
        static_cast<uint32_t*>(v.color)[pix] = q;
        break;
    }
    case FMT_RGBA16F: {
        uint2 q;
        q.x = (uint32_t)__half_as_ushort(__float2half_rn(c[0])) | ((uint32_t)__half_as_ushort(__float2half_rn(c[1])) << 16);
        q.y = (uint32_t)__half_as_ushort(__float2half_rn(c[2])) | ((uint32_t)__half_as_ushort(__float2half_rn(c[3])) << 16);
        static_cast<uint2*>(v.color)[pix] = q;
        break;
    }
    case FMT_RGBA32F: static_cast<float4*>(v.color)[pix] = make_float4(c[0], c[1], c[2], c[3]); break;
    default: {
        float* p = static_cast<float*>(v.color) + pix * 3;
        p[0] = c[0]; p[1] = c[1]; p[2] = c[2];
        break;
    }
    }
}

// ---------------------------------------------------------------------------- visibility keys
// Every sample holds one 64-bit key in shared memory; a fragment that passes the depth test
// lowers it with atomicMin, so the final key is the same whatever the order fragments arrive in:
//   high word: depth order  (LESS/LEQUAL: z ascending, GREATER/GEQUAL: descending; 0 for the
//              functions whose pass test is an explicit compare against the initial depth)
//   low word:  entry order  (entry = global triangle << 3 | fan index; "earliest wins" modes
//              store entry + 1 with the background at 0, "latest wins" modes store
//              0xFFFFFFFE - entry with the background at 0xFFFFFFFF)
// Ties therefore resolve exactly as submission-order processing does.
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
// The depth a depth-order word stands for (inverse of depth_order).
__device__ __forceinline__ float order_depth(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Whether ordered entry e may pass its depth test anywhere in a tile whose farthest prefix depth
// is dmax (its samples' depths only decrease from there: ViewArgs::ordered_cull).  Conservative:
// true unless the entry is an unclipped filled triangle under LESS / LEQUAL / EQUAL (or NEVER)
// whose depth plane, over its bounding box clipped to the tile's sample positions, lies beyond
// dmax by more than the rounding of the per-sample evaluation (2^-20 of the terms' magnitudes).
__device__ __forceinline__ bool may_pass_tile(const PassArgs& a, const PassConst& c, uint32_t e, int tx0, int ty0,
                                              int xmax, int ymax, float dmax) {
    const int g = (int)(e >> 3);
    if ((e & 7u) != 0u) return true;
    const TriRecord* rp = a.records + g;
    const int4 q1 = __ldg(reinterpret_cast<const int4*>(rp) + 1);  // X2, Y2, flags, draw
    if (!(q1.z & REC_VALID)) return true;
    const DrawDev& d = a.draws[q1.w];
    if (d.polygon_mode != POLY_FILL) return true;
    const int f = d.depth_func;
    if (f == 0) return false;  // NEVER
    if (f != 1 && f != 3 && f != 2) return true;
    const int4 q0 = __ldg(reinterpret_cast<const int4*>(rp));
    const float4 q2 = __ldg(reinterpret_cast<const float4*>(rp) + 2);  // z0, dz/dx, dz/dy
    const int32_t sx0 = max(min(q0.x, min(q0.z, q1.x)), tx0 * 256 + c.smin_x);
    const int32_t sx1 = min(max(q0.x, max(q0.z, q1.x)), xmax * 256 + c.smax_x);
    const int32_t sy0 = max(min(q0.y, min(q0.w, q1.y)), ty0 * 256 + c.smin_y);
    const int32_t sy1 = min(max(q0.y, max(q0.w, q1.y)), ymax * 256 + c.smax_y);
    if (sx0 > sx1 || sy0 > sy1) return false;  // no sample of the tile inside its bounding box
    const float ax = q2.y * (float)(sx0 - q0.x), bx = q2.y * (float)(sx1 - q0.x);
    const float ay = q2.z * (float)(sy0 - q0.y), by = q2.z * (float)(sy1 - q0.y);
    const float zmin = (q2.x + fminf(ax, bx)) + fminf(ay, by);
    const float margin = (fabsf(q2.x) + fmaxf(fabsf(ax), fabsf(bx)) + fmaxf(fabsf(ay), fabsf(by))) * 0x1p-20f;
    return !(zmin - margin > dmax);
}

// ---------------------------------------------------------------------------- atomic visibility
// Alternative to binning + the tile raster stage for deferred views: the thread of each triangle
// resolves its own samples straight into per-sample 64-bit keys in global memory with atomicMin
// (the tile stage's keys, so the winners are the same); the shade stage then reads the keys.
// Suited to views of small triangles, where binning and per-tile set-up dominate.
template <int S>
__global__ void __launch_bounds__(256) init_keys_kernel(PassArgs a, int npix) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const ViewArgs& v = a.views[0];
    const KeyRule rule = key_rule(v.depth_func, v.depth_write);
#pragma unroll
    for (int k = 0; k < S; k++) {
        const float d0 = v.clear ? v.clear_depth : v.depth[(size_t)p * S + k];
        v.keys[(size_t)p * S + k] = background_key(rule, d0);
    }
}

template <int S>
struct GlobalRasterEmit {
    __device__ void mark(int) const {}
    __device__ void operator()(const ViewArgs& v, const DrawDev& d, SubTri s, uint32_t entry) const {
        if (!scissor_clamp(d, s)) return;
        const KeyRule rule = key_rule(v.depth_func, v.depth_write);
        if (rule.func == 0) return;  // NEVER
        const uint32_t lo_word = rule.mode == KM_EARLIEST ? entry + 1u : 0xFFFFFFFEu - entry;
        for (int py = s.py0; py <= s.py1; py++) {
            for (int px = s.px0; px <= s.px1; px++) {
                if (d.scissor_count && !scissor_pass(d, px, py)) continue;
                const size_t pix = (size_t)py * v.c.W + px;
                // the tile stage's depth expression (see raster_tile)
                const float fbx = (float)(px * 256 - s.X[0]), fby = (float)(py * 256 - s.Y[0]);
#pragma unroll
                for (int k = 0; k < S; k++) {
                    if (!covered(s.A, s.B, s.Cb, px * 256 + sample_x<S>(k), py * 256 + sample_y<S>(k))) continue;
                    const float z = (s.z[0] + s.dzdx * (fbx + (float)sample_x<S>(k))) + s.dzdy * (fby + (float)sample_y<S>(k));
                    uint32_t hi_word;
                    if (rule.explicit_) {
                        if (!depth_cmp(rule.func, z, d0_of(v, px, py, k))) continue;
                        hi_word = 0u;
                    } else {
                        hi_word = rule.invert ? ~depth_order(z) : depth_order(z);
                    }
                    const unsigned long long kv = ((unsigned long long)hi_word << 32) | lo_word;
                    unsigned long long* kp = v.keys + pix * S + k;
                    if (kv < *kp) atomicMin(kp, kv);  // keys only fall: a stale read only costs an atomic
                }
            }
        }
    }
};

template <int S>
__global__ void __launch_bounds__(256) atomic_front_kernel(PassArgs a) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int di = find_draw_warp(a, min(g, a.total_tris - 1));
    if (g >= a.total_tris) return;
    front_end(a, g, di, GlobalRasterEmit<S>{});
}

// Set-up of entry e (global triangle << 3 | fan index) for shading: geometry + depth plane.
__device__ __noinline__ void setup_entry(const PassArgs& a, const PassConst& c, int e, ShadeGeom* g, RecordPlane* pl) {
    int gi = e >> 3, sub = e & 7;
    int di = record_draw(a, gi);
    SubTri s;
    setup_entry_sub(c, a.draws[di], a.records, gi, gi - __ldg(a.draw_start + di), sub, s);
    shade_geom_from(s, *g);
    pl->z0 = s.z[0];
    pl->dzdx = s.dzdx;
    pl->dzdy = s.dzdy;
    pl->X0 = s.X[0];
    pl->Y0 = s.Y[0];
}

// Raster set-up of entry e for the batch phase (out of line: one copy of the clip path).
__device__ __noinline__ bool setup_raster_entry(const PassArgs& a, const PassConst& c, uint32_t e, SubTri* s, int* draw) {
    int g = (int)(e >> 3), sub = (int)(e & 7u);
    int di = record_draw(a, g);
    *draw = di;
    const DrawDev& d = a.draws[di];
    return setup_entry_sub(c, d, a.records, g, g - __ldg(a.draw_start + di), sub, *s) && scissor_clamp(d, *s);
}

// Set-up and shading of one entry at one pixel (out of line: the rare paths share one copy).
__device__ __noinline__ void shade_uncached(const PassArgs& a, const PassConst& c, int e, int px, int py, float* col,
                                            RecordPlane* pl) {
    ShadeGeom g;
    setup_entry(a, c, e, &g, pl);
    int gi = e >> 3, sub = e & 7;
    int di = record_draw(a, gi);
    shade_fragment(c, a.draws[di], g, gi - __ldg(a.draw_start + di), sub, px, py, col);
}

// ---------------------------------------------------------------------------- persistent tiles
// Pulls the next tile of the group from its queue and stages its view's arguments in shared
// memory (the copy is skipped when the view did not change).  Returns false when the queue is
// empty.  Must be called by the whole CTA.
template <int NT>
__device__ __forceinline__ bool next_tile(const PassArgs& a, const GroupArgs& g, int qslot, ViewArgs& sv, int& s_tile,
                                          int& s_view) {
    const int tid = threadIdx.x;
    __syncthreads();  // everyone is done with the previous tile's staged data
    if (tid == 0) {
        int t = g.tile_begin + (int)atomicAdd(a.queues + qslot, 1u);
        int vi = -1;
        if (t < g.tile_end) {
            int lo = g.view_begin, hi = g.view_end - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (__ldg(a.view_tile_start + mid) <= t) lo = mid; else hi = mid - 1;
            }
            vi = lo;
        }
        s_tile = t;
        if (vi != s_view) s_view = vi | 0x40000000;  // mark: copy needed
    }
    __syncthreads();
    if (s_tile >= g.tile_end) return false;
    if (s_view & 0x40000000) {
        const int vi = s_view & 0x3fffffff;
        const int* src = reinterpret_cast<const int*>(a.views + vi);
        int* dst = reinterpret_cast<int*>(&sv);
        for (int i = tid; i < (int)(sizeof(ViewArgs) / 4); i += NT) dst[i] = src[i];
        __syncthreads();
        if (tid == 0) s_view = vi;
        __syncthreads();
    }
    return true;
}

// Pixel of lane `tid` in a TS x TS tile: 2x2 quads on consecutive lanes, quads row-major.
template <int TS>
__device__ __forceinline__ void tile_pixel(int tid, int& lx, int& ly) {
    constexpr int QR = TS / 2;
    lx = ((tid >> 2) % QR) * 2 + (tid & 1);
    ly = ((tid >> 2) / QR) * 2 + ((tid >> 1) & 1);
}

// ---------------------------------------------------------------------------- raster stage
// Edge functions are kept relative to the tile origin.  A record whose snapped vertices span
// less than 32 pixels in x and in y has |A|, |B| < 8192 (1/256 pixel units) and every sample of
// a 16x16 tile overlapping its bbox lies within 48 pixels (12288 units) of vertex 0, so each edge
// function there is below 2^28 in magnitude and coverage is evaluated exactly in 32-bit
// arithmetic.  Larger records keep the 64-bit edge functions.
constexpr int kLargeRecord = 1;
constexpr int32_t kSmallSpan = 32 * 256;

// Spans of one batch: a span is one tile row of one record's conservative column range.
template <int NT>
__host__ __device__ constexpr int span_capacity() { return NT >= 256 ? 2048 : 8 * NT; }

template <int NT>
struct TileRecords {
    int32_t A[3][NT], B[3][NT];
    long long Et[3][NT];  // biased edge functions at the tile origin
    float z0[NT], dzdx[NT], dzdy[NT];
    int32_t X0[NT], Y0[NT];
    int32_t meta[NT];     // kLargeRecord | (draw + 1) << 1 when the draw has a scissor test
    int32_t key[NT];      // entry
    // pixel offset of the span in the batch (16 bits) | record << 16 | row << 24 | first column << 28
    uint32_t span[span_capacity<NT>()];
};

// Conservative covered columns of every tile row of a record.  A pixel (c, r) of the tile can
// hold a covered sample only if, for every edge, E(256c, 256r) + max_k (A sx_k + B sy_k) >= 0
// (the largest value of the edge over the pixel's sample pattern).  Each edge with A != 0 bounds c
// from one side at the crossing column t = -(E(0, 256r) + max_k(..)) / (256 A), computed in float
// from the exact integer with a relative error below 2^-21 (three roundings), i.e. below 10^-5
// columns where it matters (|t| <= TS + 2); rounding t -+ 2^-10 up / down keeps the bound
// conservative without widening it by a column.  An edge with A == 0 empties the row when its
// largest value is negative.  A record's rows are packed as lo | hi << 4 per row, row r in bits
// 8(r mod 4) of word r / 4; an empty row is 0x0f.
template <int TS>
struct RowSpans {
    uint32_t w[TS / 4];
    int nspan, npix;
    bool large;  // the record needs the 64-bit coverage test
};

// What a row job needs of its record: the largest value of each edge over the pixel's sample
// pattern at tile column 0, row 0 (exact), -1 / (256 A) (0 for A == 0), B, and the record's
// clipped column range and first row.
struct SpanEdges {
    long long base0[3];
    float rcp[3];
    int32_t B[3];
    int box;  // cx0 | cx1 << 4 | ry0 << 8
};

template <int S>
__device__ __forceinline__ void span_edges(const int32_t A[3], const int32_t B[3], const long long Et[3], int cx0,
                                           int cx1, int ry0, SpanEdges& o) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        long long m = (long long)A[i] * sample_x<S>(0) + (long long)B[i] * sample_y<S>(0);
#pragma unroll
        for (int k = 1; k < S; k++) m = max(m, (long long)A[i] * sample_x<S>(k) + (long long)B[i] * sample_y<S>(k));
        o.base0[i] = Et[i] + m;
        o.rcp[i] = A[i] != 0 ? -1.0f / (256.0f * (float)A[i]) : 0.0f;
        o.B[i] = B[i];
    }
    o.box = cx0 | (cx1 << 4) | (ry0 << 8);
}

// Span code of tile row r of a record (lo | hi << 4, or 0x0f when empty).
template <int TS>
__device__ __forceinline__ uint32_t span_code(const SpanEdges& q, int r) {
    constexpr float kEps = 1.0f / 1024.0f;
    int lo = q.box & 15, hi = (q.box >> 4) & 15;
    bool empty = false;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const long long b = q.base0[i] + (long long)q.B[i] * (256 * r);
        const float t = fminf(fmaxf((float)b * q.rcp[i], -2.0f), (float)TS + 1.0f);
        if (q.rcp[i] < 0.0f) lo = max(lo, (int)ceilf(t - kEps));        // A > 0
        else if (q.rcp[i] > 0.0f) hi = min(hi, (int)floorf(t + kEps));  // A < 0
        else empty |= b < 0;
    }
    return empty || lo > hi ? 0x0fu : (uint32_t)(lo | (hi << 4));
}

// Raster set-up of one binned entry, clipped to the tile, in registers.
struct RasterRec {
    int32_t A[3], B[3];
    long long Et[3];  // biased edge functions at the tile origin
    float z0, dzdx, dzdy;
    int32_t X0, Y0;
    int x0, x1, y0, y1;  // covered pixel range within the tile (absolute pixels)
    bool small;
};

// Unclipped fill-mode triangles are set up straight from their record: the same integers and
// stored floats as the general set-up (sub_from_record, sub_bbox, sub_edges, scissor_clamp), with
// the edge constants of small records formed in 32 bits at the tile origin.  Everything else
// (clipped fan triangles, LINE / POINT parts) goes through the general set-up.
__device__ __forceinline__ bool raster_entry(const PassArgs& a, const PassConst& c, uint32_t e, int tx0, int ty0,
                                             int xmax, int ymax, RasterRec& o, int& di) {
    const int g = (int)(e >> 3), sub = (int)(e & 7u);
    const TriRecord* rp = a.records + g;
    const int4 q1 = __ldg(reinterpret_cast<const int4*>(rp) + 1);
    di = q1.w;
    const DrawDev& d = a.draws[di];
    int32_t X[3], Y[3];
    int px0, px1, py0, py1;
    if (sub == 0 && (q1.z & REC_VALID) && d.polygon_mode == POLY_FILL) {
        const int4 q0 = __ldg(reinterpret_cast<const int4*>(rp));
        const float4 q2 = __ldg(reinterpret_cast<const float4*>(rp) + 2);
        X[0] = q0.x; Y[0] = q0.y; X[1] = q0.z; Y[1] = q0.w; X[2] = q1.x; Y[2] = q1.y;
        o.z0 = q2.x; o.dzdx = q2.y; o.dzdy = q2.z;
        const int32_t xmn = min(X[0], min(X[1], X[2])), xmx = max(X[0], max(X[1], X[2]));
        const int32_t ymn = min(Y[0], min(Y[1], Y[2])), ymx = max(Y[0], max(Y[1], Y[2]));
        // snapped coordinates are within the guard band (|X|, |Y| < 2^24): floor division by 256
        // is an arithmetic shift
        px0 = max(-((c.smax_x - xmn) >> 8), 0);
        px1 = min((xmx - c.smin_x) >> 8, c.W - 1);
        py0 = max(-((c.smax_y - ymn) >> 8), 0);
        py1 = min((ymx - c.smin_y) >> 8, c.H - 1);
        if (d.scissor_count) {
            px0 = max(px0, d.scissor_box[0]);
            py0 = max(py0, d.scissor_box[1]);
            px1 = min(px1, d.scissor_box[2]);
            py1 = min(py1, d.scissor_box[3]);
        }
        o.small = xmx - xmn < kSmallSpan && ymx - ymn < kSmallSpan;
    } else {
        SubTri s;
        int sdi;
        if (!setup_raster_entry(a, c, e, &s, &sdi)) return false;
        di = sdi;
#pragma unroll
        for (int i = 0; i < 3; i++) { X[i] = s.X[i]; Y[i] = s.Y[i]; }
        o.z0 = s.z[0]; o.dzdx = s.dzdx; o.dzdy = s.dzdy;
        px0 = s.px0; px1 = s.px1; py0 = s.py0; py1 = s.py1;
        const int32_t xmn = min(X[0], min(X[1], X[2])), xmx = max(X[0], max(X[1], X[2]));
        const int32_t ymn = min(Y[0], min(Y[1], Y[2])), ymx = max(Y[0], max(Y[1], Y[2]));
        o.small = xmx - xmn < kSmallSpan && ymx - ymn < kSmallSpan;
    }
    o.x0 = max(px0, tx0); o.x1 = min(px1, xmax);
    o.y0 = max(py0, ty0); o.y1 = min(py1, ymax);
    if (o.x0 > o.x1 || o.y0 > o.y1) return false;
    o.X0 = X[0];
    o.Y0 = Y[0];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        o.A[i] = Y[j] - Y[k];
        o.B[i] = X[k] - X[j];
        const int bias = (o.A[i] > 0) || (o.A[i] == 0 && o.B[i] > 0) ? 0 : 1;
        // E_i(x, y) = A (x - X_j) + B (y - Y_j) - bias
        if (o.small)
            o.Et[i] = (long long)(o.A[i] * (tx0 * 256 - X[j]) + o.B[i] * (ty0 * 256 - Y[j]) - bias);
        else
            o.Et[i] = (long long)o.A[i] * (tx0 * 256 - X[j]) + (long long)o.B[i] * (ty0 * 256 - Y[j]) - bias;
    }
    return true;
}

// Depth test of the covered samples of one queued pixel: record | x << 8 | y << 12 | samples << 16.
template <int S, int TS>
__device__ __forceinline__ void raster_depth(const ViewArgs& v, const KeyRule& rule, const TileRecords<TS * TS>& rec,
                                             unsigned long long* skey, int tx0, int ty0, uint32_t item) {
    const int r = (int)(item & 0xffu), qx = (int)((item >> 8) & 15u), qy = (int)((item >> 12) & 15u);
    const unsigned cov = item >> 16;
    const int gx = tx0 + qx, gy = ty0 + qy;
    const float z0 = rec.z0[r], gzx = rec.dzdx[r], gzy = rec.dzdy[r];
    const int32_t X0 = rec.X0[r], Y0 = rec.Y0[r];
    const uint32_t e = (uint32_t)rec.key[r];
    const uint32_t lo_word = rule.mode == KM_EARLIEST ? e + 1u : 0xFFFFFFFEu - e;
    // sample-major keys ([sample][pixel]): lanes on different pixels spread over the banks
    unsigned long long* kp = skey + qy * TS + qx;
    // (float)(sx - X0) == fbx + sample offset exactly: every term is an integer below
    // 2^24 in magnitude (guard-band bound), so no conversion per sample is needed.
    const float fbx = (float)(gx * 256 - X0), fby = (float)(gy * 256 - Y0);
    if (rule.explicit_) {  // pass decided by a compare against the initial depth (rare): depth word 0
#pragma unroll 1
        for (unsigned m = cov; m; m &= m - 1) {
            const int k = __ffs((int)m) - 1;
            const float z = (z0 + gzx * (fbx + (float)sample_at<S>(k, 0))) + gzy * (fby + (float)sample_at<S>(k, 1));
            if (depth_cmp(rule.func, z, d0_of(v, gx, gy, k))) atomicMin(kp + k * (TS * TS), (unsigned long long)lo_word);
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < S; k++) {
        if (!(cov & (1u << k))) continue;
        const float z = (z0 + gzx * (fbx + (float)sample_x<S>(k))) + gzy * (fby + (float)sample_y<S>(k));
        const uint32_t hi_word = rule.invert ? ~depth_order(z) : depth_order(z);
        atomicMin(kp + k * (TS * TS), ((unsigned long long)hi_word << 32) | lo_word);
    }
}

// One tile: the tile's list is consumed in batches of up to NT set-ups.  Every record's clipped
// bbox is cut into conservative row spans; the batch's spans are laid end to end and every pixel
// of them is visited by one lane (each warp walks a contiguous range, finding the span of each of
// its 32 pixels from a window of the next 32 span starts).  Each covered sample that passes the
// depth test lowers its key.  A batch holds at most span_capacity spans; records beyond that go to
// the next batch.  The winning entry of every sample (or -1) is written for the shading stage.
template <int S, int TS>
__device__ __forceinline__ void raster_tile(const PassArgs& a, const ViewArgs& v, int gtile, TileRecords<TS * TS>& rec,
                                            unsigned long long* skey, uint32_t* warp_sum) {
    constexpr int NT = TS * TS, NW = NT / 32, CAP = span_capacity<NT>();
    __shared__ uint32_t s_total[4];
    __shared__ uint32_t s_queue[NW * 64];
    uint32_t* wq = s_queue + (threadIdx.x >> 5) * 64;
    const int ltile = gtile - v.tile_start;
    const int tx = ltile % v.c.tiles_x, ty = ltile / v.c.tiles_x;
    const int tx0 = tx * TS, ty0 = ty * TS;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int lx, ly;
    tile_pixel<TS>(tid, lx, ly);
    const int px = tx0 + lx, py = ty0 + ly;
    const bool inpix = px < v.c.W && py < v.c.H;
    const size_t pix = (size_t)py * v.c.W + px;
    const KeyRule rule = key_rule(v.depth_func, v.depth_write);

#pragma unroll
    for (int k = 0; k < S; k++) {
        float d0 = v.clear ? v.clear_depth : (inpix ? v.depth[pix * S + k] : 0.0f);
        skey[k * (TS * TS) + ly * TS + lx] = background_key(rule, d0);
    }
    const bool has_list = a.total_tris > 0 && a.status[ST_OVERFLOW] == 0 && rule.func != 0;
    const uint32_t beg = has_list ? a.tile_offset[gtile] : 0u;
    const uint32_t end = has_list ? a.tile_offset[gtile + 1] : 0u;
    const int xmax = min(v.c.W, tx0 + TS) - 1, ymax = min(v.c.H, ty0 + TS) - 1;

    for (uint32_t base = beg; base < end;) {
        const int nb = (int)min((uint32_t)NT, end - base);
        RowSpans<TS> rs;  // every row empty unless the record is set up below
        rs.nspan = 0;
        rs.npix = 0;
        rs.large = false;
#pragma unroll
        for (int q = 0; q < TS / 4; q++) rs.w[q] = 0x0f0f0f0fu;
        bool in_stage = true;
        SpanEdges se;  // the record's row-span inputs (rows = 0: no spans)
        se.box = 0;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            se.base0[i] = 0;
            se.rcp[i] = 0.0f;
            se.B[i] = 0;
        }
        int rows = 0;
        if (tid < nb) {
            uint32_t e = __ldg(a.pairs + base + tid);
            RasterRec s;
            int di;
            // ordered views: only the order-independent prefix is resolved here
            in_stage = !v.ordered || (int)(e >> 3) < v.first_tri + v.ordered_prefix;
            if (in_stage && raster_entry(a, v.c, e, tx0, ty0, xmax, ymax, s, di)) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    rec.A[i][tid] = s.A[i];
                    rec.B[i][tid] = s.B[i];
                    rec.Et[i][tid] = s.Et[i];
                }
                rec.z0[tid] = s.z0;
                rec.dzdx[tid] = s.dzdx;
                rec.dzdy[tid] = s.dzdy;
                rec.X0[tid] = s.X0;
                rec.Y0[tid] = s.Y0;
                rec.meta[tid] = (s.small ? 0 : kLargeRecord) | (a.draws[di].scissor_count ? (di + 1) << 1 : 0);
                span_edges<S>(s.A, s.B, s.Et, s.x0 - tx0, s.x1 - tx0, s.y0 - ty0, se);
                rows = s.y1 - s.y0 + 1;
                rs.large = !s.small;
            }
            rec.key[tid] = (int)e;
        }
        // Row spans of the warp's records: their (record, row) jobs, rows of one record consecutive,
        // are spread over the lanes; each job's code goes to the record's bytes in the warp's
        // row-code scratch, which aliases the span list (written only after the block scan below).
        {
            uint8_t* rcode = reinterpret_cast<uint8_t*>(rec.span) + wid * 32 * TS;
            uint32_t* mine = reinterpret_cast<uint32_t*>(rcode + lane * TS);
#pragma unroll
            for (int q = 0; q < TS / 4; q++) mine[q] = 0x0f0f0f0fu;
            int jincl = rows;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int q = __shfl_up_sync(0xffffffffu, jincl, o);
                if (lane >= o) jincl += q;
            }
            const int J = __shfl_sync(0xffffffffu, jincl, 31), jpre = jincl - rows;
            __syncwarp();
            for (int c0 = 0; c0 < J; c0 += 32) {
                const int j = c0 + lane;
                int k = 0;  // the record of job j: the last lane whose first job is at or before j
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (__shfl_sync(0xffffffffu, jpre, k + step) <= j) k += step;
                SpanEdges q;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    q.base0[i] = __shfl_sync(0xffffffffu, se.base0[i], k);
                    q.rcp[i] = __shfl_sync(0xffffffffu, se.rcp[i], k);
                    q.B[i] = __shfl_sync(0xffffffffu, se.B[i], k);
                }
                q.box = __shfl_sync(0xffffffffu, se.box, k);
                const int kpre = __shfl_sync(0xffffffffu, jpre, k);
                if (j < J) {
                    const int r = ((q.box >> 8) & 15) + (j - kpre);
                    rcode[k * TS + r] = (uint8_t)span_code<TS>(q, r);
                }
            }
            __syncwarp();
#pragma unroll
            for (int q = 0; q < TS / 4; q++) {
                const uint32_t w = mine[q];
                rs.w[q] = w;
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const uint32_t lo = (w >> (8 * b)) & 15u, hi = (w >> (8 * b + 4)) & 15u;
                    rs.nspan += lo <= hi ? 1 : 0;
                    rs.npix += lo <= hi ? (int)(hi - lo + 1) : 0;
                }
            }
        }
        // block-wide exclusive scan of (pixels | spans << 17) per record, small and large records
        // counted apart: the spans of large records (64-bit coverage tests) follow those of the
        // small ones, so that warps rarely mix the two tests
        const uint32_t cnt = (uint32_t)rs.npix | ((uint32_t)rs.nspan << 17);
        const bool large = rs.large;
        uint32_t incl_s = large ? 0u : cnt, incl_l = large ? cnt : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t qs = __shfl_up_sync(0xffffffffu, incl_s, o);
            const uint32_t ql = __shfl_up_sync(0xffffffffu, incl_l, o);
            if (lane >= o) {
                incl_s += qs;
                incl_l += ql;
            }
        }
        if (lane == 31) {
            warp_sum[wid] = incl_s;
            warp_sum[NW + wid] = incl_l;
        }
        __syncthreads();
#pragma unroll
        for (int w = 0; w < NW; w++) {
            incl_s += w < wid ? warp_sum[w] : 0u;
            incl_l += w < wid ? warp_sum[NW + w] : 0u;
        }
        const bool fits = tid < nb && (incl_s >> 17) + (incl_l >> 17) <= (uint32_t)CAP;
        const int consumed = __syncthreads_count(fits);
        if (tid == consumed - 1) {
            s_total[0] = incl_s & 0x1ffffu;  // pixels and spans of the small records
            s_total[1] = incl_s >> 17;
            s_total[2] = incl_l & 0x1ffffu;  // pixels and spans of the large records
            s_total[3] = incl_l >> 17;
        }
        __syncthreads();
        const uint32_t Ps = s_total[0], Ns = s_total[1];
        const uint32_t P = Ps + s_total[2];
        const int NSP = (int)(Ns + s_total[3]);
        if (fits) {
            const uint32_t first = (large ? incl_l : incl_s) - cnt;
            uint32_t sp = (first >> 17) + (large ? Ns : 0u), p = (first & 0x1ffffu) + (large ? Ps : 0u);
            const uint32_t span_end = sp + (uint32_t)rs.nspan;
#pragma unroll
            for (int r = 0; r < TS; r++) {
                const uint32_t code = (rs.w[r / 4] >> ((r % 4) * 8)) & 0xffu;
                const uint32_t lo = code & 15u, hi = code >> 4;
                if (lo <= hi && sp < span_end) {
                    rec.span[sp++] = p | ((uint32_t)tid << 16) | ((uint32_t)r << 24) | (lo << 28);
                    p += hi - lo + 1;
                }
            }
        }
        __syncthreads();
        base += (uint32_t)consumed;
        const uint32_t per = (P + NT - 1) / NT * 32;  // per-warp pixel range, a multiple of 32
        const uint32_t pb = (uint32_t)wid * per, pe = min(P, pb + per);
        if (pb < pe) {
            int s0 = 0;
            {
                int hi = NSP - 1;
                while (s0 < hi) {  // last span starting at or before pb
                    const int mid = (s0 + hi + 1) >> 1;
                    if ((rec.span[mid] & 0xffffu) <= pb) s0 = mid; else hi = mid - 1;
                }
            }
            uint32_t w0 = rec.span[s0];
            int qh = 0, qn = 0;  // the warp's ring of covered pixels: head, count
            for (uint32_t p0 = pb; p0 < pe; p0 += 32) {
                const int si = s0 + 1 + lane;
                const uint32_t wl = si < NSP ? rec.span[si] : 0u;
                const uint32_t d = si < NSP ? (wl & 0xffffu) - p0 : 0xffffffffu;  // >= 1
                const unsigned M = __reduce_or_sync(0xffffffffu, d < 32u ? 1u << d : 0u);
                const int rank = __popc(M & ((2u << lane) - 1u));
                uint32_t sw = __shfl_sync(0xffffffffu, wl, max(rank - 1, 0));
                if (rank == 0) sw = w0;
                const int adv = __popc(__ballot_sync(0xffffffffu, d <= 32u));
                if (adv) w0 = __shfl_sync(0xffffffffu, wl, adv - 1);
                s0 += adv;
                const uint32_t p = p0 + lane;
                const int r = (int)((sw >> 16) & 0xffu);
                const int qy = (int)((sw >> 24) & 15u);
                const int qx = (int)(sw >> 28) + (int)(p - (sw & 0xffffu));
                unsigned cov = 0;  // covered samples of this pixel
                if (p < pe) {
                    const int meta = rec.meta[r];
                    if (!(meta >> 1) || scissor_pass(a.draws[(meta >> 1) - 1], tx0 + qx, ty0 + qy)) {
                        const int32_t A[3] = {rec.A[0][r], rec.A[1][r], rec.A[2][r]};
                        const int32_t B[3] = {rec.B[0][r], rec.B[1][r], rec.B[2][r]};
                        if (!(meta & kLargeRecord)) {
                            int32_t e0[3];
#pragma unroll
                            for (int i = 0; i < 3; i++)
                                e0[i] = (int32_t)rec.Et[i][r] + A[i] * (qx * 256) + B[i] * (qy * 256);
#pragma unroll
                            for (int k = 0; k < S; k++) {
                                const int32_t c0 = e0[0] + A[0] * sample_x<S>(k) + B[0] * sample_y<S>(k);
                                const int32_t c1 = e0[1] + A[1] * sample_x<S>(k) + B[1] * sample_y<S>(k);
                                const int32_t c2 = e0[2] + A[2] * sample_x<S>(k) + B[2] * sample_y<S>(k);
                                cov |= ((c0 | c1 | c2) >= 0 ? 1u : 0u) << k;
                            }
                        } else {
                            const int64_t Et[3] = {rec.Et[0][r], rec.Et[1][r], rec.Et[2][r]};
#pragma unroll
                            for (int k = 0; k < S; k++)
                                cov |= (covered(A, B, Et, qx * 256 + sample_x<S>(k), qy * 256 + sample_y<S>(k)) ? 1u : 0u)
                                       << k;
                        }
                    }
                }
                // covered pixels are queued so that the depth tests run on full warps
                const unsigned bal = __ballot_sync(0xffffffffu, cov != 0u);
                if (cov)
                    wq[(qh + qn + __popc(bal & ((1u << lane) - 1u))) & 63] =
                        (uint32_t)r | ((uint32_t)qx << 8) | ((uint32_t)qy << 12) | (cov << 16);
                qn += __popc(bal);
                if (qn >= 32) {
                    __syncwarp();
                    const uint32_t item = wq[(qh + lane) & 63];
                    __syncwarp();
                    qh = (qh + 32) & 63;
                    qn -= 32;
                    raster_depth<S, TS>(v, rule, rec, skey, tx0, ty0, item);
                }
            }
            __syncwarp();
            if (lane < qn) raster_depth<S, TS>(v, rule, rec, skey, tx0, ty0, wq[(qh + lane) & 63]);
        }
        __syncthreads();
    }
    __syncthreads();
    if (v.ordered) {
        // tiles without ordered entries that may pass the depth test are finished by the shade
        // stage; the scatter cursors are free after binning and carry the per-tile count to the
        // later stages
        float dmax = 0.0f;  // farthest prefix depth of the tile's samples (culling views)
        if (v.ordered_cull) {
            uint32_t hmax = 0u;  // depth-order words of the prefix keys (ascending in depth)
            if (inpix) {
#pragma unroll
                for (int k = 0; k < S; k++) hmax = max(hmax, (uint32_t)(skey[k * (TS * TS) + ly * TS + lx] >> 32));
            }
            hmax = __reduce_max_sync(0xffffffffu, hmax);
            if (lane == 0) warp_sum[wid] = hmax;
            __syncthreads();
#pragma unroll
            for (int w = 0; w < NW; w++) hmax = max(hmax, warp_sum[w]);
            dmax = order_depth(hmax);
            __syncthreads();
        }
        const uint32_t first_ordered = (uint32_t)(v.first_tri + v.ordered_prefix);
        uint32_t left = 0;
        for (uint32_t i = beg + tid; i < end; i += NT) {
            const uint32_t e = __ldg(a.pairs + i);
            if ((e >> 3) < first_ordered) continue;
            left += !v.ordered_cull || may_pass_tile(a, v.c, e, tx0, ty0, xmax, ymax, dmax);
        }
        left = __reduce_add_sync(0xffffffffu, left);
        if (lane == 0) warp_sum[wid] = left;
        __syncthreads();
        if (tid == 0) {
            uint32_t sum = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) sum += warp_sum[w];
            a.tile_cursor[gtile] = sum;
        }
    }
    if (!inpix) return;
    int out[S];
#pragma unroll
    for (int k = 0; k < S; k++) out[k] = key_entry(rule, skey[k * (TS * TS) + ly * TS + lx]);
    int* ep = v.entries + pix * S;
    if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) reinterpret_cast<int4*>(ep)[k / 4] = make_int4(out[k], out[k + 1], out[k + 2], out[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < S; k++) ep[k] = out[k];
    }
}

template <int S, int TS>
size_t raster_smem_bytes() {
    return sizeof(TileRecords<TS * TS>) + (size_t)TS * TS * S * sizeof(unsigned long long);
}

// Resident raster CTAs per SM the register budget is sized for: 16x16 tiles at up to 4x fit five
// in shared memory (measured best: five beat four by ~2 %, six spill too much); 8x and 16x keys
// leave room for four and three.
template <int S, int TS>
__host__ __device__ constexpr int raster_min_blocks() {
    return TS == 16 ? (S <= 4 ? 5 : (S == 8 ? 4 : 3)) : 1024 / (TS * TS);
}

template <int S, int TS>
__global__ void __launch_bounds__(TS * TS, raster_min_blocks<S, TS>()) raster_kernel(PassArgs a, GroupArgs g) {
    constexpr int NT = TS * TS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileRecords<NT>& rec = *reinterpret_cast<TileRecords<NT>*>(smem_raw);
    unsigned long long* skey = reinterpret_cast<unsigned long long*>(smem_raw + sizeof(TileRecords<NT>));
    __shared__ uint32_t warp_sum[2 * (NT / 32)];
    __shared__ ViewArgs sv;
    __shared__ int s_tile, s_view;
    if (threadIdx.x == 0) s_view = -1;
    while (next_tile<NT>(a, g, 3 * g.queue, sv, s_tile, s_view)) raster_tile<S, TS>(a, sv, s_tile, rec, skey, warp_sum);
}

// ---------------------------------------------------------------------------- shade stage
// Interpolation set-up of an unclipped fill-mode triangle straight from its record, in registers:
// the same values as sub_from_record + shade_geom_from (edges from the snapped vertices, stored
// 1/w, the vertex order permutation of an oriented triangle).  plane = (z0, dz/dx, dz/dy, X0 bits),
// plane_y = Y0.
__device__ __forceinline__ void shade_geom_record(const TriRecord* rp, const int4 q1, ShadeGeom& g, float4& plane,
                                                  int& plane_y) {
    const int4 q0 = __ldg(reinterpret_cast<const int4*>(rp));
    const float4 q2 = __ldg(reinterpret_cast<const float4*>(rp) + 2);
    const float4 q3 = __ldg(reinterpret_cast<const float4*>(rp) + 3);
    const int32_t X[3] = {q0.x, q0.z, q1.x}, Y[3] = {q0.y, q0.w, q1.y};
    const bool swapped = (q1.z & REC_SWAPPED) != 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        g.A[i] = Y[j] - Y[k];
        g.B[i] = X[k] - X[j];
        g.C[i] = (int64_t)(Y[k] - Y[j]) * X[j] - (int64_t)(X[k] - X[j]) * Y[j];
#pragma unroll
        for (int m = 0; m < 3; m++) g.bary[i][m] = 0.0f;
    }
    g.iw[0] = q2.w; g.iw[1] = q3.x; g.iw[2] = q3.y;
    g.bary[0][0] = 1.0f;
    g.bary[1][swapped ? 2 : 1] = 1.0f;
    g.bary[2][swapped ? 1 : 2] = 1.0f;
    plane = make_float4(q2.x, q2.y, q2.z, __int_as_float(X[0]));
    plane_y = Y[0];
}

// Every other entry (clipped fan triangles, LINE / POINT parts): the general set-up, out of line so
// that its arrays stay out of the shading loop's frame.
static __device__ __noinline__ void shade_geom_general(const PassConst& c, const DrawDev& d, const TriRecord* records,
                                                       int g, int t, int sub, ShadeGeom* geo, float4* plane,
                                                       int* plane_y) {
    SubTri st;
    setup_entry_sub(c, d, records, g, t, sub, st);
    shade_geom_from(st, *geo);
    *plane = make_float4(st.z[0], st.dzdx, st.dzdy, __int_as_float(st.X[0]));
    *plane_y = st.Y[0];
}

// Texture lookups of a warp's items with their probes spread over the lanes (anisotropic lookups
// take 1 to max_aniso probes each): the calling lane's item has `n` probes described by `tp` for
// draw `di` (n = 0: no lookup); every item adds its probes' results in probe order and, when it has
// probes, finishes its colour `c`.  wres: 32 float4 of the warp's shared memory.  ROLLED: see
// tex_probe.  Whole warp.
template <bool ROLLED = false>
__device__ __forceinline__ void warp_texture_probes(const DrawDev* draws, int di, const TexProbe& tp, int n, float4* wres,
                                                    float c[4]) {
    const int lane = threadIdx.x & 31;
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int q = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += q;
    }
    const int T = __shfl_sync(0xffffffffu, incl, 31);
    if (T > 0) {
        const int pre = incl - n;
        const int packed = tp.lo | (tp.hi << 8) | (tp.n << 16) | (tp.two ? 1 << 24 : 0) | (tp.aniso ? 1 << 25 : 0);
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int c0 = 0; c0 < T; c0 += 32) {
            const int j = c0 + lane;
            int k = 0;  // the item of probe j: the last lane whose first probe is at or before j
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, pre, k + step) <= j) k += step;
            TexProbe q;
            q.u = __shfl_sync(0xffffffffu, tp.u, k);
            q.v = __shfl_sync(0xffffffffu, tp.v, k);
            q.du = __shfl_sync(0xffffffffu, tp.du, k);
            q.dv = __shfl_sync(0xffffffffu, tp.dv, k);
            q.t = __shfl_sync(0xffffffffu, tp.t, k);
            const int qp = __shfl_sync(0xffffffffu, packed, k);
            const int qd = __shfl_sync(0xffffffffu, di, k);
            const int i = j - __shfl_sync(0xffffffffu, pre, k);
            q.lo = qp & 255;
            q.hi = (qp >> 8) & 255;
            q.n = (qp >> 16) & 255;
            q.two = (qp >> 24) & 1;
            q.aniso = (qp >> 25) & 1;
            float r[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (j < T) tex_probe<ROLLED>(draws[qd], q, i, r);
            wres[lane] = make_float4(r[0], r[1], r[2], r[3]);
            __syncwarp();
            const int qa = max(pre, c0), qb = min(pre + n, c0 + 32);
            for (int m = qa; m < qb; m++) {
                const float4 x = wres[m - c0];
                acc[0] = acc[0] + x.x; acc[1] = acc[1] + x.y; acc[2] = acc[2] + x.z; acc[3] = acc[3] + x.w;
            }
            __syncwarp();
        }
        if (n > 0) tex_finish(tp, acc, c);
    }
}

// Slot codes of the shade stage's per-sample entries (see shade_tile).
constexpr int kSlotLate = 4, kSlotNone = 7;

// Sample k's visible entry read again after the shading loop.  The volatile loads keep the compiler
// from reusing the values read before the loop, which would hold every sample's entry in registers
// across it.
template <int S>
__device__ __forceinline__ int sample_entry_again(const ViewArgs& v, const KeyRule& rule, size_t pix, int k) {
    if (v.keys) {
        unsigned long long key;
        asm volatile("ld.global.u64 %0, [%1];" : "=l"(key) : "l"(v.keys + pix * S + k));
        return key_entry(rule, key);
    }
    int e;
    asm volatile("ld.global.s32 %0, [%1];" : "=r"(e) : "l"(v.entries + pix * S + k));
    return e;
}

// Shade stage CTAs: warps are independent (each pulls its own 32-pixel tasks); a CTA only holds the
// warps' shared-memory slices.
constexpr int kShadeThreads = 256;
constexpr int kShadeBlocks = 4;

// Per-sample slot codes of a pixel, 3 bits per sample (see shade_tile).
template <int S>
using SlotCodesOf = typename std::conditional<(S > 8), unsigned long long, uint32_t>::type;

// The lowest bit of each of the S 3-bit slot-code fields.
template <int S>
__device__ __forceinline__ constexpr SlotCodesOf<S> slot_field_lows() {
    SlotCodesOf<S> r = 0;
    for (int k = 0; k < S; k++) r |= (SlotCodesOf<S>)1 << (3 * k);
    return r;
}

// Depths of the owner pixel's samples on slot `slot` from the item's depth plane, into column `col`
// of the per-sample depth array.
template <int S>
__device__ __forceinline__ void item_sample_depths(SlotCodesOf<S> oc, int slot, const float4& plane, int plane_y, int opx,
                                                   int opy, float (*sdep)[kShadeThreads], int col) {
    using SlotCodes = SlotCodesOf<S>;
    if constexpr (S >= 8) {  // one copy of the loop body: the samples whose code is `slot`
        const SlotCodes rep = slot_field_lows<S>();
        const SlotCodes x = oc ^ (rep * (SlotCodes)slot);  // 0 in the fields equal to slot
        SlotCodes m = ~(x | (x >> 1) | (x >> 2)) & rep;
        while (m) {
            const int k = (S > 8 ? __ffsll((long long)m) : __ffs((int)m)) - 1;
            m &= m - 1;
            const int q = k / 3;
            sdep[q][col] = sample_depth(plane.x, plane.y, plane.z, __float_as_int(plane.w), plane_y,
                                        opx * 256 + sample_at<S>(q, 0), opy * 256 + sample_at<S>(q, 1));
        }
    } else {
#pragma unroll
        for (int k = 0; k < S; k++)
            if ((int)(oc >> (3 * k) & 7) == slot)
                sdep[k][col] = sample_depth(plane.x, plane.y, plane.z, __float_as_int(plane.w), plane_y,
                                            opx * 256 + sample_x<S>(k), opy * 256 + sample_y<S>(k));
    }
}

// A shading item off the hot path (clipped fan triangles, LINE / POINT parts, draws without an
// attribute record or with primitive-id shading): the general set-up and attribute fetch, out of
// line so that the shading loop carries only the record path.  DEPTHS: also the depths of the
// owner's samples on the item's slot (shade stage).
struct ItemShade {
    float c[4];
    TexProbe tp;
    int n;
};

template <int S, bool DEPTHS = true>
static __device__ __noinline__ ItemShade shade_item_general(const PassArgs& a, const PassConst& pc, int di, int g, int t,
                                                           int sub, bool from_record, int opx, int opy,
                                                           SlotCodesOf<S> oc, int slot, float (*sdep)[kShadeThreads],
                                                           int col) {
    const DrawDev& d = a.draws[di];
    ShadeGeom geo;
    float4 plane;
    int plane_y;
    if (from_record && d.polygon_mode == POLY_FILL) {
        const TriRecord* rp = a.records + g;
        shade_geom_record(rp, __ldg(reinterpret_cast<const int4*>(rp) + 1), geo, plane, plane_y);
    } else {
        shade_geom_general(pc, d, a.records, g, t, sub, &geo, &plane, &plane_y);
    }
    if constexpr (DEPTHS) item_sample_depths<S>(oc, slot, plane, plane_y, opx, opy, sdep, col);
    float a0[4], a1[4], a2[4];
    if (from_record && a.attrs && d.shading != SHADE_PRIMID && d.attr_count > 0) {
        const float4 q0 = __ldg(&a.attrs[g].a[0]), q1 = __ldg(&a.attrs[g].a[1]), q2 = __ldg(&a.attrs[g].a[2]);
        a0[0] = q0.x; a0[1] = q0.y; a0[2] = q0.z; a0[3] = q0.w;
        a1[0] = q1.x; a1[1] = q1.y; a1[2] = q1.z; a1[3] = q1.w;
        a2[0] = q2.x; a2[1] = q2.y; a2[2] = q2.z; a2[3] = q2.w;
    } else if (d.shading != SHADE_PRIMID) {
        fetch_attrs(d, t, a0, a1, a2);
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) a0[k] = a1[k] = a2[k] = 0.0f;
    }
    ItemShade r;
    r.c[0] = r.c[1] = r.c[2] = r.c[3] = 0.0f;
    r.tp.u = r.tp.v = r.tp.du = r.tp.dv = r.tp.t = 0.0f;
    r.tp.lo = r.tp.hi = r.tp.n = 0;
    r.tp.two = r.tp.aniso = false;
    r.n = shade_prepare_attrs(pc, d, geo, t, sub, opx, opy, a0, a1, a2, r.c, r.tp) ? r.tp.n : 0;
    return r;
}

// The shade stage's per-pixel tail: each sample's colour from its slot (or the background), the
// resolve (or the per-sample hand-off to the ordered stage), depth and visibility.  `uq` holds the
// entries of slots 0..3; LATE adds samples past the U shaded slots, shaded here one by one.
template <int S, int TS, bool LATE>
__device__ __forceinline__ void resolve_pixel(const PassArgs& a, const ViewArgs& v, const KeyRule& rule,
                                              SlotCodesOf<S> codes, float4 (*scol)[kShadeThreads],
                                              float (*sdep)[kShadeThreads], int4 uq, size_t pix, int px, int py,
                                              int ltile, int part, bool keep_samples) {
    constexpr int U = S < 4 ? S : 4;
    const int tid = threadIdx.x;
    float dep[S];
#pragma unroll
    for (int k = 0; k < S; k++) dep[k] = ((int)(codes >> (3 * k)) & 7) < U ? sdep[k][tid] : 0.0f;
    float bg[4];
    if (v.clear) {
        bg[0] = v.clear_color[0]; bg[1] = v.clear_color[1]; bg[2] = v.clear_color[2]; bg[3] = v.clear_color[3];
    } else {
        decode_color(v, pix, bg);
    }
    float acc[4];
#pragma unroll
    for (int k = 0; k < S; k++) {
        float c[4];
        const int code = (int)(codes >> (3 * k)) & 7;
        const float d0v = v.clear ? v.clear_depth : v.depth[pix * S + k];
        if (code == kSlotNone) {
            c[0] = bg[0]; c[1] = bg[1]; c[2] = bg[2]; c[3] = bg[3];
            dep[k] = d0v;
        } else {
            if (!LATE || code < U) {
                float4 q = scol[code & 3][tid];
                c[0] = q.x; c[1] = q.y; c[2] = q.z; c[3] = q.w;
            } else {  // past the U shaded slots: shade this sample's primitive here
                RecordPlane pl;
                float uc[4];
                shade_uncached(a, v.c, sample_entry_again<S>(v, rule, pix, k), px, py, uc, &pl);
                c[0] = uc[0]; c[1] = uc[1]; c[2] = uc[2]; c[3] = uc[3];
                dep[k] = sample_depth(pl.z0, pl.dzdx, pl.dzdy, pl.X0, pl.Y0, px * 256 + sample_x<S>(k),
                                      py * 256 + sample_y<S>(k));
            }
            if (!rule.write) dep[k] = d0v;
        }
        if (keep_samples)  // tile-major hand-off: [tile][sample][lane], coalesced on both sides
            v.sample_colors[((size_t)ltile * S + k) * (TS * TS) + part * 32 + (tid & 31)] = make_float4(c[0], c[1], c[2], c[3]);
        if (k == 0) {
            acc[0] = c[0]; acc[1] = c[1]; acc[2] = c[2]; acc[3] = c[3];
        } else {
            acc[0] = acc[0] + c[0]; acc[1] = acc[1] + c[1]; acc[2] = acc[2] + c[2]; acc[3] = acc[3] + c[3];
        }
    }
    if (!keep_samples) {  // a tile with ordered entries is resolved by the ordered stage
        const float invS = 1.0f / (float)S;
        acc[0] = acc[0] * invS; acc[1] = acc[1] * invS; acc[2] = acc[2] * invS; acc[3] = acc[3] * invS;
        encode_color(v, pix, acc);
    }

    float* dp = v.depth + pix * S;
    if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) reinterpret_cast<float4*>(dp)[k / 4] = make_float4(dep[k], dep[k + 1], dep[k + 2], dep[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < S; k++) dp[k] = dep[k];
    }
    if (v.vis) {
        int* vp = v.vis + pix * S;
#pragma unroll
        for (int k = 0; k < S; k++) {
            const int code = (int)(codes >> (3 * k)) & 7;
            int e = code == 0 ? uq.x : code == 1 ? uq.y : code == 2 ? uq.z : uq.w;
            if (code == kSlotNone) e = -1;
            else if (LATE && code >= U) e = sample_entry_again<S>(v, rule, pix, k);
            vp[k] = e < 0 ? -1 : (e >> 3) - v.first_tri;
        }
    }
}

template <int S, int TS>
__device__ __noinline__ void resolve_pixel_late(const PassArgs& a, const ViewArgs& v, KeyRule rule, SlotCodesOf<S> codes,
                                                float4 (*scol)[kShadeThreads], float (*sdep)[kShadeThreads], int4 uq,
                                                size_t pix, int px, int py, int ltile, int part, bool keep_samples) {
    resolve_pixel<S, TS, true>(a, v, rule, codes, scol, sdep, uq, pix, px, py, ltile, part, keep_samples);
}

// One tile, one thread per pixel.  Each pixel lists its distinct visible entries in sample
// order; the warp shades the (pixel, entry) items of all its lanes together (set-up straight
// from the binner's record, the depths of the pixel's samples on that entry, quad derivatives,
// texture filtering), then the samples are resolved on chip and depth, visibility and the
// resolved colour stored once.
template <int S, int TS>
__device__ __forceinline__ void shade_tile(const PassArgs& a, const ViewArgs& v, int gtile, int part,
                                           float4 (*scol)[kShadeThreads], float (*sdep)[kShadeThreads],
                                           float4* wres,
                                           bool keep_samples) {
    const int ltile = gtile - v.tile_start;
    const int tx = ltile % v.c.tiles_x, ty = ltile / v.c.tiles_x;
    const int tid = threadIdx.x;
    int lx, ly;
    tile_pixel<TS>(part * 32 + (tid & 31), lx, ly);
    const int px = tx * TS + lx, py = ty * TS + ly;
    const bool inpix = px < v.c.W && py < v.c.H;
    const size_t pix = (size_t)py * v.c.W + px;
    const KeyRule rule = key_rule(v.depth_func, v.depth_write);
    // Distinct visible entries of this pixel, in sample order, and each sample's 3-bit slot code:
    // 0..U-1 its list slot, kSlotLate for entries past the U shaded together (shaded on their own
    // after the warp's items), kSlotNone for no visible entry.  Per-sample entries do not stay in
    // registers across the shading loop: the slots' entries (uniq) reach the item lanes by shuffles,
    // late ones are read again from memory.
    constexpr int U = S < 4 ? S : 4;  // slots shaded together across the warp
    using SlotCodes = SlotCodesOf<S>;
    SlotCodes codes = 0;
    int uniq[U];
#pragma unroll
    for (int j = 0; j < U; j++) uniq[j] = 0;
    int nu = 0;
    if constexpr (S >= 8) {
        // one copy of the per-sample body: each sample's entry against the (at most U) entries found
        // so far; entries past the U shaded slots are late (the same codes as the pairwise form)
        int4 q[S / 4];
#pragma unroll
        for (int i = 0; i < S / 4; i++) q[i] = make_int4(-1, -1, -1, -1);
        if (inpix && !v.keys) {
            const int4* ep = reinterpret_cast<const int4*>(v.entries + pix * S);
#pragma unroll
            for (int i = 0; i < S / 4; i++) q[i] = ep[i];
        }
#pragma unroll 1
        for (int k = 0; k < S; k++) {
            int4 w = q[0];
#pragma unroll
            for (int i = 1; i < S / 4; i++)
                if ((k >> 2) == i) w = q[i];
            int e = (k & 3) == 0 ? w.x : (k & 3) == 1 ? w.y : (k & 3) == 2 ? w.z : w.w;
            if (inpix && v.keys) e = key_entry(rule, v.keys[pix * S + k]);  // atomic visibility path
            int code = kSlotNone;
            if (e >= 0) {
                code = -1;
#pragma unroll
                for (int j = 0; j < U; j++)
                    if (j < nu && uniq[j] == e) code = j;
                if (code < 0) {
                    code = nu < U ? nu : kSlotLate;
#pragma unroll
                    for (int j = 0; j < U; j++)
                        if (j == nu) uniq[j] = e;
                    nu++;
                }
            }
            codes |= (SlotCodes)code << (3 * k);
        }
    } else {
        int ent[S];
        if (inpix && v.keys) {  // atomic visibility path
#pragma unroll
            for (int k = 0; k < S; k++) ent[k] = key_entry(rule, v.keys[pix * S + k]);
        } else if (inpix) {
            const int* ep = v.entries + pix * S;
            if constexpr (S % 4 == 0) {
#pragma unroll
                for (int k = 0; k < S; k += 4) {
                    int4 q = reinterpret_cast<const int4*>(ep)[k / 4];
                    ent[k] = q.x; ent[k + 1] = q.y; ent[k + 2] = q.z; ent[k + 3] = q.w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < S; k++) ent[k] = ep[k];
            }
        } else {
#pragma unroll
            for (int k = 0; k < S; k++) ent[k] = -1;
        }
        int which[S];
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
#pragma unroll
        for (int k = 0; k < S; k++) {
            const int code = which[k] < 0 ? kSlotNone : which[k] < U ? which[k] : kSlotLate;
            codes |= (SlotCodes)code << (3 * k);
        }
    }
    // The warp's (pixel, entry) shading items, compacted: item i of the warp goes to lane i % 32,
    // whatever pixel it belongs to (quad derivatives are evaluated analytically at the owner's
    // pixel, so no item depends on another lane).  Results land in the owner's slot.
    const int lane = tid & 31, wbase = tid & ~31;
    const int nc = min(nu, U);
    int incl = nc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int q = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += q;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int ibase = incl - nc;  // this lane's first item in the warp's compacted order
    for (int r0 = 0; r0 < total; r0 += 32) {
        const int b = r0 + lane;
        int owner = 0;  // the lane of item b: the last lane whose first item is at or before b
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
            if (__shfl_sync(0xffffffffu, ibase, owner + step) <= b) owner += step;
        const int slot = b - __shfl_sync(0xffffffffu, ibase, owner);
        int item = __shfl_sync(0xffffffffu, uniq[0], owner);  // the item's entry
#pragma unroll
        for (int j = 1; j < U; j++) {
            const int ej = __shfl_sync(0xffffffffu, uniq[j], owner);
            if (slot == j) item = ej;
        }
        const SlotCodes oc = __shfl_sync(0xffffffffu, codes, owner);  // the owner pixel's slot codes
        int di = 0, n = 0;  // n: texture probes of this lane's item
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        TexProbe tp;
        tp.u = tp.v = tp.du = tp.dv = tp.t = 0.0f;
        tp.lo = tp.hi = tp.n = 0;
        tp.two = tp.aniso = false;
        if (b < total) {
            int olx, oly;
            tile_pixel<TS>(part * 32 + owner, olx, oly);
            const int opx = tx * TS + olx, opy = ty * TS + oly;
            const int g = item >> 3, sub = item & 7;
            const TriRecord* rp = a.records + g;
            const int4 q1 = __ldg(reinterpret_cast<const int4*>(rp) + 1);  // X2, Y2, flags, draw
            di = q1.w;
            const DrawDev& d = a.draws[di];
            const int t = g - __ldg(a.draw_start + di);
            const bool from_record = sub == 0 && (q1.z & REC_VALID);
            if (from_record && d.polygon_mode == POLY_FILL && a.attrs && d.shading != SHADE_PRIMID && d.attr_count > 0) {
                // the hot path: set-up and vertex attributes straight from the binner's records
                ShadeGeom geo;
                float4 plane;
                int plane_y;
                shade_geom_record(rp, q1, geo, plane, plane_y);
                item_sample_depths<S>(oc, slot, plane, plane_y, opx, opy, sdep, wbase + owner);
                float a0[4], a1[4], a2[4];
                const float4 r0 = __ldg(&a.attrs[g].a[0]), r1 = __ldg(&a.attrs[g].a[1]), r2 = __ldg(&a.attrs[g].a[2]);
                a0[0] = r0.x; a0[1] = r0.y; a0[2] = r0.z; a0[3] = r0.w;
                a1[0] = r1.x; a1[1] = r1.y; a1[2] = r1.z; a1[3] = r1.w;
                a2[0] = r2.x; a2[1] = r2.y; a2[2] = r2.z; a2[3] = r2.w;
                if (shade_prepare_attrs(v.c, d, geo, t, sub, opx, opy, a0, a1, a2, c, tp)) n = tp.n;
            } else {
                const ItemShade r = shade_item_general<S>(a, v.c, di, g, t, sub, from_record, opx, opy, oc, slot, sdep,
                                                          wbase + owner);
                c[0] = r.c[0]; c[1] = r.c[1]; c[2] = r.c[2]; c[3] = r.c[3];
                tp = r.tp;
                n = r.n;
            }
        }
        warp_texture_probes<(S >= 8)>(a.draws, di, tp, n, wres, c);
        if (b < total) scol[slot][wbase + owner] = make_float4(c[0], c[1], c[2], c[3]);
    }
    __syncwarp();
    if (!inpix) return;
    const int4 uq = make_int4(uniq[0], U > 1 ? uniq[U > 1 ? 1 : 0] : 0, U > 2 ? uniq[U > 2 ? 2 : 0] : 0,
                              U > 3 ? uniq[U > 3 ? 3 : 0] : 0);
    if (nu > U)  // more than U distinct primitives in the pixel (rare): out of line
        resolve_pixel_late<S, TS>(a, v, rule, codes, scol, sdep, uq, pix, px, py, ltile, part, keep_samples);
    else
        resolve_pixel<S, TS, false>(a, v, rule, codes, scol, sdep, uq, pix, px, py, ltile, part, keep_samples);
}

// Persistent warps: each warp pulls 32-pixel tasks (8 quads of one tile) from the group's
// queue on its own, so a warp that finishes early starts its next task instead of waiting at a
// tile barrier.  View arguments are read through L1 from the descriptor array.
template <int S, int TS>
__global__ void __launch_bounds__(kShadeThreads, kShadeBlocks) shade_kernel(PassArgs a, GroupArgs g) {
    constexpr int NT = TS * TS, CT = kShadeThreads;
    constexpr int kTasksPerTile = NT / 32;
    constexpr int U = S < 4 ? S : 4;
    __shared__ float4 scol[U][CT];  // colours of each thread's (up to U) distinct entries
    __shared__ float sdep[S][CT];   // depths of its samples on those entries
    __shared__ float4 sres[CT];                // per warp: results of one round of texture probes
    const int lane = threadIdx.x & 31;
    const int ntasks = (g.tile_end - g.tile_begin) * kTasksPerTile;
    for (;;) {
        int task = 0, vi = 0;
        if (lane == 0) {
            task = (int)atomicAdd(a.queues + 3 * g.queue + 1, 1u);
            if (task < ntasks) {
                const int t = g.tile_begin + task / kTasksPerTile;
                int lo = g.view_begin, hi = g.view_end - 1;
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (__ldg(a.view_tile_start + mid) <= t) lo = mid; else hi = mid - 1;
                }
                vi = lo;
            }
        }
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= ntasks) break;
        vi = __shfl_sync(0xffffffffu, vi, 0);
        const int gtile = g.tile_begin + task / kTasksPerTile;
        // tiles of ordered views with entries left for the ordered stage keep their per-sample
        // colours for it instead of resolving
        const bool keep = a.views[vi].ordered && __ldg(a.tile_cursor + gtile) != 0u;
        shade_tile<S, TS>(a, a.views[vi], gtile, task % kTasksPerTile, scol, sdep, sres + (threadIdx.x & ~31), keep);
    }
}

// ---------------------------------------------------------------------------- ordered stage
// Used when results depend on submission order: blending, NOT_EQUAL with depth writes, or
// draws of one view with different depth state.  The tile's entries are sorted into API order
// in shared memory, then every pixel applies them one after another exactly as the reference's
// ordered CPU path does (TileRasterWorker.cpp:1517-1580): per-sample depth test and write, one
// shading per pixel and triangle when any sample passes, per-sample blend
// (TileRasterWorker.cpp:2346-2373, pixelShadingAlphaBlendKernel .cu:1648-1897), then the
// on-chip resolve.  16x16 tiles.
constexpr int kFwdThreads = 256;

// Set-ups of one batch of ordered entries.  Edge functions are kept relative to the tile origin:
// a record spanning less than 32 pixels in x and y evaluates them exactly in 32-bit arithmetic (the
// raster stage's bound, kSmallSpan), larger ones in 64 bits.
struct FwdRecords {
    int32_t A[3][kFwdThreads], B[3][kFwdThreads];
    long long Et[3][kFwdThreads];  // biased edge functions at the tile origin
    float z0[kFwdThreads], dzdx[kFwdThreads], dzdy[kFwdThreads];
    int32_t X0[kFwdThreads], Y0[kFwdThreads];
    int32_t key[kFwdThreads];
    int32_t draw[kFwdThreads];
    int32_t meta[kFwdThreads];     // kLargeRecord | depth function << 1 | depth write << 4 | scissor test << 5
    uint32_t box[kFwdThreads];     // pixel box in the tile: column mask | row mask << 16 (0: empty)
};

// Batches of up to this many records find each pixel's candidates by scanning the records' boxes;
// larger batches mark them into per-pixel bitmasks from the records' side.
constexpr int kFwdScanBatch = 64;
// Per-warp buffer of candidate coverage masks (16 bits each) on the scanning path, which leaves the
// candidate bitmasks unused: the buffers alias them (8 warps x 1 KB).
constexpr int kFwdWarpCand = 512;

// Position of the n-th (0-based) set bit of x, which has more than n set bits.
__device__ __forceinline__ int nth_set_bit(uint32_t x, int n) {
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const uint32_t low = x & ((1u << w) - 1u);
        const int c = __popc(low);
        if (n >= c) {
            n -= c;
            x >>= w;
            pos += w;
        } else {
            x = low;
        }
    }
    return pos;
}

constexpr int kFwdFrags = 8;      // fragments a pixel holds before they are shaded (in-stage form)
constexpr int kFwdListDefer = 2048;  // ordered entries of a tile the deferring form sorts (more: the tile is redone)
constexpr int kFwdFragsDefer = 6; // fragments a pixel records in the deferring form (more: the tile is redone)
constexpr int kFwdSmallBox = 24;  // candidate boxes of up to this many pixels are marked by their record's thread

// Lane of pixel (lx, ly) of a TS x TS tile (inverse of tile_pixel).
template <int TS>
__device__ __forceinline__ int tile_lane(int lx, int ly) {
    return ((((ly >> 1) * (TS / 2)) + (lx >> 1)) << 2) | ((ly & 1) << 1) | (lx & 1);
}

// Shades fragment f = (entry, sample mask | draw << 16) at pixel (px, py) and writes or blends it
// into the per-sample colours of the calling thread.
template <int S>
__device__ __forceinline__ void apply_fragment(const PassArgs& a, const ViewArgs& v, int px, int py, float4* scol,
                                               int2 f) {
    constexpr int NT = kFwdThreads;
    float c[4];
    RecordPlane pl;
    shade_uncached(a, v.c, f.x, px, py, c, &pl);
    const DrawDev& d = a.draws[(unsigned)f.y >> 16];
    const unsigned mask = (unsigned)f.y & 0xffffu;
    if (d.blend_enable && !blend_reads_dst(d)) {  // factors of the source only: once per fragment
        float fs[4], fd[4];
#pragma unroll
        for (int ch = 0; ch < 4; ch++) {
            fs[ch] = blend_factor(ch < 3 ? d.blend_src_color : d.blend_src_alpha, ch, c, c);
            fd[ch] = blend_factor(ch < 3 ? d.blend_dst_color : d.blend_dst_alpha, ch, c, c);
        }
#pragma unroll
        for (int k = 0; k < S; k++) {
            if (!(mask & (1u << k))) continue;
            float4& sc = scol[k * NT + threadIdx.x];
            sc = make_float4(sc.x * fd[0] + c[0] * fs[0], sc.y * fd[1] + c[1] * fs[1], sc.z * fd[2] + c[2] * fs[2],
                             sc.w * fd[3] + c[3] * fs[3]);
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < S; k++) {
        if (!(mask & (1u << k))) continue;
        float4& sc = scol[k * NT + threadIdx.x];
        if (d.blend_enable) {
            float dst[4] = {sc.x, sc.y, sc.z, sc.w};
            blend_into(d, c, dst);
            sc = make_float4(dst[0], dst[1], dst[2], dst[3]);
        } else {
            sc = make_float4(c[0], c[1], c[2], c[3]);
        }
    }
}

template <int S>
__device__ __noinline__ void apply_fragments(const PassArgs& a, const ViewArgs& v, int px, int py, float4* scol,
                                             const int2* frags, int n) {
    for (int i = 0; i < n; i++) apply_fragment<S>(a, v, px, py, scol, frags[i * kFwdThreads + threadIdx.x]);
}


// A pixel's per-sample depths (16-byte stores when S is a multiple of 4: the target is then
// 16-byte aligned).
template <int S>
__device__ __forceinline__ void store_depth(float* dp, const float* dep) {
    if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4)
            reinterpret_cast<float4*>(dp)[k / 4] = make_float4(dep[k], dep[k + 1], dep[k + 2], dep[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < S; k++) dp[k] = dep[k];
    }
}

// Starting colours of the calling thread's samples: the prefix's per-sample colours handed off by
// the shade stage, or the background.
template <int S>
__device__ __forceinline__ void start_colours(const ViewArgs& v, float4* scol, int ltile, bool after_raster,
                                              const float bg[4]) {
    constexpr int NT = kFwdThreads;
#pragma unroll
    for (int k = 0; k < S; k++)
        scol[k * NT + threadIdx.x] = after_raster ? v.sample_colors[((size_t)ltile * S + k) * NT + threadIdx.x]
                                                  : make_float4(bg[0], bg[1], bg[2], bg[3]);
}

// DEFER: the tile's fragments go to the fragment kernels (fa set); the per-sample colours a tile
// finished here needs live in the tile's rows of the hand-off buffer (exclusive to the tile), not in
// shared memory.
template <int S, bool DEFER>
__device__ __forceinline__ void forward_tile(const PassArgs& a, const FragArgs& fa, const ViewArgs& v, int vi, int gtile,
                                             FwdRecords& rec, float4* scol_smem, uint32_t* list, int2* frags,
                                             uint32_t* cand, uint16_t* wcov, bool after_raster, BulkState& bs) {
    constexpr int TS = 16, NT = kFwdThreads;
    // after the raster and shade stages the shade stage has finished the tiles without ordered
    // entries (uniform over the CTA)
    if (after_raster && a.tile_cursor[gtile] == 0u) return;
    const int ltile = gtile - v.tile_start;
    // Without deferral the prefix's per-sample colours of the tile (S x 256 float4, contiguous in
    // the tile-major hand-off) come in by one bulk copy (TMA) that overlaps the gathering and
    // sorting below.
    constexpr bool defer = DEFER;
    constexpr int kMaxFrags = DEFER ? kFwdFragsDefer : kFwdFrags;
    float4* scol = scol_smem;  // the in-stage form's per-sample colours (the deferring form uses none)
    const bool bulk = after_raster && bs.ok && !defer;
    if (bulk && threadIdx.x == 0)
        bulk_load(scol, v.sample_colors + (size_t)ltile * S * NT, (uint32_t)(sizeof(float4) * S * NT), bs.bar);
    const int tx = ltile % v.c.tiles_x, ty = ltile / v.c.tiles_x;
    const int tid = threadIdx.x;
    int lx, ly;
    tile_pixel<TS>(tid, lx, ly);
    const int px = tx * TS + lx, py = ty * TS + ly;
    const bool inpix = px < v.c.W && py < v.c.H;
    const size_t pix = (size_t)py * v.c.W + px;

    float dep[S];
    int vid[S];
    float bg[4];
    if (v.clear) {
        bg[0] = v.clear_color[0]; bg[1] = v.clear_color[1]; bg[2] = v.clear_color[2]; bg[3] = v.clear_color[3];
    } else if (inpix && !after_raster) {
        decode_color(v, pix, bg);
    } else {
        bg[0] = bg[1] = bg[2] = bg[3] = 0.0f;
    }
    if (after_raster) {
        // the prefix's per-sample state as the shade stage left it: colour in the per-sample
        // scratch, depth and primitive id in the outputs
        int ent[S];
        if (!inpix) {
#pragma unroll
            for (int k = 0; k < S; k++) {
                ent[k] = -1;
                dep[k] = 0.0f;
            }
        } else if constexpr (S % 4 == 0) {
#pragma unroll
            for (int k = 0; k < S; k += 4) {
                const int4 q = v.vis ? reinterpret_cast<const int4*>(v.entries + pix * S)[k / 4] : make_int4(-1, -1, -1, -1);
                const float4 z = reinterpret_cast<const float4*>(v.depth + pix * S)[k / 4];
                ent[k] = q.x; ent[k + 1] = q.y; ent[k + 2] = q.z; ent[k + 3] = q.w;
                dep[k] = z.x; dep[k + 1] = z.y; dep[k + 2] = z.z; dep[k + 3] = z.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < S; k++) {
                ent[k] = v.vis ? v.entries[pix * S + k] : -1;  // primitive ids are only written with visibility output
                dep[k] = v.depth[pix * S + k];
            }
        }
#pragma unroll
        for (int k = 0; k < S; k++) vid[k] = ent[k] < 0 ? -1 : (ent[k] >> 3) - v.first_tri;
    } else {
#pragma unroll
        for (int k = 0; k < S; k++) {
            dep[k] = v.clear ? v.clear_depth : (inpix ? v.depth[pix * S + k] : 0.0f);
            vid[k] = -1;
        }
    }
    // the depth target already holds dep[] after the raster stage; otherwise (cleared or earlier
    // content) it is written whatever happens
    bool dep_changed = !after_raster;
    bool too_many = false;  // deferring form: a pixel passed more than kFwdFragsDefer fragments
    // Per-pixel occlusion test of candidates (views where depths only decrease, as for the tile
    // test of the raster stage): a record under LESS / LEQUAL / EQUAL whose depth plane stays beyond
    // the pixel's farthest depth over the pixel's sample range, by more than the evaluation's
    // rounding bound, cannot pass at any of its samples.
    float dmax_pix = dep[0];
#pragma unroll
    for (int k = 1; k < S; k++) dmax_pix = fmaxf(dmax_pix, dep[k]);
    bool have_cols = bulk;  // scol holds this thread's starting colours (in-stage form)
    if (!defer && !bulk) {
        start_colours<S>(v, scol, ltile, after_raster, bg);
        have_cols = true;
    }
    const bool has_list = a.total_tris > 0 && a.status[ST_OVERFLOW] == 0;
    const uint32_t beg = has_list ? a.tile_offset[gtile] : 0u;
    const uint32_t end = has_list ? a.tile_offset[gtile + 1] : 0u;
    const int total = (int)(end - beg);
    // gather the entries still to apply in order (the prefix was resolved by the raster stage)
    const uint32_t first_ordered = (uint32_t)(v.first_tri + v.ordered_prefix);
    __shared__ int s_count;
    if (tid == 0) s_count = 0;
    __syncthreads();
    for (int i = tid; i < total; i += NT) {
        const uint32_t e = __ldg(a.pairs + beg + i);
        if ((e >> 3) >= first_ordered) {
            const int at = atomicAdd(&s_count, 1);
            if (at < (DEFER ? kFwdListDefer : kOrderedCap)) list[at] = e;
        }
    }
    __syncthreads();
    int n = s_count;
    if (DEFER && n > kFwdListDefer) {  // nothing written yet: the in-stage form sorts up to kOrderedCap
        if (tid == 0) fa.redo_tiles[atomicAdd(a.status + ST_REDO, 1u)] = (uint32_t)gtile;
        return;
    }
    if (n > kOrderedCap) {  // cannot order this tile on chip: report and leave it as the prefix left it
        if (tid == 0) {
            atomicOr(a.status + ST_ORDERED_LIMIT, 1u);
            atomicOr(a.status + ST_STICKY, 2u);
        }
        n = 0;
    }
    // sort them into submission order: up to one entry per thread by rank (entries are distinct, so
    // every rank is; two barriers), longer lists bitonically (padded to 2^k)
    if (n <= NT) {
        const uint32_t e = tid < n ? list[tid] : 0u;
        int rank = 0;
        if (tid < n) {
            const uint4* l4 = reinterpret_cast<const uint4*>(list);
            for (int j = 0; j < (n >> 2); j++) {
                const uint4 q = l4[j];
                rank += (int)(q.x < e) + (int)(q.y < e) + (int)(q.z < e) + (int)(q.w < e);
            }
            for (int j = n & ~3; j < n; j++) rank += list[j] < e;
        }
        __syncthreads();
        if (tid < n) list[rank] = e;
        __syncthreads();
    } else {
        int P = 1;
        while (P < n) P <<= 1;
        for (int i = n + tid; i < P; i += NT) list[i] = 0xFFFFFFFFu;
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = tid; i < P; i += NT) {
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
    }

    if (bulk) {  // the colours must have landed before the first fragment is applied
        const bool ok = mbar_wait(bs.bar, bs.phase & 1u);
        bs.phase++;
        if (!__syncthreads_and(ok)) {  // gave up: report, and load the colours from memory from now on
            bs.ok = false;
            if (threadIdx.x == 0) atomicOr(a.status + ST_STICKY, 4u);
            bs.pending = true;
#pragma unroll
            for (int k = 0; k < S; k++) scol[k * NT + tid] = v.sample_colors[((size_t)ltile * S + k) * NT + tid];
            __syncthreads();
        }
    }
    int nfrag = 0;  // fragments recorded for this thread's pixel, not yet shaded
    const int lane = tid & 31;
    for (int base = 0; base < n; base += NT) {
        const int nb = min(NT, n - base);
        // candidate masks of the batch: bit r of cand[r / 32][lane] when record r's pixel box
        // holds the lane's pixel
        if (nb > kFwdScanBatch) {
#pragma unroll
            for (int w = 0; w < NT / 32; w++) cand[w * NT + tid] = 0u;
        }
        int area = 0, cx0 = 0, cy0 = 0, cw = 1;
        uint32_t box = 0;
        if (tid < nb) {
            uint32_t e = list[base + tid];
            SubTri s;
            int di;
            if (setup_raster_entry(a, v.c, e, &s, &di)) {
                const int64_t X_t = (int64_t)tx * TS * 256, Y_t = (int64_t)ty * TS * 256;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    rec.A[i][tid] = s.A[i];
                    rec.B[i][tid] = s.B[i];
                    rec.Et[i][tid] = s.Cb[i] + (int64_t)s.A[i] * X_t + (int64_t)s.B[i] * Y_t;
                }
                const int32_t xmn = min(s.X[0], min(s.X[1], s.X[2])), xmx = max(s.X[0], max(s.X[1], s.X[2]));
                const int32_t ymn = min(s.Y[0], min(s.Y[1], s.Y[2])), ymx = max(s.Y[0], max(s.Y[1], s.Y[2]));
                const bool small = xmx - xmn < kSmallSpan && ymx - ymn < kSmallSpan;
                const DrawDev& d = a.draws[di];
                rec.meta[tid] = (small ? 0 : kLargeRecord) | (d.depth_func << 1) | ((d.depth_write ? 1 : 0) << 4) |
                                ((d.scissor_count ? 1 : 0) << 5);
                rec.z0[tid] = s.z[0];
                rec.dzdx[tid] = s.dzdx;
                rec.dzdy[tid] = s.dzdy;
                rec.X0[tid] = s.X[0];
                rec.Y0[tid] = s.Y[0];
                cx0 = max(s.px0 - tx * TS, 0);
                cy0 = max(s.py0 - ty * TS, 0);
                const int cx1 = min(s.px1 - tx * TS, TS - 1), cy1 = min(s.py1 - ty * TS, TS - 1);
                if (cx1 >= cx0 && cy1 >= cy0) {
                    cw = cx1 - cx0 + 1;
                    area = cw * (cy1 - cy0 + 1);
                    box = (((2u << cx1) - 1u) & ~((1u << cx0) - 1u)) | ((((2u << cy1) - 1u) & ~((1u << cy0) - 1u)) << 16);
                }
            }
            rec.key[tid] = (int)e;
            rec.draw[tid] = di;
            rec.box[tid] = box;
        }
        const bool scan = nb <= kFwdScanBatch;  // uniform
        __syncthreads();
        // Coverage of record r at tile pixel (qlx, qly) (absolute (qpx, qpy), farthest depth qdmax):
        // 0 when the per-pixel occlusion test or the scissor test rejects the record there.
        auto cover = [&](int r, int qlx, int qly, int qpx, int qpy, float qdmax) -> unsigned {
            const int meta = rec.meta[r];
            const int func = (meta >> 1) & 7;
            if (v.ordered_cull && func >= 1 && func <= 3) {
                const float z0 = rec.z0[r], gx = rec.dzdx[r], gy = rec.dzdy[r];
                const int32_t qx0 = qpx * 256 + v.c.smin_x, qx1 = qpx * 256 + v.c.smax_x;
                const int32_t qy0 = qpy * 256 + v.c.smin_y, qy1 = qpy * 256 + v.c.smax_y;
                const float ax = gx * (float)(qx0 - rec.X0[r]), bx = gx * (float)(qx1 - rec.X0[r]);
                const float ay = gy * (float)(qy0 - rec.Y0[r]), by = gy * (float)(qy1 - rec.Y0[r]);
                const float zmin = (z0 + fminf(ax, bx)) + fminf(ay, by);
                const float margin = (fabsf(z0) + fmaxf(fabsf(ax), fabsf(bx)) + fmaxf(fabsf(ay), fabsf(by))) * 0x1p-20f;
                if (zmin - margin > qdmax) return 0u;
            }
            if ((meta & 32) && !scissor_pass(a.draws[rec.draw[r]], qpx, qpy)) return 0u;
            const int32_t A[3] = {rec.A[0][r], rec.A[1][r], rec.A[2][r]};
            const int32_t B[3] = {rec.B[0][r], rec.B[1][r], rec.B[2][r]};
            unsigned cov = 0;  // tile-relative edge functions
            if (!(meta & kLargeRecord)) {
                int32_t e0[3];
#pragma unroll
                for (int i = 0; i < 3; i++) e0[i] = (int32_t)rec.Et[i][r] + A[i] * (qlx * 256) + B[i] * (qly * 256);
#pragma unroll
                for (int k = 0; k < S; k++) {
                    const int32_t c0 = e0[0] + A[0] * sample_x<S>(k) + B[0] * sample_y<S>(k);
                    const int32_t c1 = e0[1] + A[1] * sample_x<S>(k) + B[1] * sample_y<S>(k);
                    const int32_t c2 = e0[2] + A[2] * sample_x<S>(k) + B[2] * sample_y<S>(k);
                    cov |= ((c0 | c1 | c2) >= 0 ? 1u : 0u) << k;
                }
            } else {
                const int64_t Et[3] = {rec.Et[0][r], rec.Et[1][r], rec.Et[2][r]};
#pragma unroll
                for (int k = 0; k < S; k++)
                    cov |= (covered(A, B, Et, qlx * 256 + sample_x<S>(k), qly * 256 + sample_y<S>(k)) ? 1u : 0u) << k;
            }
            return cov;
        };
        // Depth tests of this thread's covered samples of record r, then the fragment record.
        auto apply = [&](int r, unsigned cov) {
            const int meta = rec.meta[r];
            const int func = (meta >> 1) & 7, write = (meta >> 4) & 1;
            const int e = rec.key[r];
            unsigned mask = 0;
            // (float)(sx - X0) == fbx + sample offset exactly (integers below 2^24), as in raster_depth
            const float z0 = rec.z0[r], gzx = rec.dzdx[r], gzy = rec.dzdy[r];
            const float fbx = (float)(px * 256 - rec.X0[r]), fby = (float)(py * 256 - rec.Y0[r]);
#pragma unroll
            for (int k = 0; k < S; k++) {
                if (!(cov & (1u << k))) continue;
                const float z = (z0 + gzx * (fbx + (float)sample_x<S>(k))) + gzy * (fby + (float)sample_y<S>(k));
                if (!depth_cmp(func, z, dep[k])) continue;
                if (write) {
                    dep_changed |= __float_as_uint(dep[k]) != __float_as_uint(z);
                    dep[k] = z;
                }
                vid[k] = (e >> 3) - v.first_tri;
                mask |= 1u << k;
            }
            if (!mask) return;
            // colours never change depth: record the fragment now, shade it later
            if (nfrag == kMaxFrags) {
                if constexpr (DEFER) {  // the in-stage form redoes this tile
                    too_many = true;
                    return;
                } else {  // a full list is applied on the spot (rare)
                    if (!have_cols) start_colours<S>(v, scol, ltile, after_raster, bg);
                    have_cols = true;
                    apply_fragments<S>(a, v, px, py, scol, frags, nfrag);
                    nfrag = 0;
                }
            }
            frags[nfrag * NT + tid] = make_int2(e, (int)(mask | ((unsigned)rec.draw[r] << 16)));
            nfrag++;
        };
        if (scan) {
            // this pixel's candidates: the records whose box holds it (bit r of got[r / 32])
            uint32_t got0 = 0, got1 = 0;
            if (inpix) {
                const int n0 = min(nb, 32);
                for (int r = 0; r < n0; r++) {
                    const uint32_t b = rec.box[r];
                    got0 |= ((b >> lx) & (b >> (16 + ly)) & 1u) << r;
                }
                for (int r = 32; r < nb; r++) {
                    const uint32_t b = rec.box[r];
                    got1 |= ((b >> lx) & (b >> (16 + ly)) & 1u) << (r - 32);
                }
            }
            // The warp's (pixel, record) candidates in lane-major order; their coverage tests are
            // spread over all lanes (chunks of kFwdWarpCand), then every lane applies its own in
            // submission order.
            const int myc = __popc(got0) + __popc(got1);
            int incl = myc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int q = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += q;
            }
            const int T = __shfl_sync(0xffffffffu, incl, 31), pre = incl - myc;
            uint16_t* wc = wcov + (tid >> 5) * kFwdWarpCand;
            uint32_t left0 = got0, left1 = got1;  // this lane's candidates not applied yet
            for (int c0 = 0; c0 < T; c0 += kFwdWarpCand) {
                const int cn = min(kFwdWarpCand, T - c0);
                for (int jb = 0; jb < cn; jb += 32) {
                    const int j = c0 + jb + lane;
                    int o = 0;  // owner lane: the last lane whose first candidate is at or before j
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1)
                        if (__shfl_sync(0xffffffffu, pre, o + step) <= j) o += step;
                    const int opre = __shfl_sync(0xffffffffu, pre, o);
                    const uint32_t og0 = __shfl_sync(0xffffffffu, got0, o), og1 = __shfl_sync(0xffffffffu, got1, o);
                    const float odmax = __shfl_sync(0xffffffffu, dmax_pix, o);
                    if (jb + lane < cn) {
                        const int idx = j - opre, n0 = __popc(og0);
                        const int r = idx < n0 ? nth_set_bit(og0, idx) : 32 + nth_set_bit(og1, idx - n0);
                        int olx, oly;
                        tile_pixel<TS>((tid & ~31) + o, olx, oly);
                        wc[jb + lane] = (uint16_t)cover(r, olx, oly, tx * TS + olx, ty * TS + oly, odmax);
                    }
                }
                __syncwarp();
                const int lo = max(pre, c0), hi = min(pre + myc, c0 + cn);
                for (int jj = lo; jj < hi; jj++) {
                    int r;
                    if (left0) {
                        r = __ffs(left0) - 1;
                        left0 &= left0 - 1;
                    } else {
                        r = 32 + __ffs(left1) - 1;
                        left1 &= left1 - 1;
                    }
                    const unsigned cov = wc[jj - c0];
                    if (cov) apply(r, cov);
                }
                __syncwarp();
            }
        } else {
            // mark the candidates: small boxes by their record's thread, larger ones by the whole warp
            uint32_t* crow = cand + (tid >> 5) * NT;
            if (area > 0 && area <= kFwdSmallBox) {
                const unsigned bit = 1u << lane;
                for (int y = cy0, i = 0; i < area; y++)
                    for (int x = cx0; x < cx0 + cw; x++, i++) atomicOr(crow + tile_lane<TS>(x, y), bit);
            }
            unsigned big = __ballot_sync(0xffffffffu, area > kFwdSmallBox);
            while (big) {
                const int l = __ffs(big) - 1;
                big &= big - 1;
                const int na = __shfl_sync(0xffffffffu, area, l), x0 = __shfl_sync(0xffffffffu, cx0, l);
                const int y0 = __shfl_sync(0xffffffffu, cy0, l), w0 = __shfl_sync(0xffffffffu, cw, l);
                for (int i = lane; i < na; i += 32) atomicOr(crow + tile_lane<TS>(x0 + i % w0, y0 + i / w0), 1u << l);
            }
            __syncthreads();
            if (inpix) {
                // this pixel's candidates in submission order
                for (int w = 0; w < NT / 32; w++) {
                    uint32_t bits = cand[w * NT + tid];
                    while (bits) {
                        const int r = w * 32 + __ffs(bits) - 1;
                        bits &= bits - 1;
                        const unsigned cov = cover(r, lx, ly, px, py, dmax_pix);
                        if (cov) apply(r, cov);
                    }
                }
            }
        }
        __syncthreads();
    }
    if constexpr (DEFER) {
        // Hand the tile's fragments to the fragment kernels, pixel-major in lane order.  A tile with a
        // pixel of more than kFwdFragsDefer fragments, or whose fragments do not fit the buffer, writes
        // nothing and goes to the redo list: the in-stage form finishes it from the same inputs.
        __shared__ uint32_t s_wsum[NT / 32];
        __shared__ int s_slot;
        __shared__ uint32_t s_base;
        if (__syncthreads_or(too_many)) {
            if (tid == 0) fa.redo_tiles[atomicAdd(a.status + ST_REDO, 1u)] = (uint32_t)gtile;
            return;
        }
        uint32_t incl = (uint32_t)nfrag;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t q = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += q;
        }
        if (lane == 31) s_wsum[tid >> 5] = incl;
        __syncthreads();
        uint32_t before = 0, total = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; w++) {
            const uint32_t x = s_wsum[w];
            before += w < (tid >> 5) ? x : 0u;
            total += x;
        }
        const uint32_t pre = before + incl - (uint32_t)nfrag;
        if (tid == 0) {
            int slot = -1;
            const uint32_t fbase = total ? atomicAdd(a.status + ST_FRAGS, total) : 0u;
            if ((unsigned long long)fbase + total <= fa.frag_capacity) {
                slot = (int)atomicAdd(a.status + ST_FWD_TILES, 1u);
                fa.fwd_tiles[slot] = make_uint4((uint32_t)gtile, fbase, (uint32_t)vi, after_raster ? 1u : 0u);
            } else {  // later allocations fail too: the fragments below this one are all written
                atomicMax(a.status + ST_FRAG_FAIL, 0xFFFFFFFFu - fbase);
                const unsigned long long want = (unsigned long long)fbase + total;
                atomicMax(a.status + ST_MAX_FRAGS, want > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)want);
                fa.redo_tiles[atomicAdd(a.status + ST_REDO, 1u)] = (uint32_t)gtile;
            }
            s_slot = slot;
            s_base = fbase;
        }
        __syncthreads();
        const int slot = s_slot;
        if (slot < 0) return;
        uint4* out = fa.frags + s_base + pre;
        for (int i = 0; i < nfrag; i++) {
            const int2 f = frags[i * NT + tid];
            out[i] = make_uint4((uint32_t)f.x, (uint32_t)px | ((uint32_t)py << 16), (uint32_t)f.y & 0xffffu,
                                (uint32_t)f.y >> 16);
        }
        fa.fwd_pix_end[(size_t)slot * NT + tid] = (uint16_t)(pre + nfrag);
        if (inpix) {
            if (dep_changed) store_depth<S>(v.depth + pix * S, dep);
            if (v.vis) {
                int* vp = v.vis + pix * S;
#pragma unroll
                for (int k = 0; k < S; k++) vp[k] = vid[k];
            }
        }
        return;
    } else {
    // shade the recorded fragments with the warp converged on fragment slot i of every lane, and
    // apply each one in submission order to its samples (spreading the fragments' anisotropic probes
    // over the warp's lanes, as the shade stage does, measured slower here: 5.15 vs 4.09 ms on the
    // stress frame, more instruction-cache stalls at no fewer instructions)
    const int maxn = __reduce_max_sync(0xffffffffu, nfrag);
    for (int i = 0; i < maxn; i++)
        if (i < nfrag) apply_fragment<S>(a, v, px, py, scol, frags[i * NT + tid]);
    if (!inpix) return;
    float acc[4];
#pragma unroll
    for (int k = 0; k < S; k++) {
        const float4 q = scol[k * NT + tid];
        if (k == 0) {
            acc[0] = q.x; acc[1] = q.y; acc[2] = q.z; acc[3] = q.w;
        } else {
            acc[0] = acc[0] + q.x; acc[1] = acc[1] + q.y; acc[2] = acc[2] + q.z; acc[3] = acc[3] + q.w;
        }
    }
    const float invS = 1.0f / (float)S;
    acc[0] = acc[0] * invS; acc[1] = acc[1] * invS; acc[2] = acc[2] * invS; acc[3] = acc[3] * invS;
    encode_color(v, pix, acc);
    if (dep_changed) store_depth<S>(v.depth + pix * S, dep);
    if (v.vis) {
        int* vp = v.vis + pix * S;
#pragma unroll
        for (int k = 0; k < S; k++) vp[k] = vid[k];
    }
    }
}

template <int S, bool DEFER>
size_t forward_smem_bytes() {
    return sizeof(FwdRecords) + (DEFER ? 0 : sizeof(float4) * S * kFwdThreads) +
           sizeof(uint32_t) * (DEFER ? kFwdListDefer : kOrderedCap) +
           sizeof(int2) * (DEFER ? kFwdFragsDefer : kFwdFrags) * kFwdThreads +
           sizeof(uint32_t) * kFwdThreads * (kFwdThreads / 32);
}

// The in-stage form runs two CTAs per SM (128 registers, its shading code included); the deferring
// form, which shades nothing and sorts up to kFwdListDefer entries, four up to 8 samples (64 registers,
// 49 KB of shared memory each; measured faster than three at 80 registers despite the spills) and three
// at 16 (whose spills at 64 registers would be larger).
template <int S, bool DEFER>
__global__ void __launch_bounds__(kFwdThreads, DEFER ? (S <= 8 ? 4 : 3) : 2) forward_kernel(PassArgs a, FragArgs fa, GroupArgs g,
                                                                             int qslot, int after_raster) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FwdRecords& rec = *reinterpret_cast<FwdRecords*>(smem_raw);
    float4* scol = reinterpret_cast<float4*>(smem_raw + sizeof(FwdRecords));  // [S][256] (not DEFER)
    uint32_t* list =
        reinterpret_cast<uint32_t*>(smem_raw + sizeof(FwdRecords) + (DEFER ? 0 : sizeof(float4) * S * kFwdThreads));
    int2* frags = reinterpret_cast<int2*>(list + (DEFER ? kFwdListDefer : kOrderedCap));  // [fragments per pixel][256]
    uint32_t* cand = reinterpret_cast<uint32_t*>(frags + (DEFER ? kFwdFragsDefer : kFwdFrags) * kFwdThreads);  // [8][256]
    uint16_t* wcov = reinterpret_cast<uint16_t*>(cand);  // [8][kFwdWarpCand], aliases cand
    static_assert(sizeof(uint16_t) * kFwdWarpCand * (kFwdThreads / 32) <= sizeof(uint32_t) * kFwdThreads * (kFwdThreads / 32),
                  "coverage buffers fit the candidate masks");
    __shared__ ViewArgs sv;
    __shared__ int s_tile, s_view;
    __shared__ __align__(8) uint64_t s_bar;
    BulkState bs;
    bs.bar = &s_bar;
    bs.phase = 0;
    bs.ok = true;
    bs.pending = false;
    if (threadIdx.x == 0) {
        s_view = -1;
        mbar_init(&s_bar, 1);
    }
    __syncthreads();
    while (next_tile<kFwdThreads>(a, g, qslot, sv, s_tile, s_view))
        forward_tile<S, DEFER>(a, fa, sv, s_view, s_tile, rec, scol, list, frags, cand, wcov, after_raster != 0, bs);
    if (bs.pending && threadIdx.x == 0) mbar_wait(&s_bar, (bs.phase - 1) & 1u);  // a copy that did not land in time
}

// The tiles the deferring form left (redo list), finished by the in-stage form from the same inputs:
// the deferring form wrote nothing for them.  Tiles are taken in list order, one per CTA iteration.
template <int S>
__global__ void __launch_bounds__(kFwdThreads, 2) forward_redo_kernel(PassArgs a, FragArgs fa, GroupArgs g,
                                                                   int after_raster) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FwdRecords& rec = *reinterpret_cast<FwdRecords*>(smem_raw);
    float4* scol = reinterpret_cast<float4*>(smem_raw + sizeof(FwdRecords));  // [S][256]
    uint32_t* list = reinterpret_cast<uint32_t*>(smem_raw + sizeof(FwdRecords) + sizeof(float4) * S * kFwdThreads);
    int2* frags = reinterpret_cast<int2*>(list + kOrderedCap);  // [kFwdFrags][256]
    uint32_t* cand = reinterpret_cast<uint32_t*>(frags + kFwdFrags * kFwdThreads);  // [8][256]
    uint16_t* wcov = reinterpret_cast<uint16_t*>(cand);
    __shared__ ViewArgs sv;
    __shared__ int s_view;
    __shared__ __align__(8) uint64_t s_bar;
    BulkState bs;
    bs.bar = &s_bar;
    bs.phase = 0;
    bs.ok = true;
    bs.pending = false;
    if (threadIdx.x == 0) mbar_init(&s_bar, 1);
    const uint32_t n = min(a.status[ST_REDO], (uint32_t)(g.tile_end - g.tile_begin));
    const FragArgs none{};  // the in-stage form reads no fragment buffers
    for (uint32_t slot = blockIdx.x; slot < n; slot += gridDim.x) {
        const int t = (int)fa.redo_tiles[slot];
        __syncthreads();  // the previous tile's staged data is no longer read
        if (threadIdx.x == 0) {
            int lo = g.view_begin, hi = g.view_end - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(a.view_tile_start + mid) <= t) lo = mid; else hi = mid - 1;
            }
            s_view = lo;
        }
        __syncthreads();
        const int* src = reinterpret_cast<const int*>(a.views + s_view);
        int* dst = reinterpret_cast<int*>(&sv);
        for (int i = threadIdx.x; i < (int)(sizeof(ViewArgs) / 4); i += kFwdThreads) dst[i] = src[i];
        __syncthreads();
        forward_tile<S, false>(a, none, sv, s_view, t, rec, scol, list, frags, cand, wcov, after_raster != 0, bs);
    }
    __syncthreads();
    if (bs.pending && threadIdx.x == 0) mbar_wait(&s_bar, (bs.phase - 1) & 1u);  // a copy that did not land in time
}

// ---------------------------------------------------------------------------- deferred ordered fragments
// Fragments of the ordered tiles that the ordered stage handed off: their colours do not depend
// on the order they are applied in, so they are shaded here with every thread busy (the tile
// routine would leave most threads of a tile waiting for the pixels with the most fragments),
// then blended per pixel in submission order.

// Fragments below this count were written by tiles whose allocation fitted.
__device__ __forceinline__ uint32_t deferred_fragments(const PassArgs& a, const FragArgs& fa) {
    const uint32_t fail = a.status[ST_FRAG_FAIL];
    const uint32_t n = fail ? 0xFFFFFFFFu - fail : a.status[ST_FRAGS];
    return min(n, fa.frag_capacity);
}

// Warps take 32 fragments at a time: set-up from the triangle record where there is one, the
// vertex attributes from the attribute record, then the texture probes of all 32 spread over the
// lanes (as the shade stage does).
constexpr int kFragShadeThreads = 256;

__global__ void __launch_bounds__(kFragShadeThreads, 4) frag_shade_kernel(PassArgs a, FragArgs fa) {
    __shared__ float4 s_res[kFragShadeThreads / 32][32];
    const uint32_t n = deferred_fragments(a, fa);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (;;) {
        // 32 fragments at a time from the pass's counter, so that CTAs which start late (the redo
        // kernel of the in-stage form may hold part of an SM meanwhile) take less work
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(a.status + ST_FRAG_NEXT, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        int di = 0, np = 0;
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        TexProbe tp;
        tp.u = tp.v = tp.du = tp.dv = tp.t = 0.0f;
        tp.lo = tp.hi = tp.n = 0;
        tp.two = tp.aniso = false;
        if (i < n) {
            const uint4 f = fa.frags[i];
            const int g = (int)(f.x >> 3), sub = (int)(f.x & 7u);
            const int px = (int)(f.y & 0xffffu), py = (int)(f.y >> 16);
            const TriRecord* rp = a.records + g;
            const int4 q1 = __ldg(reinterpret_cast<const int4*>(rp) + 1);  // X2, Y2, flags, draw
            di = q1.w;
            const DrawDev& d = a.draws[di];
            const PassConst& pc = a.views[d.view].c;
            const int t = g - __ldg(a.draw_start + di);
            const bool from_record = sub == 0 && (q1.z & REC_VALID);
            if (from_record && d.polygon_mode == POLY_FILL && a.attrs && d.shading != SHADE_PRIMID && d.attr_count > 0) {
                ShadeGeom geo;
                float4 plane;
                int plane_y;
                shade_geom_record(rp, q1, geo, plane, plane_y);
                float a0[4], a1[4], a2[4];
                const float4 r0 = __ldg(&a.attrs[g].a[0]), r1 = __ldg(&a.attrs[g].a[1]), r2 = __ldg(&a.attrs[g].a[2]);
                a0[0] = r0.x; a0[1] = r0.y; a0[2] = r0.z; a0[3] = r0.w;
                a1[0] = r1.x; a1[1] = r1.y; a1[2] = r1.z; a1[3] = r1.w;
                a2[0] = r2.x; a2[1] = r2.y; a2[2] = r2.z; a2[3] = r2.w;
                if (shade_prepare_attrs(pc, d, geo, t, sub, px, py, a0, a1, a2, c, tp)) np = tp.n;
            } else {
                const ItemShade r = shade_item_general<1, false>(a, pc, di, g, t, sub, from_record, px, py, 0u, 0, nullptr, 0);
                c[0] = r.c[0]; c[1] = r.c[1]; c[2] = r.c[2]; c[3] = r.c[3];
                tp = r.tp;
                np = r.n;
            }
        }
        warp_texture_probes(a.draws, di, tp, np, s_res[warp], c);
        if (i < n) fa.frag_cols[i] = make_float4(c[0], c[1], c[2], c[3]);
    }
}

// One deferred tile per CTA iteration, one pixel per thread: the starting colours (the prefix's
// hand-off or the background), the pixel's fragments applied in submission order, then the resolve.
// The hand-off of the CTA's next tile (S x 256 float4, contiguous) comes into the other half of a
// double buffer by one bulk copy (TMA) while the current tile is blended; each thread updates its
// own samples in place.  A wait that gives up reports status bit ST_STICKY & 4 and the CTA reads
// the hand-off from memory from then on.
template <int S>
constexpr int blend_min_blocks() { return S <= 4 ? 4 : S == 8 ? 3 : 1; }

template <int S>
constexpr size_t blend_smem_bytes() { return 2 * sizeof(float4) * S * kFwdThreads; }

template <int S>
__global__ void __launch_bounds__(kFwdThreads, blend_min_blocks<S>()) frag_blend_kernel(PassArgs a, FragArgs fa) {
    constexpr int TS = 16, NT = kFwdThreads;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4* buf = reinterpret_cast<float4*>(smem_raw);  // [2][S][NT]
    __shared__ __align__(8) uint64_t s_bar[2];
    const int tid = threadIdx.x;
    const uint32_t ntiles = a.status[ST_FWD_TILES];
    if (tid == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
    }
    __syncthreads();
    int lx, ly;
    tile_pixel<TS>(tid, lx, ly);
    bool use_bulk = true;          // the same in every thread
    bool inflight[2] = {false, false};
    uint32_t parity[2] = {0u, 0u};  // parity of each buffer's next completed phase
    int stuck = -1;                 // buffer whose copy a wait gave up on
    uint32_t slot = blockIdx.x;
    if (slot < ntiles) {
        const uint4 t = fa.fwd_tiles[slot];
        if (t.w) {
            if (tid == 0) {
                const ViewArgs& v = a.views[t.z];
                bulk_load(buf, v.sample_colors + (size_t)((int)t.x - v.tile_start) * S * NT,
                          (uint32_t)(sizeof(float4) * S * NT), &s_bar[0]);
            }
            inflight[0] = true;
        }
    }
    for (int b = 0; slot < ntiles; slot += gridDim.x, b ^= 1) {
        // the next tile's hand-off into the other buffer, free since the barrier that ended the
        // previous iteration
        const uint32_t next = slot + gridDim.x;
        if (next < ntiles && use_bulk) {
            const uint4 tn = fa.fwd_tiles[next];
            if (tn.w) {
                if (tid == 0) {
                    const ViewArgs& vn = a.views[tn.z];
                    bulk_load(buf + (b ^ 1) * S * NT, vn.sample_colors + (size_t)((int)tn.x - vn.tile_start) * S * NT,
                              (uint32_t)(sizeof(float4) * S * NT), &s_bar[b ^ 1]);
                }
                inflight[b ^ 1] = true;
            }
        }
        const uint4 t = fa.fwd_tiles[slot];  // global tile, first fragment, view, hand-off flag
        const ViewArgs& v = a.views[t.z];
        const int ltile = (int)t.x - v.tile_start;
        const int tx = ltile % v.c.tiles_x, ty = ltile / v.c.tiles_x;
        const int px = tx * TS + lx, py = ty * TS + ly;
        const bool inpix = px < v.c.W && py < v.c.H;
        const size_t pix = (size_t)py * v.c.W + px;
        float4* col = buf + b * S * NT + tid;  // this thread's samples, stride NT
        bool have = false;
        if (inflight[b]) {
            const bool ok = mbar_wait(&s_bar[b], parity[b]);
            parity[b] ^= 1u;
            inflight[b] = false;
            if (__syncthreads_and(ok)) {
                have = true;
            } else {  // report, and read the hand-off from memory from now on
                if (tid == 0) atomicOr(a.status + ST_STICKY, 4u);
                use_bulk = false;
                stuck = b;
            }
        }
        if (inpix) {
            if (!have) {
                if (t.w) {
#pragma unroll
                    for (int k = 0; k < S; k++) col[k * NT] = v.sample_colors[((size_t)ltile * S + k) * NT + tid];
                } else {
                    float bg[4];
                    if (v.clear) {
                        bg[0] = v.clear_color[0]; bg[1] = v.clear_color[1]; bg[2] = v.clear_color[2]; bg[3] = v.clear_color[3];
                    } else {
                        decode_color(v, pix, bg);
                    }
#pragma unroll
                    for (int k = 0; k < S; k++) col[k * NT] = make_float4(bg[0], bg[1], bg[2], bg[3]);
                }
            }
            const uint16_t* pe = fa.fwd_pix_end + (size_t)slot * NT;
            const uint32_t f0 = t.y + (tid ? pe[tid - 1] : 0u), f1 = t.y + pe[tid];
            for (uint32_t f = f0; f < f1; f++) {
                const uint4 r = fa.frags[f];  // entry, pixel, sample mask, draw
                const float4 q = fa.frag_cols[f];
                const float c[4] = {q.x, q.y, q.z, q.w};
                const DrawDev& d = a.draws[r.w];
                if (d.blend_enable && !blend_reads_dst(d)) {
                    // factors of the source only (alpha blending): once per fragment
                    float fs[4], fd[4];
#pragma unroll
                    for (int ch = 0; ch < 4; ch++) {
                        fs[ch] = blend_factor(ch < 3 ? d.blend_src_color : d.blend_src_alpha, ch, c, c);
                        fd[ch] = blend_factor(ch < 3 ? d.blend_dst_color : d.blend_dst_alpha, ch, c, c);
                    }
                    for (uint32_t m = r.z; m; m &= m - 1) {
                        const int k = __ffs(m) - 1;
                        const float4 o = col[k * NT];
                        col[k * NT] = make_float4(o.x * fd[0] + c[0] * fs[0], o.y * fd[1] + c[1] * fs[1],
                                                  o.z * fd[2] + c[2] * fs[2], o.w * fd[3] + c[3] * fs[3]);
                    }
                    continue;
                }
                for (uint32_t m = r.z; m; m &= m - 1) {  // the covered samples, one copy of the blend code
                    const int k = __ffs(m) - 1;
                    if (d.blend_enable) {
                        const float4 o = col[k * NT];
                        float dst[4] = {o.x, o.y, o.z, o.w};
                        blend_into(d, c, dst);
                        col[k * NT] = make_float4(dst[0], dst[1], dst[2], dst[3]);
                    } else {
                        col[k * NT] = q;
                    }
                }
            }
            float4 q0 = col[0];
            float acc[4] = {q0.x, q0.y, q0.z, q0.w};
#pragma unroll
            for (int k = 1; k < S; k++) {
                const float4 q = col[k * NT];
                acc[0] = acc[0] + q.x; acc[1] = acc[1] + q.y; acc[2] = acc[2] + q.z; acc[3] = acc[3] + q.w;
            }
            const float invS = 1.0f / (float)S;
            acc[0] = acc[0] * invS; acc[1] = acc[1] * invS; acc[2] = acc[2] * invS; acc[3] = acc[3] * invS;
            encode_color(v, pix, acc);
        }
        __syncthreads();
    }
    if (tid == 0) {  // copies left in flight: a prefetch past a failed wait, or the copy given up on
        for (int b = 0; b < 2; b++)
            if (inflight[b]) mbar_wait(&s_bar[b], parity[b]);
        if (stuck >= 0) mbar_wait(&s_bar[stuck], parity[stuck] ^ 1u);
    }
}

// ---------------------------------------------------------------------------- reference line / point rules
// The reference CUDA renderer's own line and point pipelines (TileRasterCoreInvocationCuda.cu:
// 2780-3334), selected by iftrSetPolygonRules for LINE / POINT polygon modes: points are the
// draw's indices truncated to pixels (:2782-2822), lines are the triangles' three edges walked by
// Bresenham between truncated endpoints (:2974-3115), and every pixel keeps its nearest candidate
// (:2855-2920, 3167-3280).  The reference leaves depth ties to atomic arrival order; here each
// candidate is a 64-bit key (ordered depth bits, submission order) lowered with atomicMin, so the
// earliest candidate wins ties and the image is deterministic.  One thread per index (points) or
// per triangle (lines, three edges each); a resolve pass per pixel applies the depth test against
// the buffer (strict less, as the reference) and shades the winner.  Single-sample targets.
__device__ __forceinline__ unsigned long long ref_key(float z, uint32_t order) {
    uint32_t u = __float_as_uint(z + 0.0f);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((unsigned long long)u << 32) | order;
}

__device__ __forceinline__ float ref_key_depth(unsigned long long k) {
    uint32_t u = (uint32_t)(k >> 32);
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(u);
}

__device__ __forceinline__ void ref_offer(unsigned long long* keys, const PassConst& c, int px, int py, float z,
                                          uint32_t order) {
    if (px < 0 || py < 0 || px >= c.W || py >= c.H || z != z) return;
    atomicMin(keys + (size_t)py * c.W + px, ref_key(z, order));
}

// Edge e of triangle t after the w < 0 clip (moved to w = 1) and the NDC mapping; false when dropped.
__device__ __forceinline__ bool ref_edge(const DrawDev& d, int t, int e, float* p1, float* p2) {
    const int ia = __ldg(d.indices + 3 * (size_t)t + e), ib = __ldg(d.indices + 3 * (size_t)t + (e + 1) % 3);
    if (ia < 0 || ia >= d.num_vertices || ib < 0 || ib >= d.num_vertices) return false;
    float v1[4], v2[4];
    xform(d.mvp, d.vertices + (size_t)ia * d.stride, v1);
    xform(d.mvp, d.vertices + (size_t)ib * d.stride, v2);
    if (v1[3] < 0.0f && v2[3] < 0.0f) return false;
    if (v1[3] < 0.0f) {
        const float t1 = __fdiv_rn(-1.0f + v2[3], v2[3] - v1[3]);
#pragma unroll
        for (int k = 0; k < 4; k++) v1[k] = v2[k] + (v1[k] - v2[k]) * t1;
    }
    if (v2[3] < 0.0f) {
        const float t2 = __fdiv_rn(-1.0f + v1[3], v1[3] - v2[3]);
#pragma unroll
        for (int k = 0; k < 4; k++) v2[k] = v1[k] + (v2[k] - v1[k]) * t2;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        v1[k] = __fdiv_rn(v1[k], v1[3]);
        v2[k] = __fdiv_rn(v2[k], v2[3]);
    }
    v1[0] = v1[0] * 0.5f + 0.5f;
    v1[1] = v1[1] * 0.5f + 0.5f;
    v2[0] = v2[0] * 0.5f + 0.5f;
    v2[1] = v2[1] * 0.5f + 0.5f;
    if (v1[0] < 0.0f || v1[1] < 0.0f || v1[0] > 1.0f || v1[1] > 1.0f) return false;
    if (v2[0] < 0.0f || v2[1] < 0.0f) return false;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        p1[k] = v1[k];
        p2[k] = v2[k];
    }
    return true;
}

// Fraction of pixel (px, py) along the edge, on its major axis in pixel units.
__device__ __forceinline__ float ref_percent(const PassConst& c, const float* p1, const float* p2, int px, int py) {
    const float ax = p1[0] * (float)c.W, ay = p1[1] * (float)c.H, bx = p2[0] * (float)c.W, by = p2[1] * (float)c.H;
    if (fabsf(bx - ax) >= fabsf(by - ay)) return __fdiv_rn((float)px - ax, bx - ax);
    return __fdiv_rn((float)py - ay, by - ay);
}

__global__ void __launch_bounds__(256) ref_keys_init_kernel(unsigned long long* keys, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        keys[i] = ~0ull;
}

__global__ void __launch_bounds__(256) ref_point_kernel(DrawDev d, PassConst c, unsigned long long* keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * d.num_triangles) return;
    const int vid = __ldg(d.indices + i);
    if (vid < 0 || vid >= d.num_vertices) return;
    float v[4];
    xform(d.mvp, d.vertices + (size_t)vid * d.stride, v);
    if (v[3] < 1e-8f) return;
    float x = __fdiv_rn(v[0], v[3]), y = __fdiv_rn(v[1], v[3]);
    const float z = __fdiv_rn(v[2], v[3]);
    x = x * 0.5f + 0.5f;
    y = y * 0.5f + 0.5f;
    if (x < 0.0f || x > 1.0f || y < 0.0f || y > 1.0f) return;
    ref_offer(keys, c, (int)(x * (float)(c.W - 1)), (int)(y * (float)(c.H - 1)), z, (uint32_t)i);
}

__global__ void __launch_bounds__(256) ref_line_kernel(DrawDev d, PassConst c, unsigned long long* keys) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.num_triangles) return;
    for (int e = 0; e < 3; e++) {
        float p1[4], p2[4];
        if (!ref_edge(d, t, e, p1, p2)) continue;
        const uint32_t order = (uint32_t)(3 * t + e);
        int x1 = (int)(p1[0] * (float)(c.W - 1)), y1 = (int)(p1[1] * (float)(c.H - 1));
        int x2 = (int)(p2[0] * (float)(c.W - 1)), y2 = (int)(p2[1] * (float)(c.H - 1));
        const bool xmajor = abs(x1 - x2) > abs(y1 - y2);
        if (xmajor ? x2 < x1 : y2 < y1) {
            int q = x1; x1 = x2; x2 = q;
            q = y1; y1 = y2; y2 = q;
        }
        // Bresenham with a float error term (:3076-3112): the major coordinate advances by one,
        // the minor one when the accumulated slope passes 1/2
        const int len = xmajor ? x2 - x1 : y2 - y1;
        const float slope = xmajor ? fabsf(__fdiv_rn(1.0f * (float)(y2 - y1), (float)(x2 - x1)))
                                   : fabsf(__fdiv_rn(1.0f * (float)(x2 - x1), (float)(y2 - y1)));
        const int step = xmajor ? ((y2 - y1) > 0 ? 1 : -1) : ((x2 - x1) > 0 ? 1 : -1);
        float err = 0.0f;
        int cx = x1, cy = y1;
        for (int i = 0; i <= len; i++) {
            if (cx < c.W && cy < c.H) {
                const float f = ref_percent(c, p1, p2, cx, cy);
                ref_offer(keys, c, cx, cy, p1[2] + (p2[2] - p1[2]) * f, order);
            }
            err = err + slope;
            if (err > 0.5f) {
                if (xmajor) cy += step; else cx += step;
                err = err - 1.0f;
            }
            if (xmajor) cx++; else cy++;
        }
    }
}

__device__ __forceinline__ void ref_attr(const DrawDev& d, int vid, float out[4]) {
    const float* a = d.vertices + (size_t)vid * d.stride + d.attr_offset;
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = k < d.attr_count ? __ldg(a + k) : 0.0f;
}

__global__ void __launch_bounds__(256) ref_resolve_kernel(DrawDev d, ViewArgs v, const unsigned long long* keys) {
    const int W = v.c.W, H = v.c.H;
    const size_t npix = (size_t)W * H;
    for (size_t pix = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pix < npix; pix += (size_t)gridDim.x * blockDim.x) {
        const int px = (int)(pix % W), py = (int)(pix / W);
        float depth = v.clear ? v.clear_depth : v.depth[pix];
        bool write = v.clear;
        float col[4] = {v.clear_color[0], v.clear_color[1], v.clear_color[2], v.clear_color[3]};
        int vis = -1;
        const unsigned long long k = keys[pix];
        if (k != ~0ull) {
            const float z = ref_key_depth(k);
            if (z < depth) {
                const uint32_t order = (uint32_t)k;
                const int t = (int)(order / 3u), e = (int)(order % 3u);
                if (d.shading == SHADE_PRIMID) {
                    col[0] = (float)(d.prim_base + t); col[1] = (float)e; col[2] = 0.0f; col[3] = 1.0f;
                } else if (d.polygon_mode == POLY_POINT) {
                    ref_attr(d, __ldg(d.indices + order), col);
                    if (d.attr_count < 4) col[3] = 1.0f;
                } else {
                    float p1[4], p2[4], a1[4], a2[4];
                    ref_edge(d, t, e, p1, p2);
                    const float f = ref_percent(v.c, p1, p2, px, py);
                    const float z1 = p1[3], z2 = p2[3];
                    const float zt = __fdiv_rn(z1 * z2, z2 + f * (z1 - z2));
                    ref_attr(d, __ldg(d.indices + 3 * (size_t)t + e), a1);
                    ref_attr(d, __ldg(d.indices + 3 * (size_t)t + (e + 1) % 3), a2);
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const float u1 = __fdiv_rn(a1[q], z1), u2 = __fdiv_rn(a2[q], z2);
                        col[q] = (f * (u2 - u1) + u1) * zt;
                    }
                    if (d.attr_count < 4) col[3] = 1.0f;
                }
                depth = z;
                vis = d.prim_base + t;
                write = true;
            } else if (!v.clear) {
                continue;
            }
        } else if (!v.clear) {
            continue;
        }
        if (write) {
            encode_color(v, pix, col);
            v.depth[pix] = depth;
            if (v.vis) v.vis[pix] = vis;
        }
    }
}

cudaError_t launch_reference_rules(const DrawDev& d, const ViewArgs& v, unsigned long long* keys, cudaStream_t stream) {
    const size_t npix = (size_t)v.c.W * v.c.H;
    const int fill_blocks = (int)std::min<size_t>((npix + 255) / 256, 4096);
    ref_keys_init_kernel<<<fill_blocks, 256, 0, stream>>>(keys, npix);
    if (d.num_triangles > 0) {
        if (d.polygon_mode == POLY_POINT)
            ref_point_kernel<<<(3 * d.num_triangles + 255) / 256, 256, 0, stream>>>(d, v.c, keys);
        else
            ref_line_kernel<<<(d.num_triangles + 255) / 256, 256, 0, stream>>>(d, v.c, keys);
    }
    ref_resolve_kernel<<<fill_blocks, 256, 0, stream>>>(d, v, keys);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------- mesh-stage outputs
// Compaction of per-work-group mesh (or geometry) stage outputs into one indexed clip-space mesh,
// in work-group order (TileRasterCoreInvocationCuda.cu:384-402 compacts in atomic arrival order).
// Offsets: one CTA, each thread a run of consecutive work groups; counts above the per-group
// maxima, negative counts or index counts that are not a multiple of 3 set totals[2].
__global__ void __launch_bounds__(1024) mesh_offsets_kernel(const int* __restrict__ nv, const int* __restrict__ ni,
                                                            int groups, int max_v, int max_i, int* off_v, int* off_i,
                                                            long long* totals) {
    __shared__ long long ws[2][33];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int per = (groups + 1023) / 1024;
    const int b = min((int)threadIdx.x * per, groups), e = min(b + per, groups);
    long long sv = 0, si = 0;
    int bad = 0;
    for (int g = b; g < e; g++) {
        const int v = nv[g], i = ni[g];
        bad |= v < 0 || v > max_v || i < 0 || i > max_i || i % 3 != 0;
        sv += v < 0 ? 0 : min(v, max_v);
        si += i < 0 ? 0 : min(i, max_i) / 3 * 3;
    }
    long long iv = sv, ii = si;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long qv = __shfl_up_sync(0xffffffffu, iv, o), qi = __shfl_up_sync(0xffffffffu, ii, o);
        if (lane >= o) { iv += qv; ii += qi; }
    }
    if (lane == 31) { ws[0][wid] = iv; ws[1][wid] = ii; }
    bad = __syncthreads_or(bad);
    if (wid == 0) {
        long long a = ws[0][lane], c = ws[1][lane], ai = a, ci = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long qa = __shfl_up_sync(0xffffffffu, ai, o), qc = __shfl_up_sync(0xffffffffu, ci, o);
            if (lane >= o) { ai += qa; ci += qc; }
        }
        ws[0][lane] = ai - a;
        ws[1][lane] = ci - c;
        if (lane == 31) { ws[0][32] = ai; ws[1][32] = ci; }
    }
    __syncthreads();
    long long rv = ws[0][wid] + iv - sv, ri = ws[1][wid] + ii - si;
    for (int g = b; g < e; g++) {
        const int v = nv[g], i = ni[g];
        off_v[g] = (int)min(rv, (long long)INT32_MAX);
        off_i[g] = (int)min(ri, (long long)INT32_MAX);
        rv += v < 0 ? 0 : min(v, max_v);
        ri += i < 0 ? 0 : min(i, max_i) / 3 * 3;
    }
    if (threadIdx.x == 0) {
        totals[0] = ws[0][32];
        totals[1] = ws[1][32];
        totals[2] = bad;
    }
}

// Work group g (one CTA): its vertices become rows [x y z w a0 a1 a2 a3] of the compacted vertex
// array, its indices are rebased by the group's first vertex.
__global__ void __launch_bounds__(128) mesh_compact_kernel(const float4* __restrict__ pos, const float4* __restrict__ attr,
                                                           const int* __restrict__ idx, const int* __restrict__ nv,
                                                           const int* __restrict__ ni, const int* __restrict__ off_v,
                                                           const int* __restrict__ off_i, int max_v, int max_i,
                                                           float4* __restrict__ out_v, int* __restrict__ out_i) {
    const int g = blockIdx.x;
    const int v = min(max(nv[g], 0), max_v), n = min(max(ni[g], 0), max_i) / 3 * 3;
    const int ov = off_v[g], oi = off_i[g];
    for (int k = threadIdx.x; k < v; k += blockDim.x) {
        const size_t src = (size_t)g * max_v + k;
        out_v[2 * ((size_t)ov + k)] = pos[src];
        out_v[2 * ((size_t)ov + k) + 1] = attr ? attr[src] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int l = idx[(size_t)g * max_i + k];
        // an index outside the group's vertices becomes -1, which the front end rejects
        out_i[(size_t)oi + k] = l >= 0 && l < v ? ov + l : -1;
    }
}

cudaError_t launch_mesh_offsets(const int* nv, const int* ni, int groups, int max_v, int max_i, int* off_v, int* off_i,
                                long long* totals, cudaStream_t stream) {
    mesh_offsets_kernel<<<1, 1024, 0, stream>>>(nv, ni, groups, max_v, max_i, off_v, off_i, totals);
    return cudaGetLastError();
}

cudaError_t launch_mesh_compact(const float* pos, const float* attr, const int* idx, const int* nv, const int* ni,
                                const int* off_v, const int* off_i, int groups, int max_v, int max_i, float* out_v,
                                int* out_i, cudaStream_t stream) {
    if (groups > 0)
        mesh_compact_kernel<<<groups, 128, 0, stream>>>(reinterpret_cast<const float4*>(pos),
                                                        reinterpret_cast<const float4*>(attr), idx, nv, ni, off_v,
                                                        off_i, max_v, max_i, reinterpret_cast<float4*>(out_v), out_i);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------- mips
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

// ---------------------------------------------------------------------------- launches
template <int S, int TS>
cudaError_t configure_deferred() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(raster_kernel<S, TS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)raster_smem_bytes<S, TS>());
    if (e == cudaSuccess) done = true;
    return e;
}

template <int S, bool DEFER>
cudaError_t configure_forward() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(forward_kernel<S, DEFER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)forward_smem_bytes<S, DEFER>());
    if (e == cudaSuccess) done = true;
    return e;
}

template <int S, int TS>
cudaError_t launch_deferred(const PassArgs& a, const GroupArgs& g, int ctas, cudaStream_t stream, bool shade) {
    cudaError_t e = configure_deferred<S, TS>();
    if (e != cudaSuccess) return e;
    if (!shade) raster_kernel<S, TS><<<ctas, TS * TS, raster_smem_bytes<S, TS>(), stream>>>(a, g);
    else shade_kernel<S, TS><<<ctas, kShadeThreads, 0, stream>>>(a, g);
    return cudaSuccess;
}

template <int S, bool DEFER>
cudaError_t launch_forward_form(const PassArgs& a, const FragArgs& fa, const GroupArgs& g, int ctas,
                                cudaStream_t stream, int qslot) {
    cudaError_t e = configure_forward<S, DEFER>();
    if (e != cudaSuccess) return e;
    forward_kernel<S, DEFER><<<ctas, kFwdThreads, forward_smem_bytes<S, DEFER>(), stream>>>(a, fa, g, qslot,
                                                                                           qslot % 3 == 2);
    return cudaSuccess;
}

template <int S>
cudaError_t configure_redo() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(forward_redo_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)forward_smem_bytes<S, false>());
    if (e == cudaSuccess) done = true;
    return e;
}

// The deferring form when there are fragment buffers (its redo list is finished by launch_redo),
// else the in-stage form.
template <int S>
cudaError_t launch_forward(const PassArgs& a, const FragArgs& fa, const GroupArgs& g, int ctas, cudaStream_t stream,
                           int qslot) {
    if (!fa.frags) return launch_forward_form<S, false>(a, fa, g, ctas, stream, qslot);
    return launch_forward_form<S, true>(a, fa, g, ctas, stream, qslot);
}

// The in-stage form over the tiles the deferring form left (usually none or a few: one CTA per SM
// reads the count, those without a tile exit).
template <int S>
cudaError_t launch_redo(const PassArgs& a, const FragArgs& fa, const GroupArgs& g, bool after_raster,
                        cudaStream_t stream) {
    cudaError_t e = configure_redo<S>();
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    forward_redo_kernel<S><<<sms > 0 ? sms : 1, kFwdThreads, forward_smem_bytes<S, false>(), stream>>>(a, fa, g,
                                                                                                     after_raster);
    return cudaSuccess;
}

cudaError_t launch_group_redo(const PassArgs& a, const FragArgs& fa, const GroupArgs& g, int S, bool after_raster,
                              cudaStream_t stream) {
    switch (S) {
    case 1: return launch_redo<1>(a, fa, g, after_raster, stream);
    case 2: return launch_redo<2>(a, fa, g, after_raster, stream);
    case 4: return launch_redo<4>(a, fa, g, after_raster, stream);
    case 8: return launch_redo<8>(a, fa, g, after_raster, stream);
    case 16: return launch_redo<16>(a, fa, g, after_raster, stream);
    default: return cudaErrorInvalidValue;
    }
}

template <int S>
cudaError_t configure_blend() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(frag_blend_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)blend_smem_bytes<S>());
    if (e == cudaSuccess) done = true;
    return e;
}

template <int S>
cudaError_t launch_frag_kernels(const PassArgs& a, const FragArgs& fa, int ctas_shade, int ctas_blend,
                                cudaStream_t stream) {
    cudaError_t e = configure_blend<S>();
    if (e != cudaSuccess) return e;
    frag_shade_kernel<<<ctas_shade, kFragShadeThreads, 0, stream>>>(a, fa);
    frag_blend_kernel<S><<<ctas_blend, kFwdThreads, blend_smem_bytes<S>(), stream>>>(a, fa);
    return cudaSuccess;
}

cudaError_t launch_group_frags(const PassArgs& a, const FragArgs& fa, int S, int ctas_shade, int ctas_blend,
                               cudaStream_t stream) {
    switch (S) {
    case 1: return launch_frag_kernels<1>(a, fa, ctas_shade, ctas_blend, stream);
    case 2: return launch_frag_kernels<2>(a, fa, ctas_shade, ctas_blend, stream);
    case 4: return launch_frag_kernels<4>(a, fa, ctas_shade, ctas_blend, stream);
    case 8: return launch_frag_kernels<8>(a, fa, ctas_shade, ctas_blend, stream);
    case 16: return launch_frag_kernels<16>(a, fa, ctas_shade, ctas_blend, stream);
    default: return cudaErrorInvalidValue;
    }
}

// One tile stage (raster or shade) of a deferred group.
cudaError_t launch_group_stage(const PassArgs& a, const GroupArgs& g, int S, int TS, int ctas, cudaStream_t stream,
                               bool shade) {
    if (TS == 8) {
        switch (S) {
        case 1: return launch_deferred<1, 8>(a, g, ctas, stream, shade);
        case 4: return launch_deferred<4, 8>(a, g, ctas, stream, shade);
        default: break;
        }
    }
    switch (S) {
    case 1: return launch_deferred<1, 16>(a, g, ctas, stream, shade);
    case 2: return launch_deferred<2, 16>(a, g, ctas, stream, shade);
    case 4: return launch_deferred<4, 16>(a, g, ctas, stream, shade);
    case 8: return launch_deferred<8, 16>(a, g, ctas, stream, shade);
    case 16: return launch_deferred<16, 16>(a, g, ctas, stream, shade);
    default: return cudaErrorInvalidValue;
    }
}

// The ordered stage of a group; `second` when it follows the group's raster stage (its queue
// counter is then the group's second one).
cudaError_t launch_group_forward(const PassArgs& a, const FragArgs& fa, const GroupArgs& g, int S, int ctas,
                                 cudaStream_t stream, bool second) {
    const int q = 3 * g.queue + (second ? 2 : 0);
    switch (S) {
    case 1: return launch_forward<1>(a, fa, g, ctas, stream, q);
    case 2: return launch_forward<2>(a, fa, g, ctas, stream, q);
    case 4: return launch_forward<4>(a, fa, g, ctas, stream, q);
    case 8: return launch_forward<8>(a, fa, g, ctas, stream, q);
    case 16: return launch_forward<16>(a, fa, g, ctas, stream, q);
    default: return cudaErrorInvalidValue;
    }
}

template <class K>
int occupancy_of(K kernel, int threads, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

template <int S, int TS>
int deferred_occupancy(int stage) {
    configure_deferred<S, TS>();
    return stage == 0 ? occupancy_of(raster_kernel<S, TS>, TS * TS, raster_smem_bytes<S, TS>())
                      : occupancy_of(shade_kernel<S, TS>, kShadeThreads, 0);
}

template <int S, bool DEFER = false>
int forward_occupancy() {
    configure_forward<S, DEFER>();
    return occupancy_of(forward_kernel<S, DEFER>, kFwdThreads, forward_smem_bytes<S, DEFER>());
}

static int frag_kernel_occupancy_query(int S, int stage) {
    if (stage == 0) return occupancy_of(frag_shade_kernel, kFragShadeThreads, 0);
    if (stage == 2) {
        switch (S) {
        case 1: return forward_occupancy<1, true>();
        case 2: return forward_occupancy<2, true>();
        case 4: return forward_occupancy<4, true>();
        case 8: return forward_occupancy<8, true>();
        default: return forward_occupancy<16, true>();
        }
    }
    switch (S) {
    case 1: return configure_blend<1>(), occupancy_of(frag_blend_kernel<1>, kFwdThreads, blend_smem_bytes<1>());
    case 2: return configure_blend<2>(), occupancy_of(frag_blend_kernel<2>, kFwdThreads, blend_smem_bytes<2>());
    case 4: return configure_blend<4>(), occupancy_of(frag_blend_kernel<4>, kFwdThreads, blend_smem_bytes<4>());
    case 8: return configure_blend<8>(), occupancy_of(frag_blend_kernel<8>, kFwdThreads, blend_smem_bytes<8>());
    default: return configure_blend<16>(), occupancy_of(frag_blend_kernel<16>, kFwdThreads, blend_smem_bytes<16>());
    }
}

static int tile_kernel_occupancy_query(int S, int TS, int ordered, int stage) {
    if (ordered) {
        switch (S) {
        case 1: return forward_occupancy<1>();
        case 2: return forward_occupancy<2>();
        case 4: return forward_occupancy<4>();
        case 8: return forward_occupancy<8>();
        default: return forward_occupancy<16>();
        }
    }
    if (TS == 8 && S == 1) return deferred_occupancy<1, 8>(stage);
    if (TS == 8 && S == 4) return deferred_occupancy<4, 8>(stage);
    switch (S) {
    case 1: return deferred_occupancy<1, 16>(stage);
    case 2: return deferred_occupancy<2, 16>(stage);
    case 4: return deferred_occupancy<4, 16>(stage);
    case 8: return deferred_occupancy<8, 16>(stage);
    default: return deferred_occupancy<16, 16>(stage);
    }
}

template <int S>
void launch_atomic_front(const PassArgs& a, int npix, cudaStream_t stream, cudaEvent_t* ev) {
    init_keys_kernel<S><<<(npix + 255) / 256, 256, 0, stream>>>(a, npix);
    if (ev) {
        cudaEventRecord(ev[1], stream);
        cudaEventRecord(ev[2], stream);
    }
    if (a.total_tris > 0) atomic_front_kernel<S><<<(a.total_tris + 255) / 256, 256, 0, stream>>>(a);
    if (ev) {
        cudaEventRecord(ev[3], stream);
        cudaEventRecord(ev[4], stream);
    }
}

// Occupancy answers do not change for a kernel: asked once per (samples, tile size, form, stage).
static int sample_slot(int S) { return S == 1 ? 0 : S == 2 ? 1 : S == 4 ? 2 : S == 8 ? 3 : 4; }

int tile_kernel_occupancy(int S, int TS, int ordered, int stage) {
    static std::atomic<int> cache[5][2][2][2];  // 0: not asked yet (zero-initialised static storage)
    std::atomic<int>& c = cache[sample_slot(S)][TS == 8][ordered != 0][stage != 0];
    int n = c.load(std::memory_order_relaxed);
    if (n == 0) c.store(n = tile_kernel_occupancy_query(S, TS, ordered, stage), std::memory_order_relaxed);
    return n;
}

int frag_kernel_occupancy(int S, int stage) {
    static std::atomic<int> cache[5][3];
    std::atomic<int>& c = cache[sample_slot(S)][stage < 0 ? 0 : stage > 2 ? 2 : stage];
    int n = c.load(std::memory_order_relaxed);
    if (n == 0) c.store(n = frag_kernel_occupancy_query(S, stage), std::memory_order_relaxed);
    return n;
}

cudaError_t launch_pass(const PassArgs& a, const LaunchPlan& plan, cudaStream_t stream, cudaEvent_t* ev,
                        const FragArgs* fa_in, const SideStream* side) {
    const int T = a.total_tiles;
    FragArgs fa, nofa;
    std::memset(&fa, 0, sizeof(fa));
    std::memset(&nofa, 0, sizeof(nofa));
    if (fa_in && plan.defer_group >= 0) fa = *fa_in;
    if (ev) cudaEventRecord(ev[0], stream);
    cudaError_t err = cudaMemsetAsync(a.queues, 0, sizeof(uint32_t) * 3 * plan.ngroups, stream);
    if (err != cudaSuccess) return err;
    if (plan.atomic) {  // one deferred view: keys by atomics, then the shade stage
        switch (plan.samples[0]) {
        case 1: launch_atomic_front<1>(a, plan.atomic_pixels, stream, ev); break;
        case 2: launch_atomic_front<2>(a, plan.atomic_pixels, stream, ev); break;
        case 4: launch_atomic_front<4>(a, plan.atomic_pixels, stream, ev); break;
        case 8: launch_atomic_front<8>(a, plan.atomic_pixels, stream, ev); break;
        default: launch_atomic_front<16>(a, plan.atomic_pixels, stream, ev); break;
        }
        err = launch_group_stage(a, plan.groups[0], plan.samples[0], plan.tile_size[0], plan.ctas_shade[0], stream, true);
        if (ev) {
            cudaEventRecord(ev[5], stream);
            cudaEventRecord(ev[6], stream);
        }
        return err != cudaSuccess ? err : cudaGetLastError();
    }
    if (a.total_tris > 0) {
        int blocks = (a.total_tris + 255) / 256;
        bin_count_kernel<<<blocks, 256, 0, stream>>>(a);
        if (ev) cudaEventRecord(ev[1], stream);
        if (T <= kScanSingle) {
            scan_single_kernel<<<1, kScanThreads, 0, stream>>>(a, T);
        } else {
            const int nb = (T + kScanTile - 1) / kScanTile;
            scan_local_kernel<<<nb, kScanThreads, 0, stream>>>(a, T);
            scan_blocks_kernel<<<1, kScanThreads, 0, stream>>>(a, T, nb);
            scan_apply_kernel<<<nb, kScanThreads, 0, stream>>>(a, T);
        }
        if (ev) cudaEventRecord(ev[2], stream);
        bin_scatter_kernel<<<blocks, 256, 0, stream>>>(a);
        if (ev) cudaEventRecord(ev[3], stream);
    } else if (ev) {
        cudaEventRecord(ev[1], stream);
        cudaEventRecord(ev[2], stream);
        cudaEventRecord(ev[3], stream);
    }
    // first stages of all groups (raster; ordered for ordered groups without a prefix), then the
    // second stages (shade; ordered on top of the prefix for hybrid groups)
    for (int i = 0; i < plan.ngroups && err == cudaSuccess; i++) {
        if (plan.ordered[i] && !plan.hybrid[i])
            err = launch_group_forward(a, i == plan.defer_group ? fa : nofa, plan.groups[i], plan.samples[i],
                                       i == plan.defer_group && fa.frags ? plan.ctas_fwd_defer : plan.ctas[i], stream, false);
        else
            err = launch_group_stage(a, plan.groups[i], plan.samples[i], plan.tile_size[i], plan.ctas[i], stream, false);
    }
    if (ev) cudaEventRecord(ev[4], stream);
    for (int i = 0; i < plan.ngroups && err == cudaSuccess; i++)
        if (!plan.ordered[i] || plan.hybrid[i])
            err = launch_group_stage(a, plan.groups[i], plan.samples[i], plan.tile_size[i], plan.ctas_shade[i], stream, true);
    if (ev) cudaEventRecord(ev[5], stream);
    for (int i = 0; i < plan.ngroups && err == cudaSuccess; i++)
        if (plan.hybrid[i])
            err = launch_group_forward(a, i == plan.defer_group ? fa : nofa, plan.groups[i], plan.samples[i],
                                       i == plan.defer_group && fa.frags ? plan.ctas_fwd_defer : plan.ctas_fwd[i], stream,
                                       true);
    if (err == cudaSuccess && fa.frags) {
        // the redo list's tiles and the deferred fragments' tiles are disjoint: with a side stream
        // the in-stage form runs beside the fragment kernels (which take their work from a counter,
        // so the SM share it holds costs them nothing but that share)
        const int dg = plan.defer_group;
        cudaStream_t rs = stream;
        if (side) {
            err = cudaEventRecord(side->fork, stream);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(side->stream, side->fork, 0);
            rs = side->stream;
        }
        if (err == cudaSuccess) err = launch_group_redo(a, fa, plan.groups[dg], plan.samples[dg], plan.hybrid[dg] != 0, rs);
        if (err == cudaSuccess)
            err = launch_group_frags(a, fa, plan.samples[dg], plan.ctas_frag_shade, plan.ctas_frag_blend, stream);
        if (side) {  // joined even after an error, so that the side stream holds no work of this pass
            const cudaError_t j = cudaEventRecord(side->join, side->stream);
            const cudaError_t w = j == cudaSuccess ? cudaStreamWaitEvent(stream, side->join, 0) : j;
            if (err == cudaSuccess) err = w;
        }
    }
    if (ev) cudaEventRecord(ev[6], stream);
    return err != cudaSuccess ? err : cudaGetLastError();
}

}  // namespace ifr
