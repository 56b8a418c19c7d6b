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

template <bool kScatter>
__global__ void __launch_bounds__(256) bin_kernel(PassArgs a) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.total_tris) return;
    if (kScatter && a.status[ST_OVERFLOW]) return;
    int di = find_draw(a, g);
    const DrawDev& d = a.draws[di];
    int t = g - __ldg(a.draw_start + di);
    CVert poly[kMaxPoly];
    bool inside, rejected;
    if (!fetch_triangle(a.c, d, t, poly, inside, rejected)) return;
    int n = inside ? 3 : clip_polygon(a.c, poly);
    for (int i = 1; i + 1 < n; i++) {
        SubTri s;
        if (!setup_sub(a.c, d, poly[0], poly[i], poly[i + 1], s)) continue;
        int tx0 = s.px0 >> kTileShift, tx1 = s.px1 >> kTileShift;
        int ty0 = s.py0 >> kTileShift, ty1 = s.py1 >> kTileShift;
        uint32_t entry = ((uint32_t)g << 3) | (uint32_t)(i - 1);
        for (int ty = ty0; ty <= ty1; ty++)
            for (int tx = tx0; tx <= tx1; tx++) {
                int tile = ty * a.c.tiles_x + tx;
                if (kScatter) {
                    uint32_t pos = atomicAdd(a.tile_cursor + tile, 1u);
                    if (pos < a.pair_capacity) a.pairs[pos] = entry;
                } else {
                    atomicAdd(a.tile_count + tile, 1u);
                }
            }
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

// Order-independent depth test with API-order tie break (see file comment).
__device__ __forceinline__ bool depth_key_pass(int func, int write, float z, float dd, int prim, int cur) {
    if (!write) return depth_cmp(func, z, dd) && prim > cur;
    switch (func) {
    case 1: return z < dd || (z == dd && prim < cur);
    case 2: return z == dd && prim > cur;
    case 3: return z < dd || (z == dd && prim > cur);
    case 4: return z > dd || (z == dd && prim < cur);
    case 6: return z > dd || (z == dd && prim > cur);
    case 7: return prim > cur;
    default: return false;
    }
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

struct TileRecords {
    int32_t A[3][kTileThreads], B[3][kTileThreads];
    long long Cb[3][kTileThreads];
    float z0[kTileThreads], dzdx[kTileThreads], dzdy[kTileThreads];
    int32_t X0[kTileThreads], Y0[kTileThreads];
    int32_t bx[kTileThreads], by[kTileThreads];  // packed px0 | px1 << 16, py0 | py1 << 16
    int32_t key[kTileThreads];                   // global triangle << 3 | fan index
};

template <int S>
__global__ void __launch_bounds__(kTileThreads, 2) tile_kernel(PassArgs a) {
    __shared__ TileRecords rec;
    const int tile = blockIdx.x;
    const int tx = tile % a.c.tiles_x, ty = tile / a.c.tiles_x;
    const int tid = threadIdx.x;
    // 2x2 quads on consecutive lanes; a warp covers a 16x2 pixel strip
    const int lx = ((tid >> 2) & 7) * 2 + (tid & 1);
    const int ly = (tid >> 5) * 2 + ((tid >> 1) & 1);
    const int px = tx * kTileSize + lx, py = ty * kTileSize + ly;
    const bool inpix = px < a.c.W && py < a.c.H;
    const size_t pix = (size_t)py * a.c.W + px;

    float dep[S];
    int id[S];
#pragma unroll
    for (int k = 0; k < S; k++) {
        dep[k] = a.clear ? a.clear_depth : (inpix ? a.depth[pix * S + k] : 0.0f);
        id[k] = -1;
    }
    const bool has_list = a.total_tris > 0 && a.status[ST_OVERFLOW] == 0;
    const uint32_t beg = has_list ? a.tile_offset[tile] : 0u;
    const uint32_t end = has_list ? a.tile_offset[tile + 1] : 0u;
    int sxk[S], syk[S];
#pragma unroll
    for (int k = 0; k < S; k++) {
        sxk[k] = px * 256 + a.c.sx[k];
        syk[k] = py * 256 + a.c.sy[k];
    }

    for (uint32_t base = beg; base < end; base += kTileThreads) {
        const int nb = (int)min((uint32_t)kTileThreads, end - base);
        if (tid < nb) {
            uint32_t e = __ldg(a.pairs + base + tid);
            int g = (int)(e >> 3), sub = (int)(e & 7u);
            int di = find_draw(a, g);
            SubTri s;
            bool ok = setup_triangle_sub(a.c, a.draws[di], g - __ldg(a.draw_start + di), sub, s);
            if (ok) {
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
                rec.bx[tid] = 1;  // empty range: px0 = 1 > px1 = 0
                rec.by[tid] = 1;
            }
            rec.key[tid] = (int)e;
        }
        __syncthreads();
        if (inpix) {
            for (int r = 0; r < nb; r++) {
                int bx = rec.bx[r], by = rec.by[r];
                if (px < (bx & 0xffff) || px > (bx >> 16) || py < (by & 0xffff) || py > (by >> 16)) continue;
                int32_t A[3] = {rec.A[0][r], rec.A[1][r], rec.A[2][r]};
                int32_t B[3] = {rec.B[0][r], rec.B[1][r], rec.B[2][r]};
                int64_t Cb[3] = {rec.Cb[0][r], rec.Cb[1][r], rec.Cb[2][r]};
                float z0 = rec.z0[r], gx = rec.dzdx[r], gy = rec.dzdy[r];
                int32_t X0 = rec.X0[r], Y0 = rec.Y0[r];
                int key = rec.key[r];
                int prim = key >> 3;
#pragma unroll
                for (int k = 0; k < S; k++) {
                    if (!covered(A, B, Cb, sxk[k], syk[k])) continue;
                    float z = sample_depth(z0, gx, gy, X0, Y0, sxk[k], syk[k]);
                    int cur = id[k] < 0 ? -1 : (id[k] >> 3);
                    if (depth_key_pass(a.depth_func, a.depth_write, z, dep[k], prim, cur)) {
                        if (a.depth_write) dep[k] = z;
                        id[k] = key;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!inpix) return;

    // ---- deferred shading of the visible primitives + resolve
    float bg[4];
    if (a.clear) {
        bg[0] = a.clear_color[0]; bg[1] = a.clear_color[1]; bg[2] = a.clear_color[2]; bg[3] = a.clear_color[3];
    } else {
        decode_color(a, pix, bg);
    }
    int ckey[2] = {-1, -1};
    float ccol[2][4];
    float acc[4];
#pragma unroll
    for (int k = 0; k < S; k++) {
        float c[4];
        if (id[k] < 0) {
            c[0] = bg[0]; c[1] = bg[1]; c[2] = bg[2]; c[3] = bg[3];
        } else if (id[k] == ckey[0]) {
            c[0] = ccol[0][0]; c[1] = ccol[0][1]; c[2] = ccol[0][2]; c[3] = ccol[0][3];
        } else if (id[k] == ckey[1]) {
            c[0] = ccol[1][0]; c[1] = ccol[1][1]; c[2] = ccol[1][2]; c[3] = ccol[1][3];
        } else {
            int g = id[k] >> 3, sub = id[k] & 7;
            int di = find_draw(a, g);
            const DrawDev& d = a.draws[di];
            int t = g - __ldg(a.draw_start + di);
            SubTri s;
            setup_triangle_sub(a.c, d, t, sub, s);
            shade_fragment(a.c, d, s, t, sub, px, py, c);
            // keep the two most recent distinct primitives
            ckey[1] = ckey[0];
            ccol[1][0] = ccol[0][0]; ccol[1][1] = ccol[0][1]; ccol[1][2] = ccol[0][2]; ccol[1][3] = ccol[0][3];
            ckey[0] = id[k];
            ccol[0][0] = c[0]; ccol[0][1] = c[1]; ccol[0][2] = c[2]; ccol[0][3] = c[3];
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
        for (int k = 0; k < S; k++) vp[k] = id[k] < 0 ? -1 : (id[k] >> 3);
    }
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

cudaError_t launch_pass(const PassArgs& a, cudaStream_t stream, cudaEvent_t* ev) {
    const int T = a.c.tiles_x * a.c.tiles_y;
    if (ev) cudaEventRecord(ev[0], stream);
    if (a.total_tris > 0) {
        int blocks = (a.total_tris + 255) / 256;
        bin_kernel<false><<<blocks, 256, 0, stream>>>(a);
        if (ev) cudaEventRecord(ev[1], stream);
        scan_kernel<<<1, 1024, 0, stream>>>(a, T);
        if (ev) cudaEventRecord(ev[2], stream);
        bin_kernel<true><<<blocks, 256, 0, stream>>>(a);
        if (ev) cudaEventRecord(ev[3], stream);
    } else if (ev) {
        cudaEventRecord(ev[1], stream);
        cudaEventRecord(ev[2], stream);
        cudaEventRecord(ev[3], stream);
    }
    cudaError_t err = cudaSuccess;
    switch (a.c.S) {
    case 1: tile_kernel<1><<<T, kTileThreads, 0, stream>>>(a); break;
    case 2: tile_kernel<2><<<T, kTileThreads, 0, stream>>>(a); break;
    case 4: tile_kernel<4><<<T, kTileThreads, 0, stream>>>(a); break;
    case 8: tile_kernel<8><<<T, kTileThreads, 0, stream>>>(a); break;
    case 16: tile_kernel<16><<<T, kTileThreads, 0, stream>>>(a); break;
    default: err = cudaErrorInvalidValue;
    }
    if (ev) cudaEventRecord(ev[4], stream);
    return err != cudaSuccess ? err : cudaGetLastError();
}

}  // namespace ifr
