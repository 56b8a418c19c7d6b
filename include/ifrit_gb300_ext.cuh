/*
 * ifrit_gb300_ext.cuh -- device-side extension point of the GB300 rasterizer (header-only CUDA).
 *
 * The reference binds user shaders as C function pointers or C++ objects with virtual execute()
 * methods (include/ifrit/softgraphics/engine/base/Shaders.h:46-120) and calls them per vertex /
 * fragment / work group; its CUDA renderer copies the objects to the device and fixes up their
 * vtables (core/cuda/CudaUtils.cuh:26-38).  A host function or a host object cannot run on the
 * GPU here, so iftrBind*ShaderFunc / iftrBind*Shader return IFTR_ERR_UNSUPPORTED.  This header is
 * the replacement: the caller writes its shader as a functor in its own CUDA translation unit
 * (compiled with nvcc for sm_103a, --fmad=false to keep the library's float evaluation order),
 * and the templates below compile it into kernels that use the library's own rasterization
 * arithmetic.  No virtual call, no function pointer, no relocatable device code.
 *
 * Fragment shading (the reference's FragmentShader::execute, Shaders.h:58-78):
 *   struct MyShader { __device__ void operator()(const ifrit_ext::Fragment& f, float out[4]) const; };
 *   ifrit_ext::shade_visibility(pass, MyShader{...}, stream);
 * runs after a draw that wrote its visibility buffer (iftrSetVisibilityOutput, then
 * iftrGetDeviceAttachments): for every pixel and every distinct triangle visible in its samples,
 * the triangle is set up again (clipping and 16.8 snapping as the draw did), its attribute is
 * interpolated perspective-correctly at the pixel centre with the 2x2-quad derivatives (exactly
 * the built-in shading's values), the functor is called once, and the samples' colours are
 * averaged into the caller's output as the built-in resolve does.  ifrit_ext::Gouraud is the
 * built-in GOURAUD model as a functor (bit-identical to the renderer's own output).
 *
 * Vertex stage (the reference's VertexShader::execute, Shaders.h:46-56):
 *   struct MyVertex { __device__ void operator()(int i, float clip[4], float attr[4]) const; };
 *   ifrit_ext::draw_vertex_stage(renderer, MyVertex{...}, num_vertices, d_indices, num_indices,
 *                                d_positions, d_attributes, d_counts, attr_count, clear, stream);
 * runs the functor once per vertex (clip-space position and one float4 varying out) and draws the
 * caller's triangle list over its outputs (iftrDrawMeshOutputs with one work group).
 *
 * Mesh / task / geometry stage (the reference's MeshShader / TaskShader / GeometryShader
 * objects, MeshShadingStage / GeneralGeometryStage, TileRasterCoreInvocationCuda.cu:355-561):
 *   struct MyMesh {
 *     __device__ void counts(int group, int& num_vertices, int& num_indices) const;
 *     __device__ void vertex(int group, int i, float clip[4], float attr[4]) const;
 *     __device__ int  index(int group, int j) const;   // group-local vertex index
 *   };
 *   ifrit_ext::draw_mesh_stage(renderer, MyMesh{...}, groups, max_v, max_i, slots, attr_count, clear);
 * launches the functor as the stage kernel (one CTA per work group) on the renderer's stream into
 * the caller's slot arrays and draws them through iftrDrawMeshOutputs (group-order compaction,
 * the current state, clip-space input).
 *
 * Task stage (the reference's TaskShader, taskShadingKernel + prefix scan +
 * taskShadingLaunchSubGroupsKernel):
 *   struct MyTask { __device__ int mesh_groups(int task) const; };
 *   struct MyMesh { counts(task, sub, nv, ni); vertex(task, sub, i, clip, attr); index(task, sub, j); };
 *   ifrit_ext::draw_task_mesh_stage(renderer, MyTask{...}, MyMesh{...}, tasks, max_groups, max_v, max_i,
 *                                   slots, d_offsets, attr_count, clear, stream);
 * runs the task functor once per task group, scans the mesh-group counts, runs the mesh functor
 * once per spawned group (task, sub) and draws the groups in (task, sub) order.
 *
 * Compile with -I<repository>/include; this header includes the library's device arithmetic from
 * ifrit-v2_gb300/csrc (relative to this file).
 */
#ifndef IFRIT_GB300_EXT_CUH
#define IFRIT_GB300_EXT_CUH
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <climits>

#include "../ifrit-v2_gb300/csrc/pass_plan.h"
#include "../ifrit-v2_gb300/csrc/raster_math.cuh"
#include "ifrit_gb300.h"

namespace ifrit_ext {

// What a fragment functor sees: the pixel, the triangle (index within the draw), its attribute at
// the pixel centre and the attribute's quad derivatives (right column minus left column in the
// same row, bottom row minus top row in the same column, evaluated for this triangle).
struct Fragment {
    int x, y;
    int triangle;
    int attr_count;
    float attr[4];
    float ddx[4], ddy[4];
};

// A shading pass over a visibility buffer; device pointers and sizes only.  The geometry, MVP and
// cull state must be the ones of the draw that wrote the visibility buffer.
struct ShadePass {
    const float* vertices;    // AoS floats, `stride` per vertex, position = floats 0..2
    int stride, num_vertices, attr_offset, attr_count;
    const int* indices;       // 3 per triangle
    int num_triangles;
    float mvp[16];            // row-major
    int cull_mode, front_ccw;  // IF_CULL_MODE_*, 1 = counter-clockwise front faces
    int clip_input;           // 1: positions are clip-space x, y, z, w (a mesh stage's output; no MVP)
    int width, height, samples;
    const int* visibility;    // [H][W][S] triangle index, -1 = none
    int format;               // IFTR_FORMAT_RGBA8 / RGBA16F / RGBA32F / RGB32F
    void* color;              // resolved output
    float background[4];      // colour of samples no triangle covers
};

// The built-in GOURAUD model: the attribute itself (alpha 1 with fewer than four components).
struct Gouraud {
    __device__ void operator()(const Fragment& f, float out[4]) const {
        out[0] = f.attr[0];
        out[1] = f.attr[1];
        out[2] = f.attr[2];
        out[3] = f.attr_count >= 4 ? f.attr[3] : 1.0f;
    }
};

namespace detail {

__device__ __forceinline__ void encode(const ShadePass& p, size_t pix, const float c[4]) {
    switch (p.format) {
    case IFTR_FORMAT_RGBA8: {
        uint32_t q = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) q |= __float2uint_rn(fminf(fmaxf(c[i], 0.0f), 1.0f) * 255.0f) << (8 * i);
        static_cast<uint32_t*>(p.color)[pix] = q;
        break;
    }
    case IFTR_FORMAT_RGBA16F: {
        __half h[4];
#pragma unroll
        for (int i = 0; i < 4; i++) h[i] = __float2half_rn(c[i]);
        uint64_t q = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) q |= (uint64_t)__half_as_ushort(h[i]) << (16 * i);
        static_cast<uint64_t*>(p.color)[pix] = q;
        break;
    }
    case IFTR_FORMAT_RGBA32F:
        static_cast<float4*>(p.color)[pix] = make_float4(c[0], c[1], c[2], c[3]);
        break;
    default: {
        float* o = static_cast<float*>(p.color) + pix * 3;
        o[0] = c[0];
        o[1] = c[1];
        o[2] = c[2];
        break;
    }
    }
}

// Sets up the fan sub-triangle of triangle t whose edge functions cover sample (sx, sy); the
// draw's raster stage covered the sample with exactly that one (top-left rule on shared edges).
__device__ __forceinline__ bool setup_covering(const ifr::PassConst& c, const ifr::DrawDev& d, int t, int32_t sx,
                                               int32_t sy, ifr::SubTri& s) {
    for (int sub = 0; sub < ifr::kMaxPoly - 2; sub++)
        if (ifr::setup_triangle_sub(c, d, t, sub, s) && ifr::covered(s.A, s.B, s.Cb, sx, sy)) return true;
    return false;
}

// One thread per pixel.  The pixel's samples are grouped by the (triangle, fan sub-triangle)
// that covers them, in sample order, as the built-in shade stage groups its entries; each group
// calls the functor once with the attribute at the pixel centre, and the resolve adds the
// samples' colours in sample order and scales by 1/S.
template <int S, class Shader>
__global__ void __launch_bounds__(256) shade_visibility_kernel(ShadePass p, ifr::DrawDev d, ifr::PassConst c,
                                                               Shader shader) {
    const size_t npix = (size_t)p.width * p.height;
    for (size_t pix = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pix < npix; pix += (size_t)gridDim.x * blockDim.x) {
        const int px = (int)(pix % p.width), py = (int)(pix / p.width);
        int tri[S];
#pragma unroll
        for (int k = 0; k < S; k++) tri[k] = p.visibility[pix * S + k];
        float col[S][4];
        bool done[S];
#pragma unroll
        for (int k = 0; k < S; k++) done[k] = false;
        for (int k = 0; k < S; k++) {
            if (done[k]) continue;
            float c4[4] = {p.background[0], p.background[1], p.background[2], p.background[3]};
            const int t = tri[k];
            ifr::SubTri s;
            const bool ok = t >= 0 && t < d.num_triangles &&
                            setup_covering(c, d, t, px * 256 + ifr::sample_x<S>(k), py * 256 + ifr::sample_y<S>(k), s);
            if (ok) {
                ifr::ShadeGeom g;
                ifr::shade_geom_from(s, g);
                float a0[4], a1[4], a2[4];
                ifr::fetch_attrs(d, t, a0, a1, a2);
                Fragment f;
                f.x = px;
                f.y = py;
                f.triangle = t;
                f.attr_count = d.attr_count;
                const int32_t qx = px * 256 + ifr::kShadeOffset, qy = py * 256 + ifr::kShadeOffset;
                float ah[4], av[4];  // horizontal and vertical quad partners
                ifr::interp_attr(g, d.attr_count, a0, a1, a2, qx, qy, f.attr);
                ifr::interp_attr(g, d.attr_count, a0, a1, a2, (px ^ 1) * 256 + ifr::kShadeOffset, qy, ah);
                ifr::interp_attr(g, d.attr_count, a0, a1, a2, qx, (py ^ 1) * 256 + ifr::kShadeOffset, av);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    f.ddx[i] = (px & 1) ? f.attr[i] - ah[i] : ah[i] - f.attr[i];
                    f.ddy[i] = (py & 1) ? f.attr[i] - av[i] : av[i] - f.attr[i];
                }
                shader(f, c4);
            }
            for (int q = k; q < S; q++) {
                if (done[q] || tri[q] != t) continue;
                if (ok && q != k &&
                    !ifr::covered(s.A, s.B, s.Cb, px * 256 + ifr::sample_x<S>(q), py * 256 + ifr::sample_y<S>(q)))
                    continue;  // another fan sub-triangle of the same triangle
#pragma unroll
                for (int i = 0; i < 4; i++) col[q][i] = c4[i];
                done[q] = true;
            }
        }
        float acc[4];
#pragma unroll
        for (int i = 0; i < 4; i++) acc[i] = col[0][i];
#pragma unroll
        for (int k = 1; k < S; k++)
#pragma unroll
            for (int i = 0; i < 4; i++) acc[i] = acc[i] + col[k][i];
        const float invS = 1.0f / (float)S;
#pragma unroll
        for (int i = 0; i < 4; i++) acc[i] = acc[i] * invS;
        encode(p, pix, acc);
    }
}

template <class Mesh>
__global__ void mesh_stage_kernel(Mesh mesh, int max_v, int max_i, float* positions, float* attributes, int* indices,
                                  int* num_vertices, int* num_indices) {
    const int g = blockIdx.x;
    __shared__ int s_nv, s_ni;
    if (threadIdx.x == 0) {
        int nv = 0, ni = 0;
        mesh.counts(g, nv, ni);
        s_nv = nv;
        s_ni = ni;
        num_vertices[g] = nv;  // the draw rejects counts above the slots' maxima
        num_indices[g] = ni;
    }
    __syncthreads();
    const int nv = min(s_nv, max_v), ni = min(s_ni, max_i);
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        float clip[4], attr[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        mesh.vertex(g, i, clip, attr);
        float* pp = positions + ((size_t)g * max_v + i) * 4;
        pp[0] = clip[0]; pp[1] = clip[1]; pp[2] = clip[2]; pp[3] = clip[3];
        if (attributes) {
            float* ap = attributes + ((size_t)g * max_v + i) * 4;
            ap[0] = attr[0]; ap[1] = attr[1]; ap[2] = attr[2]; ap[3] = attr[3];
        }
    }
    for (int j = threadIdx.x; j < ni; j += blockDim.x) indices[(size_t)g * max_i + j] = mesh.index(g, j);
}

// One thread per task group: the number of mesh groups it spawns (negative counts as zero).
template <class Task>
__global__ void task_count_kernel(Task task, int tasks, int* offsets) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < tasks) offsets[t] = max(task.mesh_groups(t), 0);
}

// Exclusive scan of the counts in place (one CTA); offsets[tasks] receives the total, saturated at
// INT_MAX.
__global__ void __launch_bounds__(1024) task_scan_kernel(int* offsets, int tasks) {
    __shared__ long long s_warp[32];
    __shared__ long long s_carry;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < tasks; base += 1024) {
        const int i = base + threadIdx.x;
        const long long x = i < tasks ? offsets[i] : 0;
        long long incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long q = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += q;
        }
        if (lane == 31) s_warp[wid] = incl;
        __syncthreads();
        long long before = s_carry;
        for (int w = 0; w < wid; w++) before += s_warp[w];
        const long long ex = before + incl - x;
        if (i < tasks) offsets[i] = (int)min(ex, (long long)INT_MAX);
        __syncthreads();
        if (threadIdx.x == 1023) s_carry = before + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[tasks] = (int)min(s_carry, (long long)INT_MAX);
}

// One CTA per mesh slot: slot g runs the mesh functor for (task, sub) with offsets[task] <= g <
// offsets[task + 1]; slots past the total emit nothing.
template <class Mesh>
__global__ void task_mesh_kernel(Mesh mesh, const int* offsets, int tasks, int max_v, int max_i, float* positions,
                                 float* attributes, int* indices, int* num_vertices, int* num_indices) {
    const int g = blockIdx.x;
    __shared__ int s_nv, s_ni, s_task;
    if (threadIdx.x == 0) {
        int nv = 0, ni = 0, t = -1;
        if (g < offsets[tasks]) {
            int lo = 0, hi = tasks - 1;  // the last task whose first group is at or before g
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (offsets[mid] <= g) lo = mid; else hi = mid - 1;
            }
            t = lo;
            mesh.counts(t, g - offsets[t], nv, ni);
        }
        s_nv = nv;
        s_ni = ni;
        s_task = t;
        num_vertices[g] = nv;
        num_indices[g] = ni;
    }
    __syncthreads();
    if (s_task < 0) return;
    const int t = s_task, sub = g - offsets[t];
    const int nv = min(s_nv, max_v), ni = min(s_ni, max_i);
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        float clip[4], attr[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        mesh.vertex(t, sub, i, clip, attr);
        float* pp = positions + ((size_t)g * max_v + i) * 4;
        pp[0] = clip[0]; pp[1] = clip[1]; pp[2] = clip[2]; pp[3] = clip[3];
        if (attributes) {
            float* ap = attributes + ((size_t)g * max_v + i) * 4;
            ap[0] = attr[0]; ap[1] = attr[1]; ap[2] = attr[2]; ap[3] = attr[3];
        }
    }
    for (int j = threadIdx.x; j < ni; j += blockDim.x) indices[(size_t)g * max_i + j] = mesh.index(t, sub, j);
}

// One thread per vertex: the vertex functor's outputs; thread 0 also writes the group's counts.
template <class Vertex>
__global__ void vertex_stage_kernel(Vertex vs, int num_vertices, int num_indices, float* positions, float* attributes,
                                    int* counts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        counts[0] = num_vertices;
        counts[1] = num_indices;
    }
    if (i >= num_vertices) return;
    float clip[4], attr[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    vs(i, clip, attr);
    float* pp = positions + (size_t)i * 4;
    pp[0] = clip[0]; pp[1] = clip[1]; pp[2] = clip[2]; pp[3] = clip[3];
    if (attributes) {
        float* ap = attributes + (size_t)i * 4;
        ap[0] = attr[0]; ap[1] = attr[1]; ap[2] = attr[2]; ap[3] = attr[3];
    }
}

}  // namespace detail

// Shades every pixel of a visibility buffer with `shader` into p.color (see the file comment).
// Samples 1, 2, 4, 8 or 16; returns cudaErrorInvalidValue otherwise.
template <class Shader>
cudaError_t shade_visibility(const ShadePass& p, const Shader& shader, cudaStream_t stream) {
    if (p.width <= 0 || p.height <= 0 || !p.visibility || !p.color || p.stride < 3 || p.attr_count < 0 ||
        p.attr_count > 4)
        return cudaErrorInvalidValue;
    ifr::DrawDev d;
    std::memset(&d, 0, sizeof(d));
    d.vertices = p.vertices;
    d.stride = p.stride;
    d.num_vertices = p.num_vertices;
    d.attr_offset = p.attr_offset;
    d.attr_count = p.attr_count;
    d.indices = p.indices;
    d.num_triangles = p.num_triangles;
    std::memcpy(d.mvp, p.mvp, sizeof(d.mvp));
    d.cull_mode = p.cull_mode;
    d.front_ccw = p.front_ccw;
    d.clip_input = p.clip_input;
    ifr::PassConst c;
    ifr::fill_pass_const(c, p.width, p.height, p.samples, 16);
    const size_t npix = (size_t)p.width * p.height;
    const int blocks = (int)std::min<size_t>((npix + 255) / 256, 8192);
    switch (p.samples) {
    case 1: detail::shade_visibility_kernel<1, Shader><<<blocks, 256, 0, stream>>>(p, d, c, shader); break;
    case 2: detail::shade_visibility_kernel<2, Shader><<<blocks, 256, 0, stream>>>(p, d, c, shader); break;
    case 4: detail::shade_visibility_kernel<4, Shader><<<blocks, 256, 0, stream>>>(p, d, c, shader); break;
    case 8: detail::shade_visibility_kernel<8, Shader><<<blocks, 256, 0, stream>>>(p, d, c, shader); break;
    case 16: detail::shade_visibility_kernel<16, Shader><<<blocks, 256, 0, stream>>>(p, d, c, shader); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Slot arrays of a mesh stage (caller-owned device memory): positions and attributes
// [groups][max_v][4] floats, indices [groups][max_i], counts [groups].
struct MeshSlots {
    float* positions;
    float* attributes;  // may be NULL (attr_count 0)
    int* indices;
    int* num_vertices;
    int* num_indices;
};

// Runs `mesh` as the mesh / geometry stage over `groups` work groups on the renderer's stream and
// draws its outputs (iftrDrawMeshOutputs).  Returns an IFTR_* status.
template <class Mesh>
int draw_mesh_stage(IfritGbRenderer* h, const Mesh& mesh, int groups, int max_v, int max_i, const MeshSlots& slots,
                    int attr_count, int clear, cudaStream_t stream) {
    if (!h || groups < 0 || max_v <= 0 || max_i <= 0 || !slots.positions || !slots.indices || !slots.num_vertices ||
        !slots.num_indices)
        return IFTR_ERR_INVALID_ARG;
    int rc = iftrSetStream(h, stream);
    if (rc) return rc;
    if (groups > 0) {
        detail::mesh_stage_kernel<Mesh><<<groups, 128, 0, stream>>>(mesh, max_v, max_i, slots.positions,
                                                                     attr_count > 0 ? slots.attributes : nullptr,
                                                                     slots.indices, slots.num_vertices, slots.num_indices);
        if (cudaGetLastError() != cudaSuccess) return IFTR_ERR_CUDA;
    }
    return iftrDrawMeshOutputs(h, groups, slots.positions, attr_count > 0 ? slots.attributes : nullptr, attr_count,
                               slots.indices, slots.num_vertices, slots.num_indices, max_v, max_i, clear);
}

// Runs the vertex functor over `num_vertices` vertices into positions / attributes ([V][4] floats
// each, caller device memory; attributes may be NULL with attr_count 0) and draws the triangle list
// indices[num_indices] (device, a multiple of 3) over them with the current state.  counts: caller
// device memory of 2 ints.  Returns an IFTR_* status.
template <class Vertex>
int draw_vertex_stage(IfritGbRenderer* h, const Vertex& vs, int num_vertices, const int* indices, int num_indices,
                      float* positions, float* attributes, int* counts, int attr_count, int clear, cudaStream_t stream) {
    if (!h || num_vertices <= 0 || num_indices <= 0 || num_indices % 3 || !indices || !positions || !counts ||
        (attr_count > 0 && !attributes))
        return IFTR_ERR_INVALID_ARG;
    int rc = iftrSetStream(h, stream);
    if (rc) return rc;
    detail::vertex_stage_kernel<Vertex><<<(num_vertices + 255) / 256, 256, 0, stream>>>(
        vs, num_vertices, num_indices, positions, attr_count > 0 ? attributes : nullptr, counts);
    if (cudaGetLastError() != cudaSuccess) return IFTR_ERR_CUDA;
    return iftrDrawMeshOutputs(h, 1, positions, attr_count > 0 ? attributes : nullptr, attr_count, indices, counts,
                               counts + 1, num_vertices, num_indices, clear);
}

// Runs `task` over `tasks` task groups, then `mesh` over the mesh groups they spawn (at most
// `max_groups`, the slot arrays' group count), and draws them through iftrDrawMeshOutputs in
// (task, sub) order.  offsets: caller device memory of tasks + 1 ints.  Returns an IFTR_* status;
// IFTR_ERR_OVERFLOW (nothing drawn) when the tasks spawn more than max_groups groups.
template <class Task, class Mesh>
int draw_task_mesh_stage(IfritGbRenderer* h, const Task& task, const Mesh& mesh, int tasks, int max_groups, int max_v,
                         int max_i, const MeshSlots& slots, int* offsets, int attr_count, int clear,
                         cudaStream_t stream) {
    if (!h || tasks < 0 || max_groups < 0 || max_v <= 0 || max_i <= 0 || !offsets || !slots.positions ||
        !slots.indices || !slots.num_vertices || !slots.num_indices)
        return IFTR_ERR_INVALID_ARG;
    int rc = iftrSetStream(h, stream);
    if (rc) return rc;
    if (tasks > 0) detail::task_count_kernel<Task><<<(tasks + 255) / 256, 256, 0, stream>>>(task, tasks, offsets);
    detail::task_scan_kernel<<<1, 1024, 0, stream>>>(offsets, tasks);
    if (max_groups > 0)
        detail::task_mesh_kernel<Mesh><<<max_groups, 128, 0, stream>>>(mesh, offsets, tasks, max_v, max_i,
                                                                       slots.positions,
                                                                       attr_count > 0 ? slots.attributes : nullptr,
                                                                       slots.indices, slots.num_vertices,
                                                                       slots.num_indices);
    if (cudaGetLastError() != cudaSuccess) return IFTR_ERR_CUDA;
    int total = 0;
    if (cudaMemcpyAsync(&total, offsets + tasks, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
        return IFTR_ERR_CUDA;
    if (total > max_groups) return IFTR_ERR_OVERFLOW;
    return iftrDrawMeshOutputs(h, max_groups, slots.positions, attr_count > 0 ? slots.attributes : nullptr, attr_count,
                               slots.indices, slots.num_vertices, slots.num_indices, max_v, max_i, clear);
}

}  // namespace ifrit_ext

#endif
