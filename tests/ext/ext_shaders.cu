// Shaders written against the device-side extension point (include/ifrit_gb300_ext.cuh), built
// by the extension tests into a shared library and called through ctypes (test code).
//
//   ext_shade(which, ...)   which 0: ifrit_ext::Gouraud, 1: AttrDerivShader (below)
//   ext_draw_grid(...)      GridMesh as the mesh stage, drawn through iftrDrawMeshOutputs
//   ext_draw_task_grid(...) TaskSpawn + TaskGrid as the task and mesh stages
//   ext_draw_vertices(...)  ScaleVertex as the vertex stage over an indexed mesh
#include "ifrit_gb300_ext.cuh"

// Uses the attribute, both quad derivatives and the triangle index, so every field of the
// fragment is checked (scaling by a power of two is exact).
struct AttrDerivShader {
    __device__ void operator()(const ifrit_ext::Fragment& f, float out[4]) const {
        out[0] = f.attr[0] * f.attr[0] + f.attr[2];
        out[1] = f.ddy[1] * 64.0f;
        out[2] = f.ddx[0] * 64.0f;
        out[3] = (float)f.triangle;
    }
};

// A grid of nx x ny cells on z = z(cell); work group g emits cell g as two triangles (every 7th
// group emits nothing, every 5th only its first triangle).  Vertices are world positions with
// exactly representable coordinates transformed by `mvp` with the vertex stage's row order,
// ((m0 x + m1 y) + m2 z) + m3, so a host-side indexed mesh of the same positions draws the same
// clip coordinates.
// Vertex i (0..3) of the quad of grid cell `cell` (nx cells per row).
__device__ void cell_vertex(const float* mvp, int nx, int cell, int i, float clip[4], float attr[4]) {
    const int cx = cell % nx, cy = cell / nx;
    const int vx = cx + (i & 1), vy = cy + (i >> 1);
    const float p[3] = {(float)vx * 0.125f - 1.0f, (float)vy * 0.125f - 1.0f, -2.0f - (float)((cx * 3 + cy * 5) % 8) * 0.0625f};
    for (int r = 0; r < 4; r++)
        clip[r] = ((mvp[4 * r + 0] * p[0] + mvp[4 * r + 1] * p[1]) + mvp[4 * r + 2] * p[2]) + mvp[4 * r + 3];
    attr[0] = (float)vx * 0.0625f;
    attr[1] = (float)vy * 0.0625f;
    attr[2] = (float)((cell * 5) % 9) * 0.125f;
    attr[3] = 1.0f;
}

__device__ int quad_index(int j) {
    const int tri[6] = {0, 1, 2, 2, 1, 3};
    return tri[j];
}

struct GridMesh {
    int nx, ny;
    float mvp[16];
    __device__ void counts(int g, int& nv, int& ni) const {
        if (g % 7 == 3) { nv = 0; ni = 0; return; }
        nv = 4;
        ni = (g % 5 == 1) ? 3 : 6;
    }
    __device__ void vertex(int g, int i, float clip[4], float attr[4]) const { cell_vertex(mvp, nx, g, i, clip, attr); }
    __device__ int index(int g, int j) const { return quad_index(j); }
};

// Task group t spawns t % 4 mesh groups; mesh group (t, sub) draws cell 3 t + sub (one triangle when
// (t + sub) % 3 == 1, else two).
struct TaskSpawn {
    __device__ int mesh_groups(int t) const { return t % 4; }
};

struct TaskGrid {
    int nx;
    float mvp[16];
    __device__ void counts(int t, int sub, int& nv, int& ni) const {
        nv = 4;
        ni = ((t + sub) % 3 == 1) ? 3 : 6;
    }
    __device__ void vertex(int t, int sub, int i, float clip[4], float attr[4]) const {
        cell_vertex(mvp, nx, 3 * t + sub, i, clip, attr);
    }
    __device__ int index(int t, int sub, int j) const { return quad_index(j); }
};

extern "C" int ext_shade(int which, const float* vertices, int stride, int num_vertices, int attr_offset,
                         int attr_count, const int* indices, int num_triangles, const float* mvp, int cull_mode,
                         int front_ccw, int width, int height, int samples, const int* visibility, int format,
                         void* color, const float* background, void* stream) {
    ifrit_ext::ShadePass p;
    std::memset(&p, 0, sizeof(p));
    p.vertices = vertices;
    p.stride = stride;
    p.num_vertices = num_vertices;
    p.attr_offset = attr_offset;
    p.attr_count = attr_count;
    p.indices = indices;
    p.num_triangles = num_triangles;
    std::memcpy(p.mvp, mvp, sizeof(p.mvp));
    p.cull_mode = cull_mode;
    p.front_ccw = front_ccw;
    p.width = width;
    p.height = height;
    p.samples = samples;
    p.visibility = visibility;
    p.format = format;
    p.color = color;
    for (int i = 0; i < 4; i++) p.background[i] = background[i];
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = which == 0 ? ifrit_ext::shade_visibility(p, ifrit_ext::Gouraud{}, s)
                               : ifrit_ext::shade_visibility(p, AttrDerivShader{}, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return (int)e;
}

extern "C" int ext_draw_grid(IfritGbRenderer* h, int nx, int ny, const float* mvp, float* positions,
                             float* attributes, int* indices, int* num_vertices, int* num_indices, int clear,
                             void* stream) {
    GridMesh m;
    m.nx = nx;
    m.ny = ny;
    std::memcpy(m.mvp, mvp, sizeof(m.mvp));
    ifrit_ext::MeshSlots slots{positions, attributes, indices, num_vertices, num_indices};
    return ifrit_ext::draw_mesh_stage(h, m, nx * ny, 4, 6, slots, 4, clear, static_cast<cudaStream_t>(stream));
}

extern "C" int ext_draw_task_grid(IfritGbRenderer* h, int tasks, int nx, const float* mvp, float* positions,
                                  float* attributes, int* indices, int* num_vertices, int* num_indices, int* offsets,
                                  int max_groups, int clear, void* stream) {
    TaskGrid m;
    m.nx = nx;
    std::memcpy(m.mvp, mvp, sizeof(m.mvp));
    ifrit_ext::MeshSlots slots{positions, attributes, indices, num_vertices, num_indices};
    return ifrit_ext::draw_task_mesh_stage(h, TaskSpawn{}, m, tasks, max_groups, 4, 6, slots, offsets, 4, clear,
                                           static_cast<cudaStream_t>(stream));
}

// Vertex i of an (x y z r g b) AoS array scaled by 1 + (i % 3) / 8 about the origin (exact factors),
// transformed by `mvp` in the vertex stage's row order; the varying is the colour with alpha 0.5.
struct ScaleVertex {
    const float* vertices;
    float mvp[16];
    __device__ void operator()(int i, float clip[4], float attr[4]) const {
        const float* v = vertices + (size_t)i * 6;
        const float f = 1.0f + (float)(i % 3) * 0.125f;
        const float p[3] = {v[0] * f, v[1] * f, v[2] * f};
        for (int r = 0; r < 4; r++)
            clip[r] = ((mvp[4 * r + 0] * p[0] + mvp[4 * r + 1] * p[1]) + mvp[4 * r + 2] * p[2]) + mvp[4 * r + 3];
        attr[0] = v[3];
        attr[1] = v[4];
        attr[2] = v[5];
        attr[3] = 0.5f;
    }
};

extern "C" int ext_draw_vertices(IfritGbRenderer* h, const float* vertices, int num_vertices, const int* indices,
                                 int num_indices, const float* mvp, float* positions, float* attributes, int* counts,
                                 int clear, void* stream) {
    ScaleVertex vs;
    vs.vertices = vertices;
    std::memcpy(vs.mvp, mvp, sizeof(vs.mvp));
    return ifrit_ext::draw_vertex_stage(h, vs, num_vertices, indices, num_indices, positions, attributes, counts, 4,
                                        clear, static_cast<cudaStream_t>(stream));
}
