// Test infrastructure only: a thin driver that renders one seeded scene through the
// reference's own multithreaded CPU tile rasterizer (TileRasterRenderer, compiled from
// the reference sources by oracle/build_ref.py into oracle/_ref/).  It is never part of
// the product; tests and the golden-fixture script call it through ctypes to pin the
// CPU oracle against the reference.
//
// Reference interfaces used:
//   TileRasterRenderer::{Init,bindFrameBuffer,bindVertexBuffer,bindIndexBuffer,
//     bindVertexShaderLegacy,bindFragmentShader,SetDepthFunc,drawElements}
//     (projects/softgraphics/src/engine/tileraster/TileRasterRenderer.cpp:49-457)
//   VertexShader / FragmentShader (include/ifrit/softgraphics/engine/base/Shaders.h:46-78)
//   VertexBuffer (include/ifrit/softgraphics/engine/base/VertexBuffer.h:35-90)
//   TrivialBufferManager (include/ifrit/softgraphics/engine/bufferman/BufferManager.h:64-77)
#include "ifrit/softgraphics/engine/tileraster/TileRasterRenderer.h"
#include "ifrit/softgraphics/engine/bufferman/BufferManager.h"
#include <chrono>
#include <cstring>
#include <memory>
#include <vector>

using namespace Ifrit;
using namespace Ifrit::Graphics::SoftGraphics;
using namespace Ifrit::Graphics::SoftGraphics::TileRaster;

namespace {

struct MvpVS : public VertexShader {
    float m[16];
    void execute(const void* const* input, Vector4f* outPos, Vector4f* const* outVaryings) override {
        const float* p = reinterpret_cast<const float*>(input[0]);
        const float* c = reinterpret_cast<const float*>(input[1]);
        float x = p[0], y = p[1], z = p[2];
        outPos->x = m[0] * x + m[1] * y + m[2] * z + m[3];
        outPos->y = m[4] * x + m[5] * y + m[6] * z + m[7];
        outPos->z = m[8] * x + m[9] * y + m[10] * z + m[11];
        outPos->w = m[12] * x + m[13] * y + m[14] * z + m[15];
        outVaryings[0]->x = c[0];
        outVaryings[0]->y = c[1];
        outVaryings[0]->z = c[2];
        outVaryings[0]->w = c[3];
    }
};

struct PassFS : public FragmentShader {
    void execute(const void* varyings, void* colorOutput, float* fragmentDepth) override {
        const Vector4f* v = reinterpret_cast<const Vector4f*>(varyings);
        Vector4f* o = reinterpret_cast<Vector4f*>(colorOutput);
        *o = v[0];
    }
};

} // namespace

extern "C" {

// Renders `ntris` indexed triangles.  `verts` holds nverts x 8 floats: xyz, pad, rgba.
// depth_func uses the reference's IfritCompareOp numbering.  deterministic selects the
// reference's ordered (optForceDeterministic) path.  Outputs: rgba (W*H*4 floats, row-major)
// and depth (W*H floats).  Returns the median wall time of `timed` frames in milliseconds
// after `warm` untimed frames (one frame when both are zero).
// blend: NULL, or 5 ints {enable, srcColor, dstColor, srcAlpha, dstAlpha} (IfritBlendFactor
// numbering), set through TileRasterRenderer::setBlendFunc (TileRasterRenderer.cpp:212-333); a
// blended draw takes the reference's in-order path (TileRasterWorker.cpp:410).
double ref_render_ex(const float* verts, int nverts, const int* indices, int ntris, const float* mvp,
                     int W, int H, int depth_func, int deterministic, const int* blend, float* rgba, float* depth,
                     int warm, int timed) {
    auto renderer = std::make_shared<TileRasterRenderer>();
    renderer->Init();

    ImageF32 color(W, H, 4);
    ImageF32 depthImg(W, H, 1);
    FrameBuffer fb;
    fb.SetColorAttachments({&color});
    fb.SetDepthAttachment(depthImg);

    VertexBuffer vb;
    vb.setLayout({TypeDescriptors.FLOAT4, TypeDescriptors.FLOAT4});
    vb.allocateBuffer(nverts);
    for (int i = 0; i < nverts; i++) {
        vb.setValue<Vector4f>(i, 0, Vector4f(verts[i * 8 + 0], verts[i * 8 + 1], verts[i * 8 + 2], 1.0f));
        vb.setValue<Vector4f>(i, 1, Vector4f(verts[i * 8 + 4], verts[i * 8 + 5], verts[i * 8 + 6], verts[i * 8 + 7]));
    }

    auto bufman = std::make_shared<BufferManager::TrivialBufferManager>();
    bufman->Init();
    IfritBufferCreateInfo ci;
    ci.bufferSize = sizeof(int) * (size_t)ntris * 3;
    auto ib = bufman->CreateBuffer(ci);
    bufman->bufferData(ib, indices, 0, ci.bufferSize);

    VaryingDescriptor vd;
    vd.setVaryingDescriptors({TypeDescriptors.FLOAT4});

    MvpVS vs;
    std::memcpy(vs.m, mvp, sizeof(float) * 16);
    PassFS fs;

    renderer->bindFrameBuffer(fb);
    renderer->bindVertexBuffer(vb);
    renderer->bindIndexBuffer(ib);
    renderer->bindVertexShaderLegacy(vs, vd);
    renderer->bindFragmentShader(fs);
    renderer->SetDepthFunc((IfritCompareOp)depth_func);
    renderer->optsetForceDeterministic(deterministic != 0);
    if (blend) {
        IfritColorAttachmentBlendState bs;
        bs.blendEnable = blend[0] != 0;
        bs.srcColorBlendFactor = (IfritBlendFactor)blend[1];
        bs.dstColorBlendFactor = (IfritBlendFactor)blend[2];
        bs.srcAlphaBlendFactor = (IfritBlendFactor)blend[3];
        bs.dstAlphaBlendFactor = (IfritBlendFactor)blend[4];
        renderer->setBlendFunc(bs);
    }

    std::vector<double> times;
    int total = warm + timed;
    if (total <= 0) total = 1;
    for (int f = 0; f < total; f++) {
        auto t0 = std::chrono::steady_clock::now();
        renderer->drawElements(ntris * 3, true);
        auto t1 = std::chrono::steady_clock::now();
        if (f >= warm) times.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    std::memcpy(rgba, color.getData(), sizeof(float) * (size_t)W * H * 4);
    std::memcpy(depth, depthImg.getData(), sizeof(float) * (size_t)W * H);
    std::sort(times.begin(), times.end());
    return times.empty() ? 0.0 : times[times.size() / 2];
}

double ref_render(const float* verts, int nverts, const int* indices, int ntris, const float* mvp,
                  int W, int H, int depth_func, int deterministic, float* rgba, float* depth,
                  int warm, int timed) {
    return ref_render_ex(verts, nverts, indices, ntris, mvp, W, H, depth_func, deterministic, nullptr, rgba, depth,
                         warm, timed);
}

int ref_num_threads() { return TileRasterContext::numThreads; }

} // extern "C"
