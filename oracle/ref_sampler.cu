// Test infrastructure only: a host-side driver around the reference's own texture sampler
// (TextureSampleImpl in include/ifrit/softgraphics/engine/math/ShaderBuiltinCuda.cuh:96-272,
// IFRIT_DUAL code), compiled for the host by oracle/build_ref.py into oracle/_ref/.  It pins the
// CPU oracle's reference-compatible sampler (oracle_fx.c, `compat`) against the reference
// itself; it is never part of the product.
//
// The reference header is included where it lies.  Its CUDA renderer does not build with this
// toolkit (namespace drift), so the driver brings the two namespaces the sampler needs into
// scope before including it.  The dispatch below mirrors the reference's public `texture()`
// (ShaderBuiltinCuda.cuh:357-377): anisotropic filtering when the sampler enables it, otherwise
// the adaptive-LOD path, each with the quad derivatives of the UV varying
// (ndx = (du/dx, dv/dx), ndy = (du/dy, dv/dy), :262-272).
#include "ifrit/softgraphics/engine/base/Structures.h"
#include "ifrit/softgraphics/engine/tilerastercuda/TileRasterConstantsCuda.h"
using namespace Ifrit::Graphics::SoftGraphics;
using namespace Ifrit::Graphics::SoftGraphics::TileRaster::CUDA;
#include "ifrit/softgraphics/engine/math/ShaderBuiltinCuda.cuh"

namespace TS = Ifrit::SoftRenderer::Math::ShaderOps::CUDA::TextureSampleImpl;

extern "C" {

// Samples `n` points.  params: n x 7 floats (u, v, du/dx, dv/dx, du/dy, dv/dy, lod bias).
// texels: the float RGBA mip chain, level after level, padded past the chain as the caller
// needs (the reference reads level floor(lod)+1 unclamped).  out: n x 4 floats.
int ref_sample_batch(int n, const float* params, const float* texels, int width, int height, int filter,
                     int address_u, int address_v, int border_white, int anisotropy_enable, float max_anisotropy,
                     float* out) {
    IfritSamplerT s;
    s.filterMode = (IfritFilter)filter;
    s.addressModeU = (IfritSamplerAddressMode)address_u;
    s.addressModeV = (IfritSamplerAddressMode)address_v;
    s.borderColor = border_white ? IF_BORDER_COLOR_WHITE : IF_BORDER_COLOR_BLACK;
    s.anisotropyEnable = anisotropy_enable != 0;
    s.maxAnisotropy = max_anisotropy;
    const float4* tex = reinterpret_cast<const float4*>(texels);
    for (int i = 0; i < n; i++) {
        const float* p = params + 7 * i;
        float2 uv{p[0], p[1]};
        float2 ndx{p[2], p[3]};
        float2 ndy{p[4], p[5]};
        float4 r;
        if (s.anisotropyEnable)
            r = TS::textureImplAnisotropicFilter(s, tex, width, height, 1, s.maxAnisotropy, uv, ndx, ndy, p[6], {0, 0});
        else
            r = TS::textureImplAdaptiveLod(s, tex, width, height, 1, uv, ndx, ndy, p[6], {0, 0});
        out[4 * i + 0] = r.x;
        out[4 * i + 1] = r.y;
        out[4 * i + 2] = r.z;
        out[4 * i + 3] = r.w;
    }
    return 0;
}

}  // extern "C"
