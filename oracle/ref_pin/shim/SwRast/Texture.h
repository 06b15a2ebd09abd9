// Stand-in for the reference's software texture sampler: the sky and blue-noise
// textures only shade misses and bounce directions, which the pin driver never
// evaluates.  Types exist so CpuRenderer.cpp compiles in place.
#pragma once
#include <memory>
#include <string_view>
#include <SwRast/SIMD.h>
namespace swr {
enum class FilterMode { Nearest, Linear };
struct SamplerDesc {
    FilterMode MagFilter = FilterMode::Linear, MinFilter = FilterMode::Linear;
    bool EnableMips = false;
};
struct StbImage {
    std::unique_ptr<uint8_t[]> Data;
    static StbImage Load(std::string_view) {
        StbImage img;
        img.Data.reset(new uint8_t[128 * 128 * 64 * 4]());
        return img;
    }
};
struct HdrTexture2D {
    template <SamplerDesc SD, bool B>
    VFloat3 SampleCube(VFloat3, int) const { return VFloat3(0.0f); }
};
namespace texutil {
inline HdrTexture2D LoadCubemapFromPanoramaHDR(std::string_view) { return {}; }
}  // namespace texutil
namespace pixfmt {
struct RG16f {
    static VInt Pack(VFloat2) { return VInt(0); }
    static VFloat2 Unpack(VInt) { return VFloat2(0.0f); }
};
struct RGBA8u {
    static VInt Pack(VFloat4) { return VInt(0); }
};
}  // namespace pixfmt
}  // namespace swr
