// gbuffer.cu - the consumer of the primary hits: a headless G-buffer (albedo with the
// packed normal, and projected depth) per pixel of a view.
//
// The reference's renderers write it from the primary hit of every pixel:
// VoxelRender.comp:39-46,91-93 (rgba8 albedo + packGNormal in alpha, GBuffer.glsl:18-21;
// r32f depth) and CpuRenderer.cpp:364-376 (RGBA8 albedo with the normal in bits 24-29,
// the same bit layout; depth).  Here one thread per pixel traces the view's primary
// ray (either traversal mode) and writes the texel and depth, and optionally the hit
// record, so the normal comes from the full hit state: the GLSL mode's normal can have
// several axes (VoxelTraversal.glsl:190-192), which the record's face cannot carry.
// Shading (irradiance, sky, bounces' light) stays out of scope.

#include <cuda_runtime.h>

#include <cstring>

#include "batch_internal.h"
#include "trace_core.cuh"
#include "world.h"

namespace vrt {
namespace {

struct GbufferParams {
    uint32_t palette[256];  // Material::Data.x: RGB565 color in bits 0-15 (GpuRenderer.cpp:101)
    float proj[16];         // column-major projection of ray-frame positions / 16
};

// Albedo + packed normal and depth of one primary hit: every op rounded on its own in the
// order the oracle states (getMaterialColor and its square, round-half-even to 8 bits,
// packGNormal; proj * (pos / 16, 1) then z / w).
template <bool kGlsl>
__device__ __forceinline__ void gbuffer_texel(const RayState& s, bool hit, const uint32_t* pal, const float* m,
                                              uint32_t& texel, float& depth) {
    if (!hit) {
        texel = 0x00FFFFFFu;
        depth = -1.0f;
        return;
    }
    const uint32_t c = pal[s.material];
    const float r = __fmul_rn(__uint2float_rn((c >> 11) & 31u), 1.0f / 31);
    const float g = __fmul_rn(__uint2float_rn((c >> 5) & 63u), 1.0f / 63);
    const float b = __fmul_rn(__uint2float_rn(c & 31u), 1.0f / 31);
    texel = (uint32_t)__float2int_rn(__fmul_rn(__fmul_rn(r, r), 255.0f)) |
            (uint32_t)__float2int_rn(__fmul_rn(__fmul_rn(g, g), 255.0f)) << 8 |
            (uint32_t)__float2int_rn(__fmul_rn(__fmul_rn(b, b), 255.0f)) << 16;
    float ox, oy, oz, nx, ny, nz;
    hit_frame<kGlsl>(s, ox, oy, oz, nx, ny, nz);
    texel |= ((uint32_t)__fadd_rn(nx, 1.0f) | (uint32_t)__fadd_rn(ny, 1.0f) << 2 | (uint32_t)__fadd_rn(nz, 1.0f) << 4)
             << 24;
    const float px = __fmul_rn(s.cx, 0.0625f), py = __fmul_rn(s.cy, 0.0625f), pz = __fmul_rn(s.cz, 0.0625f);
    const float z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[2], px), __fmul_rn(m[6], py)), __fmul_rn(m[10], pz)), m[14]);
    const float w = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[3], px), __fmul_rn(m[7], py)), __fmul_rn(m[11], pz)), m[15]);
    depth = __fdiv_rn(z, w);
}

// 8x8 pixels per block; the palette and the matrix go to shared memory first.
template <bool kGlsl, bool kAniso>
__global__ void __launch_bounds__(64) gbuffer_kernel(DevWorld w, ViewDev v, GbufferParams gp,
                                                    uint32_t* __restrict__ tex, float* __restrict__ depth,
                                                    uint4* __restrict__ out) {
    if constexpr (kAniso) fill_forward_lut();
    __shared__ uint32_t s_pal[256];
    __shared__ float s_proj[16];
    const uint32_t t = threadIdx.y * 8 + threadIdx.x;
    for (uint32_t i = t; i < 256; i += 64) s_pal[i] = gp.palette[i];
    if (t < 16) s_proj[t] = gp.proj[t];
    __syncthreads();
    const uint32_t px = blockIdx.x * 8 + threadIdx.x, py = blockIdx.y * 8 + threadIdx.y;
    if (px >= v.width || py >= v.height) return;
    const uint32_t pixel = py * v.width + px;
    float dx, dy, dz;
    camera_ray(v.d0, v.du, v.dv, px, py, dx, dy, dz);
    RayState s;
    const bool safe = ray_start<kGlsl>(s, w, v.ox, v.oy, v.oz, dx, dy, dz, v.wo[0], v.wo[1], v.wo[2]);
    TraceCounters cnt{0, 0};
    uint32_t i = 0;
    uint32_t st = dda_steps_mode<false, kGlsl>(s, w, v.wo[0], v.wo[1], v.wo[2], cnt, safe, false, false, kAniso, 0, i,
                                                v.max_iters);
    if (v.max_iters == 0) st = kStepOut;
    const bool hit = st == kStepHit && i < v.max_iters;
    uint32_t texel;
    float d;
    gbuffer_texel<kGlsl>(s, hit, s_pal, s_proj, texel, d);
    tex[pixel] = texel;
    depth[pixel] = d;
    if (out) out[pixel] = pack_state<kGlsl>(s, hit, i, pixel);
}

vrt_status launch_gbuffer(vrt_world* w, const vrt_view* view, const uint32_t* palette, const float* proj,
                          uint32_t* tex, float* depth, vrt_hit* hits, cudaStream_t stream) {
    GbufferParams gp;
    std::memcpy(gp.palette, palette, sizeof(gp.palette));
    std::memcpy(gp.proj, proj, sizeof(gp.proj));
    const ViewDev v = make_view_dev(*view);
    dim3 block(8, 8), grid((v.width + 7) / 8, (v.height + 7) / 8);
    uint4* out = reinterpret_cast<uint4*>(hits);
    if (view_glsl(*view) && view_aniso(*view))
        gbuffer_kernel<true, true><<<grid, block, 0, stream>>>(w->dev(), v, gp, tex, depth, out);
    else if (view_glsl(*view))
        gbuffer_kernel<true, false><<<grid, block, 0, stream>>>(w->dev(), v, gp, tex, depth, out);
    else
        gbuffer_kernel<false, false><<<grid, block, 0, stream>>>(w->dev(), v, gp, tex, depth, out);
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

// Makes w's device current until `ds` ends.
vrt_status check_gbuffer_args(vrt_world* w, const vrt_view* view, const uint32_t* palette, const float* proj,
                              const void* tex, const void* depth, DeviceScope& ds) {
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK || (st = check_view(view)) != VRT_OK) return st;
    if (!palette || !proj || !tex || !depth) {
        set_error("G-buffer needs a palette, a projection and albedo/depth buffers");
        return VRT_ERR_INVALID_ARG;
    }
    return VRT_OK;
}

}  // namespace
}  // namespace vrt

using namespace vrt;

extern "C" vrt_status vrt_render_gbuffer_device(vrt_world* w, const vrt_view* view, const uint32_t* palette,
                                                const float* proj, uint32_t* albedo_normal, float* depth,
                                                vrt_hit* hits, void* stream) {
    DeviceScope ds;
    vrt_status st = check_gbuffer_args(w, view, palette, proj, albedo_normal, depth, ds);
    if (st != VRT_OK) return st;
    return launch_gbuffer(w, view, palette, proj, albedo_normal, depth, hits, (cudaStream_t)stream);
}

extern "C" vrt_status vrt_render_gbuffer(vrt_world* w, const vrt_view* view, const uint32_t* palette,
                                         const float* proj, uint32_t* albedo_normal, float* depth, void* stream_) {
    DeviceScope ds;
    vrt_status st = check_gbuffer_args(w, view, palette, proj, albedo_normal, depth, ds);
    if (st != VRT_OK) return st;
    std::lock_guard<std::mutex> lock(w->mu);
    cudaStream_t stream = (cudaStream_t)stream_;
    const size_t n = (size_t)view->cam.width * view->cam.height;
    VRT_CUDA(w->d_io.reserve(n * 8));
    uint32_t* d_tex = (uint32_t*)w->d_io.ptr;
    float* d_depth = (float*)(d_tex + n);
    if ((st = launch_gbuffer(w, view, palette, proj, d_tex, d_depth, nullptr, stream)) != VRT_OK) return st;
    VRT_CUDA(cudaMemcpyAsync(albedo_normal, d_tex, n * 4, cudaMemcpyDeviceToHost, stream));
    VRT_CUDA(cudaMemcpyAsync(depth, d_depth, n * 4, cudaMemcpyDeviceToHost, stream));
    VRT_CUDA(cudaStreamSynchronize(stream));
    return VRT_OK;
}
