// trace.cu - per-view and explicit-ray traversal kernels and their C ABI.
//
// vrt_render_view* is the one-launch-per-view path of GpuRenderer::RenderFrame
// (src/VoxelRT/GpuRenderer.cpp:239-273): 8x8 thread blocks over the image, one
// primary ray per pixel (Shaders/VoxelRender.comp:27-30), writing a headless hit
// buffer instead of the G-buffer.  vrt_cast* traverses caller-supplied rays.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "trace_core.cuh"
#include "world.h"

namespace vrt {
namespace {

uint32_t eff_iters(uint32_t max_iters, bool glsl = false) {
    if (max_iters == 0) return glsl ? VRT_GLSL_MAX_ITERS : VRT_DEFAULT_MAX_ITERS;
    return max_iters > 65535u ? 65535u : max_iters;
}

__global__ void __launch_bounds__(64) render_view_kernel(DevWorld w, vrt_camera cam, uint32_t max_iters,
                                                        uint4* __restrict__ out) {
    const uint32_t px = blockIdx.x * 8 + threadIdx.x;
    const uint32_t py = blockIdx.y * 8 + threadIdx.y;
    if (px >= cam.width || py >= cam.height) return;
    float dx, dy, dz;
    camera_ray(cam, px, py, dx, dy, dz);
    TraceResult r;
    TraceCounters cnt;
    trace_ray<false>(w, cam.origin[0], cam.origin[1], cam.origin[2], dx, dy, dz, cam.world_origin[0],
                     cam.world_origin[1], cam.world_origin[2], max_iters, r, cnt);
    const uint32_t pix = py * cam.width + px;
    out[pix] = pack_hit(r, dx, dy, dz, pix);
}

template <bool kGlsl, bool kAniso = false>
__global__ void __launch_bounds__(256) cast_kernel(DevWorld w, const float4* __restrict__ rays, uint32_t n,
                                                  int32_t wox, int32_t woy, int32_t woz, uint32_t max_iters,
                                                  uint4* __restrict__ out, bool coarse) {
    if constexpr (kAniso) fill_forward_lut();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = rays[2 * (size_t)i], b = rays[2 * (size_t)i + 1];
    TraceResult r;
    TraceCounters cnt;
    trace_ray<false, kGlsl>(w, a.x, a.y, a.z, a.w, b.x, b.y, wox, woy, woz, max_iters, r, cnt, coarse, kAniso);
    out[i] = pack_hit<kGlsl>(r, a.w, b.x, b.y, __float_as_uint(b.z));
}

// Explicit rays whose lengths vary widely (random origins and directions: some hit at
// once, others run to the iteration cap) leave most lanes of a thread-per-ray warp idle
// behind its longest ray.  Here each warp walks its own grid-strided sequence of 32-ray
// chunks (warp g takes rays [32 (g + k G), +32) for k = 0, 1, ...), traces in rounds
// of `inner` DDA steps, and between rounds stores the records of the rays that ended
// and refills those lanes from its chunks once fewer than `refill` lanes trace.  No
// device queue: calls on different streams stay independent.  Same records as
// cast_kernel: a lane's steps continue from where its ray left off, and a ray's record
// is packed from the state at its exit.
template <bool kGlsl, bool kAniso = false>
__global__ void __maxnreg__(48) cast_persistent_kernel(DevWorld w, const float4* __restrict__ rays, uint32_t n,
                                                             int32_t wox, int32_t woy, int32_t woz, uint32_t max_iters,
                                                             uint32_t inner, uint32_t refill, uint4* __restrict__ out,
                                                             bool coarse) {
    if constexpr (kAniso) fill_forward_lut();
    const uint32_t lane = threadIdx.x & 31, lt = (1u << lane) - 1u;
    const uint32_t stride = (gridDim.x * blockDim.x) & ~31u;  // rays between a warp's chunks
    uint32_t next = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;  // first ray of the warp's next chunk
    uint32_t q_next = 0, q_end = 0;
    bool active = false, ended = false, hit = false, safe = false;
    uint32_t ri = 0, iter = 0, tag = 0;
    RayState s;
    TraceCounters cnt{0, 0};
    for (;;) {
        if (ended) {
            out[ri] = pack_state<kGlsl>(s, hit, iter, tag);
            ended = false;
            active = false;
        }
        const uint32_t act = __ballot_sync(0xffffffffu, active);
        if ((uint32_t)__popc(act) < refill) {
            uint32_t idle = ~act;
            while (idle) {
                if (q_next >= q_end) {
                    if (next >= n) break;
                    q_next = next;
                    q_end = min(next + 32u, n);
                    next = next + stride < next ? n : next + stride;  // no wrap past 2^32
                }
                const uint32_t take = min(q_end - q_next, (uint32_t)__popc(idle));
                const uint32_t rank = __popc(idle & lt);
                const bool mine = ((idle >> lane) & 1u) && rank < take;
                const uint32_t assigned = __ballot_sync(0xffffffffu, mine);
                if (mine) {
                    ri = q_next + rank;
                    const float4 a = __ldg(rays + 2 * (size_t)ri), b = __ldg(rays + 2 * (size_t)ri + 1);
                    tag = __float_as_uint(b.z);
                    safe = ray_start<kGlsl>(s, w, a.x, a.y, a.z, a.w, b.x, b.y, wox, woy, woz, false, coarse);
                    iter = 0;
                    active = true;
                }
                idle &= ~assigned;
                q_next += take;
            }
        }
        if (__ballot_sync(0xffffffffu, active) == 0) break;
        const bool all_safe = __all_sync(0xffffffffu, !active || safe);
        if (active) {
            const uint32_t kmax = min(inner, max_iters - iter);
            uint32_t k = 0;
            // GLSL variants (rayCastCoarse, anisotropic LODs) are uniform over the launch
            const uint32_t st = dda_steps_mode<false, kGlsl>(s, w, wox, woy, woz, cnt, all_safe, coarse, coarse, kAniso,
                                                             iter, k, kmax);
            iter += k;
            if (st != kStepContinue || iter >= max_iters) {
                ended = true;
                hit = st == kStepHit;
            }
        }
    }
}

vrt_status check_camera(const vrt_camera* cam) {
    if (!cam || cam->width == 0 || cam->height == 0 || cam->width > 16384 || cam->height > 16384 ||
        !world_origin_ok(cam->world_origin)) {
        set_error("camera must be 1..16384 pixels on each side with |world origin| <= 2^30");
        return VRT_ERR_INVALID_ARG;
    }
    return VRT_OK;
}

vrt_status launch_render(vrt_world* w, const vrt_camera* cam, uint32_t max_iters, vrt_hit* hits,
                         cudaStream_t stream) {
    dim3 block(8, 8);
    dim3 grid((cam->width + 7) / 8, (cam->height + 7) / 8);
    L2Window l2;
    vrt_status st = l2.enter(w, stream);
    if (st != VRT_OK) return st;
    render_view_kernel<<<grid, block, 0, stream>>>(w->dev(), *cam, eff_iters(max_iters),
                                                   reinterpret_cast<uint4*>(hits));
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

// Launch shape of cast_persistent_kernel (also capped at 48 registers, for more warps to hide
// L2 latency): measured on GB300 with the 2^26 random rays
// of the incoherent workload.
constexpr uint32_t kCastThreads = 128, kCastInner = 12, kCastRefill = 28;
// Below this many rays the thread-per-ray kernel is used (too few rays to fill the
// persistent grid's lanes twice).
constexpr uint32_t kCastPersistentMin = 1u << 18;

vrt_status launch_cast(vrt_world* w, const vrt_ray* rays, uint32_t n, const vrt_cast_params* p, vrt_hit* hits,
                       cudaStream_t stream) {
    if (n == 0) return VRT_OK;
    const bool glsl = (p->flags & VRT_CAST_GLSL) != 0, coarse = (p->flags & VRT_CAST_GLSL_COARSE) != 0,
               aniso = (p->flags & VRT_CAST_GLSL_ANISO) != 0;
    const float4* r4 = reinterpret_cast<const float4*>(rays);
    uint4* o4 = reinterpret_cast<uint4*>(hits);
    uint32_t iters = eff_iters(p->max_iters, glsl);
    if (coarse) iters = std::min<uint32_t>(iters, VRT_GLSL_COARSE_MAX_ITERS);
    L2Window l2;
    vrt_status st = l2.enter(w, stream);
    if (st != VRT_OK) return st;
    if (n < kCastPersistentMin) {
        auto kernel = glsl ? (aniso ? cast_kernel<true, true> : cast_kernel<true>) : cast_kernel<false>;
        kernel<<<(n + 255) / 256, 256, 0, stream>>>(w->dev(), r4, n, p->world_origin[0], p->world_origin[1],
                                                    p->world_origin[2], iters, o4, coarse);
    } else {
        auto kernel = glsl ? (aniso ? cast_persistent_kernel<true, true> : cast_persistent_kernel<true>)
                           : cast_persistent_kernel<false>;
        int dev = 0, sms = 0, occ = 0;
        VRT_CUDA(cudaGetDevice(&dev));
        VRT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        VRT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kCastThreads, 0));
        const uint32_t blocks = (uint32_t)(sms * std::max(occ, 1));
        kernel<<<blocks, kCastThreads, 0, stream>>>(w->dev(), r4, n, p->world_origin[0], p->world_origin[1],
                                                    p->world_origin[2], iters, kCastInner, kCastRefill, o4, coarse);
    }
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

vrt_status check_params(const vrt_cast_params* p) {
    const uint32_t glsl_opts = VRT_CAST_GLSL_COARSE | VRT_CAST_GLSL_ANISO;
    if (!p || (p->flags & ~(VRT_CAST_GLSL | glsl_opts)) != 0 ||
        ((p->flags & glsl_opts) && !(p->flags & VRT_CAST_GLSL)) || !world_origin_ok(p->world_origin)) {
        set_error("cast params missing, flags other than VRT_CAST_GLSL [| VRT_CAST_GLSL_COARSE | "
                  "VRT_CAST_GLSL_ANISO], or |world origin| > 2^30");
        return VRT_ERR_INVALID_ARG;
    }
    return VRT_OK;
}

}  // namespace
}  // namespace vrt

using namespace vrt;

extern "C" {

vrt_status vrt_cast_device(vrt_world* w, const vrt_ray* rays, uint32_t n, const vrt_cast_params* params,
                           vrt_hit* hits, void* stream) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK || (st = check_params(params)) != VRT_OK) return st;
    if (n && (!rays || !hits)) {
        set_error("null ray or hit buffer");
        return VRT_ERR_INVALID_ARG;
    }
    return launch_cast(w, rays, n, params, hits, (cudaStream_t)stream);
}

vrt_status vrt_cast(vrt_world* w, const vrt_ray* rays, uint32_t n, const vrt_cast_params* params, vrt_hit* hits,
                    void* stream_) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK || (st = check_params(params)) != VRT_OK) return st;
    if (n == 0) return VRT_OK;
    if (!rays || !hits) {
        set_error("null ray or hit buffer");
        return VRT_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(w->mu);
    cudaStream_t stream = (cudaStream_t)stream_;
    const size_t rb = (size_t)n * sizeof(vrt_ray), hb = (size_t)n * sizeof(vrt_hit);
    VRT_CUDA(w->d_io.reserve(rb + hb));
    vrt_ray* d_rays = (vrt_ray*)w->d_io.ptr;
    vrt_hit* d_hits = (vrt_hit*)((uint8_t*)w->d_io.ptr + rb);
    VRT_CUDA(cudaMemcpyAsync(d_rays, rays, rb, cudaMemcpyHostToDevice, stream));
    if ((st = launch_cast(w, d_rays, n, params, d_hits, stream)) != VRT_OK) return st;
    VRT_CUDA(cudaMemcpyAsync(hits, d_hits, hb, cudaMemcpyDeviceToHost, stream));
    VRT_CUDA(cudaStreamSynchronize(stream));
    return VRT_OK;
}

vrt_status vrt_render_view_device(vrt_world* w, const vrt_camera* cam, uint32_t max_iters, vrt_hit* hits,
                                  void* stream) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK || (st = check_camera(cam)) != VRT_OK) return st;
    if (!hits) {
        set_error("null hit buffer");
        return VRT_ERR_INVALID_ARG;
    }
    return launch_render(w, cam, max_iters, hits, (cudaStream_t)stream);
}

vrt_status vrt_render_view(vrt_world* w, const vrt_camera* cam, uint32_t max_iters, vrt_hit* hits, void* stream_) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK || (st = check_camera(cam)) != VRT_OK) return st;
    if (!hits) {
        set_error("null hit buffer");
        return VRT_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(w->mu);
    cudaStream_t stream = (cudaStream_t)stream_;
    const size_t hb = (size_t)cam->width * cam->height * sizeof(vrt_hit);
    VRT_CUDA(w->d_io.reserve(hb));
    if ((st = launch_render(w, cam, max_iters, (vrt_hit*)w->d_io.ptr, stream)) != VRT_OK) return st;
    VRT_CUDA(cudaMemcpyAsync(hits, w->d_io.ptr, hb, cudaMemcpyDeviceToHost, stream));
    VRT_CUDA(cudaStreamSynchronize(stream));
    return VRT_OK;
}

}  // extern "C"
