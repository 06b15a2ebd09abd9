// pick.cu - the picking ray cast (VoxelMap::RayCast, src/VoxelRT/VoxelMap.cpp:125-170)
// on the device brickmap: one thread per ray, double precision, every op rounded
// on its own in the reference's order.  Step level 5 (32 voxels) when the sector is
// absent, 3 (8 voxels) when the brick is absent, 0 on an empty voxel, a hit on a
// solid one (GetStepLevel, VoxelMap.cpp:125-139).

#include <cuda_runtime.h>

#include "world.h"

namespace vrt {
namespace {

// glm::min(x, y) = y < x ? y : x
__device__ __forceinline__ double glm_min(double x, double y) { return y < x ? y : x; }

// double -> int32 as x86 cvttsd2si: out of range and NaN give INT32_MIN
__device__ __forceinline__ int32_t d2i_x86(double f) {
    return (f >= -2147483648.0 && f < 2147483648.0) ? (int32_t)f : INT32_MIN;
}

__global__ void pick_kernel(DevWorld w, uint32_t sy, const double* __restrict__ rays, uint32_t n, uint32_t max_iters,
                            vrt_pick_hit* __restrict__ out) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const double* ray = rays + (size_t)r * 6;
    double o[3], d[3], inv[3], ts[3];
    int32_t pos[3];
    for (int c = 0; c < 3; c++) {
        o[c] = ray[c];
        d[c] = ray[3 + c];
        inv[c] = __ddiv_rn(1.0, d[c]);
        ts[c] = __dmul_rn(__dsub_rn(d[c] < 0.0 ? 0.0 : 1.0, o[c]), inv[c]);  // glm::step(0, dir)
        pos[c] = d2i_x86(floor(o[c]));
    }
    vrt_pick_hit h;
    h.distance = -1.0;
    h.voxel[0] = h.voxel[1] = h.voxel[2] = 0;
    h.normal[0] = h.normal[1] = h.normal[2] = 0.0f;
    h.uv[0] = h.uv[1] = 0.0f;
    h.iters = max_iters;
    h.reserved = 0;
    for (uint32_t i = 0; i < max_iters; i++) {
        double side[3];
        for (int c = 0; c < 3; c++) side[c] = __dadd_rn(ts[c], __dmul_rn((double)pos[c], inv[c]));
        const double tmin = __dadd_rn(glm_min(glm_min(side[0], side[1]), side[2]), 0.0001);
        double hp[3];
        for (int c = 0; c < 3; c++) {
            hp[c] = __dadd_rn(o[c], __dmul_rn(tmin, d[c]));
            pos[c] = d2i_x86(floor(hp[c]));
        }
        // GetStepLevel: the sector key wraps as WorldSectorIndexer's 12/8/12 bits do
        const int32_t sxk = ((pos[0] >> 5) << 20) >> 20, syk = ((pos[1] >> 5) << 24) >> 24,
                      szk = ((pos[2] >> 5) << 20) >> 20;
        int32_t k = 5;
        if ((uint32_t)sxk < w.sx && (uint32_t)syk < sy && (uint32_t)szk < w.sz) {
            const SectorRec rec = w.sectors[(uint32_t)sxk + (uint32_t)szk * w.sx + (uint32_t)syk * w.sxz];
            const uint64_t mask = (uint64_t)rec.mask_lo | (uint64_t)rec.mask_hi << 32;
            if (mask != 0) {
                const uint32_t b = ((pos[0] >> 3) & 3) | ((pos[2] >> 3) & 3) << 2 | ((pos[1] >> 3) & 3) << 4;
                k = 3;
                if ((mask >> b) & 1) {
                    const uint32_t slot = rec.base + (uint32_t)__popcll(mask & ((1ull << b) - 1));
                    const uint32_t vi = (pos[0] & 7) | (pos[2] & 7) << 3 | (pos[1] & 7) << 6;
                    k = w.payload[(size_t)slot * 512 + vi] == 0 ? 0 : -1;
                }
            }
        }
        if (k < 0) {
            bool m[3];
            for (int c = 0; c < 3; c++) m[c] = tmin >= side[c];
            h.distance = tmin;
            for (int c = 0; c < 3; c++) {
                const double sg = (0.0 < d[c]) - (d[c] < 0.0);  // glm::sign
                h.normal[c] = m[c] ? (float)(-sg) : 0.0f;
                h.voxel[c] = pos[c];
            }
            // fract(mix(vec2(hp.x, hp.z), vec2(hp.y), vec2(m.x, m.z))), float ops in GLM's order
            const float ax = (float)hp[0], az = (float)hp[2], b = (float)hp[1];
            const float tx = m[0] ? 1.0f : 0.0f, tz = m[2] ? 1.0f : 0.0f;
            const float ux = __fadd_rn(__fmul_rn(ax, __fsub_rn(1.0f, tx)), __fmul_rn(b, tx));
            const float uz = __fadd_rn(__fmul_rn(az, __fsub_rn(1.0f, tz)), __fmul_rn(b, tz));
            h.uv[0] = __fsub_rn(ux, floorf(ux));
            h.uv[1] = __fsub_rn(uz, floorf(uz));
            h.iters = i;
            break;
        }
        const int32_t msk = (1 << k) - 1;
        for (int c = 0; c < 3; c++) pos[c] = d[c] < 0.0 ? (pos[c] & ~msk) : (pos[c] | msk);
    }
    out[r] = h;
}

}  // namespace
}  // namespace vrt

using namespace vrt;

extern "C" vrt_status vrt_pick(vrt_world* w, const vrt_pick_ray* rays, uint32_t n, uint32_t max_iters,
                               vrt_pick_hit* hits, void* stream_) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK) return st;
    if (n == 0) return VRT_OK;
    if (!rays || !hits) {
        set_error("null pick buffers");
        return VRT_ERR_INVALID_ARG;
    }
    if (max_iters == 0) max_iters = 1024;
    std::lock_guard<std::mutex> lock(w->mu);
    cudaStream_t stream = (cudaStream_t)stream_;
    const size_t rb = (size_t)n * sizeof(vrt_pick_ray), hb = (size_t)n * sizeof(vrt_pick_hit);
    VRT_CUDA(w->d_io.reserve(rb + hb));
    uint8_t* base = (uint8_t*)w->d_io.ptr;
    VRT_CUDA(cudaMemcpyAsync(base, rays, rb, cudaMemcpyHostToDevice, stream));
    pick_kernel<<<(n + 127) / 128, 128, 0, stream>>>(w->dev(), w->sy, (const double*)base, n, max_iters,
                                                      (vrt_pick_hit*)(base + rb));
    VRT_CUDA(cudaGetLastError());
    VRT_CUDA(cudaMemcpyAsync(hits, base + rb, hb, cudaMemcpyDeviceToHost, stream));
    VRT_CUDA(cudaStreamSynchronize(stream));
    return VRT_OK;
}
