// trace_core.cuh - per-ray brickmap traversal on the device.
//
// One thread walks one ray through sector mask -> brick cell mask -> voxel, the
// loop of RayCast/GetStepPos (src/VoxelRT/CpuRenderer.cpp:135-224) with the entry
// clip of clipRayToAABB (src/VoxelRT/Shaders/VoxelTraversal.glsl:133-145).
// Every float op is an explicitly rounded intrinsic (__fadd_rn, __fmul_rn,
// __fdiv_rn, __fsqrt_rn) in the reference's source order, so results do not
// depend on -fmad; min/max use the x86 minps/maxps NaN rule and floor->int uses
// the x86 out-of-range value INT32_MIN (SIMD_AVX512.h:109,123).
#pragma once

#include <cstdint>

#include "vrt_internal.h"

namespace vrt {

__device__ __forceinline__ float min_x86(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float max_x86(float a, float b) { return a > b ? a : b; }

// floor to int; NaN and out-of-range give INT32_MIN as cvtps2dq does.
__device__ __forceinline__ int32_t floor2i(float x) {
    return (x >= -2147483648.0f && x < 2147483648.0f) ? __float2int_rd(x) : INT32_MIN;
}
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

struct TraceResult {
    float cx, cy, cz;  // final position (HitResult.Pos)
    float sx, sy, sz;  // final side distances
    int32_t vx, vy, vz;
    uint32_t steps;
    uint32_t material;
    bool hit;
};

struct TraceCounters {
    uint32_t step_calls;
    uint32_t occ_fetches;
};

// Ray entry point of a camera pixel (the ray generation of vrt_camera).
__device__ __forceinline__ void camera_ray(const vrt_camera& cam, uint32_t px, uint32_t py, float& dx,
                                           float& dy, float& dz) {
    float u = __fadd_rn(__uint2float_rn(px), 0.5f);
    float v = __fadd_rn(__uint2float_rn(py), 0.5f);
    float x = __fadd_rn(__fadd_rn(cam.d0[0], __fmul_rn(u, cam.du[0])), __fmul_rn(v, cam.dv[0]));
    float y = __fadd_rn(__fadd_rn(cam.d0[1], __fmul_rn(u, cam.du[1])), __fmul_rn(v, cam.dv[1]));
    float z = __fadd_rn(__fadd_rn(cam.d0[2], __fmul_rn(u, cam.du[2])), __fmul_rn(v, cam.dv[2]));
    float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
    dx = __fdiv_rn(x, len);
    dy = __fdiv_rn(y, len);
    dz = __fdiv_rn(z, len);
}

template <bool kCount>
__device__ __forceinline__ void trace_ray(const DevWorld& w, float ox, float oy, float oz, float dx,
                                          float dy, float dz, int32_t wox, int32_t woy, int32_t woz,
                                          uint32_t max_iters, TraceResult& r, TraceCounters& cnt) {
    const float ix = __fdiv_rn(1.0f, dx), iy = __fdiv_rn(1.0f, dy), iz = __fdiv_rn(1.0f, dz);
    const float tsx = __fmul_rn(__fsub_rn(dx < 0.0f ? 0.0f : 1.0f, ox), ix);
    const float tsy = __fmul_rn(__fsub_rn(dy < 0.0f ? 0.0f : 1.0f, oy), iy);
    const float tsz = __fmul_rn(__fsub_rn(dz < 0.0f ? 0.0f : 1.0f, oz), iz);

    // clipRayToAABB(origin, dir, 1 - wo, size - wo - 1)
    float cx, cy, cz;
    {
        float t1x = __fmul_rn(__fsub_rn(__int2float_rn(1 - wox), ox), ix);
        float t1y = __fmul_rn(__fsub_rn(__int2float_rn(1 - woy), oy), iy);
        float t1z = __fmul_rn(__fsub_rn(__int2float_rn(1 - woz), oz), iz);
        float t2x = __fmul_rn(__fsub_rn(__fsub_rn(__fsub_rn(__uint2float_rn(w.size_x), __int2float_rn(wox)), 1.0f), ox), ix);
        float t2y = __fmul_rn(__fsub_rn(__fsub_rn(__fsub_rn(__uint2float_rn(w.size_y), __int2float_rn(woy)), 1.0f), oy), iy);
        float t2z = __fmul_rn(__fsub_rn(__fsub_rn(__fsub_rn(__uint2float_rn(w.size_z), __int2float_rn(woz)), 1.0f), oz), iz);
        float tmin = max_x86(min_x86(t1x, t2x), max_x86(min_x86(t1y, t2y), min_x86(t1z, t2z)));
        float tmax = min_x86(max_x86(t1x, t2x), min_x86(max_x86(t1y, t2y), max_x86(t1z, t2z)));
        bool clip = tmin > 0.0f && tmin < tmax;
        cx = clip ? __fadd_rn(ox, __fmul_rn(dx, tmin)) : ox;
        cy = clip ? __fadd_rn(oy, __fmul_rn(dy, tmin)) : oy;
        cz = clip ? __fadd_rn(oz, __fmul_rn(dz, tmin)) : oz;
    }
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    int32_t vx = 0, vy = 0, vz = 0;
    uint32_t steps = max_iters, material = 0;
    bool hit = false;

    for (uint32_t i = 0; i < max_iters; i++) {
        vx = wadd(wox, floor2i(cx));
        vy = wadd(woy, floor2i(cy));
        vz = wadd(woz, floor2i(cz));
        if (!((uint32_t)vx < w.size_x && (uint32_t)vy < w.size_y && (uint32_t)vz < w.size_z)) {
            steps = i;
            break;
        }
        // GetStepPos: sector allocation mask at lod 3
        const uint32_t sidx = (uint32_t)(vx >> 5) + (uint32_t)(vz >> 5) * w.sx + (uint32_t)(vy >> 5) * w.sxz;
        const uint4 rec = __ldg(reinterpret_cast<const uint4*>(w.sectors) + sidx);
        uint32_t lo = rec.x, hi = rec.y;
        uint32_t idx = ((vx >> 3) & 3) | ((vz >> 3) & 3) << 2 | ((vy >> 3) & 3) << 4;
        int32_t lod = 3;
        if (kCount) cnt.step_calls++;
        if ((((idx < 32 ? lo : hi) >> (idx & 31)) & 1u) != 0) {
            // brick allocated: slot = base + popcount of the mask below the brick bit
            const uint32_t below = (1u << (idx & 31)) - 1u;
            const uint32_t slot = rec.z + (idx < 32 ? __popc(lo & below) : __popc(lo) + __popc(hi & below));
            const uint32_t cell = ((vx >> 2) & 1) | ((vz >> 2) & 1) << 1 | ((vy >> 2) & 1) << 2;
            const uint2 cm = __ldg(reinterpret_cast<const uint2*>(w.occ) + (size_t)slot * 8 + cell);
            lo = cm.x;
            hi = cm.y;
            idx = (vx & 3) | (vz & 3) << 2 | (vy & 3) << 4;
            lod = 0;
            if (kCount) cnt.occ_fetches++;
            if ((((idx < 32 ? lo : hi) >> (idx & 31)) & 1u) != 0) {
                const uint32_t vi = (vx & 7) | (vz & 7) << 3 | (vy & 7) << 6;
                material = __ldg(w.payload + (size_t)slot * 512 + vi);
                hit = true;
                steps = i;
                break;
            }
        }
        const uint32_t half = idx < 32 ? lo : hi;
        lod += (lo | hi) == 0 ? 2 : (((half >> (idx & 0xA)) & 0x00330033u) == 0 ? 1 : 0);
        const int32_t m = (1 << lod) - 1;
        vx = dx < 0.0f ? (vx & ~m) : (vx | m);
        vy = dy < 0.0f ? (vy & ~m) : (vy | m);
        vz = dz < 0.0f ? (vz & ~m) : (vz | m);

        sx = __fadd_rn(tsx, __fmul_rn(__int2float_rn(wsub(vx, wox)), ix));
        sy = __fadd_rn(tsy, __fmul_rn(__int2float_rn(wsub(vy, woy)), iy));
        sz = __fadd_rn(tsz, __fmul_rn(__int2float_rn(wsub(vz, woz)), iz));
        const float t = __fadd_rn(min_x86(min_x86(sx, sy), sz), 0.001f);
        cx = __fadd_rn(ox, __fmul_rn(t, dx));
        cy = __fadd_rn(oy, __fmul_rn(t, dy));
        cz = __fadd_rn(oz, __fmul_rn(t, dz));
    }
    r.cx = cx;
    r.cy = cy;
    r.cz = cz;
    r.sx = sx;
    r.sy = sy;
    r.sz = sz;
    r.vx = vx;
    r.vy = vy;
    r.vz = vz;
    r.steps = steps;
    r.material = material;
    r.hit = hit;
}

// The 16-byte vrt_hit record as one vector store.
__device__ __forceinline__ uint4 pack_hit(const TraceResult& r, float dx, float dy, float dz, uint32_t tag) {
    if (!r.hit) return make_uint4(VRT_MISS_VOXEL, VRT_MISS_FACE | (r.steps << 16), 0x7F800000u, tag);
    const float t = min_x86(min_x86(r.sx, r.sy), r.sz);
    uint32_t face;
    if (r.sx == t)
        face = dx < 0.0f ? 1u : 0u;
    else if (r.sy == t)
        face = dy < 0.0f ? 3u : 2u;
    else
        face = dz < 0.0f ? 5u : 4u;
    const uint32_t voxel = (uint32_t)r.vx | (uint32_t)r.vy << 11 | (uint32_t)r.vz << 21;
    return make_uint4(voxel, face | r.material << 8 | r.steps << 16, __float_as_uint(t), tag);
}

__device__ __forceinline__ uint4 no_ray_hit() {
    return make_uint4(VRT_MISS_VOXEL, VRT_MISS_FACE, 0x7F800000u, VRT_NO_RAY);
}

// HitResult.Normal (CpuRenderer.cpp:213-217) and origin = Pos + Normal*0.01 (:389).
__device__ __forceinline__ void secondary_origin(const TraceResult& r, float dx, float dy, float dz, float& ox,
                                                 float& oy, float& oz, float& nx, float& ny, float& nz) {
    const float t = min_x86(min_x86(r.sx, r.sy), r.sz);
    const bool mx = r.sx == t, my = r.sy == t, mz = !mx && !my;
    nx = mx ? (signbit(dx) ? 1.0f : -1.0f) : 0.0f;
    ny = my ? (signbit(dy) ? 1.0f : -1.0f) : 0.0f;
    nz = mz ? (signbit(dz) ? 1.0f : -1.0f) : 0.0f;
    ox = __fadd_rn(r.cx, __fmul_rn(nx, 0.01f));
    oy = __fadd_rn(r.cy, __fmul_rn(ny, 0.01f));
    oz = __fadd_rn(r.cz, __fmul_rn(nz, 0.01f));
}

}  // namespace vrt
