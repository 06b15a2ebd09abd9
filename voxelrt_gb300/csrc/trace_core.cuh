// trace_core.cuh - per-ray brickmap traversal on the device.
//
// One thread walks one ray through brick table -> voxel code -> voxel, the
// loop of RayCast/GetStepPos (src/VoxelRT/CpuRenderer.cpp:135-224) with the entry
// clip of clipRayToAABB (src/VoxelRT/Shaders/VoxelTraversal.glsl:133-145).
// Every float op is an explicitly rounded intrinsic (__fadd_rn, __fmul_rn,
// __fdiv_rn, __frcp_rn, __fsqrt_rn) in the reference's source order, so results do not
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

// a * b + c (mod 2^32) on the integer multiply-add unit.  The step loop is bound by
// the ALU pipe (bit ops, compares, shifts) while the FMA pipe, which also executes
// integer multiply-add, has room; inline PTX keeps the compiler from folding these
// back into masks and adds (x - 8*(x >> 3) would become x & 7).
__device__ __forceinline__ uint32_t imad(uint32_t a, uint32_t b, uint32_t c) {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
#else
    return a * b + c;
#endif
}
// v - worldOrigin (wrapping), the ray-frame coordinate of a voxel
__device__ __forceinline__ float rel_voxel(int32_t v, int32_t wo) {
    return __int2float_rn((int32_t)imad((uint32_t)wo, 0xFFFFFFFFu, (uint32_t)v));
}

struct TraceResult {
    float cx, cy, cz;  // final position (HitResult.Pos)
    float sx, sy, sz;  // final side distances
    float tb;          // GLSL mode: biased tmin of the last step (hit.dist)
    int32_t vx, vy, vz;
    uint32_t steps;
    uint32_t material;
    bool hit;
};

struct TraceCounters {
    uint32_t step_calls;
    uint32_t occ_fetches;
};

// 1/sqrt(l2) for the normalisation of camera rays: the integer first estimate
// 0x5F3759DF - (bits(l2) >> 1) (C. Lomont, "Fast Inverse Square Root", 2003), then
// three Newton steps r <- r * (1.5 - (l2/2) * r*r), each one exactly rounded multiply,
// one fused multiply-add and one multiply, so any IEEE machine gets the same bits.
// For l2 in [2^-126, 2^126] the result is within 2.5 ulp of 1/sqrt(l2); the reference
// normalises with a 14-bit hardware estimate (SIMD.h normalize, rsqrt14).
__device__ __forceinline__ float camera_rsqrt(float l2) {
    const float h = __fmul_rn(0.5f, l2);
    float r = __uint_as_float(0x5F3759DFu - (__float_as_uint(l2) >> 1));
#pragma unroll
    for (int i = 0; i < 3; i++) r = __fmul_rn(r, __fmaf_rn(-h, __fmul_rn(r, r), 1.5f));
    return r;
}

// Ray entry point of a camera pixel (the ray generation of vrt_camera) from the
// camera's d0, du, dv vectors.
__device__ __forceinline__ void camera_ray(const float* d0, const float* du, const float* dv, uint32_t px,
                                           uint32_t py, float& dx, float& dy, float& dz) {
    float u = __fadd_rn(__uint2float_rn(px), 0.5f);
    float v = __fadd_rn(__uint2float_rn(py), 0.5f);
    float x = __fadd_rn(__fadd_rn(d0[0], __fmul_rn(u, du[0])), __fmul_rn(v, dv[0]));
    float y = __fadd_rn(__fadd_rn(d0[1], __fmul_rn(u, du[1])), __fmul_rn(v, dv[1]));
    float z = __fadd_rn(__fadd_rn(d0[2], __fmul_rn(u, du[2])), __fmul_rn(v, dv[2]));
    const float r = camera_rsqrt(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
    dx = __fmul_rn(x, r);
    dy = __fmul_rn(y, r);
    dz = __fmul_rn(z, r);
}
__device__ __forceinline__ void camera_ray(const vrt_camera& cam, uint32_t px, uint32_t py, float& dx,
                                           float& dy, float& dz) {
    camera_ray(cam.d0, cam.du, cam.dv, px, py, dx, dy, dz);
}

// Per-ray traversal state: RayCast's loop-carried values (CpuRenderer.cpp:173-184).
struct RayState {
    float ox, oy, oz, dx, dy, dz;
    float ix, iy, iz;     // invDir
    float tsx, tsy, tsz;  // tStart
    float cx, cy, cz;     // currPos
    float sx, sy, sz;     // sideDist
    float tb;             // GLSL mode: biased tmin of the last step
    int32_t vx, vy, vz;   // voxel of the last step (hit voxel on a hit)
    int32_t gx, gy, gz;   // -1 where dir < 0, else 0 (cell alignment side)
    uint32_t material;
};

// Bounds that keep a ray free of NaN and infinities inside the DDA loop: with
// |origin| < 2^30 and |1/dir| < 2^95, |tStart| and |(voxel - worldOrigin) * invDir|
// stay below 2^126 (voxel - worldOrigin < 2^31), so side distances and t are finite,
// and the position o + t*dir is finite or an infinity (never NaN) that leaves the grid.
constexpr float kSafeOrigin = 0x1p30f, kSafeInvDir = 0x1p95f;

// The clip box [1 - worldOrigin, size - 1 - worldOrigin] (VoxelTraversal.glsl:166) holds
// the origin strictly inside, and the origin is within the safe bound: ray_init then
// needs neither the slab test nor the origin's bound check.  Camera rays of a view
// share their origin, so the persistent kernel evaluates this once per queue chunk.
__device__ __forceinline__ bool origin_inside_safe(const DevWorld& w, float ox, float oy, float oz, int32_t wox,
                                                   int32_t woy, int32_t woz) {
    const float lx = __int2float_rn(1 - wox), ly = __int2float_rn(1 - woy), lz = __int2float_rn(1 - woz);
    const float hx = __fsub_rn(__fsub_rn(__uint2float_rn(w.size_x), __int2float_rn(wox)), 1.0f);
    const float hy = __fsub_rn(__fsub_rn(__uint2float_rn(w.size_y), __int2float_rn(woy)), 1.0f);
    const float hz = __fsub_rn(__fsub_rn(__uint2float_rn(w.size_z), __int2float_rn(woz)), 1.0f);
    return lx < ox && ox < hx && ly < oy && oy < hy && lz < oz && oz < hz && fabsf(ox) < kSafeOrigin &&
           fabsf(oy) < kSafeOrigin && fabsf(oz) < kSafeOrigin;
}

// invDir, tStart and the clipped start position (VoxelTraversal.glsl:133-145,163-167).
// Returns whether the ray is safe in the sense above (ray_step<kCount, true> applies).
// inside_safe: origin_inside_safe() is known to hold for this origin.
__device__ __forceinline__ bool ray_init(RayState& s, const DevWorld& w, float ox, float oy, float oz, float dx,
                                         float dy, float dz, int32_t wox, int32_t woy, int32_t woz,
                                         bool inside_safe = false) {
    s.ox = ox;
    s.oy = oy;
    s.oz = oz;
    s.dx = dx;
    s.dy = dy;
    s.dz = dz;
    // correctly rounded 1/dir, the same value as the IEEE division 1.0f / dir
    s.ix = __frcp_rn(dx);
    s.iy = __frcp_rn(dy);
    s.iz = __frcp_rn(dz);
    s.tsx = __fmul_rn(__fsub_rn(dx < 0.0f ? 0.0f : 1.0f, ox), s.ix);
    s.tsy = __fmul_rn(__fsub_rn(dy < 0.0f ? 0.0f : 1.0f, oy), s.iy);
    s.tsz = __fmul_rn(__fsub_rn(dz < 0.0f ? 0.0f : 1.0f, oz), s.iz);
    // An origin strictly inside the clip box never clips: per axis l - o < 0 < h - o,
    // so min(t1, t2) is negative (or -inf, or NaN when dir is NaN, which minps/maxps
    // drop) and tmin <= 0 on every path.  Camera rays of a view share the origin, so
    // the slab test below runs only for views from outside the world.
    bool clip = false;
    float tmin = 0.0f;
    bool origin_ok = true;
    if (!inside_safe && !origin_inside_safe(w, ox, oy, oz, wox, woy, woz)) {
        // clip box [1 - worldOrigin, size - 1 - worldOrigin] (VoxelTraversal.glsl:166)
        const float lx = __int2float_rn(1 - wox), ly = __int2float_rn(1 - woy), lz = __int2float_rn(1 - woz);
        const float hx = __fsub_rn(__fsub_rn(__uint2float_rn(w.size_x), __int2float_rn(wox)), 1.0f);
        const float hy = __fsub_rn(__fsub_rn(__uint2float_rn(w.size_y), __int2float_rn(woy)), 1.0f);
        const float hz = __fsub_rn(__fsub_rn(__uint2float_rn(w.size_z), __int2float_rn(woz)), 1.0f);
        const float t1x = __fmul_rn(__fsub_rn(lx, ox), s.ix);
        const float t1y = __fmul_rn(__fsub_rn(ly, oy), s.iy);
        const float t1z = __fmul_rn(__fsub_rn(lz, oz), s.iz);
        const float t2x = __fmul_rn(__fsub_rn(hx, ox), s.ix);
        const float t2y = __fmul_rn(__fsub_rn(hy, oy), s.iy);
        const float t2z = __fmul_rn(__fsub_rn(hz, oz), s.iz);
        tmin = max_x86(min_x86(t1x, t2x), max_x86(min_x86(t1y, t2y), min_x86(t1z, t2z)));
        const float tmax = min_x86(max_x86(t1x, t2x), min_x86(max_x86(t1y, t2y), max_x86(t1z, t2z)));
        clip = tmin > 0.0f && tmin < tmax;
        origin_ok = fabsf(ox) < kSafeOrigin && fabsf(oy) < kSafeOrigin && fabsf(oz) < kSafeOrigin;
    }
    s.cx = clip ? __fadd_rn(ox, __fmul_rn(dx, tmin)) : ox;
    s.cy = clip ? __fadd_rn(oy, __fmul_rn(dy, tmin)) : oy;
    s.cz = clip ? __fadd_rn(oz, __fmul_rn(dz, tmin)) : oz;
    s.sx = s.sy = s.sz = 0.0f;
    s.vx = s.vy = s.vz = INT32_MIN;
    s.gx = dx < 0.0f ? -1 : 0;
    s.gy = dy < 0.0f ? -1 : 0;
    s.gz = dz < 0.0f ? -1 : 0;
    s.material = 0;
    return origin_ok && fabsf(s.ix) < kSafeInvDir && fabsf(s.iy) < kSafeInvDir && fabsf(s.iz) < kSafeInvDir;
}

// GLSL mode (VoxelTraversal.glsl rayCast): the start voxel worldOrigin + floor(start),
// from which iteration 0 takes its side distances (:164-167).
template <bool kGlsl>
// coarse_origin (GLSL mode, a rayCastCoarse ray): the clipped start replaces the origin,
// so tStart, positions and the hit distance count from it (VoxelTraversal.glsl:207-210);
// rayCast keeps the origin and starts from the clipped voxel only (:162-167).  Without
// a clip the start is the origin and nothing changes.
__device__ __forceinline__ bool ray_start(RayState& s, const DevWorld& w, float ox, float oy, float oz, float dx,
                                          float dy, float dz, int32_t wox, int32_t woy, int32_t woz,
                                          bool inside_safe = false, bool coarse_origin = false) {
    const bool safe = ray_init(s, w, ox, oy, oz, dx, dy, dz, wox, woy, woz, inside_safe);
    if (kGlsl && coarse_origin) {
        s.ox = s.cx;
        s.oy = s.cy;
        s.oz = s.cz;
        s.tsx = __fmul_rn(__fsub_rn(dx < 0.0f ? 0.0f : 1.0f, s.ox), s.ix);
        s.tsy = __fmul_rn(__fsub_rn(dy < 0.0f ? 0.0f : 1.0f, s.oy), s.iy);
        s.tsz = __fmul_rn(__fsub_rn(dz < 0.0f ? 0.0f : 1.0f, s.oz), s.iz);
    }
    if (kGlsl) {
        s.vx = wadd(wox, floor2i(s.cx));
        s.vy = wadd(woy, floor2i(s.cy));
        s.vz = wadd(woz, floor2i(s.cz));
        s.tb = 0.0f;
    }
    return safe;
}

enum : uint32_t { kStepContinue = 0, kStepHit = 1, kStepOut = 2 };

// Anisotropic LODs: RayCellInteractionMaskLUT (GpuRenderer.cpp:193-210) in shared
// memory, entry idx + 64 * octant (octant = (dx >= 0) | (dy >= 0) << 1 | (dz >= 0) << 2),
// [0] the forward box of cell idx and [1] its part inside idx's aligned 2^3 block, so
// that getIsotropicLod of the masked mask (VoxelTraversal.glsl:24-34) is two tests.
// Every kernel that traces with anisotropic LODs fills it first (fill_forward_lut).
#if defined(__CUDACC__)
static __shared__ uint64_t s_forward_lut[2][512];
#else
inline uint64_t s_forward_lut[2][512];
#endif

__device__ __forceinline__ void fill_forward_lut_entries(uint32_t first, uint32_t step) {
    for (uint32_t i = first; i < 512; i += step) {
        const uint32_t idx = i & 63u, o = i >> 6;
        const uint64_t f = forward_cells(idx, (o & 1u) ? 0 : -1, (o & 2u) ? 0 : -1, (o & 4u) ? 0 : -1);
        s_forward_lut[0][i] = f;
        s_forward_lut[1][i] = f & (0x330033ull << (idx & 0x2Au));
    }
}

#if defined(__CUDACC__)
// all threads of the block, before any of them returns
__device__ __forceinline__ void fill_forward_lut() {
    fill_forward_lut_entries(threadIdx.x + threadIdx.y * blockDim.x, blockDim.x * blockDim.y);
    __syncthreads();
}
#endif

// GLSL mode: rayCastCoarse (VoxelTraversal.glsl:206-240), the GPU renderer's shadow and
// bounce rays (VoxelRender.comp:56,74,81): kCoarseRay for every step of such a ray,
// kCoarseNow from its iteration 31 on (`coarse = i > 30`, :218).
enum : uint32_t { kCoarseRay = 1, kCoarseNow = 2 };
constexpr uint32_t kCoarseFrom = 31, kCoarseMaxIters = 96;
__device__ __forceinline__ uint32_t coarse_bits(bool coarse_ray, uint32_t i) {
    return coarse_ray ? (kCoarseRay | (i >= kCoarseFrom ? kCoarseNow : 0u)) : 0u;
}

// One iteration of RayCast (CpuRenderer.cpp:186-201) with GetStepPos (:135-171).
// kSafe: the ray passed the bounds of ray_init, so no NaN can occur; the NaN test
// is skipped and min uses fminf, which equals the minps rule on non-NaN operands up
// to the sign of a zero result, which the +0.001 bias removes.
// kGlsl: one iteration of rayCast (VoxelTraversal.glsl:170-199) instead: side
// distances of the current voxel, tmin + 5 ulp (kept as the hit distance, so min
// keeps the minps rule), position, bounds, then getStepPos (:100-131) whose empty
// sectors take the 4th-level mask from the brick table.  kCoarse (with kGlsl): the
// step may belong to a rayCastCoarse ray, as `coarse` (coarse_bits) says: tmin + 0.001
// (:213) instead, and from iteration 31 an empty voxel whose 4^3 cell holds a solid
// voxel stops the ray at the cell's first solid voxel in mask order (getStepPos with
// coarse, :125-128, and findAnyOccupiedPos, :41-53).  Without kCoarse `coarse` is 0.
// kAniso (with kGlsl): anisotropic LODs (u_UseAnisotropicLods, :116-121): the mask of
// the current level (cell, sector or sector group, read raw instead of through the
// precomputed codes) is restricted to the cells ahead of the ray before its LOD is taken.
template <bool kCount, bool kSafe = false, bool kGlsl = false, bool kCoarse = false, bool kAniso = false>
__device__ __forceinline__ uint32_t ray_step(RayState& s, const DevWorld& w, int32_t wox, int32_t woy, int32_t woz,
                                             TraceCounters& cnt, uint32_t coarse = 0) {
    if (kGlsl) {
        s.sx = __fadd_rn(s.tsx, __fmul_rn(rel_voxel(s.vx, wox), s.ix));
        s.sy = __fadd_rn(s.tsy, __fmul_rn(rel_voxel(s.vy, woy), s.iy));
        s.sz = __fadd_rn(s.tsz, __fmul_rn(rel_voxel(s.vz, woz), s.iz));
        // +5 ulp as an integer add on the bits; a NaN tmin stays NaN (its bit pattern
        // differs between platforms: the GPU's 0x7FFFFFFF would wrap to a denormal)
        const float m = min_x86(min_x86(s.sx, s.sy), s.sz);
        const float t = (kCoarse && (coarse & kCoarseRay)) ? __fadd_rn(m, 0.001f)
                        : (!kSafe && m != m) ? m
                                             : __uint_as_float(__float_as_uint(m) + 5u);
        s.tb = t;
        s.cx = __fadd_rn(s.ox, __fmul_rn(t, s.dx));
        s.cy = __fadd_rn(s.oy, __fmul_rn(t, s.dy));
        s.cz = __fadd_rn(s.oz, __fmul_rn(t, s.dz));
    }
    // floor2i: a NaN coordinate converts to INT32_MIN on x86 and leaves the grid;
    // cvt.rmi saturates infinities and out-of-range values, which leave the grid
    // too (|world origin| <= 2^30 is enforced at the API), so only NaN needs a test
    // and one NaN among the three shows in their sum.
    if (!kSafe) {
        const float nan_probe = __fadd_rn(__fadd_rn(s.cx, s.cy), s.cz);
        if (nan_probe != nan_probe) {
            s.vx = s.vy = s.vz = INT32_MIN;
            return kStepOut;
        }
    }
    int32_t vx = (int32_t)imad((uint32_t)__float2int_rd(s.cx), 1u, (uint32_t)wox);
    int32_t vy = (int32_t)imad((uint32_t)__float2int_rd(s.cy), 1u, (uint32_t)woy);
    int32_t vz = (int32_t)imad((uint32_t)__float2int_rd(s.cz), 1u, (uint32_t)woz);
    if (!((uint32_t)vx < w.size_x && (uint32_t)vy < w.size_y && (uint32_t)vz < w.size_z)) {
        s.vx = vx;
        s.vy = vy;
        s.vz = vz;
        return kStepOut;
    }
    if (kCount) cnt.step_calls++;
    // The brick table holds the slot of an allocated brick, or for an empty one the
    // alignment mask of the level GetStepPos reaches from the sector mask
    // (3 + skip_levels).  An allocated brick's voxel code is kCodeSolid (the hit) or
    // the alignment mask of the skip level of the voxel's 4^3 cell; both replace the
    // two mask fetches of the reference with their precomputed outcome.
    const uint32_t bx = (uint32_t)vx >> 3, by = (uint32_t)vy >> 3, bz = (uint32_t)vz >> 3;
    const uint32_t e = __ldg(w.bricks + bx + bz * w.bsx + by * w.bsxz);
    int32_t m;
    if (kGlsl && kAniso) {
        if (e < kBrickEmpty) {
            if (kCount) cnt.occ_fetches++;
            const uint32_t lx = (uint32_t)vx & 7u, ly = (uint32_t)vy & 7u, lz = (uint32_t)vz & 7u;
            const uint64_t cm = __ldg(w.cells + (size_t)e * 8 + ((lx >> 2) | (lz >> 2) << 1 | (ly >> 2) << 2));
            const uint32_t idx = (lx & 3u) | (lz & 3u) << 2 | (ly & 3u) << 4;
            if ((cm >> idx) & 1u) {
                s.material = __ldg(w.payload + (size_t)e * 512 + (lx | lz << 3 | ly << 6));
                s.vx = vx;
                s.vy = vy;
                s.vz = vz;
                return kStepHit;
            }
            const uint32_t li = idx + 64u * ((uint32_t)(s.gx + 1) | (uint32_t)(s.gy + 1) << 1 | (uint32_t)(s.gz + 1) << 2);
            const uint64_t am = cm & s_forward_lut[0][li];
            if (kCoarse && (coarse & kCoarseNow) && am != 0) {
                // findAnyOccupiedPos on the masked cell mask: its lowest set bit
                const uint32_t j = (uint32_t)__ffsll((long long)am) - 1u;
                s.vx = (vx & ~3) | (int32_t)(j & 3u);
                s.vy = (vy & ~3) | (int32_t)(j >> 4);
                s.vz = (vz & ~3) | (int32_t)((j >> 2) & 3u);
                s.material = __ldg(w.payload + (size_t)e * 512 +
                                   (((uint32_t)s.vx & 7u) | ((uint32_t)s.vz & 7u) << 3 | ((uint32_t)s.vy & 7u) << 6));
                return kStepHit;
            }
            m = am == 0 ? 3 : ((cm & s_forward_lut[1][li]) == 0 ? 1 : 0);
        } else {
            // an empty brick: the sector mask (scale 8) or, in an empty sector, the
            // sector-group mask (scale 32) restricted to the ray's octant, whose skip level
            // the table entry carries per octant
            const uint32_t oct2 = ((uint32_t)(s.gx + 1) | (uint32_t)(s.gy + 1) << 1 | (uint32_t)(s.gz + 1) << 2) * 2u;
            const uint32_t skip = ((e >> (kAnisoShift + oct2)) & 3u) + ((e >> 4) & 2u);
            m = (int32_t)((8u << skip) - 1u);
        }
    } else if (e < kBrickEmpty) {
        if (kCount) cnt.occ_fetches++;
        // voxel in brick v = x | z<<3 | y<<6 from v - 8*(v >> 3) per axis; its code byte
        const uint32_t lx = imad(bx, 0xFFFFFFF8u, (uint32_t)vx), ly = imad(by, 0xFFFFFFF8u, (uint32_t)vy),
                       lz = imad(bz, 0xFFFFFFF8u, (uint32_t)vz);
        const uint32_t vi = imad(ly, 64u, imad(lz, 8u, lx));
        const uint32_t code = __ldg(w.codes + (size_t)e * 512 + vi);
        if (code == kCodeSolid) {
            s.material = __ldg(w.payload + (size_t)e * 512 + vi);
            s.vx = vx;
            s.vy = vy;
            s.vz = vz;
            return kStepHit;
        }
        if (kGlsl && kCoarse && (coarse & kCoarseNow) && code != 3u) {
            // the cell's mask is not empty (lod < 4): its first solid voxel, bit
            // x + z*4 + y*16 of the cell mask, is the hit (mask-order scan of the payload)
            const uint8_t* cell = w.payload + (size_t)e * 512 + ((lx & 4u) | (lz & 4u) << 3 | (ly & 4u) << 6);
            for (uint32_t j = 0; j < 64; j++) {
                const uint32_t mat = __ldg(cell + ((j & 3u) | ((j >> 2) & 3u) << 3 | (j >> 4) << 6));
                if (mat) {
                    s.material = mat;
                    s.vx = (vx & ~3) | (int32_t)(j & 3u);
                    s.vy = (vy & ~3) | (int32_t)(j >> 4);
                    s.vz = (vz & ~3) | (int32_t)((j >> 2) & 3u);
                    return kStepHit;
                }
            }
        }
        m = (int32_t)code;
    } else {
        m = kGlsl ? (int32_t)((e >> 8) & 127u) : (int32_t)(e & 31u);
    }
    // dir < 0 ? pos & ~m : pos | m, as (pos | m) ^ (g & m) with g = -1 for dir < 0
    vx = (vx | m) ^ (s.gx & m);
    vy = (vy | m) ^ (s.gy & m);
    vz = (vz | m) ^ (s.gz & m);
    if (kGlsl) {  // the next GLSL iteration starts from this voxel
        s.vx = vx;
        s.vy = vy;
        s.vz = vz;
        return kStepContinue;
    }
    // (the CPU loop needs the voxel only in the record of a hit or of a ray that left the
    // grid, whose paths above set it)
    s.sx = __fadd_rn(s.tsx, __fmul_rn(rel_voxel(vx, wox), s.ix));
    s.sy = __fadd_rn(s.tsy, __fmul_rn(rel_voxel(vy, woy), s.iy));
    s.sz = __fadd_rn(s.tsz, __fmul_rn(rel_voxel(vz, woz), s.iz));
    const float t = kSafe ? __fadd_rn(fminf(fminf(s.sx, s.sy), s.sz), 0.001f)
                          : __fadd_rn(min_x86(min_x86(s.sx, s.sy), s.sz), 0.001f);
    s.cx = __fadd_rn(s.ox, __fmul_rn(t, s.dx));
    s.cy = __fadd_rn(s.oy, __fmul_rn(t, s.dy));
    s.cz = __fadd_rn(s.oz, __fmul_rn(t, s.dz));
    return kStepContinue;
}

// Steps k = k .. kmax-1 of a ray whose first step here is its iteration i0 + k, until
// one ends it (the returned status) or kmax is reached (kStepContinue).  safe: the
// fast step (ray_init's bounds hold); coarse_ray: a rayCastCoarse ray (kCoarse only).
template <bool kCount, bool kGlsl, bool kCoarse, bool kAniso>
__device__ __forceinline__ uint32_t dda_steps(RayState& s, const DevWorld& w, int32_t wox, int32_t woy, int32_t woz,
                                              TraceCounters& cnt, bool safe, bool coarse_ray, uint32_t i0,
                                              uint32_t& k, uint32_t kmax) {
    uint32_t st = kStepContinue;
    if (safe) {
        for (; k < kmax; k++) {
            st = ray_step<kCount, true, kGlsl, kCoarse, kAniso>(s, w, wox, woy, woz, cnt,
                                                                kCoarse ? coarse_bits(coarse_ray, i0 + k) : 0u);
            if (st != kStepContinue) break;
        }
    } else {
        for (; k < kmax; k++) {
            st = ray_step<kCount, false, kGlsl, kCoarse, kAniso>(s, w, wox, woy, woz, cnt,
                                                                 kCoarse ? coarse_bits(coarse_ray, i0 + k) : 0u);
            if (st != kStepContinue) break;
        }
    }
    return st;
}

// dda_steps with the GLSL variants picked at run time: coarse (some ray of the caller's
// group may be a rayCastCoarse ray; coarse_ray says whether this one is) and aniso.
template <bool kCount, bool kGlsl>
__device__ __forceinline__ uint32_t dda_steps_mode(RayState& s, const DevWorld& w, int32_t wox, int32_t woy,
                                                   int32_t woz, TraceCounters& cnt, bool safe, bool coarse,
                                                   bool coarse_ray, bool aniso, uint32_t i0, uint32_t& k,
                                                   uint32_t kmax) {
    if constexpr (!kGlsl) {
        return dda_steps<kCount, false, false, false>(s, w, wox, woy, woz, cnt, safe, false, i0, k, kmax);
    } else {
        if (aniso)
            return coarse ? dda_steps<kCount, true, true, true>(s, w, wox, woy, woz, cnt, safe, coarse_ray, i0, k, kmax)
                          : dda_steps<kCount, true, false, true>(s, w, wox, woy, woz, cnt, safe, false, i0, k, kmax);
        return coarse ? dda_steps<kCount, true, true, false>(s, w, wox, woy, woz, cnt, safe, coarse_ray, i0, k, kmax)
                      : dda_steps<kCount, true, false, false>(s, w, wox, woy, woz, cnt, safe, false, i0, k, kmax);
    }
}

// Whole RayCast (or rayCast / rayCastCoarse, kGlsl) for one ray.
template <bool kCount, bool kGlsl = false>
__device__ __forceinline__ void trace_ray(const DevWorld& w, float ox, float oy, float oz, float dx, float dy,
                                          float dz, int32_t wox, int32_t woy, int32_t woz, uint32_t max_iters,
                                          TraceResult& r, TraceCounters& cnt, bool coarse_ray = false,
                                          bool aniso = false) {
    RayState s;
    const bool safe = ray_start<kGlsl>(s, w, ox, oy, oz, dx, dy, dz, wox, woy, woz, false, coarse_ray);
    uint32_t i = 0;
    uint32_t st = dda_steps_mode<kCount, kGlsl>(s, w, wox, woy, woz, cnt, safe, coarse_ray, coarse_ray, aniso, 0, i,
                                                max_iters);
    if (max_iters == 0) st = kStepOut;
    r.cx = s.cx;
    r.cy = s.cy;
    r.cz = s.cz;
    r.sx = s.sx;
    r.sy = s.sy;
    r.sz = s.sz;
    r.tb = s.tb;
    r.vx = s.vx;
    r.vy = s.vy;
    r.vz = s.vz;
    r.steps = i;  // == max_iters when the cap ran out
    r.material = s.material;
    r.hit = st == kStepHit && i < max_iters;
}

// The 16-byte vrt_hit record as one vector store.  kGlsl: t is the biased tmin and
// the face the first axis with tmin >= side (hit.normal's sideMask, VoxelTraversal.glsl:190).
template <bool kGlsl = false>
__device__ __forceinline__ uint4 pack_hit(const TraceResult& r, float dx, float dy, float dz, uint32_t tag) {
    if (!r.hit) return make_uint4(VRT_MISS_VOXEL, VRT_MISS_FACE | (r.steps << 16), 0x7F800000u, tag);
    float t;
    uint32_t face;
    if (kGlsl) {
        t = r.tb;
        if (t >= r.sx)
            face = dx < 0.0f ? 1u : 0u;
        else if (t >= r.sy)
            face = dy < 0.0f ? 3u : 2u;
        else
            face = dz < 0.0f ? 5u : 4u;
    } else {
        t = min_x86(min_x86(r.sx, r.sy), r.sz);
        if (r.sx == t)
            face = dx < 0.0f ? 1u : 0u;
        else if (r.sy == t)
            face = dy < 0.0f ? 3u : 2u;
        else
            face = dz < 0.0f ? 5u : 4u;
    }
    const uint32_t voxel = (uint32_t)r.vx | (uint32_t)r.vy << 11 | (uint32_t)r.vz << 21;
    return make_uint4(voxel, face | r.material << 8 | r.steps << 16, __float_as_uint(t), tag);
}

__device__ __forceinline__ uint4 no_ray_hit() {
    return make_uint4(VRT_MISS_VOXEL, VRT_MISS_FACE, 0x7F800000u, VRT_NO_RAY);
}

// HitResult.Normal (CpuRenderer.cpp:213-217) and origin = Pos + Normal*0.01 (:389).
// kGlsl: hit.normal = mix(0, -sign(dir), tmin >= sideDist) (VoxelTraversal.glsl:190-192),
// every axis within the bias, sign(+-0) = 0.
template <bool kGlsl = false>
__device__ __forceinline__ void secondary_origin(const TraceResult& r, float dx, float dy, float dz, float& ox,
                                                 float& oy, float& oz, float& nx, float& ny, float& nz) {
    if (kGlsl) {
        nx = r.tb >= r.sx ? (dx > 0.0f ? -1.0f : (dx < 0.0f ? 1.0f : 0.0f)) : 0.0f;
        ny = r.tb >= r.sy ? (dy > 0.0f ? -1.0f : (dy < 0.0f ? 1.0f : 0.0f)) : 0.0f;
        nz = r.tb >= r.sz ? (dz > 0.0f ? -1.0f : (dz < 0.0f ? 1.0f : 0.0f)) : 0.0f;
    } else {
        const float t = min_x86(min_x86(r.sx, r.sy), r.sz);
        const bool mx = r.sx == t, my = r.sy == t, mz = !mx && !my;
        nx = mx ? (signbit(dx) ? 1.0f : -1.0f) : 0.0f;
        ny = my ? (signbit(dy) ? 1.0f : -1.0f) : 0.0f;
        nz = mz ? (signbit(dz) ? 1.0f : -1.0f) : 0.0f;
    }
    ox = __fadd_rn(r.cx, __fmul_rn(nx, 0.01f));
    oy = __fadd_rn(r.cy, __fmul_rn(ny, 0.01f));
    oz = __fadd_rn(r.cz, __fmul_rn(nz, 0.01f));
}

}  // namespace vrt

namespace vrt {

// PCG32 (O'Neill, pcg-random.org: 64-bit LCG state, XSH-RR output).
struct DevPcg32 {
    uint64_t state, inc;
    __device__ __forceinline__ DevPcg32(uint64_t initstate, uint64_t initseq) {
        state = 0;
        inc = (initseq << 1) | 1u;
        next();
        state += initstate;
        next();
    }
    __device__ __forceinline__ uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
        const uint32_t rot = (uint32_t)(old >> 59);
        return (xs >> rot) | (xs << ((32 - rot) & 31));
    }
    // uniform in [-1, 1) with 2^-23 spacing; every op exact
    __device__ __forceinline__ float next_signed() {
        return __fsub_rn(__fmul_rn(__uint2float_rn(next() >> 8), 0x1p-23f), 1.0f);
    }
};

constexpr uint64_t kBounceStream = 0x9E3779B97F4A7C15ULL;

// Lambertian bounce normalize(n + s), s uniform on the sphere by rejection from the
// cube (the structure of CpuRenderer.cpp:392 with IEEE-exact sampling).
__device__ __forceinline__ void bounce_dir(uint32_t pixel, uint32_t bounce, float nx, float ny, float nz, float& dx,
                                           float& dy, float& dz) {
    DevPcg32 rng(pixel ^ bounce, kBounceStream);
    for (int attempt = 0; attempt < 64; attempt++) {
        const float x = rng.next_signed(), y = rng.next_signed(), z = rng.next_signed();
        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
        if (!(r2 > 1e-6f && r2 <= 1.0f)) continue;
        const float r = __fsqrt_rn(r2);
        const float ax = __fadd_rn(nx, __fdiv_rn(x, r)), ay = __fadd_rn(ny, __fdiv_rn(y, r)),
                    az = __fadd_rn(nz, __fdiv_rn(z, r));
        const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)), __fmul_rn(az, az));
        if (!(l2 > 1e-12f)) continue;
        const float l = __fsqrt_rn(l2);
        dx = __fdiv_rn(ax, l);
        dy = __fdiv_rn(ay, l);
        dz = __fdiv_rn(az, l);
        return;
    }
    const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz)));
    dx = __fdiv_rn(nx, l);
    dy = __fdiv_rn(ny, l);
    dz = __fdiv_rn(nz, l);
}

// Hit record from a finished RayState (steps = iteration index at exit).
template <bool kGlsl = false>
__device__ __forceinline__ uint4 pack_state(const RayState& s, bool hit, uint32_t steps, uint32_t tag) {
    TraceResult r;
    r.sx = s.sx;
    r.sy = s.sy;
    r.sz = s.sz;
    r.tb = s.tb;
    r.vx = s.vx;
    r.vy = s.vy;
    r.vz = s.vz;
    r.steps = steps;
    r.material = s.material;
    r.hit = hit;
    return pack_hit<kGlsl>(r, s.dx, s.dy, s.dz, tag);
}

// Where the secondary rays of a hit start and the hit's normal (secondary_origin).
template <bool kGlsl = false>
__device__ __forceinline__ void hit_frame(const RayState& s, float& ox, float& oy, float& oz, float& nx, float& ny,
                                          float& nz) {
    TraceResult r;
    r.cx = s.cx;
    r.cy = s.cy;
    r.cz = s.cz;
    r.sx = s.sx;
    r.sy = s.sy;
    r.sz = s.sz;
    r.tb = s.tb;
    secondary_origin<kGlsl>(r, s.dx, s.dy, s.dz, ox, oy, oz, nx, ny, nz);
}

// The GPU renderer's whole path (VoxelRender.comp:51-86), a view with a sun direction
// and bounces: record plane k >= 1 holds a sun ray for k = 1, 3, 5 (after the primary
// hit and the first two bounce hits) and otherwise bounce k/2 (k <= 4) or k - 3
// (k >= 6).  Flag in ViewDev::path.
constexpr uint32_t kPathFull = 1u << 20;
__host__ __device__ __forceinline__ bool full_is_sun(uint32_t k) { return k <= 5u && (k & 1u); }
__host__ __device__ __forceinline__ uint32_t full_bounce(uint32_t k) { return k <= 4u ? k >> 1 : k - 3u; }

// Origin and direction of the next ray of a path after a hit: the shadow ray
// (kind 1 with shadows) or bounce `bounce` (1-based).
template <bool kGlsl = false>
__device__ __forceinline__ void next_path_ray(const RayState& s, bool shadow, const float* sun, uint32_t pixel,
                                              uint32_t bounce, float& ox, float& oy, float& oz, float& dx, float& dy,
                                              float& dz) {
    TraceResult r;
    r.cx = s.cx;
    r.cy = s.cy;
    r.cz = s.cz;
    r.sx = s.sx;
    r.sy = s.sy;
    r.sz = s.sz;
    r.tb = s.tb;
    float nx, ny, nz;
    secondary_origin<kGlsl>(r, s.dx, s.dy, s.dz, ox, oy, oz, nx, ny, nz);
    if (shadow) {
        dx = sun[0];
        dy = sun[1];
        dz = sun[2];
    } else {
        bounce_dir(pixel, bounce, nx, ny, nz, dx, dy, dz);
    }
}

}  // namespace vrt
