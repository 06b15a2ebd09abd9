// glsl_driver.cpp - host entry points around the reference's traversal shaders compiled
// as C++ (oracle/glsl_pin/build_glsl.py): load one world into the shaders' buffers
// (ssbo_VoxelData, ssbo_VoxelOccupancy, the ray-cell LUT; GpuRenderer.cpp:45-167,
// 193-210) and cast rays through rayCast or rayCastCoarse.  Test infrastructure: used
// only by tests/golden/make_golden_glsl.py to record the pin of the GLSL mode.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "glsl_shim.h"

#include GLSL_TRAVERSAL_SOURCE

namespace {
std::vector<uint32_t> g_bricks;  // 4-byte words, as BrickData reads them
std::vector<uvec2> g_occupancy;
}  // namespace

extern "C" {

// The sizes this build was compiled for: sectors along x and z, sectors along y,
// voxels per brick edge.
void glsl_ref_dims(uint32_t* out) {
    out[0] = NUM_SECTORS_XZ;
    out[1] = NUM_SECTORS_Y;
    out[2] = BRICK_SIZE;
}

// base_slots, brick_masks: per sector (index x + z*XZ + y*XZ*XZ); sector_masks: per
// group of 4^3 sectors; bricks: 512 B per slot; occupancy: 8 cell masks per slot;
// lut: 512 entries, index cell + 64 * octant.  Palette entry i encodes id i.
void glsl_ref_load(const uint32_t* base_slots, const uint64_t* brick_masks, const uint64_t* sector_masks,
                   const uint8_t* bricks, uint64_t n_slots, const uint64_t* occupancy, const uint64_t* lut) {
    for (uint32_t i = 0; i < 256; i++) b_VoxelData.Palette[i].Data = uvec2(i, 0u);
    for (uint32_t s = 0; s < NUM_SECTORS; s++) {
        b_VoxelData.BaseSlots[s] = base_slots[s];
        b_VoxelData.BrickMasks[s] = uvec2((uint)brick_masks[s], (uint)(brick_masks[s] >> 32));
    }
    for (uint32_t g = 0; g < NUM_SECTORS / 64; g++)
        b_VoxelData.SectorMasks[g] = uvec2((uint)sector_masks[g], (uint)(sector_masks[g] >> 32));
    g_bricks.assign(n_slots * 128 + 1, 0u);
    std::memcpy(g_bricks.data(), bricks, n_slots * 512);
    b_VoxelData.BrickData = g_bricks.data();
    g_occupancy.resize(n_slots * 8 + 1);
    for (uint64_t i = 0; i < n_slots * 8; i++) g_occupancy[i] = uvec2((uint)occupancy[i], (uint)(occupancy[i] >> 32));
    b_VoxelOccupancy.Data = g_occupancy.data();
    for (uint32_t i = 0; i < 512; i++) RayCellInteractionMaskLUT[i] = uvec2((uint)lut[i], (uint)(lut[i] >> 32));
}

// rays: origin xyz, dir xyz per ray, relative to the world origin wo.  Per ray: hit
// flag, dist, pos (3), normal (3), iters (0xFFFFFFFF where the shader leaves it
// unset: the iteration cap ran out), material id.
void glsl_ref_cast(const float* rays, uint32_t n, const int32_t* wo, int coarse, int aniso, uint8_t* hit,
                   float* dist, float* pos, float* normal, uint32_t* iters, uint32_t* mat) {
    u_WorldOrigin = ivec3(wo[0], wo[1], wo[2]);
    u_UseAnisotropicLods = aniso != 0;
    for (uint32_t i = 0; i < n; i++) {
        const float* r = rays + 6 * (size_t)i;
        HitInfo h;
        std::memset(&h, 0, sizeof(h));
        h.iters = 0xFFFFFFFFu;
        h.dist = NAN;
        const vec3 o(r[0], r[1], r[2]), d(r[3], r[4], r[5]);
        const bool ok = coarse ? rayCastCoarse(o, d, h) : rayCast(o, d, h);
        hit[i] = ok ? 1 : 0;
        dist[i] = h.dist;
        pos[3 * i] = h.pos.x, pos[3 * i + 1] = h.pos.y, pos[3 * i + 2] = h.pos.z;
        normal[3 * i] = h.normal.x, normal[3 * i + 1] = h.normal.y, normal[3 * i + 2] = h.normal.z;
        iters[i] = h.iters;
        mat[i] = h.mat.Data.x;
    }
}

// A primary rayCast per ray and, for the rays that hit, the shadow ray the GPU renderer
// casts toward the sun (VoxelRender.comp:56: rayCastCoarse(hit.pos + hit.normal*0.01,
// sunDir, sunHit)).  Primary outputs as glsl_ref_cast; shadow: hit flag (2 where no
// shadow ray was cast), dist, iters (0xFFFFFFFF where unset), material id.
void glsl_ref_shadow(const float* rays, uint32_t n, const int32_t* wo, const float* sun, int aniso, uint8_t* hit,
                     float* dist, float* pos, float* normal, uint32_t* iters, uint32_t* mat, uint8_t* s_hit,
                     float* s_dist, uint32_t* s_iters, uint32_t* s_mat) {
    u_WorldOrigin = ivec3(wo[0], wo[1], wo[2]);
    u_UseAnisotropicLods = aniso != 0;
    const vec3 sunDir(sun[0], sun[1], sun[2]);
    for (uint32_t i = 0; i < n; i++) {
        const float* r = rays + 6 * (size_t)i;
        HitInfo h, sh;
        std::memset(&h, 0, sizeof(h));
        std::memset(&sh, 0, sizeof(sh));
        h.iters = sh.iters = 0xFFFFFFFFu;
        h.dist = sh.dist = NAN;
        const bool ok = rayCast(vec3(r[0], r[1], r[2]), vec3(r[3], r[4], r[5]), h);
        hit[i] = ok ? 1 : 0;
        dist[i] = h.dist;
        pos[3 * i] = h.pos.x, pos[3 * i + 1] = h.pos.y, pos[3 * i + 2] = h.pos.z;
        normal[3 * i] = h.normal.x, normal[3 * i + 1] = h.normal.y, normal[3 * i + 2] = h.normal.z;
        iters[i] = h.iters;
        mat[i] = h.mat.Data.x;
        s_hit[i] = 2;
        if (ok) s_hit[i] = rayCastCoarse(h.pos + h.normal * 0.01f, sunDir, sh) ? 1 : 0;
        s_dist[i] = sh.dist;
        s_iters[i] = sh.iters;
        s_mat[i] = sh.mat.Data.x;
    }
}
}
