// vrt_internal.h - shared host/device definitions of the device brickmap.
//
// Device layout of one world (all arrays in HBM, owned by the library):
//   sectors  dense table over the world's sector grid, 16-byte records
//            {mask lo, mask hi, base slot (0-based), flags}, index
//            x + z*SX + y*SX*SZ (the order of LinearIndexer3D, VoxelMap.h:95-97);
//            the storage of record: sync, edit, read-back and picking use it;
//   bricks   the brick table derived from it, one u32 per brick position of the
//            world, index bx + bz*BX + by*BX*BZ (BX = 4*SX, BZ = 4*SZ): the brick's
//            slot when its bit is set in the sector mask, else kBrickEmpty | the
//            alignment mask (1 << level) - 1 of the level GetStepPos reaches there,
//            level = 3 + skip_levels of the sector mask (CpuRenderer.cpp:139-167),
//            in bits 0-7, and in bits 8-15 the mask of the GLSL mode's getStepPos
//            (VoxelTraversal.glsl:100-131): the same where the sector holds a brick,
//            else (32 << skip_levels of the sector-group mask) - 1, cells of 32, 64
//            or 128 voxels; bit 5 and bits 15-30 hold the anisotropic LODs' skip
//            levels per ray octant (kAnisoGroupBit, kAnisoShift);
//   codes    voxel codes, one byte per voxel (512 B per brick slot), voxel
//            v = x | z<<3 | y<<6 at byte v (as the payload): kCodeSolid, or
//            for an empty voxel the alignment mask (1 << level) - 1 (0, 1 or 3) of
//            level = skip_levels of its 4^3 cell's occupancy mask (cell
//            cx | cz<<1 | cy<<2, bit vx + vz*4 + vy*16: UpdateOccupancy,
//            CpuRenderer.cpp:63-83, and GetStepPos :146-167);
//   payload  512 B of u8 voxel ids per brick slot, voxel x | z<<3 | y<<6;
//   cells    the 8 cell masks of each brick slot (UpdateOccupancy, cell cx | cz<<1 |
//            cy<<2, bit vx + vz*4 + vy*16), read only by the GLSL mode's anisotropic
//            LODs, which mask them per ray octant;
//   groups   per group of 4^3 sectors, bit x | z<<2 | y<<4 set per non-empty sector.
// A brick's slot is base + popcount(mask & ((1<<b)-1)) (VoxelMap.glsl:45-64,
// BrickSlotAllocator.h:37-41).  The traversal reads bricks, codes and payload
// only: one 4-byte load per step, one byte more on an allocated brick (the
// anisotropic LODs read the brick's 8-byte cell mask instead of its code byte).
#pragma once

#include <cstdint>

#include "../../include/vrt.h"

namespace vrt {

struct SectorRec {
    uint32_t mask_lo, mask_hi;
    uint32_t base;   // 0-based slot of the sector's first brick
    uint32_t flags;  // reserved
};
static_assert(sizeof(SectorRec) == 16, "sector record is one 16-byte load");

#if defined(__CUDACC__)
#define VRT_HD __host__ __device__
#else
#define VRT_HD
#endif

// Brick-table entry of an unallocated brick position; the low bits hold the mask.
constexpr uint32_t kBrickEmpty = 0x80000000u;
// Voxel code of a solid voxel (the masks of empty voxels are 0, 1 and 3).
constexpr uint32_t kCodeSolid = 2u;

// Extra levels GetStepPos skips at position idx (0..63) of an empty bit of the
// 64-bit mask (lo, hi): 2 when the whole mask is 0, 1 when the 2x2x2 block holding
// idx is empty (bits (idx & 0xA) + {0,1,4,5,16,17,20,21} of the half idx falls
// in), else 0 (CpuRenderer.cpp:157-159).
VRT_HD inline uint32_t skip_levels(uint32_t lo, uint32_t hi, uint32_t idx) {
    const uint32_t half = idx < 32 ? lo : hi;
    return (lo | hi) == 0 ? 2u : (((half >> (idx & 0xA)) & 0x00330033u) == 0 ? 1u : 0u);
}

// The 4^3 cells ahead of cell idx (x | z<<2 | y<<4) along the ray: on each axis idx's
// coordinate and above (dir >= 0) or and below (dir < 0); g = -1 where dir < 0.  The
// entry idx + octant*64 of RayCellInteractionMaskLUT (GpuRenderer.cpp:193-210, octant
// bit per axis set for dir >= 0, VoxelTraversal.glsl:119), built here from 4-bit
// ranges: x bits, spread to z rows at bits 4z and y planes at bits 16y.
VRT_HD inline uint64_t forward_cells(uint32_t idx, int32_t gx, int32_t gy, int32_t gz) {
    const uint32_t x = idx & 3u, z = (idx >> 2) & 3u, y = idx >> 4;
    const uint32_t xr = gx ? (0xFu >> (3u - x)) : ((0xFu << x) & 0xFu);
    const uint32_t zr = gz ? (0xFu >> (3u - z)) : ((0xFu << z) & 0xFu);
    const uint32_t yr = gy ? (0xFu >> (3u - y)) : ((0xFu << y) & 0xFu);
    const uint32_t zs = (zr & 1u) | (zr & 2u) << 3 | (zr & 4u) << 6 | (zr & 8u) << 9;
    const uint64_t ys = (uint64_t)(yr & 1u) | (uint64_t)(yr & 2u) << 15 | (uint64_t)(yr & 4u) << 30 |
                        (uint64_t)(yr & 8u) << 45;
    return (uint64_t)(xr * zs) * ys;
}

// An empty brick's table entry also carries what the anisotropic LODs need there:
// kAnisoGroupBit when its sector is empty (the step then works at the sector-group
// scale 32, else at the brick scale 8), and at bit kAnisoShift + 2*octant
// (octant = (dx >= 0) | (dy >= 0) << 1 | (dz >= 0) << 2) the skip level (0-2) of that
// level's mask restricted to forward_cells of the brick's (or sector's) index.
constexpr uint32_t kAnisoGroupBit = 1u << 5;
constexpr uint32_t kAnisoShift = 15;

// Kernel-side view of one world (passed by value or stored in a world table).
struct alignas(16) DevWorld {
    const uint32_t* bricks;
    const uint8_t* codes;
    const uint8_t* payload;
    const SectorRec* sectors;
    uint32_t bsx, bsxz;               // brick-table strides: 4*SX, 4*SX * 4*SZ
    uint32_t size_x, size_y, size_z;  // voxels
    uint32_t sx, sz, sxz;             // sector-table strides
    const uint64_t* cells;            // 8 cell masks per brick slot (GLSL anisotropic LODs)
};
static_assert(sizeof(DevWorld) == 80, "world table entries are 80 bytes");

// World origins stay within +-2^30 so that saturated float->int conversions of
// far-away positions always land outside the grid (the traversal relies on it).
constexpr int32_t kMaxWorldOrigin = 1 << 30;
inline bool world_origin_ok(const int32_t wo[3]) {
    for (int c = 0; c < 3; c++)
        if (wo[c] > kMaxWorldOrigin || wo[c] < -kMaxWorldOrigin) return false;
    return true;
}

inline int32_t sector_index_pack(int32_t x, int32_t y, int32_t z) {
    return (int32_t)(((uint32_t)x & 4095u) | ((uint32_t)z & 4095u) << 12 | ((uint32_t)y & 255u) << 24);
}
inline void sector_index_unpack(int32_t idx, int32_t& x, int32_t& y, int32_t& z) {
    uint32_t u = (uint32_t)idx;
    x = (int32_t)(u << 20) >> 20;
    z = (int32_t)(u << 8) >> 20;
    y = (int32_t)u >> 24;
}

}  // namespace vrt
