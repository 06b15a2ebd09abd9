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
//            or 128 voxels;
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
// only: one 4-byte load per step, one byte more on an allocated brick.
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
    const uint64_t* groups;           // sector-group masks (GLSL anisotropic LODs)
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
