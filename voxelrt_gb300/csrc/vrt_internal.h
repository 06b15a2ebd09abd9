// vrt_internal.h - shared host/device definitions of the device brickmap.
//
// Device layout of one world (all arrays in HBM, owned by the library):
//   sectors  dense table over the world's sector grid, 16-byte records
//            {mask lo, mask hi, base slot (0-based), flags}, index
//            x + z*SX + y*SX*SZ (the order of LinearIndexer3D, VoxelMap.h:95-97);
//   occ      8 x u64 voxel-cell masks per brick slot (64 B, one line per brick),
//            cell c = cx | cz<<1 | cy<<2, bit vx + vz*4 + vy*16
//            (UpdateOccupancy, CpuRenderer.cpp:63-83);
//   payload  512 B of u8 voxel ids per brick slot, voxel x | z<<3 | y<<6.
// A brick's slot is base + popcount(mask & ((1<<b)-1)) (VoxelMap.glsl:45-64,
// BrickSlotAllocator.h:37-41).
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

// Kernel-side view of one world (passed by value or stored in a world table).
struct DevWorld {
    const SectorRec* sectors;
    const uint64_t* occ;
    const uint8_t* payload;
    uint32_t sx, sz;         // sectors along x and z
    uint32_t sxz;            // sx * sz
    uint32_t size_x, size_y, size_z;  // voxels
};

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
