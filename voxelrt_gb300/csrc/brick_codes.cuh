// brick_codes.cuh - occupancy of one brick, derived by a warp from its 512 voxel bytes.
//
// UpdateOccupancy (CpuRenderer.cpp:63-83, Shaders/UpdateOccupancy.comp) builds eight
// 64-bit masks of 4^3-voxel cells per brick; GetStepPos (CpuRenderer.cpp:146-160)
// then tests the voxel's bit and, when it is clear, derives the skip level from the
// same mask.  Both are functions of the brick's bytes and the voxel position alone,
// so the device stores their result per voxel: a code byte, kCodeSolid, or the
// alignment mask (1 << level) - 1 of an empty voxel (vrt_internal.h has the layout).
#pragma once

#include <cstdint>

#include "vrt_internal.h"

namespace vrt {

// Round r tests, in lane l, voxel (4cx + (l&3), 4cy + 2h + (l>>4), 4cz + ((l>>2)&3)) of
// cell c = r>>1 (cx = c&1, cz = (c>>1)&1, cy = c>>2), half h = r&1, so the ballot is
// bits 32h..32h+31 of cell c's mask (bit vx + vz*4 + vy*16, CpuRenderer.cpp:78).
// Lane c < 8 returns cell c's 64-bit mask; the other lanes return 0.
__device__ __forceinline__ uint64_t warp_cell_mask(const uint8_t* sb, uint32_t lane) {
    uint64_t mine = 0;
#pragma unroll
    for (uint32_t r = 0; r < 16; r++) {
        const uint32_t c = r >> 1, h = r & 1;
        const uint32_t x = (c & 1) * 4 + (lane & 3);
        const uint32_t z = ((c >> 1) & 1) * 4 + ((lane >> 2) & 3);
        const uint32_t y = (c >> 2) * 4 + 2 * h + (lane >> 4);
        const uint32_t bits = __ballot_sync(0xffffffffu, sb[x | z << 3 | y << 6] != 0);
        if (lane == c) mine |= (uint64_t)bits << (32 * h);
    }
    return mine;
}

// 16-byte group `lane` of the brick's voxel codes (voxels 16*lane .. 16*lane+15, one
// byte each), given the brick in shared memory and the cell masks of warp_cell_mask.
// Lane l covers y = l>>2, z = 2(l&3) + (j>>3), x = j&7 for j = 0..15, so it needs the
// masks of cells (0, cz, cy) and (1, cz, cy).
__device__ __forceinline__ uint4 warp_voxel_codes(const uint8_t* sb, uint64_t cell_masks, uint32_t lane) {
    const uint32_t y = lane >> 2, z0 = 2 * (lane & 3);
    const uint32_t cbase = (z0 >> 2) << 1 | (y >> 2) << 2;
    const uint32_t lo0 = __shfl_sync(0xffffffffu, (uint32_t)cell_masks, cbase);
    const uint32_t hi0 = __shfl_sync(0xffffffffu, (uint32_t)(cell_masks >> 32), cbase);
    const uint32_t lo1 = __shfl_sync(0xffffffffu, (uint32_t)cell_masks, cbase | 1);
    const uint32_t hi1 = __shfl_sync(0xffffffffu, (uint32_t)(cell_masks >> 32), cbase | 1);
    uint32_t word[4] = {0, 0, 0, 0};
#pragma unroll
    for (uint32_t j = 0; j < 16; j++) {
        const uint32_t x = j & 7, z = z0 + (j >> 3);
        const uint32_t idx = (x & 3) | (z & 3) << 2 | (y & 3) << 4;  // bit in the cell mask
        const uint32_t level = x < 4 ? skip_levels(lo0, hi0, idx) : skip_levels(lo1, hi1, idx);
        const uint32_t code = sb[x | z << 3 | y << 6] != 0 ? kCodeSolid : (1u << level) - 1u;
        word[j >> 2] |= code << (8 * (j & 3));
    }
    return make_uint4(word[0], word[1], word[2], word[3]);
}

// Codes of an all-empty brick: every cell mask is 0, so every voxel skips 2 levels
// (mask 3 in every byte).
constexpr uint32_t kEmptyCodeWord = 0x03030303u;
__device__ __forceinline__ uint4 empty_brick_codes() {
    return make_uint4(kEmptyCodeWord, kEmptyCodeWord, kEmptyCodeWord, kEmptyCodeWord);
}

}  // namespace vrt
