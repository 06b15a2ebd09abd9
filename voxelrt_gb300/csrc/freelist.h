// freelist.h - brick-slot allocation for the device brick pool.
//
// Behaviour follows the reference's FreeList / BrickSlotAllocator
// (src/VoxelRT/BrickSlotAllocator.h:6-65, BrickSlotAllocator.cpp:5-94):
//   * slots are 1-based, 0 means "no allocation";
//   * a sector's bricks occupy one contiguous range; brick b sits at
//     base + popcount(mask & ((1 << b) - 1));
//   * Realloc grows in place when the free range right after the allocation is
//     strictly larger than the growth, otherwise frees the range and takes the
//     smallest free range that fits (first one on ties);
//   * Free returns the range tail and coalesces neighbours.
// Departures: a failed Realloc restores the previous allocation and returns 0
// (the reference throws after having freed it, BrickSlotAllocator.cpp:14-16),
// and the pool can grow (the GPU renderer instead rebuilds a bigger buffer,
// GpuRenderer.cpp:82-97).
#pragma once

#include <cstdint>
#include <map>
#include <utility>
#include <vector>

namespace vrt {

class FreeList {
  public:
    explicit FreeList(uint32_t capacity = 0) { reset(capacity); }

    void reset(uint32_t capacity) {
        ranges_.clear();
        capacity_ = capacity;
        allocated_ = 0;
        if (capacity) ranges_[1] = capacity;
    }
    // Make slots capacity+1 .. new_capacity free (coalesced with the tail).
    void grow(uint32_t new_capacity);
    // Allocate or grow [base, base+cur) to `want` slots. Returns the new base or 0.
    uint32_t realloc(uint32_t base, uint32_t cur, uint32_t want);
    void free(uint32_t base, uint32_t size);

    uint32_t capacity() const { return capacity_; }
    uint32_t allocated() const { return allocated_; }
    size_t num_ranges() const { return ranges_.size(); }
    const std::map<uint32_t, uint32_t>& ranges() const { return ranges_; }
    // Largest slot index in use + 1 (1 when nothing is allocated).
    uint32_t high_water() const;
    // Reset to `capacity` slots of which exactly the given ranges (1-based start, length;
    // sorted by start, disjoint) are allocated: the free ranges are the gaps between them.
    void assign_used(uint32_t capacity, const std::vector<std::pair<uint32_t, uint32_t>>& used);

  private:
    void take_front(std::map<uint32_t, uint32_t>::iterator it, uint32_t count);
    void take_exact(uint32_t start, uint32_t count);

    std::map<uint32_t, uint32_t> ranges_;  // start -> length of free ranges
    uint32_t capacity_ = 0;
    uint32_t allocated_ = 0;
};

// Per-sector allocation record (BrickSlotAllocator::SectorInfo, BrickSlotAllocator.h:33-42).
struct SectorSlots {
    uint32_t base = 0;  // 1-based, 0 = nothing allocated
    uint64_t mask = 0;
    uint32_t slot_of(uint32_t brick) const {
        return base + (uint32_t)__builtin_popcountll(mask & ((1ull << brick) - 1));
    }
};

// Sector-level operations of BrickSlotAllocator::Alloc/Free.  Both return false
// only when the pool has no fitting range (state is then unchanged).
bool sector_free(FreeList& fl, SectorSlots& s, uint64_t remove);
bool sector_alloc(FreeList& fl, SectorSlots& s, uint64_t add);

}  // namespace vrt
