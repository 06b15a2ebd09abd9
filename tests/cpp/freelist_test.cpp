// freelist_test.cpp - the host brick-slot allocator of libvrt.so (vrt::FreeList,
// vrt::sector_alloc, vrt::sector_free) over runs of sector edits, for the comparison with
// the reference's own BrickSlotAllocator in tests/test_alloc_pin_cpu.py.
//
// Input file: u32 runs; per run u32 bounds_xz, u32 bounds_y, u32 n, then u32 sector[n],
// u64 add[n], u64 remove[n].  Output file: per run u32 base[n], u64 mask[n] (the sector's
// state after each op), u32 n_ranges, u32 (start, length)[n_ranges] (the free ranges at the
// end), u32 failed_op (n when every allocation found room).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "freelist.h"

template <typename T>
static bool get(std::FILE* f, T* p, size_t n) {
    return std::fread(p, sizeof(T), n, f) == n;
}
template <typename T>
static void put(std::FILE* f, const T* p, size_t n) {
    std::fwrite(p, sizeof(T), n, f);
}

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: freelist_test <ops file> <out file>\n");
        return 2;
    }
    std::FILE* in = std::fopen(argv[1], "rb");
    std::FILE* out = std::fopen(argv[2], "wb");
    if (!in || !out) return 2;
    uint32_t runs = 0;
    if (!get(in, &runs, 1)) return 2;
    for (uint32_t r = 0; r < runs; r++) {
        uint32_t hdr[3];
        if (!get(in, hdr, 3)) return 2;
        const uint32_t bxz = hdr[0], by = hdr[1], n = hdr[2];
        std::vector<uint32_t> sector(n), base(n, 0);
        std::vector<uint64_t> add(n), remove(n), mask(n, 0);
        if (!get(in, sector.data(), n) || !get(in, add.data(), n) || !get(in, remove.data(), n)) return 2;
        // the reference's arena: bounds_xz^2 * bounds_y sectors of 64 slots, slots 1..capacity
        vrt::FreeList fl(bxz * bxz * by * 64);
        std::vector<vrt::SectorSlots> slots(bxz * bxz * by);
        uint32_t failed = n;
        for (uint32_t i = 0; i < n; i++) {
            vrt::SectorSlots& s = slots.at(sector[i]);
            if (!vrt::sector_alloc(fl, s, add[i])) {
                failed = i;
                break;
            }
            vrt::sector_free(fl, s, remove[i]);
            base[i] = s.base;
            mask[i] = s.mask;
        }
        put(out, base.data(), n);
        put(out, mask.data(), n);
        const uint32_t nr = (uint32_t)fl.num_ranges();
        put(out, &nr, 1);
        for (const auto& kv : fl.ranges()) {
            const uint32_t pr[2] = {kv.first, kv.second};
            put(out, pr, 2);
        }
        put(out, &failed, 1);
    }
    std::fclose(in);
    std::fclose(out);
    return 0;
}
