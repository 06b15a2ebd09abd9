// ref_driver.cpp - TEST INFRASTRUCTURE.  Compiles the reference's own CPU traversal
// (src/VoxelRT/CpuRenderer.cpp) and host world model (src/VoxelRT/VoxelMap.cpp) in
// place from the reference checkout, with the shim headers of oracle/ref_pin/shim/
// standing in for GLM, ImGui and the OpenGL wrapper, and exposes a C entry point
// that runs the reference's static RayCast (CpuRenderer.cpp:172-224) over
// FlatVoxelStorage (CpuRenderer.cpp:20-84) filled through VoxelMap and SyncBuffers.
// The AVX-512 code only runs on x86-64; its outputs are committed as golden
// vectors (tests/golden/) that pin the portable oracle.  World files go through the
// reference's own VoxelMap::Serialize / Deserialize (VoxelMap.cpp:211-273) and
// BinaryIO.cpp framing, compiled in place with the system's libzstd.
#include "CpuRenderer.cpp"
#include "VoxelMap.cpp"
#include "BrickSlotAllocator.cpp"

#include <algorithm>
#include <stdexcept>
#include <vector>

#if !VRT_REF_BINARY_IO
// no libzstd: the world-file entry points below report failure
namespace glim::io {
void WriteCompressed(std::ostream&, const void*, size_t) { throw std::runtime_error("zstd is not available"); }
void ReadCompressed(std::istream&, void*, size_t) { throw std::runtime_error("zstd is not available"); }
}  // namespace glim::io
#endif

namespace {
struct RefWorld {
    std::shared_ptr<VoxelMap> map = std::make_shared<VoxelMap>();
    std::unique_ptr<FlatVoxelStorage> storage = std::make_unique<FlatVoxelStorage>();
};
}  // namespace

extern "C" {

uint32_t ref_lanes(void) { return simd::VectorWidth; }

// View extent of FlatVoxelStorage in sectors (x, y, z): CpuRenderer.cpp:14-16.
void ref_view_sectors(uint32_t out[3]) {
    out[0] = ViewSectorIndexer::SizeXZ;
    out[1] = ViewSectorIndexer::SizeY;
    out[2] = ViewSectorIndexer::SizeXZ;
}

void* ref_world_create(void) {
    auto* w = new RefWorld;
    // palette entry i encodes i in its RGB565 bits, so MaterialData & 0xFFFF is the voxel id
    for (uint32_t i = 0; i < 256; i++) {
        Material& m = w->map->Palette[i];
        m.Color[0] = 0;
        m.Color[1] = (uint8_t)((i >> 5) << 2);
        m.Color[2] = (uint8_t)((i & 31) << 3);
        m.Emission = 0.0f;
    }
    return w;
}

void ref_world_destroy(void* p) { delete static_cast<RefWorld*>(p); }

// Sector records (WorldSectorIndexer index, allocation mask, bricks in bit order)
// go into VoxelMap::Sectors and DirtyLocs; SyncBuffers then builds the flat layout.
int ref_world_load(void* p, uint32_t n, const int32_t* sector_idx, const uint64_t* masks, const uint8_t* bricks) {
    auto* w = static_cast<RefWorld*>(p);
    for (uint32_t i = 0; i < n; i++) {
        Sector& s = w->map->Sectors[(uint32_t)sector_idx[i]];
        for (uint64_t m = masks[i]; m; m &= m - 1) {
            uint32_t b = (uint32_t)std::countr_zero(m);
            std::memcpy(s.GetBrick(b, true)->Data, bricks, 512);
            bricks += 512;
        }
        w->map->DirtyLocs[(uint32_t)sector_idx[i]] |= masks[i];
    }
    w->storage->SyncBuffers(*w->map);
    return 0;
}

// RayCast over n rays in SIMD groups; per ray: hit flag, Pos (3), Normal (3),
// Distance, MaterialData.
int ref_raycast(void* p, uint64_t n, const float* origins, const float* dirs, const int32_t wo[3], uint8_t* hit,
                float* pos, float* normal, float* dist, int32_t* material) {
    auto* w = static_cast<RefWorld*>(p);
    const uint32_t L = simd::VectorWidth;
    for (uint64_t base = 0; base < n; base += L) {
        VFloat3 o, d;
        VMask mask = 0;
        for (uint32_t l = 0; l < L; l++) {
            uint64_t i = base + l < n ? base + l : n - 1;
            o.x[l] = origins[i * 3 + 0];
            o.y[l] = origins[i * 3 + 1];
            o.z[l] = origins[i * 3 + 2];
            d.x[l] = dirs[i * 3 + 0];
            d.y[l] = dirs[i * 3 + 1];
            d.z[l] = dirs[i * 3 + 2];
            if (base + l < n) mask |= (VMask)(1u << l);
        }
        VHitResult r = RayCast(*w->storage, o, d, mask, glm::ivec3(wo[0], wo[1], wo[2]));
        for (uint32_t l = 0; l < L && base + l < n; l++) {
            uint64_t i = base + l;
            hit[i] = (r.Mask >> l) & 1;
            pos[i * 3 + 0] = r.Pos.x[l];
            pos[i * 3 + 1] = r.Pos.y[l];
            pos[i * 3 + 2] = r.Pos.z[l];
            normal[i * 3 + 0] = r.Normal.x[l];
            normal[i * 3 + 1] = r.Normal.y[l];
            normal[i * 3 + 2] = r.Normal.z[l];
            dist[i] = r.Distance[l];
            material[i] = r.MaterialData[l];
        }
    }
    return 0;
}

// VoxelMap::Serialize (VoxelMap.cpp:246-273) of the loaded map to `path`; 0 or -1.
int ref_serialize(void* p, const char* path) {
    try {
        static_cast<RefWorld*>(p)->map->Serialize(path);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// A world read by VoxelMap::Deserialize (VoxelMap.cpp:211-244), or NULL when it throws.
void* ref_world_from_file(const char* path) {
    auto* w = new RefWorld;
    try {
        w->map->Deserialize(path);
    } catch (const std::exception&) {
        delete w;
        return nullptr;
    }
    return w;
}

// Sectors of the map in ascending index order: count, then (index, allocation mask,
// bricks in bit order) into the given arrays (bricks: total popcount x 512 bytes).
uint32_t ref_world_sector_count(void* p, uint64_t* n_bricks) {
    auto* w = static_cast<RefWorld*>(p);
    uint64_t nb = 0;
    for (auto& [idx, sector] : w->map->Sectors) nb += (uint64_t)std::popcount(sector.GetAllocationMask());
    *n_bricks = nb;
    return (uint32_t)w->map->Sectors.size();
}

void ref_world_export(void* p, int32_t* idx_out, uint64_t* mask_out, uint8_t* bricks_out) {
    auto* w = static_cast<RefWorld*>(p);
    std::vector<uint32_t> keys;
    for (auto& kv : w->map->Sectors) keys.push_back(kv.first);
    std::sort(keys.begin(), keys.end());
    for (uint32_t idx : keys) {
        Sector& sector = w->map->Sectors[idx];
        const uint64_t mask = sector.GetAllocationMask();
        *idx_out++ = (int32_t)idx;
        *mask_out++ = mask;
        for (uint64_t m = mask; m; m &= m - 1) {
            std::memcpy(bricks_out, sector.GetBrick((uint32_t)std::countr_zero(m))->Data, 512);
            bricks_out += 512;
        }
    }
}

// VoxelMap::RayCast (VoxelMap.cpp:140-170) on the loaded map; rays: 6 doubles each.
int ref_pick(void* p, uint64_t n, const double* rays, uint32_t max_iters, double* dist, float* normal, float* uv,
             int32_t* voxel) {
    auto* w = static_cast<RefWorld*>(p);
    for (uint64_t i = 0; i < n; i++) {
        const double* r = rays + i * 6;
        HitResult h = w->map->RayCast(glm::dvec3(r[0], r[1], r[2]), glm::dvec3(r[3], r[4], r[5]), max_iters);
        dist[i] = h.Distance;
        for (int c = 0; c < 3; c++) {
            normal[i * 3 + c] = h.Normal[c];
            voxel[i * 3 + c] = h.VoxelPos[c];
        }
        uv[i * 2 + 0] = h.UV.x;
        uv[i * 2 + 1] = h.UV.y;
    }
    return 0;
}

// The 4^3-cell occupancy masks FlatVoxelStorage::UpdateOccupancy (CpuRenderer.cpp:63-83)
// derived for the bricks at the given brick positions (x, y, z), 8 masks each in
// BrickMaskIndexer order; bricks outside the storage's view get zeros.
void ref_world_occupancy(void* p, uint32_t n, const int32_t* brick_pos, uint64_t* out) {
    auto* w = static_cast<RefWorld*>(p);
    for (uint32_t i = 0; i < n; i++) {
        const glm::ivec3 bp(brick_pos[3 * i], brick_pos[3 * i + 1], brick_pos[3 * i + 2]);
        const glm::ivec3 sp = bp >> glm::ivec3(MaskIndexer::ShiftXZ, MaskIndexer::ShiftY, MaskIndexer::ShiftXZ);
        uint64_t* o = out + 8 * (size_t)i;
        if (!ViewSectorIndexer::CheckInBounds(sp)) {
            for (int c = 0; c < 8; c++) o[c] = 0;
            continue;
        }
        const uint32_t view_idx = ViewSectorIndexer::GetIndex(sp);
        const uint32_t offset = view_idx * (sizeof(Brick) * 64) + MaskIndexer::GetIndex(bp) * sizeof(Brick);
        for (int c = 0; c < 8; c++) o[c] = w->storage->OccupancyStorage[offset / 64 + c];
    }
}

// Sphere edits through the reference's own region dispatch and brick GC:
// VoxelMap::RegionDispatchSIMD (VoxelMap.h:222-263) called as BrushSession::Dispatch calls
// it (Brush.cpp:10-31): region center -/+ radius, bricks created unless the edit erases,
// Replace restricted to non-empty voxels, set_if + any.  The capsule SDF of the brush is
// replaced by the library's exact integer sphere |v - center|^2 <= radius^2 (vrt_edit).
int ref_world_edit_spheres(void* p, uint32_t n, const int32_t* centers, const uint32_t* radii,
                           const uint8_t* materials, const uint8_t* modes) {
    auto* w = static_cast<RefWorld*>(p);
    for (uint32_t k = 0; k < n; k++) {
        const glm::ivec3 c(centers[3 * k], centers[3 * k + 1], centers[3 * k + 2]);
        const int32_t r = (int32_t)radii[k];
        const int32_t r2 = r * r;
        const uint8_t material = materials[k];
        const bool replace = modes[k] == 1;
        w->map->RegionDispatchSIMD(c - r, c + r, material != 0, [&](VoxelDispatchInvocationPars& invoc) {
            VInt dx = invoc.X - c.x, dy = invoc.Y - c.y, dz = invoc.Z - c.z;
            VMask mask = (dx * dx + dy * dy + dz * dz) <= r2;
            if (replace) mask &= invoc.VoxelIds != 0;
            invoc.VoxelIds.set_if(mask, (int32_t)material);
            return simd::any(mask);
        });
    }
    // the edited bricks reach the flat storage and their cell masks, as a frame's sync does
    w->storage->SyncBuffers(*w->map);
    return 0;
}

// BrickSlotAllocator (BrickSlotAllocator.cpp:5-94, .h:6-65) over a run of sector edits:
// op i adds the bricks add[i] to sector sector[i] (Alloc), then drops remove[i] (Free).
// After each op the sector's BaseSlot and AllocMask are recorded; at the end the free
// ranges (start, length), up to max_ranges of them.  The reference throws when no range
// fits, after freeing the sector's old range, so the run stops before such an op.
// Returns the number of ops run; *n_ranges receives the number of free ranges.
uint32_t ref_alloc_run(uint32_t bounds_xz, uint32_t bounds_y, uint32_t n, const uint32_t* sector, const uint64_t* add,
                       const uint64_t* remove, uint32_t* base_out, uint64_t* mask_out, uint32_t* ranges_out,
                       uint32_t max_ranges, uint32_t* n_ranges) {
    BrickSlotAllocator alloc(glm::uvec2(bounds_xz, bounds_y));
    const uint32_t n_sectors = alloc.Arena.Capacity / 64;
    uint32_t i = 0;
    for (; i < n; i++) {
        if (sector[i] >= n_sectors) break;
        BrickSlotAllocator::SectorInfo* s = &alloc.Sectors[sector[i]];
        // would Alloc find room? (the same test as FreeList::Realloc, without its side effects)
        const uint64_t nm = s->AllocMask | add[i];
        if (nm != s->AllocMask) {
            const uint32_t cur = (uint32_t)std::popcount(s->AllocMask), want = (uint32_t)std::popcount(nm);
            bool fits = false;
            if (s->BaseSlot != 0) {
                auto it = alloc.Arena.FreeRanges.lower_bound(s->BaseSlot);
                fits = it != alloc.Arena.FreeRanges.end() && it->first == s->BaseSlot + cur &&
                       s->BaseSlot + want < it->first + it->second;
            }
            uint32_t largest = 0;
            for (const auto& r : alloc.Arena.FreeRanges) largest = std::max(largest, r.second);
            // freeing the old range first can merge it with its neighbours
            if (!fits) {
                BrickSlotAllocator trial = BrickSlotAllocator(glm::uvec2(bounds_xz, bounds_y));
                trial.Arena.FreeRanges = alloc.Arena.FreeRanges;
                trial.Arena.NumAllocated = alloc.Arena.NumAllocated;
                if (s->BaseSlot != 0) trial.Arena.Free(s->BaseSlot, cur);
                largest = 0;
                for (const auto& r : trial.Arena.FreeRanges) largest = std::max(largest, r.second);
                fits = largest >= want;
            }
            if (!fits) break;
            alloc.Alloc(s, add[i]);
        }
        alloc.Free(s, remove[i]);
        base_out[i] = s->BaseSlot;
        mask_out[i] = s->AllocMask;
    }
    uint32_t k = 0;
    for (const auto& r : alloc.Arena.FreeRanges) {
        if (k < max_ranges) {
            ranges_out[2 * k] = r.first;
            ranges_out[2 * k + 1] = r.second;
        }
        k++;
    }
    *n_ranges = k;
    return i;
}

}  // extern "C"
