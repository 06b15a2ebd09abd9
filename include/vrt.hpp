// vrt.hpp - C++ host-side mirror of the reference's storage and renderer interface,
// header-only, over the C ABI of vrt.h.
//
// A caller of the reference keeps its host world model and swaps the device side:
//   VoxelMap / Sector / Brick         src/VoxelRT/VoxelMap.h:9-264 (host model, DirtyLocs)
//   GpuVoxelStorage::SyncBuffers       src/VoxelRT/GpuRenderer.cpp:45-167
//   GpuRenderer::RenderFrame           src/VoxelRT/GpuRenderer.cpp:239-273 (hit records
//                                      instead of a G-buffer; no graphics API)
// Errors: every failing ABI call throws vrt::Error (std::runtime_error), as the
// reference throws on slot exhaustion (BrickSlotAllocator.cpp:14-16).
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "vrt.h"

namespace vrt {

struct Error : std::runtime_error {
    vrt_status status;
    Error(vrt_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(vrt_status s) {
    if (s != VRT_OK) throw Error(s, vrt_last_error());
}

struct IVec3 {
    int32_t x, y, z;
};

// ---- host world model (VoxelMap.h) ----

struct Voxel {
    uint8_t Data = 0;
    bool IsEmpty() const { return Data == 0; }
};

struct Brick {
    Voxel Data[512] = {};
    static uint32_t Index(int32_t x, int32_t y, int32_t z) { return (x & 7) | (z & 7) << 3 | (y & 7) << 6; }
    bool IsEmpty() const {
        for (const Voxel& v : Data)
            if (!v.IsEmpty()) return false;
        return true;
    }
};

// 4x4x4 bricks; slot table maps brick index -> 1-based storage slot (0 = absent).
struct Sector {
    std::vector<Brick> Storage;
    uint8_t BrickSlots[64] = {};

    static uint32_t Index(int32_t bx, int32_t by, int32_t bz) { return (bx & 3) | (bz & 3) << 2 | (by & 3) << 4; }

    Brick* GetBrick(uint32_t index, bool create = false) {
        uint8_t& slot = BrickSlots[index];
        if (slot) return &Storage[slot - 1];
        if (!create) return nullptr;
        Storage.emplace_back();
        slot = (uint8_t)Storage.size();
        return &Storage.back();
    }
    uint64_t GetAllocationMask() const {
        uint64_t m = 0;
        for (uint32_t i = 0; i < 64; i++) m |= (uint64_t)(BrickSlots[i] != 0) << i;
        return m;
    }
    // Drops the bricks in `mask`, compacting storage in brick order.
    void DeleteBricks(uint64_t mask) {
        const uint64_t keep = GetAllocationMask() & ~mask;
        std::vector<Brick> kept;
        kept.reserve((size_t)__builtin_popcountll(keep));
        uint8_t slots[64] = {};
        for (uint64_t r = keep; r; r &= r - 1) {
            const uint32_t b = (uint32_t)__builtin_ctzll(r);
            kept.push_back(Storage[BrickSlots[b] - 1]);
            slots[b] = (uint8_t)kept.size();
        }
        Storage = std::move(kept);
        std::memcpy(BrickSlots, slots, 64);
    }
};

// Sector map keyed by WorldSectorIndexer index, with the DirtyLocs set of
// bricks changed since the last SyncBuffers.
struct VoxelMap {
    std::unordered_map<uint32_t, Sector> Sectors;
    std::map<uint32_t, uint64_t> DirtyLocs;

    static uint32_t SectorKey(int32_t sx, int32_t sy, int32_t sz) { return (uint32_t)vrt_sector_index(sx, sy, sz); }

    Brick* GetBrick(IVec3 brickPos, bool create = false, bool markAsDirty = false) {
        const uint32_t key = SectorKey(brickPos.x >> 2, brickPos.y >> 2, brickPos.z >> 2);
        auto it = Sectors.find(key);
        if (it == Sectors.end()) {
            if (!create) return nullptr;
            it = Sectors.emplace(key, Sector{}).first;
        }
        const uint32_t b = Sector::Index(brickPos.x, brickPos.y, brickPos.z);
        if (markAsDirty) DirtyLocs[key] |= 1ull << b;
        return it->second.GetBrick(b, create);
    }
    Voxel Get(IVec3 p) {
        Brick* br = GetBrick({p.x >> 3, p.y >> 3, p.z >> 3});
        return br ? br->Data[Brick::Index(p.x, p.y, p.z)] : Voxel{};
    }
    void Set(IVec3 p, Voxel v) {
        Brick* br = GetBrick({p.x >> 3, p.y >> 3, p.z >> 3}, true, true);
        br->Data[Brick::Index(p.x, p.y, p.z)] = v;
    }
    void MarkAllDirty() {
        for (auto& kv : Sectors) DirtyLocs[kv.first] = kv.second.GetAllocationMask();
    }
    // Calls fn(x, y, z, voxel&) for every voxel of the bricks overlapping
    // [regionMin, regionMax] (voxel units); fn returns true when it changed the
    // voxel.  Bricks are created first when createEmpty; changed or empty bricks
    // are marked dirty and empty bricks are freed afterwards (RegionDispatchSIMD).
    template <typename F>
    void RegionDispatch(IVec3 regionMin, IVec3 regionMax, bool createEmpty, F&& fn) {
        std::map<uint32_t, uint64_t> empty;
        for (int32_t by = regionMin.y >> 3; by <= regionMax.y >> 3; by++)
            for (int32_t bz = regionMin.z >> 3; bz <= regionMax.z >> 3; bz++)
                for (int32_t bx = regionMin.x >> 3; bx <= regionMax.x >> 3; bx++) {
                    Brick* br = GetBrick({bx, by, bz}, createEmpty);
                    if (!br) continue;
                    bool changed = false;
                    for (uint32_t i = 0; i < 512; i++)
                        changed |= fn(bx * 8 + (int32_t)(i & 7), by * 8 + (int32_t)(i >> 6),
                                      bz * 8 + (int32_t)((i >> 3) & 7), br->Data[i]);
                    const bool isEmpty = br->IsEmpty();
                    if (changed || isEmpty) {
                        const uint32_t key = SectorKey(bx >> 2, by >> 2, bz >> 2);
                        const uint64_t bit = 1ull << Sector::Index(bx, by, bz);
                        DirtyLocs[key] |= bit;
                        if (isEmpty) empty[key] |= bit;
                    }
                }
        for (auto& kv : empty) {
            Sector& s = Sectors[kv.first];
            if (s.GetAllocationMask() & ~kv.second)
                s.DeleteBricks(kv.second);
            else
                Sectors.erase(kv.first);
        }
    }
};

// ---- device storage (GpuVoxelStorage) ----

class GpuVoxelStorage {
  public:
    GpuVoxelStorage(uint32_t sectorsX, uint32_t sectorsY, uint32_t sectorsZ, int device = 0) {
        vrt_world_desc d{sectorsX, sectorsY, sectorsZ, 0, device, 0};
        check(vrt_world_create(&d, &world_));
    }
    ~GpuVoxelStorage() { vrt_world_destroy(world_); }
    GpuVoxelStorage(const GpuVoxelStorage&) = delete;
    GpuVoxelStorage& operator=(const GpuVoxelStorage&) = delete;

    // Uploads the dirty bricks of `map` and clears DirtyLocs (GpuRenderer.cpp:45-167).
    void SyncBuffers(VoxelMap& map, void* stream = nullptr) {
        std::vector<int32_t> idx;
        std::vector<uint64_t> alloc, dirty;
        std::vector<uint8_t> bricks;
        for (const auto& [key, mask] : map.DirtyLocs) {
            auto it = map.Sectors.find(key);
            const uint64_t am = it == map.Sectors.end() ? 0 : it->second.GetAllocationMask();
            const uint64_t dm = mask & am;
            idx.push_back((int32_t)key);
            alloc.push_back(am);
            dirty.push_back(dm);
            for (uint64_t r = dm; r; r &= r - 1) {
                const Brick* b = it->second.GetBrick((uint32_t)__builtin_ctzll(r));
                const uint8_t* p = &b->Data[0].Data;
                bricks.insert(bricks.end(), p, p + 512);
            }
        }
        check(vrt_world_sync_sectors(world_, (uint32_t)idx.size(), idx.data(), alloc.data(), dirty.data(),
                                     bricks.data(), stream));
        map.DirtyLocs.clear();
    }
    vrt_world* handle() const { return world_; }

  private:
    vrt_world* world_ = nullptr;
};

// ---- renderer (GpuRenderer) ----

class GpuRenderer {
  public:
    GpuRenderer(std::shared_ptr<VoxelMap> map, uint32_t sectorsX, uint32_t sectorsY, uint32_t sectorsZ, int device = 0)
        : map_(std::move(map)), storage_(sectorsX, sectorsY, sectorsZ, device) {
        map_->MarkAllDirty();
    }
    // One frame: sync dirty bricks, then primary rays (+ secondary rays per
    // `view`'s flags) into host records laid out as vrt_view_records().  With
    // UseAnisotropicLods the frame traces in the GLSL mode with anisotropic LODs.
    std::vector<vrt_hit> RenderFrame(const vrt_view& view, void* stream = nullptr) {
        storage_.SyncBuffers(*map_, stream);
        vrt_view v = view;
        if (UseAnisotropicLods) v.flags |= VRT_VIEW_GLSL | VRT_VIEW_GLSL_ANISO;
        std::vector<vrt_hit> hits(vrt_view_records(&v));
        check(vrt_render_path(storage_.handle(), &v, hits.data(), stream));
        return hits;
    }
    GpuVoxelStorage& storage() { return storage_; }

    // the renderer setting of the same name (Renderer.h:45, VoxelTraversal.glsl:116-121)
    bool UseAnisotropicLods = false;

  private:
    std::shared_ptr<VoxelMap> map_;
    GpuVoxelStorage storage_;
};

inline vrt_camera LookAt(const double pos[3], const double target[3], double vfovDeg, uint32_t w, uint32_t h) {
    vrt_camera c;
    check(vrt_camera_look_at(pos, target, vfovDeg, w, h, &c));
    return c;
}

}  // namespace vrt
