// world.h - host-side state of one device-resident world (vrt_world).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "freelist.h"
#include "vrt_internal.h"

namespace vrt {

// thread-local error message behind vrt_last_error()
void set_error(const std::string& msg);
const char* last_error_cstr();
vrt_status cuda_fail(cudaError_t e, const char* what);

#define VRT_CUDA(call)                                             \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return ::vrt::cuda_fail(e_, #call); \
    } while (0)

// Grow-only device buffer.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    // geometric: at least double, for buffers that grow call by call (each growth frees
    // the old buffer, and cudaFree waits for the whole device)
    cudaError_t reserve(size_t n, bool geometric = false) {
        if (n <= bytes) return cudaSuccess;
        if (geometric && bytes * 2 > n) n = bytes * 2;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) return e;
        if (ptr) cudaFree(ptr);
        ptr = p;
        bytes = n;
        return cudaSuccess;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

}  // namespace vrt

struct vrt_world {
    int device = 0;
    uint32_t sx = 0, sy = 0, sz = 0;
    uint32_t flags = 0;
    std::mutex mu;

    // host mirror of the allocation state (BrickSlotAllocator, GpuRenderer.cpp:23)
    std::vector<vrt::SectorSlots> slots;
    vrt::FreeList arena;

    // device storage
    vrt::SectorRec* d_sectors = nullptr;
    uint32_t* d_bricks = nullptr;  // brick table, derived from the sector table on the device
    uint64_t* d_groups = nullptr;  // sector-group masks of the GLSL mode's 4th level
    uint4* d_codes = nullptr;      // byte voxel codes, 512 B (32 x 16 B) per slot
    uint64_t* d_cells = nullptr;   // 8 cell masks per slot
    uint8_t* d_payload = nullptr;
    uint32_t capacity = 0;  // brick slots in the device pools

    // scratch reused across sync/edit calls
    vrt::DevBuf d_stage;    // uploaded brick bytes
    vrt::DevBuf d_ops;      // brick operation lists
    vrt::DevBuf d_scratch;  // bricks in flight during a repack
    vrt::DevBuf d_glist;    // sector groups whose brick-table entries an edit re-derives
    vrt::DevBuf d_io;       // ray/hit staging for host-buffer calls
    std::vector<vrt::SectorRec> h_table;  // host copy of the sector table

    uint32_t num_sectors() const { return sx * sy * sz; }
    size_t num_brick_positions() const { return (size_t)num_sectors() * 64; }
    uint32_t num_groups() const { return ((sx + 3) / 4) * ((sy + 3) / 4) * ((sz + 3) / 4); }
    uint32_t lin(int32_t x, int32_t y, int32_t z) const {
        return (uint32_t)x + (uint32_t)z * sx + (uint32_t)y * sx * sz;
    }
    bool sector_in(int32_t x, int32_t y, int32_t z) const {
        return (uint32_t)x < sx && (uint32_t)y < sy && (uint32_t)z < sz;
    }
    vrt::DevWorld dev() const {
        vrt::DevWorld w;
        w.bricks = d_bricks;
        w.codes = reinterpret_cast<const uint8_t*>(d_codes);
        w.payload = d_payload;
        w.sectors = d_sectors;
        w.bsx = sx * 4;
        w.bsxz = sx * 4 * sz * 4;
        w.sx = sx;
        w.sz = sz;
        w.sxz = sx * sz;
        w.cells = d_cells;
        w.size_x = sx * 32;
        w.size_y = sy * 32;
        w.size_z = sz * 32;
        return w;
    }
};

namespace vrt {
// Make `world` current on the calling thread.
vrt_status world_enter(vrt_world* world);
}  // namespace vrt
