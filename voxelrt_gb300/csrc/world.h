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

// Pinned host buffer for asynchronous uploads.  A pageable source may still be read
// after cudaMemcpyAsync returns (a device with a coherent host link reads it during the
// copy), so uploads go through this buffer, and a call that rewrites it first waits for
// the copy that last read it (the `read` event).
struct HostStage {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaEvent_t read = nullptr;
    cudaError_t acquire(size_t n) {
        if (!read) {
            cudaError_t e = cudaEventCreateWithFlags(&read, cudaEventDisableTiming);
            if (e != cudaSuccess) return e;
        }
        cudaError_t e = cudaEventSynchronize(read);
        if (e != cudaSuccess || n <= bytes) return e;
        if (bytes * 2 > n) n = bytes * 2;
        void* p = nullptr;
        if ((e = cudaHostAlloc(&p, n, cudaHostAllocDefault)) != cudaSuccess) return e;
        if (ptr) cudaFreeHost(ptr);
        ptr = p;
        bytes = n;
        return cudaSuccess;
    }
    cudaError_t release(cudaStream_t stream) { return cudaEventRecord(read, stream); }
    void destroy() {
        if (read) cudaEventSynchronize(read), cudaEventDestroy(read);
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        read = nullptr;
        bytes = 0;
    }
};

// Device side of the brick-slot allocator: slots [0, top) have been handed out (live
// bricks and the garbage left behind by relocated sectors), `live` are in use, `cap`
// is the pool size; `overflow` is set when an allocation did not fit (it is skipped).
struct DevAlloc {
    uint32_t top, live, cap, overflow;
};

}  // namespace vrt

struct vrt_world {
    int device = 0;
    uint32_t sx = 0, sy = 0, sz = 0;
    uint32_t flags = 0;
    std::mutex mu;
    // VRT_WORLD_L2_PERSIST: the access-policy window over the brick table
    size_t l2_window_bytes = 0;
    float l2_hit_ratio = 0.0f;

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

    // device-side edits (alloc.cu): the bump allocator in device memory, the edit batch
    // upload, and what the host knows of the device's layout
    vrt::DevAlloc* d_alloc = nullptr;
    vrt::HostStage edit_stage[4];  // pinned uploads of the last edit batches, used in turn
    uint32_t edit_stage_next = 0;
    vrt::DevBuf d_edit;         // the edit batch on the device
    vrt::DevBuf d_gc;           // per touched sector: bricks an edit emptied
    cudaEvent_t edited = nullptr;  // recorded behind the last device edit
    bool host_stale = false;    // slots / arena / h_table predate device edits
    uint64_t top_bound = 0;     // upper bound of d_alloc->top without reading it
    uint32_t compactions = 0;   // pool compactions so far (vrt_world_defrag and edits)

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
// Makes a device current for the length of an ABI call and gives the caller's current
// device back when the call returns, so the library never leaves it switched.
struct DeviceScope {
    int prev = -1;
    bool switched = false;
    DeviceScope() = default;
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
    cudaError_t enter(int device) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return e;
        if (prev == device) return cudaSuccess;
        e = cudaSetDevice(device);
        switched = e == cudaSuccess;
        return e;
    }
    ~DeviceScope() {
        if (switched) cudaSetDevice(prev);
    }
};

// Make `world`'s device current on the calling thread until `scope` ends.
vrt_status world_enter(vrt_world* world, DeviceScope& scope);

// While alive, kernels launched on `stream` carry an L2 access-policy window that keeps the
// brick table of a VRT_WORLD_L2_PERSIST world persisting in L2 (the table is the mask
// level every DDA step reads); the stream's previous window comes back when it ends.  A
// no-op for other worlds and for the legacy default stream, whose attributes cannot be set.
struct L2Window {
    cudaStream_t stream = nullptr;
    bool set = false;
    cudaStreamAttrValue prev{};
    vrt_status enter(const vrt_world* w, cudaStream_t s);
    ~L2Window();
};

// alloc.cu (callers hold world->mu)
// Rebuild the host mirror (slots, arena, h_table) from the device after device edits.
vrt_status refresh_host_mirror(vrt_world* w);
// After host planning: publish the host allocator's state to the device allocator.
vrt_status alloc_publish(vrt_world* w, cudaStream_t stream);
// Make room for `need` more bump-allocated slots: compacts (and grows) the pool when
// the bound of the bump pointer says it may not fit.
vrt_status ensure_headroom(vrt_world* w, uint64_t need, cudaStream_t stream);
// Pack the live bricks from slot 0 in sector order into a pool of `capacity` slots.
vrt_status world_compact(vrt_world* w, uint32_t capacity, cudaStream_t stream);
// Brick-table entries of the listed sector groups (device list of n groups), or of the
// whole world when they are a quarter of it or more.
vrt_status rebuild_table_groups(vrt_world* w, const uint32_t* d_groups, uint32_t n, cudaStream_t stream);
}  // namespace vrt
