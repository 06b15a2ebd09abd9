// noalloc.cu - batched traversal for callers that cannot allocate device memory.
//
// vrt_batch keeps its world table, view table, tile-queue counter and launch
// counters in device memory it allocates with cudaMalloc.  Some callers cannot
// allow that: a renderer whose frame loop must never call cudaMalloc (the call can
// synchronise the device and stall every other stream), or a host application
// that hands the library a fixed memory budget up front and forbids allocations
// afterwards.  vrt_render_views_static runs the same persistent kernel with that
// scratch in one file-scope device array of fixed size instead; the caller still
// passes the worlds, the views and the device record buffer.

#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "batch_internal.h"
#include "world.h"

namespace vrt {
namespace {

constexpr uint32_t kStaticMaxWorlds = 256;
constexpr uint32_t kStaticMaxViews = 1024;
constexpr int kStaticMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kQueueOff = 0;  // tile-queue counter + 4 launch counters (64 bytes used)
constexpr size_t kWorldsOff = 256;
constexpr size_t kViewsOff = align256(kWorldsOff + kStaticMaxWorlds * sizeof(DevWorld));
constexpr size_t kChunkOff = align256(kViewsOff + kStaticMaxViews * sizeof(ViewDev));
constexpr size_t kScratchBytes = align256(kChunkOff + (kStaticMaxViews + 1) * sizeof(uint32_t));

// The scratch itself: every GPU that loads the library holds these bytes until
// the process exits.  In host code the name is only a host-side stand-in; the
// device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) uint8_t g_static_scratch[kScratchBytes];

// Host side of the calls.  The tables below are the sources of the call's
// host-to-device copies.  Those copies are from pageable memory, which a device with a
// coherent host link (GB300 over NVLink-C2C) may read while the copy runs, after
// cudaMemcpyAsync has returned.  So each device's `copied` event is recorded behind the
// three copies, and the next call waits for it before it rewrites the tables.  The
// events are created with the scratch address at a device's first call; creating an
// event allocates no device memory.
struct StaticState {
    std::mutex mu;
    uint8_t* scratch[kStaticMaxDevices] = {};  // device address per device ordinal
    cudaEvent_t copied[kStaticMaxDevices] = {};
    DevWorld worlds[kStaticMaxWorlds];
    ViewDev views[kStaticMaxViews];
    uint32_t chunk_base[kStaticMaxViews + 1];
};
StaticState g_state;

uint32_t log2u_static(uint32_t v) {
    uint32_t r = 0;
    while ((1u << r) < v) r++;
    return r;
}

}  // namespace
}  // namespace vrt

using namespace vrt;

extern "C" vrt_status vrt_render_views_static(vrt_world* const* worlds, uint32_t n_worlds, const vrt_view* views,
                                              uint32_t n_views, const vrt_batch_config* cfg_in, vrt_hit* hits_device,
                                              void* stream_) {
    if (!worlds || n_worlds == 0 || !views || n_views == 0 || !hits_device) {
        set_error("vrt_render_views_static needs worlds, views and a device record buffer");
        return VRT_ERR_INVALID_ARG;
    }
    if (n_worlds > kStaticMaxWorlds || n_views > kStaticMaxViews) {
        set_error("vrt_render_views_static takes at most 256 worlds and 1024 views per call");
        return VRT_ERR_INVALID_ARG;
    }
    for (uint32_t i = 0; i < n_worlds; i++)
        if (!worlds[i] || worlds[i]->device != worlds[0]->device) {
            set_error("worlds must be non-null and on one device");
            return VRT_ERR_INVALID_ARG;
        }
    const int device = worlds[0]->device;
    if (device < 0 || device >= kStaticMaxDevices) {
        set_error("device ordinal out of range for the static scratch table");
        return VRT_ERR_INVALID_ARG;
    }
    vrt_batch_config cfg;
    vrt_status st = normalize_batch_config(cfg_in, cfg);
    if (st != VRT_OK) return st;
    for (uint32_t i = 0; i < n_views; i++) {
        if ((st = check_view(&views[i])) != VRT_OK) return st;
        if (views[i].world >= n_worlds) {
            set_error("view references a world outside the list");
            return VRT_ERR_INVALID_ARG;
        }
    }
    if ((st = check_same_mode(views, n_views)) != VRT_OK) return st;
    const bool glsl = n_views > 0 && view_glsl(views[0]);
    std::lock_guard<std::mutex> lock(g_state.mu);
    DeviceScope scope;
    VRT_CUDA(scope.enter(device));
    // first call on this device: look up the device address of the scratch array, and
    // create the event that guards the host tables
    if (!g_state.scratch[device]) {
        void* p = nullptr;
        VRT_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
        cudaEvent_t ev = nullptr;
        VRT_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        g_state.copied[device] = ev;
        g_state.scratch[device] = static_cast<uint8_t*>(p);
    }
    uint8_t* scratch = g_state.scratch[device];
    // the copies of the last call on this device have read the host tables
    VRT_CUDA(cudaEventSynchronize(g_state.copied[device]));
    // the launch grid, and what the config leaves to the library
    const bool aniso = view_aniso(views[0]);
    bool full = false;
    for (uint32_t i = 0; i < n_views; i++) full |= view_full_path(views[i]);
    int blocks = 0, threads = 0;
    if ((st = persistent_grid(device, cfg, false, glsl, aniso, false, full, blocks, threads)) != VRT_OK) return st;
    resolve_batch_defaults(cfg, views, n_views, (uint64_t)blocks * (threads / 32));
    // lay the views out behind one tile queue (same layout as vrt_batch)
    const uint32_t tw_log2 = log2u_static(cfg.tile_w), ts_log2 = log2u_static(cfg.tile_w * cfg.tile_h);
    uint64_t chunks = 0, records = 0;
    for (uint32_t i = 0; i < n_views; i++) {
        const vrt_view& v = views[i];
        ViewDev& d = g_state.views[i];
        d = make_view_dev(v);
        const uint32_t tx = (v.cam.width + cfg.tile_w - 1) / cfg.tile_w;
        const uint32_t ty = (v.cam.height + cfg.tile_h - 1) / cfg.tile_h;
        const uint64_t tiles = (uint64_t)tx * ty;
        d.tiles_x = tx;
        d.tiles_x_magic = div_magic(tx);
        d.n_rays = (uint32_t)(tiles << ts_log2);
        d.chunk_base = (uint32_t)chunks;
        d.out_base = records;
        g_state.chunk_base[i] = (uint32_t)chunks;
        chunks += (tiles + cfg.chunk_tiles - 1) / cfg.chunk_tiles;
        records += view_record_count(v);
        if (chunks >= 0xffffffffull) {
            set_error("too many ray tiles for one call");
            return VRT_ERR_INVALID_ARG;
        }
    }
    g_state.chunk_base[n_views] = (uint32_t)chunks;
    for (uint32_t i = 0; i < n_worlds; i++) g_state.worlds[i] = worlds[i]->dev();

    cudaStream_t stream = (cudaStream_t)stream_;
    VRT_CUDA(cudaMemcpyAsync(scratch + kWorldsOff, g_state.worlds, n_worlds * sizeof(DevWorld), cudaMemcpyHostToDevice,
                             stream));
    VRT_CUDA(cudaMemcpyAsync(scratch + kViewsOff, g_state.views, n_views * sizeof(ViewDev), cudaMemcpyHostToDevice,
                             stream));
    VRT_CUDA(cudaMemcpyAsync(scratch + kChunkOff, g_state.chunk_base, (n_views + 1) * sizeof(uint32_t),
                             cudaMemcpyHostToDevice, stream));
    VRT_CUDA(cudaEventRecord(g_state.copied[device], stream));
    BatchParams p{};
    p.worlds = reinterpret_cast<const DevWorld*>(scratch + kWorldsOff);
    p.views = reinterpret_cast<const ViewDev*>(scratch + kViewsOff);
    p.chunk_base = reinterpret_cast<const uint32_t*>(scratch + kChunkOff);
    p.n_views = n_views;
    p.total_chunks = (uint32_t)chunks;
    p.queue = reinterpret_cast<uint32_t*>(scratch + kQueueOff);
    p.counters = reinterpret_cast<unsigned long long*>(scratch + kQueueOff + 16);
    p.out = reinterpret_cast<uint4*>(hits_device);
    p.tile_w_log2 = tw_log2;
    p.tile_size_log2 = ts_log2;
    p.morton = cfg.morton;
    p.chunk_rays = cfg.chunk_tiles << ts_log2;
    p.refill = std::max(1u, cfg.refill_threshold);
    p.inner = std::max(1u, cfg.inner_iters);
    p.glsl = glsl ? 1u : 0u;
    p.aniso = aniso ? 1u : 0u;
    p.full = full ? 1u : 0u;
    // launch_persistent zeroes the queue counter and the launch counters first
    return launch_persistent(p, blocks, threads, false, stream);
}
