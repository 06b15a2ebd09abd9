// batch_internal.h - launch planning shared by vrt_batch and the request server.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "vrt_internal.h"

namespace vrt {

// Device view-table entry of the persistent kernel: 128 bytes, 16-byte aligned, so ray
// setup reads it with 128-bit loads (the camera's ray generation in the first three
// vectors, world origin and world index in the fourth, the tile geometry in the fifth).
struct alignas(16) ViewDev {
    float d0[3], ox;          // camera: d0 and origin.x
    float du[3], oy;          // du and origin.y
    float dv[3], oz;          // dv and origin.z
    int32_t wo[3];            // camera world origin
    uint32_t world;
    uint32_t width, height;
    uint32_t tiles_x;
    uint32_t tiles_x_magic;   // ceil(2^32 / tiles_x): tile row by a multiply-high
    uint32_t max_iters;
    uint32_t path;            // last kind of a pixel's path << 8 | shadow << 16
    uint32_t n_rays;          // tile-padded ray space of the view
    uint32_t chunk_base;      // first queue chunk of the view
    uint64_t out_base;        // first record of the view
    float sun[3];
    uint32_t aniso;           // GLSL mode with anisotropic LODs (VRT_VIEW_GLSL_ANISO)
    uint32_t pad[2];
    VRT_HD uint32_t shadow() const { return (path >> 16) & 1u; }
    VRT_HD uint32_t last_kind() const { return (path >> 8) & 0xFFu; }
};
static_assert(sizeof(ViewDev) == 128, "view table entry is 128 bytes (copied per camera update)");

// The camera fields of a view-table entry.
void set_view_camera(ViewDev& d, const vrt_camera& c);
// A view-table entry for view `v` (camera, world, path, iteration cap, sun); the
// planner adds the tile and queue fields.
ViewDev make_view_dev(const vrt_view& v);

// ceil(2^32 / d) for 2 <= d < 2^32; 0 marks d == 1 (the quotient is the numerator).
inline uint32_t div_magic(uint32_t d) {
    return d <= 1 ? 0u : (uint32_t)((0x100000000ull + d - 1) / d);
}

struct BatchParams {
    const DevWorld* worlds;
    const ViewDev* views;
    const uint32_t* chunk_base;  // n_views + 1 entries
    uint32_t n_views;
    uint32_t total_chunks;
    uint32_t chunk_first;  // absolute queue chunk of the first view (views may be a sub-range)
    uint32_t* queue;
    unsigned long long* counters;  // rays, step calls, occ fetches, hits
    uint4* out;
    uint32_t tile_w_log2, tile_size_log2, morton;
    uint32_t chunk_rays;
    uint32_t refill;
    uint32_t inner;
    uint32_t glsl;  // traversal mode of every view (VRT_VIEW_GLSL)
    uint32_t aniso;  // ... with anisotropic LODs (VRT_VIEW_GLSL_ANISO)
    uint32_t full;   // some view traces the GPU renderer's whole path (sun rays among bounces)
    // resident launches (request server): views are published while the kernel runs
    unsigned long long* mailbox;  // host-mapped: published chunks | published views << 32 | closed << 63
    uint32_t* next_chunk;         // device: next chunk to claim
    const unsigned long long* hint;  // device copy of the mailbox word the host writes after each change
                                     // (never ahead of it): idle warps poll it instead of host memory
    uint32_t* remaining;          // device, per view: pixels whose path is not finished
    uint32_t* done_flags;         // host-mapped, per view: 1 once every record of the view is stored
    uint32_t idle_us;             // sleep an idle warp accumulates before it closes the mailbox
    uint32_t n_worlds;            // bounds the kernel checks views of a resident launch against:
    unsigned long long out_records;  // a bad entry is skipped, never accessed
};

// Mailbox word of a resident launch.
constexpr unsigned long long kMailboxClosed = 1ull << 63;
VRT_HD inline unsigned long long mailbox_word(uint32_t chunks, uint32_t views) {
    return (unsigned long long)chunks | (unsigned long long)(views & 0x7FFFFFFFu) << 32;
}

// Views laid out behind one tile queue.
struct LaunchPlan {
    vrt_batch_config cfg{};
    uint32_t tile_w_log2 = 3, tile_size_log2 = 6;
    std::vector<ViewDev> views;
    std::vector<uint32_t> chunk_base;  // n_views + 1
    uint64_t records = 0;
    uint32_t chunks = 0;
    bool glsl = false;   // every view traces in the GLSL mode
    bool aniso = false;  // ... with anisotropic LODs
    bool full = false;   // some view traces the GPU renderer's whole path
};

// Dynamic shared memory of a persistent launch: the hit frame a lane keeps across a sun
// ray of the GPU renderer's whole path (6 floats per thread), only where a view needs it.
inline size_t pend_bytes(const BatchParams& p, int threads) { return p.full ? (size_t)threads * 6 * sizeof(float) : 0; }

// Iteration cap of a view or cast: 0 = the mode's default, at most 65535.
uint32_t eff_iters(uint32_t max_iters, bool glsl = false);
inline bool view_glsl(const vrt_view& v) { return (v.flags & VRT_VIEW_GLSL) != 0; }
inline bool view_aniso(const vrt_view& v) { return (v.flags & VRT_VIEW_GLSL_ANISO) != 0; }
// A view's traversal mode: the CPU traversal, GLSL, or GLSL with anisotropic LODs.
inline uint32_t view_mode(const vrt_view& v) { return v.flags & (VRT_VIEW_GLSL | VRT_VIEW_GLSL_ANISO); }
// A sun direction and bounces: the GPU renderer's whole path (VoxelRender.comp:51-86).
inline bool view_full_path(const vrt_view& v) { return (v.flags & VRT_VIEW_SHADOW) && v.n_bounces; }
// All views of one launch share a traversal mode (VRT_ERR_INVALID_ARG otherwise).
vrt_status check_same_mode(const vrt_view* views, uint32_t n);
uint64_t view_record_count(const vrt_view& v);
vrt_status check_view(const vrt_view* v);
// Fill defaults and validate a batch config.
vrt_status normalize_batch_config(const vrt_batch_config* in, vrt_batch_config& out);
// Tiles per queue chunk when a config leaves it to the library (chunk_tiles 0): about
// eight chunks per warp of the launch, 1..16 tiles.  Fixed chunks too large for a small
// launch leave most warps without work; the tuned table names its chunks explicitly.
uint32_t auto_chunk_tiles(uint64_t tiles, uint64_t warps);
// Fill the fields a config leaves to the library (0): views with diffuse bounces (long,
// uneven, incoherent paths per pixel) refill below 28 lanes and claim one tile at a time;
// camera and sun rays refill below 16 and claim auto_chunk_tiles.
void resolve_batch_defaults(vrt_batch_config& cfg, const vrt_view* views, uint32_t n, uint64_t warps);
// Validate views against n_worlds and lay them out (tiles, queue chunks, record offsets).
// Fields left to the library are resolved for a launch of `warps` warps
// (resolve_batch_defaults), and plan.cfg holds the config used.
vrt_status plan_views(const vrt_view* views, uint32_t n, uint32_t n_worlds, const vrt_batch_config& cfg,
                      LaunchPlan& plan, uint64_t warps = 0);
// Grid of the persistent kernel: every SM, as many blocks of the launched instantiation
// (counting, traversal mode, resident) as fit, or cfg.blocks_per_sm of them.
vrt_status persistent_grid(int device, const vrt_batch_config& cfg, bool count, bool glsl, bool aniso, bool resident,
                           bool full, int& blocks, int& threads);
BatchParams make_params(const LaunchPlan& plan, const DevWorld* worlds, const ViewDev* views,
                        const uint32_t* chunk_base, uint32_t* queue, vrt_hit* out);
// Queue reset (the tile counter, and with reset_counters the launch counters: 64
// bytes at params.queue) + persistent kernel launch.
vrt_status launch_persistent(const BatchParams& p, int blocks, int threads, bool count, cudaStream_t stream,
                             bool reset_counters = true);
// A resident launch: the kernel claims chunks the host publishes through p.mailbox
// while it runs, and exits once the mailbox is closed and its work is done.  The
// caller zeroes the block at p.queue (claim counter and launch counters in the first
// 64 bytes, the hint on its own line at kResidentHintOffset) before publishing the
// first views.
constexpr size_t kResidentHintOffset = 128;
vrt_status launch_resident(const BatchParams& p, int blocks, int threads, cudaStream_t stream);

}  // namespace vrt
