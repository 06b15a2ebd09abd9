// world.cu - device-resident brickmap storage: create/destroy, dirty-brick sync,
// brick-slot repacking, occupancy re-derivation and the brick table.
//
// Replaces GpuVoxelStorage (src/VoxelRT/GpuRenderer.cpp:17-167) and the
// UpdateOccupancy dispatch (GpuRenderer.cpp:163-166, Shaders/UpdateOccupancy.comp).
// Unlike the reference, bricks that keep their content but change slot are moved
// on the device instead of being re-uploaded from the host
// (BrickSlotAllocator.cpp:84-87 marks the whole sector dirty).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <unordered_set>
#include <vector>

#include "brick_codes.cuh"
#include "world.h"

namespace vrt {

vrt_status cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return VRT_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return VRT_ERR_NO_DEVICE;
    return VRT_ERR_DEVICE;
}

vrt_status world_enter(vrt_world* world, DeviceScope& scope) {
    if (!world) {
        set_error("null world");
        return VRT_ERR_INVALID_ARG;
    }
    VRT_CUDA(scope.enter(world->device));
    return VRT_OK;
}

vrt_status L2Window::enter(const vrt_world* w, cudaStream_t s) {
    if (!w || !(w->flags & VRT_WORLD_L2_PERSIST) || !s || w->l2_window_bytes == 0) return VRT_OK;
    VRT_CUDA(cudaStreamGetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &prev));
    cudaStreamAttrValue a{};
    a.accessPolicyWindow.base_ptr = w->d_bricks;
    a.accessPolicyWindow.num_bytes = w->l2_window_bytes;
    a.accessPolicyWindow.hitRatio = w->l2_hit_ratio;
    a.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    a.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    VRT_CUDA(cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &a));
    stream = s;
    set = true;
    return VRT_OK;
}

L2Window::~L2Window() {
    if (set) cudaStreamSetAttribute(stream, cudaStreamAttributeAccessPolicyWindow, &prev);
}

namespace {

// The window of a VRT_WORLD_L2_PERSIST world: its brick table, up to the device's largest
// window, with the context's persisting L2 set-aside raised to cover it (up to the
// device's maximum; the set-aside lasts as long as this process's context).
vrt_status setup_l2_window(vrt_world* w) {
    int max_window = 0, max_persist = 0;
    VRT_CUDA(cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, w->device));
    VRT_CUDA(cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, w->device));
    if (max_window <= 0 || max_persist <= 0) return VRT_OK;  // no persisting L2: the flag does nothing
    const size_t table = w->num_brick_positions() * sizeof(uint32_t);
    w->l2_window_bytes = std::min(table, (size_t)max_window);
    size_t limit = 0;
    VRT_CUDA(cudaDeviceGetLimit(&limit, cudaLimitPersistingL2CacheSize));
    const size_t want = std::min(w->l2_window_bytes, (size_t)max_persist);
    if (want > limit) VRT_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want));
    VRT_CUDA(cudaDeviceGetLimit(&limit, cudaLimitPersistingL2CacheSize));
    w->l2_hit_ratio = (float)std::min(1.0, (double)limit / (double)w->l2_window_bytes);
    return VRT_OK;
}

// ---------------------------------------------------------------------------
// Brick operations, one warp per brick.

enum : uint32_t { kOpMove = 0u, kOpUpload = 1u, kOpZero = 2u };

struct BrickOp {
    uint32_t dst;  // 0-based destination slot
    uint32_t src;  // kind << 30 | index (scratch brick or staged brick)
};

constexpr int kOpsWarps = 8;

__global__ void gather_bricks_kernel(const uint32_t* __restrict__ src_slots, uint32_t n,
                                     const uint8_t* __restrict__ payload, const uint4* __restrict__ codes,
                                     const uint64_t* __restrict__ cells, uint8_t* __restrict__ scratch_payload,
                                     uint4* __restrict__ scratch_codes, uint64_t* __restrict__ scratch_cells) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = warp; k < n; k += nwarps) {
        const size_t s = src_slots[k];
        const uint4 v = reinterpret_cast<const uint4*>(payload + s * 512)[lane];
        reinterpret_cast<uint4*>(scratch_payload + (size_t)k * 512)[lane] = v;
        scratch_codes[(size_t)k * 32 + lane] = codes[s * 32 + lane];
        if (lane < 8) scratch_cells[(size_t)k * 8 + lane] = cells[s * 8 + lane];
    }
}

__global__ void __launch_bounds__(kOpsWarps * 32)
    brick_ops_kernel(const BrickOp* __restrict__ ops, uint32_t n, const uint8_t* __restrict__ stage,
                     const uint8_t* __restrict__ scratch_payload, const uint4* __restrict__ scratch_codes,
                     const uint64_t* __restrict__ scratch_cells, uint8_t* __restrict__ payload,
                     uint4* __restrict__ codes, uint64_t* __restrict__ cells) {
    __shared__ __align__(16) uint8_t sbrick[kOpsWarps][512];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    const uint32_t warp = blockIdx.x * kOpsWarps + wib;
    const uint32_t nwarps = gridDim.x * kOpsWarps;
    for (uint32_t k = warp; k < n; k += nwarps) {
        const BrickOp op = ops[k];
        const uint32_t kind = op.src >> 30, si = op.src & 0x3fffffffu;
        const size_t d = op.dst;
        if (kind == kOpMove) {
            const uint4 v = reinterpret_cast<const uint4*>(scratch_payload + (size_t)si * 512)[lane];
            reinterpret_cast<uint4*>(payload + d * 512)[lane] = v;
            codes[d * 32 + lane] = scratch_codes[(size_t)si * 32 + lane];
            if (lane < 8) cells[d * 8 + lane] = scratch_cells[(size_t)si * 8 + lane];
        } else if (kind == kOpZero) {
            reinterpret_cast<uint4*>(payload + d * 512)[lane] = make_uint4(0, 0, 0, 0);
            codes[d * 32 + lane] = empty_brick_codes();
            if (lane < 8) cells[d * 8 + lane] = 0;
        } else {
            const uint4 v = reinterpret_cast<const uint4*>(stage + (size_t)si * 512)[lane];
            reinterpret_cast<uint4*>(payload + d * 512)[lane] = v;
            reinterpret_cast<uint4*>(sbrick[wib])[lane] = v;
            __syncwarp();
            const uint64_t m = warp_cell_mask(sbrick[wib], lane);
            codes[d * 32 + lane] = warp_voxel_codes(sbrick[wib], m, lane);
            if (lane < 8) cells[d * 8 + lane] = m;
            __syncwarp();
        }
    }
}

// Sector-group masks of the GLSL mode's 4th level (VoxelTraversal.glsl:114-118): per
// group of 4^3 sectors, bit x | z<<2 | y<<4 set when that sector holds a brick
// (GpuRenderer.cpp:139-149); groups indexed x + z*GX + y*GX*GZ, one warp each (lane l
// tests sectors l and l + 32 of the group, a ballot gathers each half).
__global__ void group_masks_kernel(const SectorRec* __restrict__ sectors, uint32_t sx, uint32_t sy, uint32_t sz,
                                   unsigned long long* __restrict__ groups) {
    const uint32_t gx = (sx + 3) / 4, gy = (sy + 3) / 4, gz = (sz + 3) / 4;
    const uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (g >= gx * gy * gz) return;  // whole warps leave together
    const uint32_t x0 = (g % gx) * 4, z0 = ((g / gx) % gz) * 4, y0 = (g / (gx * gz)) * 4;
    uint32_t half[2];
    for (uint32_t h = 0; h < 2; h++) {
        const uint32_t b = lane + 32 * h;
        const uint32_t x = x0 + (b & 3), z = z0 + ((b >> 2) & 3), y = y0 + (b >> 4);
        bool nonempty = false;
        if (x < sx && y < sy && z < sz) {
            const SectorRec r = sectors[x + z * sx + y * sx * sz];
            nonempty = (r.mask_lo | r.mask_hi) != 0;
        }
        half[h] = __ballot_sync(0xffffffffu, nonempty);
    }
    if (lane == 0) groups[g] = (unsigned long long)half[0] | (unsigned long long)half[1] << 32;
}

// The brick-table entry of brick b of sector s, written at its brick position.
__device__ __forceinline__ void write_table_entry(const SectorRec* __restrict__ sectors,
                                                  const unsigned long long* __restrict__ groups, uint32_t s,
                                                  uint32_t b, uint32_t sx, uint32_t sz, uint32_t* __restrict__ bricks) {
    const SectorRec rec = sectors[s];
    const uint32_t x = s % sx, z = (s / sx) % sz, y = s / (sx * sz);
    const uint32_t bx = x * 4 + (b & 3), bz = z * 4 + ((b >> 2) & 3), by = y * 4 + (b >> 4);
    const uint32_t lo = rec.mask_lo, hi = rec.mask_hi;
    uint32_t e;
    if ((((b < 32 ? lo : hi) >> (b & 31)) & 1u) != 0) {
        const uint32_t below = (1u << (b & 31)) - 1u;
        e = rec.base + (b < 32 ? __popc(lo & below) : __popc(lo) + __popc(hi & below));
    } else {
        const uint32_t cpu_m = (8u << skip_levels(lo, hi, b)) - 1u;
        e = kBrickEmpty | cpu_m;
        // the level the GLSL mode and its anisotropic LODs read: the sector's mask, or
        // where the sector is empty its group's mask, at the sector's index in the group
        uint64_t lm = (uint64_t)hi << 32 | lo;
        uint32_t li = b;
        if ((lo | hi) == 0) {
            const uint32_t gx = (sx + 3) / 4, gz = (sz + 3) / 4;
            lm = groups[(x >> 2) + (z >> 2) * gx + (y >> 2) * gx * gz];
            li = (x & 3) | (z & 3) << 2 | (y & 3) << 4;
            e |= kAnisoGroupBit | ((32u << skip_levels((uint32_t)lm, (uint32_t)(lm >> 32), li)) - 1u) << 8;
        } else {
            e |= cpu_m << 8;
        }
        // anisotropic LODs: that mask's skip level per ray octant
        for (uint32_t o = 0; o < 8; o++) {
            const uint64_t f = lm & forward_cells(li, (o & 1u) ? 0 : -1, (o & 2u) ? 0 : -1, (o & 4u) ? 0 : -1);
            e |= skip_levels((uint32_t)f, (uint32_t)(f >> 32), li) << (kAnisoShift + 2 * o);
        }
    }
    bricks[bx + bz * (sx * 4) + by * (sx * 4) * (sz * 4)] = e;
}

// Brick-table entries of sectors [s_lo, s_hi), one thread per brick position.
__global__ void brick_table_kernel(const SectorRec* __restrict__ sectors, const unsigned long long* __restrict__ groups,
                                   uint32_t s_lo, uint32_t s_hi, uint32_t sx, uint32_t sz,
                                   uint32_t* __restrict__ bricks) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (s_hi - s_lo) * 64u) return;
    write_table_entry(sectors, groups, s_lo + (i >> 6), i & 63u, sx, sz, bricks);
}

// Brick-table entries of the sectors of listed sector groups (4^3 sectors, index
// x + z*GX + y*GX*GZ), 4096 threads per group: after an edit, only the groups of the
// sectors it changed are re-derived (a sector's emptiness changes its group's mask,
// which the GLSL entries of the group's empty sectors read).
__global__ void brick_table_groups_kernel(const SectorRec* __restrict__ sectors,
                                          const unsigned long long* __restrict__ groups,
                                          const uint32_t* __restrict__ list, uint32_t n, uint32_t sx, uint32_t sy,
                                          uint32_t sz, uint32_t* __restrict__ bricks) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * 4096u) return;
    const uint32_t g = list[i >> 12], si = (i >> 6) & 63u, gx = (sx + 3) / 4, gz = (sz + 3) / 4;
    const uint32_t x = (g % gx) * 4 + (si & 3u), z = ((g / gx) % gz) * 4 + ((si >> 2) & 3u),
                   y = (g / (gx * gz)) * 4 + (si >> 4);
    if (x >= sx || y >= sy || z >= sz) return;
    write_table_entry(sectors, groups, x + z * sx + y * sx * sz, i & 63u, sx, sz, bricks);
}

uint32_t ops_grid(uint32_t n) {
    uint32_t blocks = (n + kOpsWarps - 1) / kOpsWarps;
    return std::max(1u, std::min(blocks, 152u * 16u));
}

// ---------------------------------------------------------------------------

// Grow the brick pools to at least min_capacity slots (at least doubling);
// slots keep their content, so planned moves stay valid.
vrt_status grow_pool(vrt_world* w, uint32_t min_capacity, cudaStream_t stream) {
    uint64_t want = std::max<uint64_t>({(uint64_t)w->capacity * 2, (uint64_t)min_capacity, 1024});
    want = std::min<uint64_t>(want, 0x3fffffffull);
    if (want <= w->capacity) {
        set_error("brick pool cannot grow further");
        return VRT_ERR_SLOTS_EXHAUSTED;
    }
    uint32_t cap = (uint32_t)want;
    uint4* codes = nullptr;
    uint8_t* payload = nullptr;
    uint64_t* cells = nullptr;
    cudaError_t e = cudaMalloc(&codes, (size_t)cap * 512);
    if (e == cudaSuccess) e = cudaMalloc(&payload, (size_t)cap * 512);
    if (e == cudaSuccess) e = cudaMalloc(&cells, (size_t)cap * 64);
    if (e != cudaSuccess) {
        if (codes) cudaFree(codes);
        if (payload) cudaFree(payload);
        cudaGetLastError();
        return cuda_fail(e, "grow brick pool");
    }
    if (w->capacity) {
        VRT_CUDA(cudaMemcpyAsync(codes, w->d_codes, (size_t)w->capacity * 512, cudaMemcpyDeviceToDevice, stream));
        VRT_CUDA(cudaMemcpyAsync(payload, w->d_payload, (size_t)w->capacity * 512, cudaMemcpyDeviceToDevice, stream));
        VRT_CUDA(cudaMemcpyAsync(cells, w->d_cells, (size_t)w->capacity * 64, cudaMemcpyDeviceToDevice, stream));
        VRT_CUDA(cudaStreamSynchronize(stream));
    }
    if (w->d_codes) cudaFree(w->d_codes);
    if (w->d_payload) cudaFree(w->d_payload);
    if (w->d_cells) cudaFree(w->d_cells);
    w->d_codes = codes;
    w->d_payload = payload;
    w->d_cells = cells;
    w->capacity = cap;
    w->arena.grow(cap);
    return VRT_OK;
}

// One self-consistent batch of sector updates: plan, then move, upload, zero.
struct SyncBatch {
    std::vector<uint32_t> gathers;   // old slots copied to scratch first
    std::vector<BrickOp> ops;
    const uint8_t* src = nullptr;    // first input brick of the batch
    uint64_t n_stage = 0;            // bricks staged from the input
    std::vector<uint32_t> touched;   // sector linear indices
};

vrt_status plan_sector(vrt_world* w, SyncBatch& b, uint32_t s, uint64_t am, uint64_t dm, uint64_t stage_first,
                       cudaStream_t stream) {
    SectorSlots& cur = w->slots[s];
    const SectorSlots old = cur;
    sector_free(w->arena, cur, old.mask & ~am);
    while (!sector_alloc(w->arena, cur, am)) {
        vrt_status st = grow_pool(w, w->capacity + 64, stream);
        if (st != VRT_OK) return st;
    }
    uint64_t rank_in = 0;
    for (uint64_t r = cur.mask; r; r &= r - 1) {
        const uint32_t brick = (uint32_t)__builtin_ctzll(r);
        const uint32_t dst = cur.slot_of(brick) - 1;
        const uint64_t bit = 1ull << brick;
        if (dm & bit) {
            rank_in = (uint64_t)__builtin_popcountll(dm & (bit - 1));
            b.ops.push_back({dst, kOpUpload << 30 | (uint32_t)(stage_first + rank_in)});
        } else if (old.mask & bit) {
            const uint32_t src = old.slot_of(brick) - 1;
            if (src != dst) {
                b.ops.push_back({dst, kOpMove << 30 | (uint32_t)b.gathers.size()});
                b.gathers.push_back(src);
            }
        } else {
            b.ops.push_back({dst, kOpZero << 30});
        }
    }
    SectorRec& rec = w->h_table[s];
    rec.mask_lo = (uint32_t)cur.mask;
    rec.mask_hi = (uint32_t)(cur.mask >> 32);
    rec.base = cur.base ? cur.base - 1 : 0;
    rec.flags = 0;
    b.touched.push_back(s);
    return VRT_OK;
}

// Re-derive the sector-group masks and the whole brick table from the device sector
// table (a sector's emptiness changes the GLSL-mode entries of its whole group).
cudaError_t rebuild_brick_table(vrt_world* w, cudaStream_t stream) {
    const uint32_t ng = w->num_groups();
    group_masks_kernel<<<(ng + 3) / 4, 128, 0, stream>>>(w->d_sectors, w->sx, w->sy, w->sz,
                                                       (unsigned long long*)w->d_groups);
    const uint32_t ns = w->num_sectors(), n = ns * 64;
    brick_table_kernel<<<(n + 255) / 256, 256, 0, stream>>>(w->d_sectors, (const unsigned long long*)w->d_groups, 0,
                                                           ns, w->sx, w->sz, w->d_bricks);
    return cudaGetLastError();
}

// The same for the groups of the given sectors only (device list in `list`, at most
// num_groups entries); the whole table when they are most of the world.
vrt_status rebuild_brick_table_for(vrt_world* w, const std::vector<uint32_t>& sectors, cudaStream_t stream) {
    const uint32_t gx = (w->sx + 3) / 4, gz = (w->sz + 3) / 4;
    std::vector<uint32_t> gl;
    gl.reserve(sectors.size());
    for (uint32_t s : sectors) {
        const uint32_t x = s % w->sx, z = (s / w->sx) % w->sz, y = s / (w->sx * w->sz);
        gl.push_back((x >> 2) + (z >> 2) * gx + (y >> 2) * gx * gz);
    }
    std::sort(gl.begin(), gl.end());
    gl.erase(std::unique(gl.begin(), gl.end()), gl.end());
    if ((uint64_t)gl.size() * 4 >= w->num_groups()) {
        VRT_CUDA(rebuild_brick_table(w, stream));
        return VRT_OK;
    }
    VRT_CUDA(w->d_glist.reserve(gl.size() * sizeof(uint32_t)));
    VRT_CUDA(cudaMemcpyAsync(w->d_glist.ptr, gl.data(), gl.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
    const uint32_t ng = w->num_groups();
    group_masks_kernel<<<(ng + 3) / 4, 128, 0, stream>>>(w->d_sectors, w->sx, w->sy, w->sz,
                                                       (unsigned long long*)w->d_groups);
    const uint32_t n = (uint32_t)gl.size() * 4096u;
    brick_table_groups_kernel<<<(n + 255) / 256, 256, 0, stream>>>(
        w->d_sectors, (const unsigned long long*)w->d_groups, (const uint32_t*)w->d_glist.ptr, (uint32_t)gl.size(),
        w->sx, w->sy, w->sz, w->d_bricks);
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

}  // namespace

vrt_status rebuild_table_groups(vrt_world* w, const uint32_t* d_groups, uint32_t n, cudaStream_t stream) {
    if (!d_groups || (uint64_t)n * 4 >= w->num_groups()) {
        VRT_CUDA(rebuild_brick_table(w, stream));
        return VRT_OK;
    }
    if (n == 0) return VRT_OK;
    const uint32_t ng = w->num_groups();
    group_masks_kernel<<<(ng + 3) / 4, 128, 0, stream>>>(w->d_sectors, w->sx, w->sy, w->sz,
                                                       (unsigned long long*)w->d_groups);
    const uint32_t k = n * 4096u;
    brick_table_groups_kernel<<<(k + 255) / 256, 256, 0, stream>>>(w->d_sectors, (const unsigned long long*)w->d_groups,
                                                                 d_groups, n, w->sx, w->sy, w->sz, w->d_bricks);
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

namespace {

vrt_status run_batch(vrt_world* w, SyncBatch& b, cudaStream_t stream) {
    if (b.ops.empty() && b.touched.empty()) return VRT_OK;
    const size_t stage_bytes = (size_t)b.n_stage * 512;
    if (stage_bytes) {
        VRT_CUDA(w->d_stage.reserve(stage_bytes));
        VRT_CUDA(cudaMemcpyAsync(w->d_stage.ptr, b.src, stage_bytes, cudaMemcpyHostToDevice, stream));
    }
    const size_t gbytes = b.gathers.size() * sizeof(uint32_t);
    const size_t obytes = b.ops.size() * sizeof(BrickOp);
    const size_t ooff = (gbytes + 15) & ~size_t(15);
    if (gbytes + obytes) {
        VRT_CUDA(w->d_ops.reserve(ooff + obytes, true));
        if (gbytes) VRT_CUDA(cudaMemcpyAsync(w->d_ops.ptr, b.gathers.data(), gbytes, cudaMemcpyHostToDevice, stream));
        if (obytes)
            VRT_CUDA(cudaMemcpyAsync((uint8_t*)w->d_ops.ptr + ooff, b.ops.data(), obytes, cudaMemcpyHostToDevice, stream));
    }
    const size_t ng = b.gathers.size();
    if (ng) {
        VRT_CUDA(w->d_scratch.reserve(ng * 1088, true));
        uint8_t* sp = (uint8_t*)w->d_scratch.ptr;
        uint4* sc = (uint4*)(sp + ng * 512);
        uint64_t* sm = (uint64_t*)(sp + ng * 1024);
        gather_bricks_kernel<<<ops_grid((uint32_t)ng), kOpsWarps * 32, 0, stream>>>(
            (const uint32_t*)w->d_ops.ptr, (uint32_t)ng, w->d_payload, w->d_codes, w->d_cells, sp, sc, sm);
        VRT_CUDA(cudaGetLastError());
    }
    if (!b.ops.empty()) {
        uint8_t* sp = (uint8_t*)w->d_scratch.ptr;
        uint4* sc = sp ? (uint4*)(sp + ng * 512) : nullptr;
        uint64_t* sm = sp ? (uint64_t*)(sp + ng * 1024) : nullptr;
        brick_ops_kernel<<<ops_grid((uint32_t)b.ops.size()), kOpsWarps * 32, 0, stream>>>(
            (const BrickOp*)((uint8_t*)w->d_ops.ptr + ooff), (uint32_t)b.ops.size(), (const uint8_t*)w->d_stage.ptr,
            sp, sc, sm, w->d_payload, w->d_codes, w->d_cells);
        VRT_CUDA(cudaGetLastError());
    }
    // sector headers: copy the span of touched records
    if (!b.touched.empty()) {
        auto mm = std::minmax_element(b.touched.begin(), b.touched.end());
        const uint32_t lo = *mm.first, hi = *mm.second + 1;
        VRT_CUDA(cudaMemcpyAsync(w->d_sectors + lo, w->h_table.data() + lo, (size_t)(hi - lo) * sizeof(SectorRec),
                                 cudaMemcpyHostToDevice, stream));
        vrt_status st = rebuild_brick_table_for(w, b.touched, stream);
        if (st != VRT_OK) return st;
    }
    vrt_status st = alloc_publish(w, stream);
    if (st != VRT_OK) return st;
    VRT_CUDA(cudaStreamSynchronize(stream));
    b = SyncBatch();
    return VRT_OK;
}

}  // namespace

}  // namespace vrt

using namespace vrt;

extern "C" {

const char* vrt_last_error(void) { return vrt::last_error_cstr(); }

uint32_t vrt_abi_version(void) { return VRT_ABI_VERSION; }

int32_t vrt_sector_index(int32_t sx, int32_t sy, int32_t sz) { return sector_index_pack(sx, sy, sz); }

vrt_status vrt_world_create(const vrt_world_desc* desc, vrt_world** out) {
    if (!desc || !out) {
        set_error("null argument");
        return VRT_ERR_INVALID_ARG;
    }
    *out = nullptr;
    if (desc->sectors_x == 0 || desc->sectors_y == 0 || desc->sectors_z == 0 ||
        desc->sectors_x * 32 > VRT_MAX_WORLD_X || desc->sectors_y * 32 > VRT_MAX_WORLD_Y ||
        desc->sectors_z * 32 > VRT_MAX_WORLD_Z) {
        set_error("world extent must be 1..64 x 1..32 x 1..64 sectors");
        return VRT_ERR_INVALID_ARG;
    }
    if (desc->flags & ~VRT_WORLD_L2_PERSIST) {
        set_error("unknown world flags");
        return VRT_ERR_INVALID_ARG;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return VRT_ERR_NO_DEVICE;
    }
    if (desc->device < 0 || desc->device >= ndev) {
        set_error("device ordinal out of range");
        return VRT_ERR_INVALID_ARG;
    }
    vrt_world* w = new vrt_world;
    w->device = desc->device;
    w->sx = desc->sectors_x;
    w->sy = desc->sectors_y;
    w->sz = desc->sectors_z;
    w->flags = desc->flags;
    w->slots.assign(w->num_sectors(), SectorSlots{});
    w->h_table.assign(w->num_sectors(), SectorRec{0, 0, 0, 0});
    w->arena.reset(0);
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st == VRT_OK) {
        e = cudaMalloc(&w->d_sectors, (size_t)w->num_sectors() * sizeof(SectorRec));
        if (e == cudaSuccess) e = cudaMemset(w->d_sectors, 0, (size_t)w->num_sectors() * sizeof(SectorRec));
        if (e == cudaSuccess) e = cudaMalloc(&w->d_bricks, w->num_brick_positions() * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&w->d_groups, (size_t)w->num_groups() * sizeof(uint64_t));
        // the group list of incremental table rebuilds, at its largest size: it never
        // grows (a growing buffer's cudaFree would wait for the whole device)
        if (e == cudaSuccess) e = w->d_glist.reserve((size_t)w->num_groups() * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&w->d_alloc, sizeof(DevAlloc));
        if (e == cudaSuccess) e = cudaMemset(w->d_alloc, 0, sizeof(DevAlloc));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->edited, cudaEventDisableTiming);
        // edit scratch for batches of up to a few thousand touched sectors: a buffer that
        // grows later frees its old block, and cudaFree waits for the whole device
        if (e == cudaSuccess) e = w->d_edit.reserve(256 << 10);
        if (e == cudaSuccess) e = w->d_gc.reserve(64 << 10);
        for (auto& stage : w->edit_stage)
            if (e == cudaSuccess) e = stage.acquire(64 << 10);
        if (e == cudaSuccess) e = rebuild_brick_table(w, 0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(0);
        if (e != cudaSuccess) st = cuda_fail(e, "allocate sector table");
    }
    if (st == VRT_OK) st = grow_pool(w, desc->brick_capacity ? desc->brick_capacity : 4096, 0);
    if (st == VRT_OK) st = alloc_publish(w, 0);
    if (st == VRT_OK && (w->flags & VRT_WORLD_L2_PERSIST)) st = setup_l2_window(w);
    if (st == VRT_OK && cudaStreamSynchronize(0) != cudaSuccess) st = cuda_fail(cudaGetLastError(), "create world");
    if (st != VRT_OK) {
        vrt_world_destroy(w);
        return st;
    }
    *out = w;
    return VRT_OK;
}

vrt_status vrt_world_destroy(vrt_world* w) {
    if (!w) return VRT_OK;
    DeviceScope ds;
    ds.enter(w->device);
    cudaDeviceSynchronize();
    if (w->d_sectors) cudaFree(w->d_sectors);
    if (w->d_bricks) cudaFree(w->d_bricks);
    if (w->d_groups) cudaFree(w->d_groups);
    if (w->d_codes) cudaFree(w->d_codes);
    if (w->d_payload) cudaFree(w->d_payload);
    if (w->d_cells) cudaFree(w->d_cells);
    w->d_stage.release();
    w->d_ops.release();
    w->d_scratch.release();
    w->d_io.release();
    w->d_glist.release();
    w->d_edit.release();
    w->d_gc.release();
    for (auto& stage : w->edit_stage) stage.destroy();
    if (w->d_alloc) cudaFree(w->d_alloc);
    if (w->edited) cudaEventDestroy(w->edited);
    delete w;
    return VRT_OK;
}

vrt_status vrt_world_get_stats(const vrt_world* cw, vrt_world_stats* out) {
    if (!cw || !out) {
        set_error("null argument");
        return VRT_ERR_INVALID_ARG;
    }
    // the host mirror is rebuilt from the device after device edits (a cache of the
    // device's state, not a change to the world)
    vrt_world* w = const_cast<vrt_world*>(cw);
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK) return st;
    std::lock_guard<std::mutex> lock(w->mu);
    if ((st = refresh_host_mirror(w)) != VRT_OK) return st;
    out->sectors_x = w->sx;
    out->sectors_y = w->sy;
    out->sectors_z = w->sz;
    out->allocated_bricks = w->arena.allocated();
    out->brick_capacity = w->capacity;
    out->free_ranges = (uint32_t)w->arena.num_ranges();
    out->compactions = w->compactions;
    out->reserved = 0;
    // sector records, brick table, group masks, per slot 512 B payload + 512 B codes +
    // 64 B cell masks, and the scratch buffers
    out->device_bytes = (uint64_t)w->num_sectors() * sizeof(SectorRec) + (uint64_t)w->num_brick_positions() * 4 +
                        (uint64_t)w->num_groups() * 8 + (uint64_t)w->capacity * 1088 + w->d_stage.bytes +
                        w->d_ops.bytes + w->d_scratch.bytes + w->d_io.bytes + w->d_glist.bytes + w->d_edit.bytes +
                        w->d_gc.bytes;
    return VRT_OK;
}

vrt_status vrt_world_sync_sectors(vrt_world* w, uint32_t n, const int32_t* sector_idx, const uint64_t* alloc_mask,
                                  const uint64_t* dirty_mask, const uint8_t* bricks, void* stream_) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK) return st;
    if (n && (!sector_idx || !alloc_mask)) {
        set_error("null sector arrays");
        return VRT_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(w->mu);
    if ((st = refresh_host_mirror(w)) != VRT_OK) return st;
    cudaStream_t stream = (cudaStream_t)stream_;
    const uint64_t kBatchBricks = 1ull << 19;  // 256 MiB of staged bricks per batch
    SyncBatch batch;
    std::unordered_set<uint32_t> seen;
    uint64_t in_brick = 0;  // index of the next brick in the input stream
    for (uint32_t i = 0; i < n; i++) {
        const uint64_t am = alloc_mask[i];
        const uint64_t dm = dirty_mask ? (dirty_mask[i] & am) : am;
        const uint64_t cnt = (uint64_t)__builtin_popcountll(dm);
        if (cnt && !bricks) {
            set_error("null brick data");
            return VRT_ERR_INVALID_ARG;
        }
        int32_t x, y, z;
        sector_index_unpack(sector_idx[i], x, y, z);
        if (w->sector_in(x, y, z)) {
            const uint32_t s = w->lin(x, y, z);
            if (seen.count(s) || batch.n_stage + cnt > kBatchBricks) {
                if ((st = run_batch(w, batch, stream)) != VRT_OK) return st;
                seen.clear();
            }
            if (batch.ops.empty() && batch.touched.empty()) {
                batch.src = bricks ? bricks + in_brick * 512 : nullptr;
                batch.n_stage = 0;
            }
            // stage index relative to the batch's first input brick
            const uint64_t first = (bricks ? (in_brick - (uint64_t)(batch.src - bricks) / 512) : 0);
            if ((st = plan_sector(w, batch, s, am, dm, first, stream)) != VRT_OK) return st;
            batch.n_stage = first + cnt;
            seen.insert(s);
        }
        in_brick += cnt;
    }
    return run_batch(w, batch, stream);
}

vrt_status vrt_world_save_cvox(vrt_world* w, const char* path) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK) return st;
    std::vector<int32_t> idx;
    std::vector<uint64_t> masks;
    std::vector<uint8_t> bricks;
    {
        std::lock_guard<std::mutex> lock(w->mu);
        if ((st = refresh_host_mirror(w)) != VRT_OK) return st;
        for (uint32_t y = 0; y < w->sy; y++)
            for (uint32_t z = 0; z < w->sz; z++)
                for (uint32_t x = 0; x < w->sx; x++) {
                    const SectorSlots& s = w->slots[w->lin((int32_t)x, (int32_t)y, (int32_t)z)];
                    if (!s.mask) continue;
                    idx.push_back(sector_index_pack((int32_t)x, (int32_t)y, (int32_t)z));
                    masks.push_back(s.mask);
                    const size_t nb = (size_t)__builtin_popcountll(s.mask);
                    const size_t off = bricks.size();
                    bricks.resize(off + nb * 512);
                    VRT_CUDA(cudaMemcpy(bricks.data() + off, w->d_payload + (size_t)(s.base - 1) * 512, nb * 512,
                                        cudaMemcpyDeviceToHost));
                }
    }
    return vrt_cvox_write(path, (uint32_t)idx.size(), idx.data(), masks.data(), bricks.data());
}

vrt_status vrt_world_load_cvox(vrt_world* w, const char* path, void* stream) {
    vrt_sector_stream* s = nullptr;
    vrt_status st = vrt_cvox_read(path, &s);
    if (st != VRT_OK) return st;
    st = vrt_world_sync_sectors(w, s->n_sectors, s->sector_idx, s->alloc_mask, nullptr, s->bricks, stream);
    vrt_sector_stream_free(s);
    return st;
}

vrt_status vrt_world_read_sector(vrt_world* w, int32_t sector_idx, uint64_t* alloc_mask, uint8_t* bricks,
                                 size_t bricks_capacity, void* stream_) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK) return st;
    int32_t x, y, z;
    sector_index_unpack(sector_idx, x, y, z);
    if (!w->sector_in(x, y, z)) {
        set_error("sector outside the world");
        return VRT_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(w->mu);
    if ((st = refresh_host_mirror(w)) != VRT_OK) return st;
    const SectorSlots& s = w->slots[w->lin(x, y, z)];
    if (alloc_mask) *alloc_mask = s.mask;
    const size_t need = (size_t)__builtin_popcountll(s.mask) * 512;
    if (!bricks || need == 0) return VRT_OK;
    if (bricks_capacity < need) {
        set_error("brick buffer too small");
        return VRT_ERR_INVALID_ARG;
    }
    cudaStream_t stream = (cudaStream_t)stream_;
    VRT_CUDA(cudaMemcpyAsync(bricks, w->d_payload + (size_t)(s.base - 1) * 512, need, cudaMemcpyDeviceToHost, stream));
    VRT_CUDA(cudaStreamSynchronize(stream));
    return VRT_OK;
}

}  // extern "C"
