// edit.cu - the edit path: sphere fill/carve on device bricks, brick allocation and
// empty-brick GC, with the voxel-cell masks re-derived in the same kernel.
//
// Semantics of VoxelMap::RegionDispatchSIMD + GC (src/VoxelRT/VoxelMap.h:222-263)
// driving the brush (src/VoxelRT/Brush.cpp:10-31), per edit in order: every brick
// in the edit's brick bounding box is visited (created first for fills), voxels
// with |v - c|^2 <= r^2 are set, and visited bricks that end up empty are freed.
// Because voxels are independent, the batch is applied as
//   1. host: bricks a fill reaches that are not allocated get slots (sector repack);
//   2. device: one warp per touched brick applies every edit of the batch in order,
//      derives the 8 cell masks by ballot, stores the voxel codes and flags empty
//      bricks;
//   3. host: empty bricks are freed (sector repack).
// The final state equals applying the edits one by one.

#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <vector>

#include "brick_codes.cuh"
#include "world.h"

namespace vrt {

// defined in world.cu
vrt_status world_repack(vrt_world* w, const std::map<uint32_t, uint64_t>& new_masks, cudaStream_t stream);

namespace {

struct EditDev {
    int32_t cx, cy, cz;
    int32_t r2;
    int32_t lo[3], hi[3];  // brick bounding box (inclusive)
    uint32_t material;
    uint32_t replace;
};

struct TouchedBrick {
    uint32_t slot;        // 0-based
    uint32_t bx, by, bz;  // brick coordinates in the world
};

constexpr int kEditWarps = 8;

__global__ void __launch_bounds__(kEditWarps * 32)
    edit_bricks_kernel(const TouchedBrick* __restrict__ bricks, uint32_t n, const EditDev* __restrict__ edits,
                       uint32_t n_edits, uint8_t* __restrict__ payload, uint4* __restrict__ codes,
                       uint64_t* __restrict__ cell_masks,
                       uint8_t* __restrict__ empty) {
    __shared__ __align__(16) uint8_t sb[kEditWarps][512];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (uint32_t k = blockIdx.x * kEditWarps + wib; k < n; k += gridDim.x * kEditWarps) {
        const TouchedBrick tb = bricks[k];
        uint4 v = reinterpret_cast<const uint4*>(payload + (size_t)tb.slot * 512)[lane];
        uint8_t* b = reinterpret_cast<uint8_t*>(&v);
        // lane holds voxels 16*lane .. 16*lane+15: y = lane>>2, z = 2*(lane&3) + (j>>3), x = j&7
        const int32_t y = (int32_t)(tb.by * 8 + (lane >> 2));
        const int32_t z0 = (int32_t)(tb.bz * 8 + 2 * (lane & 3));
        const int32_t x0 = (int32_t)(tb.bx * 8);
        for (uint32_t e = 0; e < n_edits; e++) {
            const EditDev ed = edits[e];
            if ((int32_t)tb.bx < ed.lo[0] || (int32_t)tb.bx > ed.hi[0] || (int32_t)tb.by < ed.lo[1] ||
                (int32_t)tb.by > ed.hi[1] || (int32_t)tb.bz < ed.lo[2] || (int32_t)tb.bz > ed.hi[2])
                continue;
            const int32_t dy = y - ed.cy;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int32_t dx = x0 + (j & 7) - ed.cx, dz = z0 + (j >> 3) - ed.cz;
                if (dx * dx + dy * dy + dz * dz > ed.r2) continue;
                if (ed.replace && b[j] == 0) continue;
                b[j] = (uint8_t)ed.material;
            }
        }
        reinterpret_cast<uint4*>(payload + (size_t)tb.slot * 512)[lane] = v;
        reinterpret_cast<uint4*>(sb[wib])[lane] = v;
        __syncwarp();
        const uint64_t cells = warp_cell_mask(sb[wib], lane);
        codes[(size_t)tb.slot * 32 + lane] = warp_voxel_codes(sb[wib], cells, lane);
        if (lane < 8) cell_masks[(size_t)tb.slot * 8 + lane] = cells;
        const bool any = __any_sync(0xffffffffu, cells != 0);
        if (lane == 0) empty[k] = any ? 0 : 1;
        __syncwarp();
    }
}

// Closest voxel of the brick to the center lies within the sphere.
bool sphere_reaches_brick(const vrt_edit& e, int32_t bx, int32_t by, int32_t bz) {
    const int32_t b[3] = {bx, by, bz};
    int64_t d2 = 0;
    for (int c = 0; c < 3; c++) {
        const int64_t lo = (int64_t)b[c] * 8, hi = lo + 7;
        const int64_t p = std::min(std::max<int64_t>(e.center[c], lo), hi);
        d2 += (p - e.center[c]) * (p - e.center[c]);
    }
    return d2 <= (int64_t)e.radius * e.radius;
}

}  // namespace
}  // namespace vrt

using namespace vrt;

extern "C" vrt_status vrt_world_edit(vrt_world* w, const vrt_edit* edits, uint32_t n, void* stream_) {
    vrt_status st = world_enter(w);
    if (st != VRT_OK) return st;
    if (n == 0) return VRT_OK;
    if (!edits) {
        set_error("null edit array");
        return VRT_ERR_INVALID_ARG;
    }
    for (uint32_t i = 0; i < n; i++)
        if (edits[i].radius > 4096 || edits[i].mode > VRT_EDIT_REPLACE || edits[i].reserved) {
            set_error("edit radius must be <= 4096, mode FILL or REPLACE, reserved 0");
            return VRT_ERR_INVALID_ARG;
        }
    std::lock_guard<std::mutex> lock(w->mu);
    cudaStream_t stream = (cudaStream_t)stream_;
    const int32_t nb[3] = {(int32_t)w->sx * 4, (int32_t)w->sy * 4, (int32_t)w->sz * 4};
    auto brick_bit = [](int32_t bx, int32_t by, int32_t bz) {
        return 1ull << ((bx & 3) | (bz & 3) << 2 | (by & 3) << 4);
    };
    // 1. touched bricks and bricks to create
    std::vector<EditDev> ed(n);
    std::map<uint32_t, uint64_t> grow;     // sector -> mask with created bricks
    std::map<uint64_t, bool> touched;      // packed brick coords
    for (uint32_t i = 0; i < n; i++) {
        const vrt_edit& e = edits[i];
        EditDev& d = ed[i];
        d.cx = e.center[0];
        d.cy = e.center[1];
        d.cz = e.center[2];
        d.r2 = (int32_t)(e.radius * e.radius);
        d.material = e.material;
        d.replace = e.mode == VRT_EDIT_REPLACE;
        bool empty_box = false;
        for (int c = 0; c < 3; c++) {
            const int64_t lo = ((int64_t)e.center[c] - e.radius) >> 3, hi = ((int64_t)e.center[c] + e.radius) >> 3;
            d.lo[c] = (int32_t)std::max<int64_t>(lo, 0);
            d.hi[c] = (int32_t)std::min<int64_t>(hi, nb[c] - 1);
            if (d.lo[c] > d.hi[c]) empty_box = true;
        }
        if (empty_box) {
            d.lo[0] = 1, d.hi[0] = 0;  // never matches
            continue;
        }
        const bool creates = e.material != 0 && e.mode == VRT_EDIT_FILL;
        for (int32_t by = d.lo[1]; by <= d.hi[1]; by++)
            for (int32_t bz = d.lo[2]; bz <= d.hi[2]; bz++)
                for (int32_t bx = d.lo[0]; bx <= d.hi[0]; bx++) {
                    const uint32_t s = w->lin(bx >> 2, by >> 2, bz >> 2);
                    const uint64_t bit = brick_bit(bx, by, bz);
                    const uint64_t have = w->slots[s].mask | (grow.count(s) ? grow[s] : 0);
                    if (have & bit) {
                        touched[(uint64_t)bx | (uint64_t)by << 21 | (uint64_t)bz << 42] = true;
                    } else if (creates && sphere_reaches_brick(e, bx, by, bz)) {
                        grow[s] |= w->slots[s].mask | bit;
                        touched[(uint64_t)bx | (uint64_t)by << 21 | (uint64_t)bz << 42] = true;
                    }
                }
    }
    if (touched.empty()) return VRT_OK;
    if (!grow.empty() && (st = world_repack(w, grow, stream)) != VRT_OK) return st;
    // 2. device edit over the touched bricks
    std::vector<TouchedBrick> tb;
    tb.reserve(touched.size());
    for (auto& kv : touched) {
        const int32_t bx = (int32_t)(kv.first & 0x1FFFFF), by = (int32_t)((kv.first >> 21) & 0x1FFFFF),
                      bz = (int32_t)(kv.first >> 42);
        const uint32_t s = w->lin(bx >> 2, by >> 2, bz >> 2);
        const uint32_t b = (uint32_t)((bx & 3) | (bz & 3) << 2 | (by & 3) << 4);
        tb.push_back({w->slots[s].slot_of(b) - 1, (uint32_t)bx, (uint32_t)by, (uint32_t)bz});
    }
    const size_t eb = ed.size() * sizeof(EditDev), bb = tb.size() * sizeof(TouchedBrick);
    const size_t boff = (eb + 15) & ~size_t(15), foff = (boff + bb + 15) & ~size_t(15);
    VRT_CUDA(w->d_ops.reserve(foff + tb.size(), true));
    uint8_t* base = (uint8_t*)w->d_ops.ptr;
    VRT_CUDA(cudaMemcpyAsync(base, ed.data(), eb, cudaMemcpyHostToDevice, stream));
    VRT_CUDA(cudaMemcpyAsync(base + boff, tb.data(), bb, cudaMemcpyHostToDevice, stream));
    const uint32_t blocks = std::max(1u, std::min<uint32_t>(((uint32_t)tb.size() + kEditWarps - 1) / kEditWarps, 152u * 16u));
    edit_bricks_kernel<<<blocks, kEditWarps * 32, 0, stream>>>((const TouchedBrick*)(base + boff), (uint32_t)tb.size(),
                                                               (const EditDev*)base, n, w->d_payload, w->d_codes,
                                                               w->d_cells,
                                                               base + foff);
    VRT_CUDA(cudaGetLastError());
    std::vector<uint8_t> empty(tb.size());
    VRT_CUDA(cudaMemcpyAsync(empty.data(), base + foff, tb.size(), cudaMemcpyDeviceToHost, stream));
    VRT_CUDA(cudaStreamSynchronize(stream));
    // 3. free the bricks that became empty
    std::map<uint32_t, uint64_t> shrink;
    for (size_t i = 0; i < tb.size(); i++) {
        if (!empty[i]) continue;
        const uint32_t s = w->lin((int32_t)tb[i].bx >> 2, (int32_t)tb[i].by >> 2, (int32_t)tb[i].bz >> 2);
        if (!shrink.count(s)) shrink[s] = w->slots[s].mask;
        shrink[s] &= ~brick_bit((int32_t)tb[i].bx, (int32_t)tb[i].by, (int32_t)tb[i].bz);
    }
    if (!shrink.empty() && (st = world_repack(w, shrink, stream)) != VRT_OK) return st;
    return VRT_OK;
}
