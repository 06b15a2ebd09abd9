// edit.cu - the edit path on the device: sphere fill/carve on device bricks, brick
// allocation for fills and empty-brick GC, with the occupancy and voxel codes of every
// edited brick re-derived in the same kernel, and no host round trip.
//
// Semantics of VoxelMap::RegionDispatchSIMD + GC (src/VoxelRT/VoxelMap.h:222-263)
// driving the brush (src/VoxelRT/Brush.cpp:10-31), per edit in order: every brick in the
// edit's brick bounding box is visited (created first for fills), voxels with
// |v - c|^2 <= r^2 are set, and visited bricks that end up empty are freed.  Because
// voxels are independent, a batch of edits is applied as
//   host (geometry only, no device state): the sectors the edits' boxes touch, per
//       sector the bricks inside a box (`visit`) and the bricks a fill sphere reaches
//       (`create`), and the sector groups whose brick-table entries follow them;
//   1. relayout_kernel<true>: sectors gaining bricks move to a fresh range from the
//      device's bump allocator (alloc.cu) and zero-fill the new bricks;
//   2. edit_bricks_kernel: one warp per visited allocated brick applies every edit of
//      the batch in order, derives the 8 cell masks by ballot, stores the voxel codes
//      and flags the brick when it is empty;
//   3. relayout_kernel<false>: sectors with emptied bricks drop them in place;
//   4. the group masks and brick-table entries of the touched groups.
// The final state equals applying the edits one by one.  The call only enqueues this
// work on the stream (one upload of the batch from pinned memory and the kernels); the
// host reads nothing back, except when its bound of the bump pointer says the pool may
// be full, and then it compacts the pool first (alloc.cu).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "brick_codes.cuh"
#include "world.h"

namespace vrt {
namespace {

struct EditDev {
    int32_t cx, cy, cz;
    int32_t r2;
    int32_t lo[3], hi[3];  // brick bounding box (inclusive)
    uint32_t material;
    uint32_t replace;
};

// A sector an edit batch touches: bricks inside an edit's box, bricks a fill creates.
struct EditSector {
    unsigned long long visit, create;
    uint32_t sector, pad;
};
static_assert(sizeof(EditSector) == 24, "edit sector records are 24 bytes");

constexpr uint32_t kNoSlot = 0xFFFFFFFFu;
constexpr int kEditWarps = 8;

// Copy brick slot src to slot dst (payload, voxel codes, cell masks: 68 16-byte words),
// or zero-fill dst (an empty brick) when src is kNoSlot; threads [0, n) share the words.
__device__ __forceinline__ void move_brick(uint8_t* __restrict__ payload, uint4* __restrict__ codes,
                                           uint64_t* __restrict__ cells, uint32_t src, uint32_t dst, uint32_t t,
                                           uint32_t n) {
    for (uint32_t k = t; k < 68; k += n) {
        if (k < 32) {
            uint4* d = reinterpret_cast<uint4*>(payload + (size_t)dst * 512) + k;
            *d = src == kNoSlot ? make_uint4(0, 0, 0, 0)
                                : reinterpret_cast<const uint4*>(payload + (size_t)src * 512)[k];
        } else if (k < 64) {
            codes[(size_t)dst * 32 + (k - 32)] =
                src == kNoSlot ? empty_brick_codes() : codes[(size_t)src * 32 + (k - 32)];
        } else {
            uint4* d = reinterpret_cast<uint4*>(cells + (size_t)dst * 8) + (k - 64);
            *d = src == kNoSlot ? make_uint4(0, 0, 0, 0)
                                : reinterpret_cast<const uint4*>(cells + (size_t)src * 8)[k - 64];
        }
    }
}

// Relayout of the touched sectors whose mask the batch changes, one block per touched
// sector.  kGrow: new mask = old | create; the sector takes popcount(new) slots at the
// bump pointer, its bricks move there, created bricks are zero-filled, and its old
// range is left as garbage.  Otherwise: new mask = old & ~emptied; the remaining bricks
// move down in place in ascending order: every brick's destination lies at or below its
// source, and a brick's source lies above the destinations of the bricks before it, so
// moving one brick at a time in that order never overwrites a brick not yet moved.
template <bool kGrow>
__global__ void __launch_bounds__(96)
    relayout_kernel(const EditSector* __restrict__ ts, uint32_t m, const unsigned long long* __restrict__ emptied,
                    SectorRec* __restrict__ sectors, DevAlloc* __restrict__ alloc, uint8_t* __restrict__ payload,
                    uint4* __restrict__ codes, uint64_t* __restrict__ cells) {
    const uint32_t i = blockIdx.x, t = threadIdx.x;
    if (i >= m) return;
    const uint32_t s = ts[i].sector;
    const SectorRec rec = sectors[s];
    const uint64_t old = (uint64_t)rec.mask_hi << 32 | rec.mask_lo;
    const uint64_t nm = kGrow ? (old | ts[i].create) : (old & ~emptied[i]);
    if (nm == old) return;  // the whole block
    __shared__ uint32_t s_dst;
    if (t == 0) {
        const uint32_t n_new = (uint32_t)__popcll(nm), n_old = (uint32_t)__popcll(old);
        if (kGrow) {
            const uint32_t b = atomicAdd(&alloc->top, n_new);
            if ((uint64_t)b + n_new > alloc->cap) {
                atomicExch(&alloc->overflow, 1u);  // never, while the host's bound of the pointer holds
                s_dst = kNoSlot;
            } else {
                atomicAdd(&alloc->live, n_new - n_old);
                s_dst = b;
            }
        } else {
            atomicSub(&alloc->live, n_old - n_new);
            s_dst = rec.base;
        }
    }
    __syncthreads();
    const uint32_t dst_base = s_dst;
    if (dst_base == kNoSlot) return;
    uint32_t k = 0;
    for (uint64_t r = nm; r; r &= r - 1, k++) {
        const uint64_t bit = r & (~r + 1);
        const uint32_t src = (old & bit) ? rec.base + (uint32_t)__popcll(old & (bit - 1)) : kNoSlot;
        if (src == dst_base + k) continue;
        move_brick(payload, codes, cells, src, dst_base + k, t, blockDim.x);
        __syncthreads();
    }
    if (t == 0) {
        SectorRec out = rec;
        out.mask_lo = (uint32_t)nm;
        out.mask_hi = (uint32_t)(nm >> 32);
        out.base = nm ? dst_base : 0;
        sectors[s] = out;
    }
}

// One warp per (touched sector i, brick b): a visited brick that is allocated takes every
// edit of the batch in order; its cell masks and voxel codes are re-derived, and an
// emptied brick is flagged in emptied[i].
__global__ void __launch_bounds__(kEditWarps * 32)
    edit_bricks_kernel(const EditSector* __restrict__ ts, uint32_t m, const EditDev* __restrict__ edits,
                       uint32_t n_edits, const SectorRec* __restrict__ sectors, uint32_t sx, uint32_t sz,
                       uint8_t* __restrict__ payload, uint4* __restrict__ codes, uint64_t* __restrict__ cell_masks,
                       unsigned long long* __restrict__ emptied) {
    __shared__ __align__(16) uint8_t sb[kEditWarps][512];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t gw = blockIdx.x * kEditWarps + wib;
    const uint32_t i = gw >> 6, b = gw & 63u;
    if (i >= m) return;  // whole warps
    const unsigned long long bit = 1ull << b;
    if (!(ts[i].visit & bit)) return;
    const uint32_t s = ts[i].sector;
    const SectorRec rec = sectors[s];
    const uint64_t mask = (uint64_t)rec.mask_hi << 32 | rec.mask_lo;
    if (!(mask & bit)) return;
    const uint32_t slot = rec.base + (uint32_t)__popcll(mask & (bit - 1));
    const uint32_t bx = (s % sx) * 4 + (b & 3u), bz = ((s / sx) % sz) * 4 + ((b >> 2) & 3u),
                   by = (s / (sx * sz)) * 4 + (b >> 4);
    uint4 v = reinterpret_cast<const uint4*>(payload + (size_t)slot * 512)[lane];
    uint8_t* bytes = reinterpret_cast<uint8_t*>(&v);
    // lane holds voxels 16*lane .. 16*lane+15: y = lane>>2, z = 2*(lane&3) + (j>>3), x = j&7
    const int32_t y = (int32_t)(by * 8 + (lane >> 2));
    const int32_t z0 = (int32_t)(bz * 8 + 2 * (lane & 3));
    const int32_t x0 = (int32_t)(bx * 8);
    for (uint32_t e = 0; e < n_edits; e++) {
        const EditDev ed = edits[e];
        if ((int32_t)bx < ed.lo[0] || (int32_t)bx > ed.hi[0] || (int32_t)by < ed.lo[1] || (int32_t)by > ed.hi[1] ||
            (int32_t)bz < ed.lo[2] || (int32_t)bz > ed.hi[2])
            continue;
        const int32_t dy = y - ed.cy;
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int32_t dx = x0 + (j & 7) - ed.cx, dz = z0 + (j >> 3) - ed.cz;
            if (dx * dx + dy * dy + dz * dz > ed.r2) continue;
            if (ed.replace && bytes[j] == 0) continue;
            bytes[j] = (uint8_t)ed.material;
        }
    }
    reinterpret_cast<uint4*>(payload + (size_t)slot * 512)[lane] = v;
    reinterpret_cast<uint4*>(sb[wib])[lane] = v;
    __syncwarp();
    const uint64_t cells = warp_cell_mask(sb[wib], lane);
    codes[(size_t)slot * 32 + lane] = warp_voxel_codes(sb[wib], cells, lane);
    if (lane < 8) cell_masks[(size_t)slot * 8 + lane] = cells;
    if (!__any_sync(0xffffffffu, cells != 0) && lane == 0) atomicOr(emptied + i, bit);
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

// Bits of the bricks of a sector whose in-sector coordinates lie in [lo, hi] per axis
// (brick bit x | z<<2 | y<<4).
uint64_t box_bits(const int32_t lo[3], const int32_t hi[3]) {
    uint64_t m = 0;
    for (int32_t y = lo[1]; y <= hi[1]; y++)
        for (int32_t z = lo[2]; z <= hi[2]; z++)
            for (int32_t x = lo[0]; x <= hi[0]; x++) m |= 1ull << (x | z << 2 | y << 4);
    return m;
}

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

}  // namespace
}  // namespace vrt

using namespace vrt;

extern "C" vrt_status vrt_world_edit(vrt_world* w, const vrt_edit* edits, uint32_t n, void* stream_) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
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
    // edits of a world follow each other whatever streams they are queued on
    VRT_CUDA(cudaStreamWaitEvent(stream, w->edited, 0));
    const int32_t nb[3] = {(int32_t)w->sx * 4, (int32_t)w->sy * 4, (int32_t)w->sz * 4};
    // host: geometry of the batch
    std::vector<EditDev> ed(n);
    std::unordered_map<uint32_t, uint32_t> index;  // sector -> position in `secs`
    std::vector<EditSector> secs;
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
        for (int32_t sy = d.lo[1] >> 2; sy <= d.hi[1] >> 2; sy++)
            for (int32_t sz = d.lo[2] >> 2; sz <= d.hi[2] >> 2; sz++)
                for (int32_t sx = d.lo[0] >> 2; sx <= d.hi[0] >> 2; sx++) {
                    int32_t lo[3], hi[3];
                    const int32_t sc[3] = {sx, sy, sz};
                    for (int c = 0; c < 3; c++) {
                        lo[c] = std::max(d.lo[c], sc[c] * 4) - sc[c] * 4;
                        hi[c] = std::min(d.hi[c], sc[c] * 4 + 3) - sc[c] * 4;
                    }
                    const uint32_t s = w->lin(sx, sy, sz);
                    auto it = index.find(s);
                    if (it == index.end()) {
                        it = index.emplace(s, (uint32_t)secs.size()).first;
                        secs.push_back(EditSector{0, 0, s, 0});
                    }
                    EditSector& es = secs[it->second];
                    es.visit |= box_bits(lo, hi);
                    if (!creates) continue;
                    for (int32_t y = lo[1]; y <= hi[1]; y++)
                        for (int32_t z = lo[2]; z <= hi[2]; z++)
                            for (int32_t x = lo[0]; x <= hi[0]; x++)
                                if (sphere_reaches_brick(e, sx * 4 + x, sy * 4 + y, sz * 4 + z))
                                    es.create |= 1ull << (x | z << 2 | y << 4);
                }
    }
    if (secs.empty()) return VRT_OK;
    // sector groups whose brick-table entries follow the touched sectors
    const uint32_t gx = (w->sx + 3) / 4, gz = (w->sz + 3) / 4;
    std::vector<uint32_t> groups;
    groups.reserve(secs.size());
    uint64_t growing = 0;
    for (const EditSector& es : secs) {
        const uint32_t x = es.sector % w->sx, z = (es.sector / w->sx) % w->sz, y = es.sector / (w->sx * w->sz);
        groups.push_back((x >> 2) + (z >> 2) * gx + (y >> 2) * gx * gz);
        growing += es.create ? 1 : 0;
    }
    std::sort(groups.begin(), groups.end());
    groups.erase(std::unique(groups.begin(), groups.end()), groups.end());
    // a growing sector takes at most 64 slots from the bump pointer
    const uint64_t need = growing * 64;
    if ((st = ensure_headroom(w, need, stream)) != VRT_OK) return st;
    // one upload: [edits][touched sectors][groups], from pinned memory; the stages are
    // used in turn, so a call waits on the host only for the upload four edits back
    const uint32_t m = (uint32_t)secs.size();
    const size_t eb = ed.size() * sizeof(EditDev), sb = secs.size() * sizeof(EditSector);
    const size_t soff = align16(eb), goff = align16(soff + sb), total = goff + groups.size() * sizeof(uint32_t);
    HostStage& stage = w->edit_stage[w->edit_stage_next];
    w->edit_stage_next = (w->edit_stage_next + 1) % 4;
    VRT_CUDA(stage.acquire(total));
    uint8_t* h = (uint8_t*)stage.ptr;
    std::memcpy(h, ed.data(), eb);
    std::memcpy(h + soff, secs.data(), sb);
    std::memcpy(h + goff, groups.data(), groups.size() * sizeof(uint32_t));
    VRT_CUDA(w->d_edit.reserve(total, true));
    VRT_CUDA(w->d_gc.reserve((size_t)m * 8, true));
    uint8_t* d = (uint8_t*)w->d_edit.ptr;
    VRT_CUDA(cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, stream));
    VRT_CUDA(stage.release(stream));
    VRT_CUDA(cudaMemsetAsync(w->d_gc.ptr, 0, (size_t)m * 8, stream));
    const EditSector* d_secs = (const EditSector*)(d + soff);
    auto* d_emptied = (unsigned long long*)w->d_gc.ptr;
    if (growing)
        relayout_kernel<true><<<m, 96, 0, stream>>>(d_secs, m, d_emptied, w->d_sectors, w->d_alloc, w->d_payload,
                                                   w->d_codes, w->d_cells);
    edit_bricks_kernel<<<(m * 64 + kEditWarps - 1) / kEditWarps, kEditWarps * 32, 0, stream>>>(
        d_secs, m, (const EditDev*)d, n, w->d_sectors, w->sx, w->sz, w->d_payload, w->d_codes, w->d_cells, d_emptied);
    relayout_kernel<false><<<m, 96, 0, stream>>>(d_secs, m, d_emptied, w->d_sectors, w->d_alloc, w->d_payload,
                                                w->d_codes, w->d_cells);
    VRT_CUDA(cudaGetLastError());
    if ((st = rebuild_table_groups(w, (const uint32_t*)(d + goff), (uint32_t)groups.size(), stream)) != VRT_OK)
        return st;
    VRT_CUDA(cudaEventRecord(w->edited, stream));
    w->host_stale = true;
    w->top_bound += need;
    return VRT_OK;
}
