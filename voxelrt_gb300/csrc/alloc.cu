// alloc.cu - the device side of brick-slot allocation: a bump allocator that device
// edits draw from without a host round trip, relayout of sectors whose brick set an
// edit changes, and compaction (defragmentation) of the brick pool.
//
// The reference allocates on the host: BrickSlotAllocator keeps a best-fit FreeList
// of slot ranges, grows a sector's range in place when it can and otherwise moves it,
// and throws when nothing fits (src/VoxelRT/BrickSlotAllocator.cpp:5-94); it leaves
// defragmentation as a TODO (:14).  Here the host free list still plans bulk uploads
// (vrt_world_sync_sectors), while edits run entirely on the device:
//   - a sector that gains bricks takes a fresh range of popcount(new mask) slots from
//     the bump pointer (one atomicAdd) and its bricks move there; its old range is
//     left behind as garbage;
//   - a sector that loses bricks is compacted in place (its range shrinks; the tail is
//     garbage);
//   - the host keeps an upper bound of the bump pointer (64 slots per sector an edit
//     may grow).  Only when the bound passes the pool's end does it read the device
//     state and compact the pool: live bricks packed from slot 0 in sector order, into
//     a pool of the same size, or a larger one when the live bricks fill most of it;
//   - the host mirror of the layout (per-sector slots, the free list, the sector table)
//     is rebuilt from the device lazily, before a host-side reader or planner needs it.
// Results never depend on slot placement: parity is on each sector's mask and bricks.

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "brick_codes.cuh"
#include "world.h"

namespace vrt {

namespace {

__global__ void set_alloc_kernel(DevAlloc* a, uint32_t top, uint32_t live, uint32_t cap) {
    a->top = top;
    a->live = live;
    a->cap = cap;
}

}  // namespace

namespace {

// Compaction, pass 1 (one block of 1024 threads): the new base of every sector, the
// exclusive prefix sum of the brick counts in sector order; the total is the new bump
// pointer and live count.
constexpr uint32_t kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads)
    compact_scan_kernel(const SectorRec* __restrict__ sectors, uint32_t n, uint32_t* __restrict__ new_base,
                        DevAlloc* __restrict__ alloc, uint32_t cap) {
    __shared__ uint32_t part[kScanThreads];
    const uint32_t t = threadIdx.x;
    const uint32_t per = (n + kScanThreads - 1) / kScanThreads;
    const uint32_t lo = min(n, t * per), hi = min(n, lo + per);
    uint32_t sum = 0;
    for (uint32_t s = lo; s < hi; s++) sum += (uint32_t)(__popc(sectors[s].mask_lo) + __popc(sectors[s].mask_hi));
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < kScanThreads; off <<= 1) {  // inclusive scan (Hillis-Steele)
        const uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t base = part[t] - sum;
    for (uint32_t s = lo; s < hi; s++) {
        new_base[s] = base;
        base += (uint32_t)(__popc(sectors[s].mask_lo) + __popc(sectors[s].mask_hi));
    }
    if (t == kScanThreads - 1) {
        alloc->top = part[t];
        alloc->live = part[t];
        alloc->cap = cap;
        alloc->overflow = 0;
    }
}

// Compaction, pass 2: one block per sector copies its bricks (68 16-byte words each:
// payload, voxel codes, cell masks) from the old pool to their packed slots in the new
// pool, every thread a strided share of the words, and rewrites the sector's base.
constexpr uint32_t kCopyThreads = 256;
__global__ void __launch_bounds__(kCopyThreads)
    compact_copy_kernel(SectorRec* __restrict__ sectors, uint32_t n, const uint32_t* __restrict__ new_base,
                        const uint8_t* __restrict__ old_payload, const uint4* __restrict__ old_codes,
                        const uint64_t* __restrict__ old_cells, uint8_t* __restrict__ payload,
                        uint4* __restrict__ codes, uint64_t* __restrict__ cells) {
    const uint32_t s = blockIdx.x, t = threadIdx.x;
    if (s >= n) return;
    const SectorRec rec = sectors[s];
    const uint32_t cnt = (uint32_t)(__popc(rec.mask_lo) + __popc(rec.mask_hi));
    if (cnt == 0) return;  // base 0 already (an empty sector's base is 0)
    const uint32_t nb = new_base[s];
    for (uint32_t c = t; c < cnt * 68u; c += kCopyThreads) {
        const uint32_t k = c / 68u, w = c - k * 68u;
        const size_t src = (size_t)rec.base + k, dst = (size_t)nb + k;
        if (w < 32)
            reinterpret_cast<uint4*>(payload + dst * 512)[w] = reinterpret_cast<const uint4*>(old_payload + src * 512)[w];
        else if (w < 64)
            codes[dst * 32 + (w - 32)] = old_codes[src * 32 + (w - 32)];
        else
            reinterpret_cast<uint4*>(cells + dst * 8)[w - 64] = reinterpret_cast<const uint4*>(old_cells + src * 8)[w - 64];
    }
    __syncthreads();  // every thread has read the old base
    if (t == 0) sectors[s].base = nb;
}

}  // namespace

vrt_status alloc_publish(vrt_world* w, cudaStream_t stream) {
    const uint32_t top = w->arena.high_water() - 1;  // 0-based: every slot from here on is free
    set_alloc_kernel<<<1, 1, 0, stream>>>(w->d_alloc, top, w->arena.allocated(), w->capacity);
    VRT_CUDA(cudaGetLastError());
    w->top_bound = top;
    return VRT_OK;
}

vrt_status refresh_host_mirror(vrt_world* w) {
    if (!w->host_stale) return VRT_OK;
    VRT_CUDA(cudaEventSynchronize(w->edited));
    DevAlloc a;
    VRT_CUDA(cudaMemcpy(&a, w->d_alloc, sizeof(a), cudaMemcpyDeviceToHost));
    VRT_CUDA(cudaMemcpy(w->h_table.data(), w->d_sectors, w->h_table.size() * sizeof(SectorRec), cudaMemcpyDeviceToHost));
    std::vector<std::pair<uint32_t, uint32_t>> used;
    for (size_t s = 0; s < w->h_table.size(); s++) {
        const SectorRec& r = w->h_table[s];
        SectorSlots& sl = w->slots[s];
        sl.mask = (uint64_t)r.mask_hi << 32 | r.mask_lo;
        sl.base = sl.mask ? r.base + 1 : 0;
        if (sl.mask) used.emplace_back(sl.base, (uint32_t)__builtin_popcountll(sl.mask));
    }
    std::sort(used.begin(), used.end());
    w->arena.assign_used(w->capacity, used);
    w->top_bound = a.top;
    w->host_stale = false;
    if (a.overflow) {
        set_error("brick pool overflowed during a device edit");
        return VRT_ERR_SLOTS_EXHAUSTED;
    }
    return VRT_OK;
}

vrt_status world_compact(vrt_world* w, uint32_t capacity, cudaStream_t stream) {
    vrt_status st = refresh_host_mirror(w);
    if (st != VRT_OK) return st;
    const uint32_t live = w->arena.allocated();
    capacity = std::max({capacity, live, 1024u});
    if (capacity > 0x3fffffffu) {
        set_error("brick pool cannot grow further");
        return VRT_ERR_SLOTS_EXHAUSTED;
    }
    uint4* codes = nullptr;
    uint8_t* payload = nullptr;
    uint64_t* cells = nullptr;
    uint32_t* new_base = nullptr;
    cudaError_t e = cudaMalloc(&codes, (size_t)capacity * 512);
    if (e == cudaSuccess) e = cudaMalloc(&payload, (size_t)capacity * 512);
    if (e == cudaSuccess) e = cudaMalloc(&cells, (size_t)capacity * 64);
    if (e == cudaSuccess) e = cudaMalloc(&new_base, (size_t)w->num_sectors() * sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaFree(codes);
        cudaFree(payload);
        cudaFree(cells);
        cudaFree(new_base);
        cudaGetLastError();
        return cuda_fail(e, "compact brick pool");
    }
    const uint32_t n = w->num_sectors();
    compact_scan_kernel<<<1, kScanThreads, 0, stream>>>(w->d_sectors, n, new_base, w->d_alloc, capacity);
    compact_copy_kernel<<<n, kCopyThreads, 0, stream>>>(w->d_sectors, n, new_base, w->d_payload, w->d_codes,
                                                        w->d_cells, payload, codes, cells);
    e = cudaGetLastError();
    if (e == cudaSuccess) {
        std::swap(w->d_codes, codes);
        std::swap(w->d_payload, payload);
        std::swap(w->d_cells, cells);
        w->capacity = capacity;
        st = rebuild_table_groups(w, nullptr, 0, stream);
        if (st == VRT_OK) e = cudaStreamSynchronize(stream);
    }
    // the old pool (or, on failure, the new one)
    cudaFree(codes);
    cudaFree(payload);
    cudaFree(cells);
    cudaFree(new_base);
    if (e != cudaSuccess) return cuda_fail(e, "compact brick pool");
    if (st != VRT_OK) return st;
    w->host_stale = true;
    w->compactions++;
    VRT_CUDA(cudaEventRecord(w->edited, stream));
    return refresh_host_mirror(w);
}

vrt_status ensure_headroom(vrt_world* w, uint64_t need, cudaStream_t stream) {
    if (w->top_bound + need <= w->capacity) return VRT_OK;
    // the device's bump pointer (16 bytes read once the world's last edit has run)
    VRT_CUDA(cudaEventSynchronize(w->edited));
    DevAlloc a;
    VRT_CUDA(cudaMemcpy(&a, w->d_alloc, sizeof(a), cudaMemcpyDeviceToHost));
    w->top_bound = a.top;
    if (w->top_bound + need <= w->capacity) return VRT_OK;
    vrt_status st = refresh_host_mirror(w);  // the live bricks, for the pool size below
    if (st != VRT_OK) return st;
    const uint64_t live = w->arena.allocated();
    uint64_t cap = w->capacity;
    // keep the pool size while the live bricks and this edit fill at most 3/4 of it
    if ((live + need) * 4 > cap * 3) cap = std::max<uint64_t>(cap * 2, (live + need) * 4 / 3 + 1024);
    if (cap > 0x3fffffffull) {
        set_error("brick pool cannot grow further");
        return VRT_ERR_SLOTS_EXHAUSTED;
    }
    return world_compact(w, (uint32_t)cap, stream);
}

}  // namespace vrt

using namespace vrt;

extern "C" vrt_status vrt_world_defrag(vrt_world* w, uint32_t capacity, void* stream) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK) return st;
    std::lock_guard<std::mutex> lock(w->mu);
    return world_compact(w, capacity ? capacity : w->capacity, (cudaStream_t)stream);
}

extern "C" vrt_status vrt_world_wait(vrt_world* w) {
    DeviceScope ds;
    vrt_status st = world_enter(w, ds);
    if (st != VRT_OK) return st;
    VRT_CUDA(cudaEventSynchronize(w->edited));
    return VRT_OK;
}
