// vrt_oracle.cpp - CPU oracle of the brickmap traversal path (test infrastructure).
//
// A scalar, per-ray restatement of the reference's CPU traversal.  Each function
// names the reference lines it follows.  Build with -O2 -ffp-contract=off and no
// -ffast-math: every float op is rounded on its own, in the source order of
// src/VoxelRT/CpuRenderer.cpp:172-224, which is the order the device kernels use.
//
// Differences from the reference that are deliberate (all shared with the device):
//   * the grid extent is the world's sector extent, not the fixed 2048x512x2048 view
//     of CpuRenderer.cpp:13-16, and the bounds test is per axis (the x|z trick of
//     CpuRenderer.cpp:114-117 needs a power-of-two XZ extent);
//   * the ray start is clipped to the grid inset by one voxel, as the GLSL path does
//     (VoxelTraversal.glsl:133-145, 164-167); tStart keeps the unclipped origin;
//   * the hit voxel's material is read at worldOrigin + floor(pos) even when the
//     iteration cap ran out (CpuRenderer.cpp:195 leaves relative coordinates in
//     voxelPos in that case, a SIMD-lane artefact);
//   * the step count mirrors GLSL hit.iters (VoxelTraversal.glsl:185,197).
//
// Mode VRT_CAST_GLSL / VRT_VIEW_GLSL restates instead the GPU renderer's rayCast
// (VoxelTraversal.glsl:100-131 getStepPos, :162-204 rayCast) with anisotropic LODs
// off: a 4th level of sector-group masks (GpuRenderer.cpp:139-149), cells of
// isotropic size 1/2/4 x scale 1/8/32, a 256-iteration cap, the +5-ulp bias on tmin,
// and side distances taken from the current voxel before each step, so the start
// voxel itself is never tested; shadow and bounce rays (and casts with
// VRT_CAST_GLSL_COARSE) follow rayCastCoarse (:206-240) as the GPU renderer's do.  Its
// parity is unpinned: the shader cannot run here.

#include "vrt_oracle.h"

#include <atomic>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t kSectorVoxels = 64 * 512;

// FlatVoxelStorage keeps one dense 32 KiB block of voxels and 512 cell masks per
// sector (CpuRenderer.cpp:20-31); here a block exists only for allocated sectors.
struct SectorBlock {
    uint8_t vox[kSectorVoxels];  // brick*512 + (x | z<<3 | y<<6)
    uint64_t occ[64 * 8];        // brick*8 + cell
};

inline int popc64(uint64_t x) { return __builtin_popcountll(x); }
inline int ctz64(uint64_t x) { return __builtin_ctzll(x); }

// x86 minps/maxps: the second operand is returned unless the compare holds, so a
// NaN in either operand yields the second one (SIMD_AVX512.h:123, SIMD_AVX2.h:129).
inline float min_x86(float a, float b) { return a < b ? a : b; }
inline float max_x86(float a, float b) { return a > b ? a : b; }

// floor2i: round toward -inf, then convert; out of range and NaN give INT32_MIN
// (the x86 "integer indefinite" value), SIMD_AVX512.h:109.
inline int32_t floor2i(float x) {
    float f = std::floor(x);
    if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int32_t)f;
}
inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

// WorldSectorIndexer::GetPos (VoxelMap.h:80-86): 12-bit signed x, z at 12, 8-bit y at 24.
inline void decode_sector(int32_t idx, int32_t& x, int32_t& y, int32_t& z) {
    uint32_t u = (uint32_t)idx;
    x = (int32_t)(u << 20) >> 20;
    z = (int32_t)(u << 8) >> 20;
    y = (int32_t)u >> 24;
}

// UpdateOccupancy (CpuRenderer.cpp:63-83): 8 cells of 4^3 voxels; bit vx + vz*4 + vy*16;
// cell index (cx | cz<<1 | cy<<2) as BrickMaskIndexer (CpuRenderer.cpp:18).
void update_occupancy(const uint8_t* brick, uint64_t* cells) {
    for (uint32_t cy = 0; cy < 8; cy += 4)
        for (uint32_t cz = 0; cz < 8; cz += 4)
            for (uint32_t cx = 0; cx < 8; cx += 4) {
                uint64_t mask = 0;
                for (uint32_t vy = 0; vy < 4; vy++)
                    for (uint32_t vz = 0; vz < 4; vz++)
                        for (uint32_t vx = 0; vx < 4; vx++) {
                            uint32_t vi = (cx + vx) | (cz + vz) << 3 | (cy + vy) << 6;
                            uint64_t occupied = brick[vi] != 0;
                            mask |= occupied << (vx + vz * 4 + vy * 16);
                        }
                cells[(cx >> 2) | (cz >> 2) << 1 | (cy >> 2) << 2] = mask;
            }
}

bool brick_is_empty(const uint8_t* brick) {
    for (int i = 0; i < 512; i++)
        if (brick[i]) return false;
    return true;
}

template <typename F>
void parallel_for(uint64_t n, int threads, F&& fn) {
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    if (threads <= 0) threads = 1;
    const uint64_t chunk = 256;
    uint64_t nchunks = (n + chunk - 1) / chunk;
    if ((uint64_t)threads > nchunks) threads = (int)(nchunks ? nchunks : 1);
    std::atomic<uint64_t> next{0};
    auto worker = [&](int tid) {
        for (;;) {
            uint64_t c = next.fetch_add(1);
            if (c >= nchunks) break;
            uint64_t b = c * chunk, e = b + chunk < n ? b + chunk : n;
            fn(tid, b, e);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(worker, t);
    worker(0);
    for (auto& th : pool) th.join();
}

struct Trace {
    bool hit;
    bool glsl;      // traced in the GLSL mode (t, face and normal follow rayCast)
    float tb;       // GLSL mode: the biased tmin of the hit step (hit.dist)
    uint16_t steps;
    uint8_t material;
    int32_t vp[3];
    float cur[3];   // final position (HitResult.Pos, CpuRenderer.cpp:212)
    float side[3];  // final side distances
    uint32_t step_calls;
    uint32_t occ_fetches;
};

}  // namespace

struct ora_world {
    uint32_t sx, sy, sz;
    std::vector<uint64_t> masks;
    // GLSL mode 4th level: per group of 4^3 sectors, bit x | z<<2 | y<<4 set when that
    // sector holds a brick (GpuRenderer.cpp:139-149), groups indexed x + z*GX + y*GX*GZ
    std::vector<uint64_t> groups;
    uint32_t gx() const { return (sx + 3) / 4; }
    uint32_t gz() const { return (sz + 3) / 4; }
    void refresh_groups() {
        groups.assign((size_t)gx() * ((sy + 3) / 4) * gz(), 0);
        for (uint32_t y = 0; y < sy; y++)
            for (uint32_t z = 0; z < sz; z++)
                for (uint32_t x = 0; x < sx; x++)
                    if (masks[lin((int32_t)x, (int32_t)y, (int32_t)z)])
                        groups[(x >> 2) + (z >> 2) * gx() + (y >> 2) * gx() * gz()] |=
                            1ull << ((x & 3) | (z & 3) << 2 | (y & 3) << 4);
    }
    std::vector<std::unique_ptr<SectorBlock>> data;

    uint32_t lin(int32_t x, int32_t y, int32_t z) const {
        return (uint32_t)x + (uint32_t)z * sx + (uint32_t)y * sx * sz;
    }
    bool sector_in(int32_t x, int32_t y, int32_t z) const {
        return (uint32_t)x < sx && (uint32_t)y < sy && (uint32_t)z < sz;
    }
    SectorBlock* block(uint32_t s) {
        if (!data[s]) {
            data[s].reset(new SectorBlock);
            std::memset(data[s].get(), 0, sizeof(SectorBlock));
        }
        return data[s].get();
    }
    void clear_brick(uint32_t s, uint32_t b) {
        if (!data[s]) return;
        std::memset(&data[s]->vox[b * 512], 0, 512);
        std::memset(&data[s]->occ[b * 8], 0, 64);
    }
};

namespace {

// GetStepPos (CpuRenderer.cpp:135-171) for one lane.  Returns true on a hit.
inline bool get_step_pos(const ora_world& w, int32_t vp[3], const float dir[3], Trace& tr) {
    uint32_t s = w.lin(vp[0] >> 5, vp[1] >> 5, vp[2] >> 5);
    uint64_t m = w.masks[s];
    uint32_t idx = ((vp[0] >> 3) & 3) | ((vp[2] >> 3) & 3) << 2 | ((vp[1] >> 3) & 3) << 4;
    int32_t lod = 3;
    tr.step_calls++;
    if ((m >> idx) & 1) {
        const SectorBlock* blk = w.data[s].get();
        uint32_t brick = idx;
        uint32_t cell = ((vp[0] >> 2) & 1) | ((vp[2] >> 2) & 1) << 1 | ((vp[1] >> 2) & 1) << 2;
        m = blk->occ[brick * 8 + cell];
        idx = (vp[0] & 3) | (vp[2] & 3) << 2 | (vp[1] & 3) << 4;
        lod = 0;
        tr.occ_fetches++;
        if ((m >> idx) & 1) {
            // GetVoxelMaterial (CpuRenderer.cpp:120-132): the raw voxel id.
            uint32_t vi = (vp[0] & 7) | (vp[2] & 7) << 3 | (vp[1] & 7) << 6;
            tr.material = blk->vox[brick * 512 + vi];
            return true;
        }
    }
    // level4: whole mask empty -> +2; level2: the 2^3 block holding idx empty -> +1.
    uint32_t half = (uint32_t)(idx < 32 ? m : m >> 32);
    if (m == 0)
        lod += 2;
    else if (((half >> (idx & 0xA)) & 0x00330033u) == 0)
        lod += 1;
    int32_t cm = (1 << lod) - 1;
    for (int c = 0; c < 3; c++) vp[c] = dir[c] < 0.0f ? (vp[c] & ~cm) : (vp[c] | cm);
    return false;
}

// getIsotropicLod (VoxelTraversal.glsl:24-34): cell size in units of the level's scale.
inline int32_t iso_lod(uint64_t m, uint32_t idx) {
    if (m == 0) return 4;
    uint32_t half = (uint32_t)(idx < 32 ? m : m >> 32);
    return ((half >> (idx & 0xA)) & 0x00330033u) == 0 ? 2 : 1;
}

// RayCellInteractionMaskLUT (GenerateRayCellInteractionMaskLUT, GpuRenderer.cpp:193-210):
// for octant o (axis a stepping +1 when bit a of o is set, else -1) and cell origin i of
// a 4^3 mask, the cells origin + j*dir for the 64 offsets j that stay inside the block.
struct RayCellLut {
    uint64_t m[512];
    RayCellLut() {
        for (uint32_t oct = 0; oct < 8; oct++) {
            const int32_t dir[3] = {(int32_t)(oct & 1) * 2 - 1, (int32_t)((oct >> 1) & 1) * 2 - 1,
                                    (int32_t)((oct >> 2) & 1) * 2 - 1};
            for (uint32_t o = 0; o < 64; o++) {
                const int32_t op[3] = {(int32_t)(o & 3), (int32_t)(o >> 4), (int32_t)((o >> 2) & 3)};  // x, y, z
                uint64_t mask = 0;
                for (uint32_t j = 0; j < 64; j++) {
                    const int32_t jp[3] = {(int32_t)(j & 3), (int32_t)(j >> 4), (int32_t)((j >> 2) & 3)};
                    int32_t p[3];
                    bool in = true;
                    for (int c = 0; c < 3; c++) {
                        p[c] = op[c] + jp[c] * dir[c];
                        in = in && p[c] >= 0 && p[c] < 4;
                    }
                    if (in) mask |= 1ull << (uint32_t)(p[0] | p[2] << 2 | p[1] << 4);
                }
                m[o + oct * 64] = mask;
            }
        }
    }
};
const RayCellLut& ray_cell_lut() {
    static const RayCellLut lut;
    return lut;
}

// getStepPos (VoxelTraversal.glsl:92-131) in the reference's order: the level's mask
// (sector at scale 8, 4^3 cell at scale 1 when the brick is allocated, sector group at
// scale 32 when the sector is empty), with aniso (u_UseAnisotropicLods, :116-121) masked
// by the ray's octant LUT entry, its isotropic LOD times the scale, and with coarse
// (rayCastCoarse from iteration 31, :218) a LOD below 4 ends the ray on the mask's
// lowest set cell (findAnyOccupiedPos, :41-53).  Returns true on a hit.
inline bool get_step_pos_glsl(const ora_world& w, int32_t vp[3], const float dir[3], Trace& tr,
                              bool coarse = false, bool aniso = false) {
    const int32_t sx = vp[0] >> 5, sy = vp[1] >> 5, sz = vp[2] >> 5;
    uint32_t s = w.lin(sx, sy, sz);
    uint64_t m = w.masks[s];
    uint32_t idx = ((vp[0] >> 3) & 3) | ((vp[2] >> 3) & 3) << 2 | ((vp[1] >> 3) & 3) << 4;
    int32_t scale = 8;
    const SectorBlock* blk = nullptr;
    uint32_t brick = 0;
    tr.step_calls++;
    if ((m >> idx) & 1) {
        blk = w.data[s].get();
        brick = idx;
        uint32_t cell = ((vp[0] >> 2) & 1) | ((vp[2] >> 2) & 1) << 1 | ((vp[1] >> 2) & 1) << 2;
        m = blk->occ[brick * 8 + cell];
        idx = (vp[0] & 3) | (vp[2] & 3) << 2 | (vp[1] & 3) << 4;
        scale = 1;
        tr.occ_fetches++;
        if ((m >> idx) & 1) {
            uint32_t vi = (vp[0] & 7) | (vp[2] & 7) << 3 | (vp[1] & 7) << 6;
            tr.material = blk->vox[brick * 512 + vi];
            return true;
        }
    } else if (m == 0) {
        m = w.groups[(uint32_t)(sx >> 2) + (uint32_t)(sz >> 2) * w.gx() + (uint32_t)(sy >> 2) * w.gx() * w.gz()];
        idx = (uint32_t)((sx & 3) | (sz & 3) << 2 | (sy & 3) << 4);
        scale = 32;
    }
    if (aniso) {
        const uint32_t oct = (dir[0] < 0.0f ? 0u : 1u) + (dir[1] < 0.0f ? 0u : 2u) + (dir[2] < 0.0f ? 0u : 4u);
        m &= ray_cell_lut().m[idx + oct * 64];
    }
    const int32_t lod = iso_lod(m, idx) * scale;
    if (coarse && lod < 4) {
        uint32_t b = 0;
        while (!((m >> b) & 1)) b++;
        vp[0] = (vp[0] & ~3) | (int32_t)(b & 3);
        vp[1] = (vp[1] & ~3) | (int32_t)(b >> 4);
        vp[2] = (vp[2] & ~3) | (int32_t)((b >> 2) & 3);
        uint32_t vi = (vp[0] & 7) | (vp[2] & 7) << 3 | (vp[1] & 7) << 6;
        tr.material = blk->vox[brick * 512 + vi];
        return true;
    }
    const int32_t cm = lod - 1;
    for (int c = 0; c < 3; c++) vp[c] = dir[c] < 0.0f ? (vp[c] & ~cm) : (vp[c] | cm);
    return false;
}

// The entry clip of VoxelTraversal.glsl:133-145 with bounds 1 - wo .. size - wo - 1
// (:166): the start position (origin when the clip does not apply).
void clip_start(const ora_world& w, const float o[3], const float d[3], const float inv[3], const int32_t wo[3],
                float cur[3]) {
    const int32_t size[3] = {(int32_t)w.sx * 32, (int32_t)w.sy * 32, (int32_t)w.sz * 32};
    float lo[3], hi[3];
    for (int c = 0; c < 3; c++) {
        float bmin = (float)(1 - wo[c]);
        float bmax = ((float)size[c] - (float)wo[c]) - 1.0f;
        float t1 = (bmin - o[c]) * inv[c];
        float t2 = (bmax - o[c]) * inv[c];
        lo[c] = min_x86(t1, t2);
        hi[c] = max_x86(t1, t2);
    }
    float tmin = max_x86(lo[0], max_x86(lo[1], lo[2]));
    float tmax = min_x86(hi[0], min_x86(hi[1], hi[2]));
    if (tmin > 0.0f && tmin < tmax) {
        for (int c = 0; c < 3; c++) cur[c] = o[c] + d[c] * tmin;
    } else {
        for (int c = 0; c < 3; c++) cur[c] = o[c];
    }
}

// rayCast (VoxelTraversal.glsl:162-204) for one ray: the voxel's side distances,
// tmin + 5 ulp, the next position, bounds, getStepPos.  coarse: rayCastCoarse
// (:206-240) instead, tmin + 0.001 and coarse steps from iteration 31.
void trace_ray_glsl(const ora_world& w, const float o[3], const float d[3], const int32_t wo[3],
                    uint32_t max_iters, Trace& tr, bool coarse = false, bool aniso = false) {
    tr.hit = false;
    tr.glsl = true;
    tr.tb = 0.0f;
    tr.material = 0;
    tr.step_calls = 0;
    tr.occ_fetches = 0;
    float inv[3], ts[3];
    for (int c = 0; c < 3; c++) inv[c] = 1.0f / d[c];
    for (int c = 0; c < 3; c++) ts[c] = ((d[c] < 0.0f ? 0.0f : 1.0f) - o[c]) * inv[c];
    const int32_t size[3] = {(int32_t)w.sx * 32, (int32_t)w.sy * 32, (int32_t)w.sz * 32};
    float* cur = tr.cur;
    clip_start(w, o, d, inv, wo, cur);
    // rayCastCoarse replaces the origin by the clipped start (VoxelTraversal.glsl:207-210):
    // tStart and positions count from it; rayCast keeps the origin (:162-167)
    float oc[3];
    const float* org = o;
    if (coarse) {
        for (int c = 0; c < 3; c++) oc[c] = cur[c];
        for (int c = 0; c < 3; c++) ts[c] = ((d[c] < 0.0f ? 0.0f : 1.0f) - oc[c]) * inv[c];
        org = oc;
    }
    int32_t* vp = tr.vp;
    for (int c = 0; c < 3; c++) vp[c] = wadd(wo[c], floor2i(cur[c]));
    float* side = tr.side;
    for (uint32_t i = 0; i < max_iters; i++) {
        for (int c = 0; c < 3; c++) side[c] = ts[c] + (float)wsub(vp[c], wo[c]) * inv[c];
        float t = min_x86(min_x86(side[0], side[1]), side[2]);
        if (coarse) {
            t = t + 0.001f;
        } else if (t == t) {  // +5 ulp on the bits; a NaN stays NaN (its bits are platform-defined)
            uint32_t bits;
            std::memcpy(&bits, &t, 4);
            bits += 5u;
            std::memcpy(&t, &bits, 4);
        }
        for (int c = 0; c < 3; c++) cur[c] = org[c] + t * d[c];
        for (int c = 0; c < 3; c++) vp[c] = wadd(wo[c], floor2i(cur[c]));
        if (!((uint32_t)vp[0] < (uint32_t)size[0] && (uint32_t)vp[1] < (uint32_t)size[1] &&
              (uint32_t)vp[2] < (uint32_t)size[2])) {
            tr.steps = (uint16_t)i;
            return;
        }
        if (get_step_pos_glsl(w, vp, d, tr, coarse && i >= 31, aniso)) {
            tr.hit = true;
            tr.tb = t;
            tr.steps = (uint16_t)i;
            return;
        }
    }
    tr.steps = (uint16_t)max_iters;
}

// RayCast (CpuRenderer.cpp:172-224) for one lane, with the GLSL entry clip.
void trace_ray(const ora_world& w, const float o[3], const float d[3], const int32_t wo[3],
               uint32_t max_iters, Trace& tr) {
    tr.hit = false;
    tr.glsl = false;
    tr.material = 0;
    tr.step_calls = 0;
    tr.occ_fetches = 0;
    float inv[3], ts[3];
    for (int c = 0; c < 3; c++) inv[c] = 1.0f / d[c];
    for (int c = 0; c < 3; c++) ts[c] = ((d[c] < 0.0f ? 0.0f : 1.0f) - o[c]) * inv[c];

    const int32_t size[3] = {(int32_t)w.sx * 32, (int32_t)w.sy * 32, (int32_t)w.sz * 32};
    // clipRayToAABB(origin, dir, 1 - wo, size - wo - 1), VoxelTraversal.glsl:133-145, 166.
    float lo[3], hi[3];
    for (int c = 0; c < 3; c++) {
        float bmin = (float)(1 - wo[c]);
        float bmax = ((float)size[c] - (float)wo[c]) - 1.0f;
        float t1 = (bmin - o[c]) * inv[c];
        float t2 = (bmax - o[c]) * inv[c];
        lo[c] = min_x86(t1, t2);
        hi[c] = max_x86(t1, t2);
    }
    float tmin = max_x86(lo[0], max_x86(lo[1], lo[2]));
    float tmax = min_x86(hi[0], min_x86(hi[1], hi[2]));
    float* cur = tr.cur;
    if (tmin > 0.0f && tmin < tmax) {
        for (int c = 0; c < 3; c++) cur[c] = o[c] + d[c] * tmin;
    } else {
        for (int c = 0; c < 3; c++) cur[c] = o[c];
    }
    float* side = tr.side;
    side[0] = side[1] = side[2] = 0.0f;
    int32_t* vp = tr.vp;

    for (uint32_t i = 0; i < max_iters; i++) {
        for (int c = 0; c < 3; c++) vp[c] = wadd(wo[c], floor2i(cur[c]));
        // GetInboundMask (CpuRenderer.cpp:114-117), per axis.
        if (!((uint32_t)vp[0] < (uint32_t)size[0] && (uint32_t)vp[1] < (uint32_t)size[1] &&
              (uint32_t)vp[2] < (uint32_t)size[2])) {
            tr.steps = (uint16_t)i;
            return;
        }
        if (get_step_pos(w, vp, d, tr)) {
            tr.hit = true;
            tr.steps = (uint16_t)i;
            return;
        }
        for (int c = 0; c < 3; c++) side[c] = ts[c] + (float)wsub(vp[c], wo[c]) * inv[c];
        float t = min_x86(min_x86(side[0], side[1]), side[2]) + 0.001f;
        for (int c = 0; c < 3; c++) cur[c] = o[c] + t * d[c];
    }
    tr.steps = (uint16_t)max_iters;
}

void fill_hit(const Trace& tr, const float d[3], uint32_t tag, vrt_hit& h) {
    h.tag = tag;
    h.steps = tr.steps;
    if (!tr.hit) {
        h.voxel = VRT_MISS_VOXEL;
        h.face = VRT_MISS_FACE;
        h.material = 0;
        h.t = INFINITY;
        return;
    }
    uint32_t axis;
    if (tr.glsl) {
        // hit.dist = biased tmin; the face is the first axis of sideMask = tmin >= sideDist
        axis = tr.tb >= tr.side[0] ? 0u : (tr.tb >= tr.side[1] ? 1u : 2u);
        h.t = tr.tb;
    } else {
        float t = min_x86(min_x86(tr.side[0], tr.side[1]), tr.side[2]);
        axis = tr.side[0] == t ? 0u : (tr.side[1] == t ? 1u : 2u);
        h.t = t;
    }
    h.face = (uint8_t)(axis * 2 + (d[axis] < 0.0f ? 1 : 0));
    h.material = tr.material;
    h.voxel = (uint32_t)tr.vp[0] | (uint32_t)tr.vp[1] << 11 | (uint32_t)tr.vp[2] << 21;
}

void fill_no_ray(vrt_hit& h) {
    h.voxel = VRT_MISS_VOXEL;
    h.face = VRT_MISS_FACE;
    h.material = 0;
    h.steps = 0;
    h.t = INFINITY;
    h.tag = VRT_NO_RAY;
}

// HitResult.Normal (CpuRenderer.cpp:213-217): sideMaskX = sx==t, sideMaskY = sy==t,
// sideMaskZ = neither; component = (sign bit of dir) ? +1 : -1.
void hit_normal(const Trace& tr, const float d[3], float n[3]) {
    if (tr.glsl) {
        // hit.normal = mix(0, -sign(dir), tmin >= sideDist) (VoxelTraversal.glsl:190-192);
        // sign(+-0) = 0
        for (int c = 0; c < 3; c++)
            n[c] = tr.tb >= tr.side[c] ? (d[c] > 0.0f ? -1.0f : (d[c] < 0.0f ? 1.0f : 0.0f)) : 0.0f;
        return;
    }
    float t = min_x86(min_x86(tr.side[0], tr.side[1]), tr.side[2]);
    bool mx = tr.side[0] == t, my = tr.side[1] == t, mz = !mx && !my;
    bool m[3] = {mx, my, mz};
    for (int c = 0; c < 3; c++) n[c] = m[c] ? (std::signbit(d[c]) ? 1.0f : -1.0f) : 0.0f;
}

// origin = hit.Pos + hit.Normal * 0.01f (CpuRenderer.cpp:389)
void offset_origin(const Trace& tr, const float n[3], float o[3]) {
    for (int c = 0; c < 3; c++) o[c] = tr.cur[c] + n[c] * 0.01f;
}

// 1/sqrt(l2): integer first estimate 0x5F3759DF - (bits >> 1) (Lomont 2003), then three
// Newton steps r * fma(-l2/2, r*r, 1.5); the vrt_camera contract of include/vrt.h.
float camera_rsqrt(float l2) {
    const float h = 0.5f * l2;
    uint32_t b;
    std::memcpy(&b, &l2, 4);
    b = 0x5F3759DFu - (b >> 1);
    float r;
    std::memcpy(&r, &b, 4);
    for (int i = 0; i < 3; i++) r = r * std::fmaf(-h, r * r, 1.5f);
    return r;
}

// The ray of pixel (px, py) of a vrt_camera: d0 + u*du + v*dv, u = px + 0.5, v = py + 0.5,
// times camera_rsqrt of its squared length.
void camera_ray(const vrt_camera& cam, uint32_t px, uint32_t py, float o[3], float d[3]) {
    float u = (float)px + 0.5f, v = (float)py + 0.5f;
    float x = (cam.d0[0] + u * cam.du[0]) + v * cam.dv[0];
    float y = (cam.d0[1] + u * cam.du[1]) + v * cam.dv[1];
    float z = (cam.d0[2] + u * cam.du[2]) + v * cam.dv[2];
    const float r = camera_rsqrt((x * x + y * y) + z * z);
    d[0] = x * r;
    d[1] = y * r;
    d[2] = z * r;
    for (int c = 0; c < 3; c++) o[c] = cam.origin[c];
}

// PCG32 (O'Neill, pcg-random.org: 64-bit LCG state, XSH-RR output).
struct Pcg32 {
    uint64_t state, inc;
    Pcg32(uint64_t initstate, uint64_t initseq) {
        state = 0;
        inc = (initseq << 1) | 1u;
        next();
        state += initstate;
        next();
    }
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
        uint32_t rot = (uint32_t)(old >> 59);
        return (xs >> rot) | (xs << ((32 - rot) & 31));
    }
    // uniform in [-1, 1) with 2^-23 spacing; every op exact
    float next_signed() { return (float)(next() >> 8) * 0x1p-23f - 1.0f; }
};

constexpr uint64_t kBounceStream = 0x9E3779B97F4A7C15ULL;

void bounce_dir(uint32_t pixel, uint32_t bounce, const float n[3], float out[3]) {
    Pcg32 rng(pixel ^ bounce, kBounceStream);
    for (int attempt = 0; attempt < 64; attempt++) {
        float x = rng.next_signed(), y = rng.next_signed(), z = rng.next_signed();
        float r2 = (x * x + y * y) + z * z;
        if (!(r2 > 1e-6f && r2 <= 1.0f)) continue;
        float r = std::sqrt(r2);
        float dx = n[0] + x / r, dy = n[1] + y / r, dz = n[2] + z / r;
        float l2 = (dx * dx + dy * dy) + dz * dz;
        if (!(l2 > 1e-12f)) continue;
        float l = std::sqrt(l2);
        out[0] = dx / l;
        out[1] = dy / l;
        out[2] = dz / l;
        return;
    }
    float l = std::sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);
    for (int c = 0; c < 3; c++) out[c] = n[c] / l;
}

// Traversal of one ray in the given mode.  secondary: a shadow or bounce ray, which the
// GPU renderer casts with rayCastCoarse (VoxelRender.comp:56,74,81; cap 96).
// mode: 0 the CPU traversal, kModeGlsl the GLSL mode, | kModeAniso its anisotropic LODs.
constexpr uint32_t kModeGlsl = 1, kModeAniso = 2;
inline void trace_mode(const ora_world& w, uint32_t mode, const float o[3], const float d[3], const int32_t wo[3],
                       uint32_t max_iters, Trace& tr, bool secondary = false) {
    const bool aniso = (mode & kModeAniso) != 0;
    if ((mode & kModeGlsl) && secondary)
        trace_ray_glsl(w, o, d, wo, std::min<uint32_t>(max_iters, VRT_GLSL_COARSE_MAX_ITERS), tr, true, aniso);
    else if (mode & kModeGlsl)
        trace_ray_glsl(w, o, d, wo, max_iters, tr, false, aniso);
    else
        trace_ray(w, o, d, wo, max_iters, tr);
}

uint32_t eff_iters_mode(uint32_t max_iters, bool glsl) {
    if (max_iters == 0) return glsl ? VRT_GLSL_MAX_ITERS : VRT_DEFAULT_MAX_ITERS;
    return max_iters > 65535u ? 65535u : max_iters;
}

uint32_t eff_iters(uint32_t max_iters) {
    if (max_iters == 0) return VRT_DEFAULT_MAX_ITERS;
    return max_iters > 65535 ? 65535 : max_iters;
}

struct StatAcc {
    std::vector<ora_stats> per;
    explicit StatAcc(int threads) {
        int t = threads <= 0 ? (int)std::thread::hardware_concurrency() : threads;
        per.assign(t > 0 ? t : 1, ora_stats{0, 0, 0, 0});
    }
    void add(int tid, const Trace& tr) {
        ora_stats& s = per[tid];
        s.rays++;
        s.step_calls += tr.step_calls;
        s.occ_fetches += tr.occ_fetches;
        s.hits += tr.hit ? 1 : 0;
    }
    void store(ora_stats* out) const {
        if (!out) return;
        *out = ora_stats{0, 0, 0, 0};
        for (auto& s : per) {
            out->rays += s.rays;
            out->step_calls += s.step_calls;
            out->occ_fetches += s.occ_fetches;
            out->hits += s.hits;
        }
    }
};

}  // namespace

extern "C" {

ora_world* ora_world_create(uint32_t sx, uint32_t sy, uint32_t sz) {
    if (sx == 0 || sy == 0 || sz == 0 || sx * 32 > VRT_MAX_WORLD_X || sy * 32 > VRT_MAX_WORLD_Y ||
        sz * 32 > VRT_MAX_WORLD_Z)
        return nullptr;
    ora_world* w = new ora_world;
    w->sx = sx;
    w->sy = sy;
    w->sz = sz;
    w->masks.assign((size_t)sx * sy * sz, 0);
    w->data.resize((size_t)sx * sy * sz);
    w->refresh_groups();
    return w;
}

void ora_world_destroy(ora_world* w) { delete w; }

// FlatVoxelStorage::SyncBuffers (CpuRenderer.cpp:33-61) for the record semantics of
// vrt_world_sync_sectors: new mask, dirty bricks copied, occupancy re-derived.
int ora_world_sync(ora_world* w, uint32_t n, const int32_t* sector_idx, const uint64_t* alloc_mask,
                   const uint64_t* dirty_mask, const uint8_t* bricks) {
    if (!w || (n && (!sector_idx || !alloc_mask))) return -1;
    const uint8_t* p = bricks;
    for (uint32_t i = 0; i < n; i++) {
        uint64_t am = alloc_mask[i];
        uint64_t dm = dirty_mask ? (dirty_mask[i] & am) : am;
        int32_t x, y, z;
        decode_sector(sector_idx[i], x, y, z);
        if (dm && !p) return -1;
        if (w->sector_in(x, y, z)) {
            uint32_t s = w->lin(x, y, z);
            uint64_t old = w->masks[s];
            for (uint64_t r = old & ~am; r; r &= r - 1) w->clear_brick(s, ctz64(r));
            if (am) {
                SectorBlock* blk = w->block(s);
                for (uint64_t r = am & ~old & ~dm; r; r &= r - 1) w->clear_brick(s, ctz64(r));
                const uint8_t* q = p;
                for (uint64_t r = dm; r; r &= r - 1) {
                    uint32_t b = ctz64(r);
                    std::memcpy(&blk->vox[b * 512], q, 512);
                    update_occupancy(&blk->vox[b * 512], &blk->occ[b * 8]);
                    q += 512;
                }
            } else {
                w->data[s].reset();
            }
            w->masks[s] = am;
        }
        if (p) p += (size_t)popc64(dm) * 512;
    }
    w->refresh_groups();
    return 0;
}

uint64_t ora_world_sector_mask(const ora_world* w, int32_t sector_idx) {
    int32_t x, y, z;
    decode_sector(sector_idx, x, y, z);
    if (!w || !w->sector_in(x, y, z)) return 0;
    return w->masks[w->lin(x, y, z)];
}

int ora_world_read_sector(const ora_world* w, int32_t sector_idx, uint64_t* mask, uint8_t* bricks) {
    int32_t x, y, z;
    decode_sector(sector_idx, x, y, z);
    if (!w || !w->sector_in(x, y, z)) return -1;
    uint32_t s = w->lin(x, y, z);
    uint64_t m = w->masks[s];
    if (mask) *mask = m;
    if (bricks) {
        for (uint64_t r = m; r; r &= r - 1) {
            std::memcpy(bricks, &w->data[s]->vox[ctz64(r) * 512], 512);
            bricks += 512;
        }
    }
    return 0;
}

uint8_t ora_world_get_voxel(const ora_world* w, int32_t x, int32_t y, int32_t z) {
    if (!w || !w->sector_in(x >> 5, y >> 5, z >> 5) || x < 0 || y < 0 || z < 0) return 0;
    uint32_t s = w->lin(x >> 5, y >> 5, z >> 5);
    uint32_t b = ((x >> 3) & 3) | ((z >> 3) & 3) << 2 | ((y >> 3) & 3) << 4;
    if (!((w->masks[s] >> b) & 1)) return 0;
    return w->data[s]->vox[b * 512 + ((x & 7) | (z & 7) << 3 | (y & 7) << 6)];
}

int ora_world_brick_occupancy(const ora_world* w, int32_t bx, int32_t by, int32_t bz, uint64_t out[8]) {
    if (!w || bx < 0 || by < 0 || bz < 0 || !w->sector_in(bx >> 2, by >> 2, bz >> 2)) return -1;
    uint32_t s = w->lin(bx >> 2, by >> 2, bz >> 2);
    uint32_t b = (bx & 3) | (bz & 3) << 2 | (by & 3) << 4;
    if (!((w->masks[s] >> b) & 1)) {
        std::memset(out, 0, 64);
        return 0;
    }
    std::memcpy(out, &w->data[s]->occ[b * 8], 64);
    return 0;
}

uint64_t ora_world_allocated_bricks(const ora_world* w) {
    uint64_t n = 0;
    for (uint64_t m : w->masks) n += (uint64_t)popc64(m);
    return n;
}

int ora_ray_cell_lut(uint64_t* out) {
    if (!out) return -1;
    std::memcpy(out, ray_cell_lut().m, sizeof(uint64_t) * 512);
    return 0;
}

int ora_cast(const ora_world* w, const vrt_ray* rays, uint64_t n, const vrt_cast_params* params,
             vrt_hit* hits, int threads, ora_stats* stats) {
    if (!w || (n && (!rays || !hits)) || !params) return -1;
    const bool glsl = (params->flags & VRT_CAST_GLSL) != 0;
    const bool coarse = glsl && (params->flags & VRT_CAST_GLSL_COARSE) != 0;
    const uint32_t mode = glsl ? (kModeGlsl | ((params->flags & VRT_CAST_GLSL_ANISO) ? kModeAniso : 0u)) : 0u;
    uint32_t iters = eff_iters_mode(params->max_iters, glsl);
    StatAcc acc(threads);
    parallel_for(n, (int)acc.per.size(), [&](int tid, uint64_t b, uint64_t e) {
        Trace tr;
        for (uint64_t i = b; i < e; i++) {
            trace_mode(*w, mode, rays[i].origin, rays[i].dir, params->world_origin, iters, tr, coarse);
            fill_hit(tr, rays[i].dir, rays[i].tag, hits[i]);
            acc.add(tid, tr);
        }
    });
    acc.store(stats);
    return 0;
}

int ora_camera_rays(const vrt_camera* cam, vrt_ray* rays) {
    if (!cam || !rays) return -1;
    for (uint32_t py = 0; py < cam->height; py++)
        for (uint32_t px = 0; px < cam->width; px++) {
            vrt_ray& r = rays[(size_t)py * cam->width + px];
            camera_ray(*cam, px, py, r.origin, r.dir);
            r.tag = py * cam->width + px;
            r.reserved = 0;
        }
    return 0;
}

int ora_render_view(const ora_world* w, const vrt_camera* cam, uint32_t max_iters, uint32_t mode, vrt_hit* hits,
                    int threads, ora_stats* stats) {
    if (!w || !cam || !hits) return -1;
    const bool glsl = (mode & kModeGlsl) != 0;
    uint32_t iters = eff_iters_mode(max_iters, glsl);
    uint64_t n = (uint64_t)cam->width * cam->height;
    StatAcc acc(threads);
    parallel_for(n, (int)acc.per.size(), [&](int tid, uint64_t b, uint64_t e) {
        Trace tr;
        float o[3], d[3];
        for (uint64_t i = b; i < e; i++) {
            camera_ray(*cam, (uint32_t)(i % cam->width), (uint32_t)(i / cam->width), o, d);
            trace_mode(*w, mode, o, d, cam->world_origin, iters, tr);
            fill_hit(tr, d, (uint32_t)i, hits[i]);
            acc.add(tid, tr);
        }
    });
    acc.store(stats);
    return 0;
}

int ora_render_view_shadow(const ora_world* w, const vrt_camera* cam, const float sun_dir[3],
                           uint32_t max_iters, uint32_t mode, vrt_hit* primary, vrt_hit* shadow, int threads,
                           ora_stats* stats) {
    if (!w || !cam || !sun_dir || !primary || !shadow) return -1;
    const bool glsl = (mode & kModeGlsl) != 0;
    uint32_t iters = eff_iters_mode(max_iters, glsl);
    uint64_t n = (uint64_t)cam->width * cam->height;
    StatAcc acc(threads);
    parallel_for(n, (int)acc.per.size(), [&](int tid, uint64_t b, uint64_t e) {
        Trace tr, ts;
        float o[3], d[3], nrm[3], so[3];
        for (uint64_t i = b; i < e; i++) {
            camera_ray(*cam, (uint32_t)(i % cam->width), (uint32_t)(i / cam->width), o, d);
            trace_mode(*w, mode, o, d, cam->world_origin, iters, tr);
            fill_hit(tr, d, (uint32_t)i, primary[i]);
            acc.add(tid, tr);
            if (!tr.hit) {
                fill_no_ray(shadow[i]);
                continue;
            }
            hit_normal(tr, d, nrm);
            offset_origin(tr, nrm, so);
            trace_mode(*w, mode, so, sun_dir, cam->world_origin, iters, ts, true);
            fill_hit(ts, sun_dir, (uint32_t)i, shadow[i]);
            acc.add(tid, ts);
        }
    });
    acc.store(stats);
    return 0;
}

int ora_render_view_bounces(const ora_world* w, const vrt_camera* cam, uint32_t n_bounces,
                            uint32_t max_iters, uint32_t mode, vrt_hit* hits, int threads, ora_stats* stats) {
    if (!w || !cam || !hits) return -1;
    const bool glsl = (mode & kModeGlsl) != 0;
    uint32_t iters = eff_iters_mode(max_iters, glsl);
    uint64_t n = (uint64_t)cam->width * cam->height;
    StatAcc acc(threads);
    parallel_for(n, (int)acc.per.size(), [&](int tid, uint64_t b, uint64_t e) {
        Trace tr;
        float o[3], d[3], nrm[3];
        for (uint64_t i = b; i < e; i++) {
            camera_ray(*cam, (uint32_t)(i % cam->width), (uint32_t)(i / cam->width), o, d);
            bool alive = true;
            for (uint32_t k = 0; k <= n_bounces; k++) {
                vrt_hit& h = hits[(uint64_t)k * n + i];
                if (!alive) {
                    fill_no_ray(h);
                    continue;
                }
                if (k > 0) {
                    hit_normal(tr, d, nrm);
                    offset_origin(tr, nrm, o);
                    bounce_dir((uint32_t)i, k, nrm, d);
                }
                trace_mode(*w, mode, o, d, cam->world_origin, iters, tr, k > 0);
                fill_hit(tr, d, (uint32_t)i, h);
                acc.add(tid, tr);
                alive = tr.hit;
            }
        }
    });
    acc.store(stats);
    return 0;
}

// The GPU renderer's whole per-pixel path (VoxelRender.comp:51-86) with u_MaxBounces =
// n_bounces > 0: the primary ray; a sun ray from its hit (:54-61); then bounce i = 1..n
// from the last hit (:63-74), stopping at the first miss (:76-79), each of the first two
// bounce hits followed by a sun ray from it (:81).  Every sun and bounce ray starts at
// hitPos + normal*0.01; the bounce direction is bounce_dir (the contract of
// vrt_view).  Records: [primary][sun 0][bounce 1][sun 1][bounce 2][sun 2][bounce 3]...
// [bounce n], planes of width*height; rays never cast are VRT_NO_RAY records.
int ora_render_view_path(const ora_world* w, const vrt_camera* cam, const float sun_dir[3], uint32_t n_bounces,
                         uint32_t max_iters, uint32_t mode, vrt_hit* hits, int threads, ora_stats* stats) {
    if (!w || !cam || !sun_dir || !hits || n_bounces == 0 || n_bounces > VRT_MAX_BOUNCES) return -1;
    const bool glsl = (mode & kModeGlsl) != 0;
    const uint32_t iters = eff_iters_mode(max_iters, glsl);
    const uint64_t n = (uint64_t)cam->width * cam->height;
    const uint32_t kinds = 2 + n_bounces + std::min<uint32_t>(n_bounces, 2);
    StatAcc acc(threads);
    parallel_for(n, (int)acc.per.size(), [&](int tid, uint64_t b, uint64_t e) {
        Trace tr, ts;
        float o[3], d[3], nrm[3], so[3];
        for (uint64_t i = b; i < e; i++) {
            uint32_t k = 0;  // next record plane
            auto put = [&](const Trace& t, const float* dir) {
                fill_hit(t, dir, (uint32_t)i, hits[(uint64_t)k++ * n + i]);
                acc.add(tid, t);
            };
            camera_ray(*cam, (uint32_t)(i % cam->width), (uint32_t)(i / cam->width), o, d);
            trace_mode(*w, mode, o, d, cam->world_origin, iters, tr);
            put(tr, d);
            for (uint32_t bnc = 0; tr.hit && bnc <= n_bounces; bnc++) {
                // from the last hit: its sun ray (after the primary and the first two
                // bounces), then the next bounce
                hit_normal(tr, d, nrm);
                offset_origin(tr, nrm, so);
                if (bnc <= 2) {
                    trace_mode(*w, mode, so, sun_dir, cam->world_origin, iters, ts, true);
                    put(ts, sun_dir);
                }
                if (bnc == n_bounces) break;
                for (int c = 0; c < 3; c++) o[c] = so[c];
                bounce_dir((uint32_t)i, bnc + 1, nrm, d);
                trace_mode(*w, mode, o, d, cam->world_origin, iters, tr, true);
                put(tr, d);
            }
            for (; k < kinds; k++) fill_no_ray(hits[(uint64_t)k * n + i]);
        }
    });
    acc.store(stats);
    return 0;
}

// G-buffer of the primary hits (VoxelRender.comp:39-46,91-93; CpuRenderer.cpp:364-376):
//   albedo_normal  RGBA8: rgb = round-half-even(255 * c*c) per channel of the material's
//                  RGB565 color (c = field / 31, / 63, / 31; getMaterialColor, its square
//                  the "srgb gamma hack"), a = the packed normal (n.x+1) | (n.y+1)<<2 |
//                  (n.z+1)<<4 (packGNormal; CpuRenderer's bits 24-29); on a miss
//                  0x00FFFFFF (white, normal bits 0);
//   depth          projPos.z / projPos.w with projPos = proj * (hitPos / 16, 1), proj
//                  column-major, every op rounded on its own in the order
//                  ((m[r]*x + m[4+r]*y) + m[8+r]*z) + m[12+r]; -1 on a miss.
static void gbuffer_texel(const Trace& tr, const float d[3], const uint32_t* palette, const float* proj, uint32_t& texel,
                   float& depth) {
    if (!tr.hit) {
        texel = 0x00FFFFFFu;
        depth = -1.0f;
        return;
    }
    const uint32_t m = palette[tr.material];
    const float c[3] = {(float)((m >> 11) & 31u) * (1.0f / 31), (float)((m >> 5) & 63u) * (1.0f / 63),
                        (float)(m & 31u) * (1.0f / 31)};
    texel = 0;
    for (int k = 0; k < 3; k++) texel |= (uint32_t)std::nearbyint(c[k] * c[k] * 255.0f) << (8 * k);
    float nrm[3];
    hit_normal(tr, d, nrm);
    const uint32_t a = (uint32_t)(nrm[0] + 1.0f) | (uint32_t)(nrm[1] + 1.0f) << 2 | (uint32_t)(nrm[2] + 1.0f) << 4;
    texel |= a << 24;
    const float p[3] = {tr.cur[0] * 0.0625f, tr.cur[1] * 0.0625f, tr.cur[2] * 0.0625f};
    const float z = ((proj[2] * p[0] + proj[6] * p[1]) + proj[10] * p[2]) + proj[14];
    const float wv = ((proj[3] * p[0] + proj[7] * p[1]) + proj[11] * p[2]) + proj[15];
    depth = z / wv;
}

int ora_render_gbuffer(const ora_world* w, const vrt_camera* cam, uint32_t max_iters, uint32_t mode,
                       const uint32_t* palette, const float* proj, uint32_t* albedo_normal, float* depth, vrt_hit* hits,
                       int threads) {
    if (!w || !cam || !palette || !proj || !albedo_normal || !depth) return -1;
    const uint32_t iters = eff_iters_mode(max_iters, (mode & kModeGlsl) != 0);
    const uint64_t n = (uint64_t)cam->width * cam->height;
    StatAcc acc(threads);
    parallel_for(n, (int)acc.per.size(), [&](int, uint64_t b, uint64_t e) {
        Trace tr;
        float o[3], d[3];
        for (uint64_t i = b; i < e; i++) {
            camera_ray(*cam, (uint32_t)(i % cam->width), (uint32_t)(i / cam->width), o, d);
            trace_mode(*w, mode, o, d, cam->world_origin, iters, tr);
            gbuffer_texel(tr, d, palette, proj, albedo_normal[i], depth[i]);
            if (hits) fill_hit(tr, d, (uint32_t)i, hits[i]);
        }
    });
    return 0;
}

// VoxelMap::RayCast (VoxelMap.cpp:140-170) with GetStepLevel (:125-139) over the
// oracle's sectors; glm::min(x, y) = y < x ? y : x, glm::step(0, d) = d < 0 ? 0 : 1,
// double -> int as x86 cvttsd2si (INT32_MIN out of range).
int ora_pick(const ora_world* w, const double* rays, uint64_t n, uint32_t max_iters, vrt_pick_hit* hits) {
    if (!w || (n && (!rays || !hits))) return -1;
    if (max_iters == 0) max_iters = 1024;
    auto gmin = [](double x, double y) { return y < x ? y : x; };
    auto d2i = [](double f) { return (f >= -2147483648.0 && f < 2147483648.0) ? (int32_t)f : INT32_MIN; };
    for (uint64_t r = 0; r < n; r++) {
        const double* ray = rays + r * 6;
        double o[3], d[3], inv[3], ts[3];
        int32_t pos[3];
        for (int c = 0; c < 3; c++) {
            o[c] = ray[c];
            d[c] = ray[3 + c];
            inv[c] = 1.0 / d[c];
            ts[c] = ((d[c] < 0.0 ? 0.0 : 1.0) - o[c]) * inv[c];
            pos[c] = d2i(std::floor(o[c]));
        }
        vrt_pick_hit h{};
        h.distance = -1.0;
        h.iters = max_iters;
        for (uint32_t i = 0; i < max_iters; i++) {
            double side[3], hp[3];
            for (int c = 0; c < 3; c++) side[c] = ts[c] + (double)pos[c] * inv[c];
            const double tmin = gmin(gmin(side[0], side[1]), side[2]) + 0.0001;
            for (int c = 0; c < 3; c++) {
                hp[c] = o[c] + tmin * d[c];
                pos[c] = d2i(std::floor(hp[c]));
            }
            // sector key wraps like WorldSectorIndexer (12/8/12 signed bits)
            const int32_t sx = (int32_t)((uint32_t)(pos[0] >> 5) << 20) >> 20;
            const int32_t sy = (int32_t)((uint32_t)(pos[1] >> 5) << 24) >> 24;
            const int32_t sz = (int32_t)((uint32_t)(pos[2] >> 5) << 20) >> 20;
            int32_t k = 5;
            if (w->sector_in(sx, sy, sz)) {
                const uint32_t s = w->lin(sx, sy, sz);
                const uint64_t mask = w->masks[s];
                if (mask) {
                    const uint32_t b = ((pos[0] >> 3) & 3) | ((pos[2] >> 3) & 3) << 2 | ((pos[1] >> 3) & 3) << 4;
                    k = 3;
                    if ((mask >> b) & 1) {
                        const uint32_t vi = (pos[0] & 7) | (pos[2] & 7) << 3 | (pos[1] & 7) << 6;
                        k = w->data[s]->vox[b * 512 + vi] == 0 ? 0 : -1;
                    }
                }
            }
            if (k < 0) {
                bool m[3];
                for (int c = 0; c < 3; c++) m[c] = tmin >= side[c];
                h.distance = tmin;
                for (int c = 0; c < 3; c++) {
                    const double sg = (double)((0.0 < d[c]) - (d[c] < 0.0));
                    h.normal[c] = m[c] ? (float)(-sg) : 0.0f;
                    h.voxel[c] = pos[c];
                }
                const float ax = (float)hp[0], az = (float)hp[2], b = (float)hp[1];
                const float tx = m[0] ? 1.0f : 0.0f, tz = m[2] ? 1.0f : 0.0f;
                const float ux = ax * (1.0f - tx) + b * tx, uz = az * (1.0f - tz) + b * tz;
                h.uv[0] = ux - std::floor(ux);
                h.uv[1] = uz - std::floor(uz);
                h.iters = i;
                break;
            }
            const int32_t msk = (1 << k) - 1;
            for (int c = 0; c < 3; c++) pos[c] = d[c] < 0.0 ? (pos[c] & ~msk) : (pos[c] | msk);
        }
        hits[r] = h;
    }
    return 0;
}

// VoxelMap::RegionDispatchSIMD + GC (VoxelMap.h:222-263) driving the sphere brush
// (Brush.cpp:10-31) with an exact integer sphere test.
int ora_world_edit(ora_world* w, const vrt_edit* edits, uint32_t n) {
    if (!w || (n && !edits)) return -1;
    const int32_t nbx = (int32_t)w->sx * 4, nby = (int32_t)w->sy * 4, nbz = (int32_t)w->sz * 4;
    for (uint32_t k = 0; k < n; k++) {
        const vrt_edit& e = edits[k];
        const int64_t r = e.radius;
        const int64_t r2 = r * r;
        const bool create = e.material != 0;  // createEmpty = !isErasing (Brush.cpp:17)
        int64_t lo[3], hi[3];
        const int32_t nb[3] = {nbx, nby, nbz};
        bool empty_range = false;
        for (int c = 0; c < 3; c++) {
            lo[c] = ((int64_t)e.center[c] - r) >> 3;
            hi[c] = ((int64_t)e.center[c] + r) >> 3;
            if (lo[c] < 0) lo[c] = 0;
            if (hi[c] > nb[c] - 1) hi[c] = nb[c] - 1;
            if (lo[c] > hi[c]) empty_range = true;
        }
        if (empty_range) continue;
        for (int64_t by = lo[1]; by <= hi[1]; by++)
            for (int64_t bz = lo[2]; bz <= hi[2]; bz++)
                for (int64_t bx = lo[0]; bx <= hi[0]; bx++) {
                    uint32_t s = w->lin((int32_t)bx >> 2, (int32_t)by >> 2, (int32_t)bz >> 2);
                    uint32_t b = (uint32_t)((bx & 3) | (bz & 3) << 2 | (by & 3) << 4);
                    bool allocated = (w->masks[s] >> b) & 1;
                    if (!allocated && !create) continue;
                    SectorBlock* blk = w->block(s);
                    if (!allocated) {
                        w->clear_brick(s, b);
                        w->masks[s] |= 1ull << b;
                    }
                    uint8_t* brick = &blk->vox[b * 512];
                    for (int vi = 0; vi < 512; vi++) {
                        int64_t x = bx * 8 + (vi & 7), z = bz * 8 + ((vi >> 3) & 7), y = by * 8 + (vi >> 6);
                        int64_t dx = x - e.center[0], dy = y - e.center[1], dz = z - e.center[2];
                        if (dx * dx + dy * dy + dz * dz > r2) continue;
                        if (e.mode == VRT_EDIT_REPLACE && brick[vi] == 0) continue;
                        brick[vi] = e.material;
                    }
                    update_occupancy(brick, &blk->occ[b * 8]);
                    if (brick_is_empty(brick)) {
                        w->clear_brick(s, b);
                        w->masks[s] &= ~(1ull << b);
                    }
                }
        // drop blocks of sectors that became empty
        for (int64_t sy = lo[1] >> 2; sy <= hi[1] >> 2; sy++)
            for (int64_t sz = lo[2] >> 2; sz <= hi[2] >> 2; sz++)
                for (int64_t sx = lo[0] >> 2; sx <= hi[0] >> 2; sx++) {
                    uint32_t s = w->lin((int32_t)sx, (int32_t)sy, (int32_t)sz);
                    if (w->masks[s] == 0) w->data[s].reset();
                }
    }
    w->refresh_groups();
    return 0;
}

}  // extern "C"
