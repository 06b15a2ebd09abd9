// synth.cpp - seeded synthetic worlds and ray sets (see include/vrt_synth.h).
//
// Built with -ffp-contract=off: the noise is evaluated in double with separately
// rounded ops so x86 and arm64 hosts produce the same voxels.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/vrt_synth.h"
#include "vrt_internal.h"

namespace vrt {
void set_error(const std::string& msg);
const char* last_error_cstr();
}

namespace {

// PCG-RXS-M-XS 32-bit permutation (the PCG family's hash form), used as the
// lattice hash of the gradient noise.
inline uint32_t pcg_hash(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

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
    double unit() { return (double)(next() >> 8) * (1.0 / 16777216.0); }
    float next_signed() { return (float)(next() >> 8) * 0x1p-23f - 1.0f; }
};

inline double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
inline double lerp(double a, double b, double t) { return a + t * (b - a); }

const double kGrad2[8][2] = {{1, 1}, {-1, 1}, {1, -1}, {-1, -1}, {1, 0}, {-1, 0}, {0, 1}, {0, -1}};
const double kGrad3[16][3] = {{1, 1, 0}, {-1, 1, 0}, {1, -1, 0}, {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1},
                              {1, 0, -1}, {-1, 0, -1}, {0, 1, 1}, {0, -1, 1}, {0, 1, -1}, {0, -1, -1},
                              {1, 1, 0}, {-1, 1, 0}, {0, -1, 1}, {0, -1, -1}};

inline double grad2(uint32_t h, double x, double z) {
    const double* g = kGrad2[h & 7];
    return g[0] * x + g[1] * z;
}
inline double grad3(uint32_t h, double x, double y, double z) {
    const double* g = kGrad3[h & 15];
    return (g[0] * x + g[1] * y) + g[2] * z;
}

double noise2(double x, double z, uint32_t seed) {
    const double fx = std::floor(x), fz = std::floor(z);
    const uint32_t ix = (uint32_t)(int32_t)fx, iz = (uint32_t)(int32_t)fz;
    const double tx = x - fx, tz = z - fz;
    const uint32_t hs = pcg_hash(seed);
    const uint32_t h0 = pcg_hash(hs ^ ix), h1 = pcg_hash(hs ^ (ix + 1));
    const double g00 = grad2(pcg_hash(h0 ^ iz), tx, tz);
    const double g10 = grad2(pcg_hash(h1 ^ iz), tx - 1.0, tz);
    const double g01 = grad2(pcg_hash(h0 ^ (iz + 1)), tx, tz - 1.0);
    const double g11 = grad2(pcg_hash(h1 ^ (iz + 1)), tx - 1.0, tz - 1.0);
    const double u = fade(tx), v = fade(tz);
    return lerp(lerp(g00, g10, u), lerp(g01, g11, u), v);
}

double noise3(double x, double y, double z, uint32_t seed) {
    const double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    const uint32_t ix = (uint32_t)(int32_t)fx, iy = (uint32_t)(int32_t)fy, iz = (uint32_t)(int32_t)fz;
    const double tx = x - fx, ty = y - fy, tz = z - fz;
    const uint32_t hs = pcg_hash(seed);
    double g[8];
    for (int c = 0; c < 8; c++) {
        const uint32_t dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
        const uint32_t h = pcg_hash(pcg_hash(pcg_hash(hs ^ (ix + dx)) ^ (iy + dy)) ^ (iz + dz));
        g[c] = grad3(h, tx - dx, ty - dy, tz - dz);
    }
    const double u = fade(tx), v = fade(ty), w = fade(tz);
    const double x00 = lerp(g[0], g[1], u), x10 = lerp(g[2], g[3], u);
    const double x01 = lerp(g[4], g[5], u), x11 = lerp(g[6], g[7], u);
    return lerp(lerp(x00, x10, v), lerp(x01, x11, v), w);
}

double fbm2(double x, double z, uint32_t octaves, uint64_t seed) {
    double sum = 0.0, amp = 1.0, f = 1.0;
    for (uint32_t o = 0; o < octaves; o++) {
        sum += amp * noise2(x * f, z * f, (uint32_t)seed + o * 0x9E3779B9u);
        f *= 2.0;
        amp *= 0.5;
    }
    return sum;
}

double fbm3(double x, double y, double z, uint32_t octaves, uint64_t seed) {
    double sum = 0.0, amp = 1.0, f = 1.0;
    for (uint32_t o = 0; o < octaves; o++) {
        sum += amp * noise3(x * f, y * f, z * f, (uint32_t)seed + o * 0x9E3779B9u);
        f *= 2.0;
        amp *= 0.5;
    }
    return sum;
}

template <typename F>
void parallel_for(uint64_t n, int threads, F&& fn) {
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    if (threads <= 0) threads = 1;
    if ((uint64_t)threads > n) threads = (int)(n ? n : 1);
    std::atomic<uint64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            uint64_t i = next.fetch_add(1);
            if (i >= n) break;
            fn(i);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
}

struct SectorOut {
    uint64_t mask = 0;
    std::vector<uint8_t> bricks;
};

// Per-sector voxel function -> sector stream in ascending linear order.
template <typename FillSector>
vrt_status build_stream(uint32_t sx, uint32_t sy, uint32_t sz, int threads, FillSector&& fill,
                        vrt_sector_stream** out) {
    const uint64_t nsec = (uint64_t)sx * sy * sz;
    std::vector<SectorOut> res(nsec);
    parallel_for(nsec, threads, [&](uint64_t s) {
        const uint32_t x = (uint32_t)(s % sx), z = (uint32_t)((s / sx) % sz), y = (uint32_t)(s / ((uint64_t)sx * sz));
        std::vector<uint8_t> vox(32 * 32 * 32);  // index lx | lz<<5 | ly<<10
        if (!fill(x, y, z, vox.data())) return;
        SectorOut& o = res[s];
        for (uint32_t b = 0; b < 64; b++) {
            const uint32_t bx = b & 3, bz = (b >> 2) & 3, by = b >> 4;
            uint8_t brick[512];
            bool any = false;
            for (uint32_t vi = 0; vi < 512; vi++) {
                const uint32_t lx = bx * 8 + (vi & 7), lz = bz * 8 + ((vi >> 3) & 7), ly = by * 8 + (vi >> 6);
                brick[vi] = vox[lx | lz << 5 | ly << 10];
                any |= brick[vi] != 0;
            }
            if (!any) continue;
            o.mask |= 1ull << b;
            o.bricks.insert(o.bricks.end(), brick, brick + 512);
        }
    });
    uint64_t nrec = 0, nbr = 0;
    for (auto& r : res)
        if (r.mask) {
            nrec++;
            nbr += r.bricks.size() / 512;
        }
    auto* st = (vrt_sector_stream*)std::calloc(1, sizeof(vrt_sector_stream));
    if (!st) return VRT_ERR_OUT_OF_MEMORY;
    st->sectors_x = sx;
    st->sectors_y = sy;
    st->sectors_z = sz;
    st->n_sectors = (uint32_t)nrec;
    st->n_bricks = nbr;
    st->sector_idx = (int32_t*)std::malloc(sizeof(int32_t) * (nrec ? nrec : 1));
    st->alloc_mask = (uint64_t*)std::malloc(sizeof(uint64_t) * (nrec ? nrec : 1));
    st->bricks = (uint8_t*)std::malloc(512 * (nbr ? nbr : 1));
    if (!st->sector_idx || !st->alloc_mask || !st->bricks) {
        vrt_sector_stream_free(st);
        return VRT_ERR_OUT_OF_MEMORY;
    }
    uint64_t k = 0, off = 0;
    for (uint64_t s = 0; s < nsec; s++) {
        if (!res[s].mask) continue;
        const uint32_t x = (uint32_t)(s % sx), z = (uint32_t)((s / sx) % sz), y = (uint32_t)(s / ((uint64_t)sx * sz));
        st->sector_idx[k] = vrt::sector_index_pack((int32_t)x, (int32_t)y, (int32_t)z);
        st->alloc_mask[k] = res[s].mask;
        std::memcpy(st->bricks + off, res[s].bricks.data(), res[s].bricks.size());
        off += res[s].bricks.size();
        k++;
    }
    *out = st;
    return VRT_OK;
}

bool valid_size(const uint32_t size[3]) {
    return size[0] && size[1] && size[2] && size[0] % 32 == 0 && size[1] % 32 == 0 && size[2] % 32 == 0 &&
           size[0] <= VRT_MAX_WORLD_X && size[1] <= VRT_MAX_WORLD_Y && size[2] <= VRT_MAX_WORLD_Z;
}

struct Sphere {
    int32_t c[3];
    double r;
    uint8_t mat;
};

}  // namespace

extern "C" {

const char* vrt_synth_last_error(void) { return vrt::last_error_cstr(); }

double vrt_synth_terrain_height(const vrt_synth_terrain* d, double x, double z) {
    return d->base + d->amplitude * fbm2(x / d->scale, z / d->scale, d->octaves, d->seed);
}

vrt_status vrt_synth_terrain_world(const vrt_synth_terrain* desc, int threads, vrt_sector_stream** out) {
    if (!desc || !out || !valid_size(desc->size) || !(desc->scale > 0.0) ||
        (desc->cave_octaves && !(desc->cave_scale > 0.0))) {
        vrt::set_error("bad terrain description");
        return VRT_ERR_INVALID_ARG;
    }
    const vrt_synth_terrain d = *desc;
    auto fill = [&](uint32_t sxi, uint32_t syi, uint32_t szi, uint8_t* vox) -> bool {
        double h[32 * 32];
        double hmax = -1e300;
        for (uint32_t lz = 0; lz < 32; lz++)
            for (uint32_t lx = 0; lx < 32; lx++) {
                const double v = vrt_synth_terrain_height(&d, (double)(sxi * 32 + lx), (double)(szi * 32 + lz));
                h[lx | lz << 5] = v;
                hmax = v > hmax ? v : hmax;
            }
        if ((double)(syi * 32) >= hmax) return false;
        bool any = false;
        for (uint32_t ly = 0; ly < 32; ly++) {
            const uint32_t y = syi * 32 + ly;
            const uint8_t mat = (uint8_t)(1 + (y / 32 < 3 ? y / 32 : 3));
            for (uint32_t lz = 0; lz < 32; lz++)
                for (uint32_t lx = 0; lx < 32; lx++) {
                    bool solid = (double)y < h[lx | lz << 5];
                    if (solid && d.cave_octaves) {
                        const double n = fbm3((double)(sxi * 32 + lx) / d.cave_scale, (double)y / d.cave_scale,
                                              (double)(szi * 32 + lz) / d.cave_scale, d.cave_octaves, d.cave_seed);
                        solid = !(n > d.cave_threshold);
                    }
                    vox[lx | lz << 5 | ly << 10] = solid ? mat : 0;
                    any |= solid;
                }
        }
        return any;
    };
    return build_stream(d.size[0] / 32, d.size[1] / 32, d.size[2] / 32, threads, fill, out);
}

vrt_status vrt_synth_mix_world(uint32_t edge, uint64_t seed, int threads, vrt_sector_stream** out) {
    const uint32_t size[3] = {edge, edge, edge};
    if (!out || !valid_size(size)) {
        vrt::set_error("edge must be a multiple of 32 in 32..1024");
        return VRT_ERR_INVALID_ARG;
    }
    Pcg32 rng(seed, 0x5EED0001u);
    const double density = 0.01 + 0.29 * rng.unit();
    const double fill_frac = 0.20 * rng.unit();
    vrt_synth_terrain t{};
    t.size[0] = t.size[1] = t.size[2] = edge;
    t.base = 0.375 * edge;
    t.amplitude = 0.1875 * edge;
    t.scale = 128.0;
    t.octaves = 4;
    t.seed = rng.next();
    const uint32_t rand_seed = rng.next();
    std::vector<Sphere> spheres;
    const double target = fill_frac * (double)edge * edge * edge;
    double vol = 0.0;
    while (vol < target && spheres.size() < 4096) {
        Sphere s;
        s.r = 2.0 + 38.0 * rng.unit();
        for (int c = 0; c < 3; c++) s.c[c] = (int32_t)(rng.next() % edge);
        s.mat = (uint8_t)(1 + rng.next() % 255);
        vol += 4.18879020478639098 * s.r * s.r * s.r;
        spheres.push_back(s);
    }
    const uint32_t ns = edge / 32;
    std::vector<std::vector<uint32_t>> bins((size_t)ns * ns * ns);
    for (uint32_t i = 0; i < spheres.size(); i++) {
        const Sphere& s = spheres[i];
        int32_t lo[3], hi[3];
        for (int c = 0; c < 3; c++) {
            lo[c] = std::max<int32_t>(0, (int32_t)std::floor(s.c[c] - s.r) >> 5);
            hi[c] = std::min<int32_t>((int32_t)ns - 1, (int32_t)std::floor(s.c[c] + s.r) >> 5);
        }
        for (int32_t y = lo[1]; y <= hi[1]; y++)
            for (int32_t z = lo[2]; z <= hi[2]; z++)
                for (int32_t x = lo[0]; x <= hi[0]; x++) bins[(size_t)x + (size_t)z * ns + (size_t)y * ns * ns].push_back(i);
    }
    const uint32_t thresh = (uint32_t)(density * 4294967296.0 > 4294967295.0 ? 4294967295.0 : density * 4294967296.0);
    auto fill = [&](uint32_t sxi, uint32_t syi, uint32_t szi, uint8_t* vox) -> bool {
        double h[32 * 32];
        for (uint32_t lz = 0; lz < 32; lz++)
            for (uint32_t lx = 0; lx < 32; lx++)
                h[lx | lz << 5] = vrt_synth_terrain_height(&t, (double)(sxi * 32 + lx), (double)(szi * 32 + lz));
        const auto& bin = bins[(size_t)sxi + (size_t)szi * ns + (size_t)syi * ns * ns];
        bool any = false;
        for (uint32_t ly = 0; ly < 32; ly++)
            for (uint32_t lz = 0; lz < 32; lz++)
                for (uint32_t lx = 0; lx < 32; lx++) {
                    const int32_t x = (int32_t)(sxi * 32 + lx), y = (int32_t)(syi * 32 + ly), z = (int32_t)(szi * 32 + lz);
                    uint8_t v = 0;
                    for (uint32_t si : bin) {
                        const Sphere& s = spheres[si];
                        const int64_t dx = x - s.c[0], dy = y - s.c[1], dz = z - s.c[2];
                        if ((double)(dx * dx + dy * dy + dz * dz) <= s.r * s.r) {
                            v = s.mat;
                            break;
                        }
                    }
                    if (!v && (double)y < h[lx | lz << 5]) v = (uint8_t)(1 + ((uint32_t)y / 32 < 3 ? (uint32_t)y / 32 : 3));
                    if (!v) {
                        const uint32_t hh = pcg_hash(pcg_hash(pcg_hash(rand_seed ^ (uint32_t)x) ^ (uint32_t)y) ^ (uint32_t)z);
                        if (hh < thresh) v = (uint8_t)(1 + pcg_hash(hh) % 255);
                    }
                    vox[lx | lz << 5 | ly << 10] = v;
                    any |= v != 0;
                }
        return any;
    };
    return build_stream(ns, ns, ns, threads, fill, out);
}

vrt_status vrt_synth_random_rays(const uint32_t size[3], uint64_t seed, uint64_t first, uint64_t n, int threads,
                                 vrt_ray* out) {
    if (!size || (n && !out)) {
        vrt::set_error("null argument");
        return VRT_ERR_INVALID_ARG;
    }
    const uint64_t chunk = 4096;
    parallel_for((n + chunk - 1) / chunk, threads, [&](uint64_t c) {
        const uint64_t b = c * chunk, e = b + chunk < n ? b + chunk : n;
        for (uint64_t i = b; i < e; i++) {
            Pcg32 rng(first + i, seed);
            vrt_ray& r = out[i];
            for (int k = 0; k < 3; k++) r.origin[k] = (float)(rng.next() >> 8) * 0x1p-24f * (float)size[k];
            float x = 1.0f, y = 0.0f, z = 0.0f, r2 = 1.0f;
            for (int attempt = 0; attempt < 64; attempt++) {
                x = rng.next_signed();
                y = rng.next_signed();
                z = rng.next_signed();
                r2 = (x * x + y * y) + z * z;
                if (r2 > 1e-6f && r2 <= 1.0f) break;
                x = 1.0f, y = 0.0f, z = 0.0f, r2 = 1.0f;
            }
            const float len = std::sqrt(r2);
            r.dir[0] = x / len;
            r.dir[1] = y / len;
            r.dir[2] = z / len;
            r.tag = (uint32_t)(first + i);
            r.reserved = 0;
        }
    });
    return VRT_OK;
}

}  // extern "C"
