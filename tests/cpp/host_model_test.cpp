// host_model_test.cpp - drives the C++ host mirror (include/vrt.hpp) the way the
// reference's application drives VoxelMap + GpuRenderer, and dumps what it built
// so the Python tests can compare it with the CPU oracle.
//
//   host_model_test edits <out>   host model only: sets + sphere edits, dump sectors
//   host_model_test render <out>  also SyncBuffers + RenderFrame on the GPU, dump hits
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "vrt.hpp"

namespace {

// Integer sphere brush through RegionDispatch (the semantics of vrt_edit).
void sphere(vrt::VoxelMap& map, int cx, int cy, int cz, int r, uint8_t material, int sectors) {
    const int lim = sectors * 32 - 1;
    vrt::IVec3 lo{std::max(cx - r, 0), std::max(cy - r, 0), std::max(cz - r, 0)};
    vrt::IVec3 hi{std::min(cx + r, lim), std::min(cy + r, lim), std::min(cz + r, lim)};
    map.RegionDispatch(lo, hi, material != 0, [&](int x, int y, int z, vrt::Voxel& v) {
        const long dx = x - cx, dy = y - cy, dz = z - cz;
        if (dx * dx + dy * dy + dz * dz > (long)r * r) return false;
        v.Data = material;
        return true;
    });
}

void build(vrt::VoxelMap& map) {
    for (int x = 0; x < 64; x++)
        for (int z = 0; z < 64; z++)
            for (int y = 0; y < 10 + (x * 7 + z * 3) % 13; y++) map.Set({x, y, z}, {(uint8_t)(1 + y / 8)});
    sphere(map, 30, 20, 30, 12, 0, 2);
    sphere(map, 10, 40, 50, 9, 77, 2);
    sphere(map, 50, 8, 10, 6, 0, 2);
    sphere(map, 0, 0, 0, 3, 200, 2);
}

void dump_sectors(const vrt::VoxelMap& map, FILE* f) {
    // records sorted by key: u32 key, u64 mask, bricks in bit order
    std::vector<uint32_t> keys;
    for (const auto& kv : map.Sectors) keys.push_back(kv.first);
    std::sort(keys.begin(), keys.end());
    uint32_t n = (uint32_t)keys.size();
    fwrite(&n, 4, 1, f);
    for (uint32_t k : keys) {
        vrt::Sector s = map.Sectors.at(k);
        uint64_t m = s.GetAllocationMask();
        fwrite(&k, 4, 1, f);
        fwrite(&m, 8, 1, f);
        for (uint64_t r = m; r; r &= r - 1) fwrite(s.GetBrick((uint32_t)__builtin_ctzll(r))->Data, 1, 512, f);
    }
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    auto map = std::make_shared<vrt::VoxelMap>();
    build(*map);
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    dump_sectors(*map, f);
    if (std::strcmp(argv[1], "render") == 0) {
        vrt::GpuRenderer renderer(map, 2, 2, 2);
        const double pos[3] = {32.5, 90.0, -20.0}, tgt[3] = {32.0, 10.0, 40.0};
        vrt_view view{};
        view.cam = vrt::LookAt(pos, tgt, 75.0, 96, 64);
        std::vector<vrt_hit> a = renderer.RenderFrame(view);
        // an edit between frames, then the next frame sees it
        sphere(*map, 32, 12, 32, 10, 0, 2);
        std::vector<vrt_hit> b = renderer.RenderFrame(view);
        renderer.UseAnisotropicLods = true;
        std::vector<vrt_hit> c = renderer.RenderFrame(view);
        uint64_t n = a.size();
        fwrite(&n, 8, 1, f);
        fwrite(a.data(), sizeof(vrt_hit), a.size(), f);
        fwrite(b.data(), sizeof(vrt_hit), b.size(), f);
        fwrite(c.data(), sizeof(vrt_hit), c.size(), f);
        fwrite(&view.cam, sizeof(vrt_camera), 1, f);
    }
    std::fclose(f);
    return 0;
}
