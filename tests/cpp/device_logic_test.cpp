// device_logic_test.cpp - compiles the device traversal step (trace_core.cuh) for the
// host, with the CUDA rounding intrinsics mapped to their IEEE host equivalents, and
// runs it over a world and ray batch dumped by the Python test; the records go back
// to be compared with the oracle.  This checks the kernel's control logic (brick
// table and voxel codes, alignment, clipping, NaN handling) on every CPU test run,
// without a GPU.
//
//   device_logic_test <world.bin> <rays.bin> <out.bin> <max_iters> <wox> <woy> <woz> [glsl]
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define __device__
#define __host__
#define __forceinline__ inline
struct uint4 {
    unsigned x, y, z, w;
};
struct uint2 {
    unsigned x, y;
};
inline uint4 make_uint4(unsigned a, unsigned b, unsigned c, unsigned d) { return uint4{a, b, c, d}; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline float __fsqrt_rn(float a) { return std::sqrt(a); }
inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
inline float __int2float_rn(int a) { return (float)a; }
inline float __uint2float_rn(unsigned a) { return (float)a; }
// cvt.rmi.s32.f32: floor, saturating, NaN -> 0
inline int __float2int_rd(float x) {
    if (x != x) return 0;
    const float f = std::floor(x);
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f < -2147483648.0f) return INT32_MIN;
    return (int)f;
}
inline unsigned __float_as_uint(float f) {
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float __uint_as_float(unsigned u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __ffsll(long long x) { return __builtin_ffsll(x); }
template <typename T>
inline T __ldg(const T* p) {
    return *p;
}
using std::signbit;

#include "../../voxelrt_gb300/csrc/trace_core.cuh"

using namespace vrt;

int main(int argc, char** argv) {
    fill_forward_lut_entries(0, 1);
    if (argc < 8) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    uint32_t dims[3], nslots;
    if (std::fread(dims, 4, 3, f) != 3 || std::fread(&nslots, 4, 1, f) != 1) return 4;
    const size_t npos = (size_t)dims[0] * dims[1] * dims[2] * 64;
    std::vector<uint32_t> bricks(npos);
    std::vector<uint8_t> codes((size_t)nslots * 512);
    std::vector<uint8_t> payload((size_t)nslots * 512);
    if (std::fread(bricks.data(), 4, npos, f) != npos) return 5;
    if (std::fread(codes.data(), 1, codes.size(), f) != codes.size()) return 6;
    if (std::fread(payload.data(), 1, payload.size(), f) != payload.size()) return 7;
    std::vector<uint64_t> cells((size_t)nslots * 8);
    if (std::fread(cells.data(), 8, cells.size(), f) != cells.size()) return 9;
    std::fclose(f);
    DevWorld w{};
    w.bricks = bricks.data();
    w.codes = codes.data();
    w.payload = payload.data();
    w.cells = cells.data();
    w.bsx = dims[0] * 4;
    w.bsxz = dims[0] * 4 * dims[2] * 4;
    w.size_x = dims[0] * 32;
    w.size_y = dims[1] * 32;
    w.size_z = dims[2] * 32;
    f = std::fopen(argv[2], "rb");
    if (!f) return 8;
    std::vector<vrt_ray> rays;
    vrt_ray r;
    while (std::fread(&r, sizeof(r), 1, f) == 1) rays.push_back(r);
    std::fclose(f);
    const uint32_t max_iters = (uint32_t)std::atoi(argv[4]);
    const bool glsl = argc > 8 && std::atoi(argv[8]) != 0;
    const bool coarse = argc > 9 && std::atoi(argv[9]) != 0;
    const bool aniso = argc > 10 && std::atoi(argv[10]) != 0;
    const int wo[3] = {std::atoi(argv[5]), std::atoi(argv[6]), std::atoi(argv[7])};
    std::vector<uint4> out(rays.size());
    for (size_t i = 0; i < rays.size(); i++) {
        TraceResult res;
        TraceCounters cnt{0, 0};
        const vrt_ray& q = rays[i];
        if (glsl) {
            trace_ray<false, true>(w, q.origin[0], q.origin[1], q.origin[2], q.dir[0], q.dir[1], q.dir[2], wo[0],
                                   wo[1], wo[2], max_iters, res, cnt, coarse, aniso);
            out[i] = pack_hit<true>(res, q.dir[0], q.dir[1], q.dir[2], q.tag);
        } else {
            trace_ray<false, false>(w, q.origin[0], q.origin[1], q.origin[2], q.dir[0], q.dir[1], q.dir[2], wo[0],
                                    wo[1], wo[2], max_iters, res, cnt);
            out[i] = pack_hit<false>(res, q.dir[0], q.dir[1], q.dir[2], q.tag);
        }
    }
    f = std::fopen(argv[3], "wb");
    if (!f) return 9;
    std::fwrite(out.data(), sizeof(uint4), out.size(), f);
    std::fclose(f);
    return 0;
}
