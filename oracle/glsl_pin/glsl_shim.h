// glsl_shim.h - the subset of GLSL that the reference's traversal shaders use
// (Shaders/VoxelTraversal.glsl, Shaders/VoxelMap.glsl), as C++, so that their source
// compiles on the host as a pin for the GLSL traversal mode.  Test infrastructure:
// built only into oracle/_ref by oracle/glsl_pin/build_glsl.py.
//
// Where GLSL leaves a result open, this header follows the traversal contract the
// oracle and the device pin (oracle/vrt_oracle.cpp):
//   * min(a, b) = a < b ? a : b and max(a, b) = a > b ? a : b (x86 minps/maxps; GLSL
//     leaves NaN operands undefined);
//   * float -> int conversion of a NaN or out-of-range value gives INT32_MIN (x86);
//   * integer vector adds and subtracts wrap (two's complement, as on a GPU).
// Vector swizzles are provided for the ones these shaders read (.xz, .yy).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

typedef unsigned int uint;

namespace glsl_shim {

template <class T>
struct Vec2 {
    T x, y;
    Vec2() = default;
    Vec2(T a, T b) : x(a), y(b) {}
};

template <class T, int A, int B>
struct Swz2 {
    T v[3];
    operator Vec2<T>() const { return Vec2<T>(v[A], v[B]); }
};

template <class T>
struct Vec3 {
    union {
        struct {
            T x, y, z;
        };
        Swz2<T, 0, 2> xz;
        Swz2<T, 1, 1> yy;
    };
    Vec3() = default;
    Vec3(T a, T b, T c) : x(a), y(b), z(c) {}
};

}  // namespace glsl_shim

using bvec2 = glsl_shim::Vec2<bool>;

struct vec2 : glsl_shim::Vec2<float> {
    vec2() = default;
    vec2(float a, float b) : Vec2(a, b) {}
    vec2(const glsl_shim::Vec2<float>& v) : Vec2(v) {}
};

struct uvec2 : glsl_shim::Vec2<uint> {
    uvec2() = default;
    uvec2(uint a, uint b) : Vec2(a, b) {}
    explicit uvec2(int s) : Vec2((uint)s, (uint)s) {}
};
inline bool operator==(uvec2 a, uvec2 b) { return a.x == b.x && a.y == b.y; }
inline bool operator!=(uvec2 a, uvec2 b) { return !(a == b); }
inline uvec2& operator&=(uvec2& a, uvec2 b) {
    a.x &= b.x;
    a.y &= b.y;
    return a;
}

struct ivec3;
struct uvec3;

struct bvec3 : glsl_shim::Vec3<bool> {
    bvec3() = default;
    bvec3(bool a, bool b, bool c) : Vec3(a, b, c) {}
};

struct vec3 : glsl_shim::Vec3<float> {
    vec3() = default;
    vec3(float a, float b, float c) : Vec3(a, b, c) {}
    explicit vec3(float s) : Vec3(s, s, s) {}
    explicit vec3(int s) : Vec3((float)s, (float)s, (float)s) {}
    vec3(const ivec3& v);            // implicit, as GLSL converts int vectors to float
    explicit vec3(const uvec3& v);
};

struct ivec3 : glsl_shim::Vec3<int> {
    ivec3() = default;
    ivec3(int a, int b, int c) : Vec3(a, b, c) {}
    explicit ivec3(int s) : Vec3(s, s, s) {}
    explicit ivec3(uint s) : Vec3((int)s, (int)s, (int)s) {}
    explicit ivec3(const vec3& v);   // the x86 conversion rule
    explicit ivec3(const uvec3& v);
};

struct uvec3 : glsl_shim::Vec3<uint> {
    uvec3() = default;
    uvec3(uint a, uint b, uint c) : Vec3(a, b, c) {}
    uvec3(int a, int b, int c) : Vec3((uint)a, (uint)b, (uint)c) {}
    explicit uvec3(uint s) : Vec3(s, s, s) {}
    explicit uvec3(const ivec3& v) : Vec3((uint)v.x, (uint)v.y, (uint)v.z) {}
};

inline int glsl_f2i(float f) {
    if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int)f;
}
inline vec3::vec3(const ivec3& v) : Vec3((float)v.x, (float)v.y, (float)v.z) {}
inline vec3::vec3(const uvec3& v) : Vec3((float)v.x, (float)v.y, (float)v.z) {}
inline ivec3::ivec3(const vec3& v) : Vec3(glsl_f2i(v.x), glsl_f2i(v.y), glsl_f2i(v.z)) {}
inline ivec3::ivec3(const uvec3& v) : Vec3((int)v.x, (int)v.y, (int)v.z) {}

// float vectors: component-wise arithmetic, each op rounded on its own
#define GLSL_F3_OP(op)                                                                               \
    inline vec3 operator op(vec3 a, vec3 b) { return vec3(a.x op b.x, a.y op b.y, a.z op b.z); }     \
    inline vec3 operator op(vec3 a, float s) { return vec3(a.x op s, a.y op s, a.z op s); }          \
    inline vec3 operator op(float s, vec3 a) { return vec3(s op a.x, s op a.y, s op a.z); }
GLSL_F3_OP(+)
GLSL_F3_OP(-)
GLSL_F3_OP(*)
GLSL_F3_OP(/)
#undef GLSL_F3_OP
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }

// integer vectors (wrapping add, subtract, multiply)
inline int glsl_wrap(int64_t v) { return (int)(uint32_t)(uint64_t)v; }
#define GLSL_I3_ARITH(op)                                                                              \
    inline ivec3 operator op(ivec3 a, ivec3 b) {                                                       \
        return ivec3(glsl_wrap((int64_t)a.x op b.x), glsl_wrap((int64_t)a.y op b.y),                   \
                     glsl_wrap((int64_t)a.z op b.z));                                                  \
    }                                                                                                  \
    inline ivec3 operator op(ivec3 a, int s) { return a op ivec3(s); }                                 \
    inline ivec3 operator op(int s, ivec3 a) { return ivec3(s) op a; }
GLSL_I3_ARITH(+)
GLSL_I3_ARITH(-)
GLSL_I3_ARITH(*)
#undef GLSL_I3_ARITH
#define GLSL_I3_BIT(op)                                                                                \
    inline ivec3 operator op(ivec3 a, ivec3 b) { return ivec3(a.x op b.x, a.y op b.y, a.z op b.z); } \
    inline ivec3 operator op(ivec3 a, int s) { return ivec3(a.x op s, a.y op s, a.z op s); }
GLSL_I3_BIT(&)
GLSL_I3_BIT(|)
GLSL_I3_BIT(^)
GLSL_I3_BIT(>>)
GLSL_I3_BIT(<<)
#undef GLSL_I3_BIT
inline ivec3 operator-(ivec3 a) { return ivec3(0) - a; }

#define GLSL_U3_OP(op)                                                                               \
    inline uvec3 operator op(uvec3 a, uvec3 b) { return uvec3(a.x op b.x, a.y op b.y, a.z op b.z); } \
    inline uvec3 operator op(uvec3 a, uint s) { return uvec3(a.x op s, a.y op s, a.z op s); }
GLSL_U3_OP(+)
GLSL_U3_OP(-)
GLSL_U3_OP(*)
GLSL_U3_OP(/)
GLSL_U3_OP(%)
GLSL_U3_OP(&)
GLSL_U3_OP(|)
GLSL_U3_OP(>>)
GLSL_U3_OP(<<)
#undef GLSL_U3_OP

// built-in functions
inline float min(float a, float b) { return a < b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline vec3 min(vec3 a, vec3 b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 floor(vec3 a) { return vec3(std::floor(a.x), std::floor(a.y), std::floor(a.z)); }
inline float glsl_fract(float a) { return a - std::floor(a); }
inline vec2 fract(glsl_shim::Vec2<float> a) { return vec2(glsl_fract(a.x), glsl_fract(a.y)); }
inline float glsl_sign(float a) { return a > 0.0f ? 1.0f : a < 0.0f ? -1.0f : 0.0f; }
inline vec3 sign(vec3 a) { return vec3(glsl_sign(a.x), glsl_sign(a.y), glsl_sign(a.z)); }
inline vec3 step(float edge, vec3 a) {
    return vec3(a.x < edge ? 0.0f : 1.0f, a.y < edge ? 0.0f : 1.0f, a.z < edge ? 0.0f : 1.0f);
}
inline bvec3 greaterThanEqual(vec3 a, vec3 b) { return bvec3(a.x >= b.x, a.y >= b.y, a.z >= b.z); }
inline vec3 mix(vec3 a, vec3 b, bvec3 s) { return vec3(s.x ? b.x : a.x, s.y ? b.y : a.y, s.z ? b.z : a.z); }
// 2-vectors as the base type, so that a swizzle (.xz, .yy) converts in one step
inline glsl_shim::Vec2<float> mix(glsl_shim::Vec2<float> a, glsl_shim::Vec2<float> b, bvec2 s) {
    return glsl_shim::Vec2<float>(s.x ? b.x : a.x, s.y ? b.y : a.y);
}
inline uint floatBitsToUint(float f) {
    uint u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float uintBitsToFloat(uint u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline int findLSB(uint v) { return v ? __builtin_ctz(v) : -1; }
inline int bitCount(uint v) { return __builtin_popcount(v); }
// IEEE binary16 -> binary32 by its definition (sign, 5-bit exponent, 10-bit fraction)
inline float glsl_half(uint h) {
    const uint s = h >> 15, e = (h >> 10) & 31u, m = h & 1023u;
    float v = e == 0 ? std::ldexp((float)m, -24) : e == 31 ? (m ? NAN : INFINITY) : std::ldexp((float)(m | 1024u), (int)e - 25);
    return s ? -v : v;
}
inline vec2 unpackHalf2x16(uint v) { return vec2(glsl_half(v & 0xFFFFu), glsl_half(v >> 16)); }
