// Minimal stand-in for the subset of GLM that the reference's CPU traversal,
// VoxelMap and renderer headers use, so those files compile in place for the
// oracle pin build (x86 only, test infrastructure).  Written from GLM's documented
// semantics; only what the pinned code paths need is exact.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

namespace glm {

template <int N, typename T>
struct vec;

template <typename T>
struct vec<2, T> {
    T x, y;
    constexpr vec() : x(0), y(0) {}
    template <typename A>
    constexpr explicit vec(A s) : x(T(s)), y(T(s)) {}
    template <typename A, typename B>
    constexpr vec(A a, B b) : x(T(a)), y(T(b)) {}
    template <typename U>
    constexpr vec(const vec<2, U>& o) : x(T(o.x)), y(T(o.y)) {}
    constexpr T& operator[](int i) { return i == 0 ? x : y; }
    constexpr const T& operator[](int i) const { return i == 0 ? x : y; }
};
template <typename T>
struct vec<3, T> {
    T x, y, z;
    constexpr vec() : x(0), y(0), z(0) {}
    template <typename A>
    constexpr explicit vec(A s) : x(T(s)), y(T(s)), z(T(s)) {}
    template <typename A, typename B, typename C>
    constexpr vec(A a, B b, C c) : x(T(a)), y(T(b)), z(T(c)) {}
    template <typename U>
    constexpr vec(const vec<3, U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    template <typename U>
    constexpr explicit vec(const vec<4, U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    constexpr T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    constexpr const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <typename T>
struct vec<4, T> {
    T x, y, z, w;
    constexpr vec() : x(0), y(0), z(0), w(0) {}
    template <typename A>
    constexpr explicit vec(A s) : x(T(s)), y(T(s)), z(T(s)), w(T(s)) {}
    template <typename A, typename B, typename C, typename D>
    constexpr vec(A a, B b, C c, D d) : x(T(a)), y(T(b)), z(T(c)), w(T(d)) {}
    template <typename U, typename D>
    constexpr vec(const vec<3, U>& o, D d) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(d)) {}
    template <typename U>
    constexpr vec(const vec<4, U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
    constexpr T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    constexpr const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

using vec2 = vec<2, float>;
using vec3 = vec<3, float>;
using vec4 = vec<4, float>;
using dvec3 = vec<3, double>;
using ivec2 = vec<2, int32_t>;
using ivec3 = vec<3, int32_t>;
using uvec2 = vec<2, uint32_t>;
using uvec3 = vec<3, uint32_t>;
using bvec2 = vec<2, bool>;
using bvec3 = vec<3, bool>;

#define GLM_SHIM_BINOP(op)                                                                   \
    template <int N, typename T>                                                             \
    constexpr vec<N, T> operator op(const vec<N, T>& a, const vec<N, T>& b) {               \
        vec<N, T> r;                                                                         \
        for (int i = 0; i < N; i++) r[i] = a[i] op b[i];                                    \
        return r;                                                                            \
    }                                                                                        \
    template <int N, typename T, typename S, typename = std::enable_if_t<std::is_arithmetic_v<S>>> \
    constexpr vec<N, T> operator op(const vec<N, T>& a, S b) {                              \
        vec<N, T> r;                                                                         \
        for (int i = 0; i < N; i++) r[i] = a[i] op T(b);                                    \
        return r;                                                                            \
    }                                                                                        \
    template <int N, typename T, typename S, typename = std::enable_if_t<std::is_arithmetic_v<S>>> \
    constexpr vec<N, T> operator op(S a, const vec<N, T>& b) {                              \
        vec<N, T> r;                                                                         \
        for (int i = 0; i < N; i++) r[i] = T(a) op b[i];                                    \
        return r;                                                                            \
    }                                                                                        \
    template <int N, typename T, typename U>                                                 \
    constexpr vec<N, T>& operator op##=(vec<N, T>& a, const U& b) {                         \
        a = a op b;                                                                          \
        return a;                                                                            \
    }

GLM_SHIM_BINOP(+)
GLM_SHIM_BINOP(-)
GLM_SHIM_BINOP(*)
GLM_SHIM_BINOP(/)
GLM_SHIM_BINOP(&)
GLM_SHIM_BINOP(|)
GLM_SHIM_BINOP(^)
GLM_SHIM_BINOP(>>)
GLM_SHIM_BINOP(<<)
#undef GLM_SHIM_BINOP

template <int N, typename T>
constexpr vec<N, T> operator-(const vec<N, T>& a) {
    vec<N, T> r;
    for (int i = 0; i < N; i++) r[i] = -a[i];
    return r;
}
template <int N, typename T>
constexpr bool operator==(const vec<N, T>& a, const vec<N, T>& b) {
    for (int i = 0; i < N; i++)
        if (!(a[i] == b[i])) return false;
    return true;
}
template <int N, typename T>
constexpr bool operator!=(const vec<N, T>& a, const vec<N, T>& b) { return !(a == b); }

#define GLM_SHIM_FN1(name, expr)                      \
    template <int N, typename T>                      \
    vec<N, T> name(const vec<N, T>& a) {              \
        vec<N, T> r;                                  \
        for (int i = 0; i < N; i++) {                 \
            T v = a[i];                               \
            r[i] = (expr);                            \
        }                                             \
        return r;                                     \
    }
GLM_SHIM_FN1(floor, std::floor(v))
GLM_SHIM_FN1(fract, v - std::floor(v))
GLM_SHIM_FN1(round, std::round(v))
GLM_SHIM_FN1(sign, T((T(0) < v) - (v < T(0))))
#undef GLM_SHIM_FN1

inline float floor(float v) { return std::floor(v); }
inline double floor(double v) { return std::floor(v); }
inline float fract(float v) { return v - std::floor(v); }
inline float round(float v) { return std::round(v); }

template <int N, typename T>
vec<N, T> min(const vec<N, T>& a, const vec<N, T>& b) {
    vec<N, T> r;
    for (int i = 0; i < N; i++) r[i] = b[i] < a[i] ? b[i] : a[i];
    return r;
}
template <int N, typename T>
vec<N, T> max(const vec<N, T>& a, const vec<N, T>& b) {
    vec<N, T> r;
    for (int i = 0; i < N; i++) r[i] = a[i] < b[i] ? b[i] : a[i];
    return r;
}
template <typename T>
T min(T a, T b) { return b < a ? b : a; }
template <typename T>
T max(T a, T b) { return a < b ? b : a; }
template <int N, typename T, typename S>
vec<N, T> clamp(const vec<N, T>& x, S lo, S hi) {
    vec<N, T> r;
    for (int i = 0; i < N; i++) r[i] = min(max(x[i], T(lo)), T(hi));
    return r;
}
template <int N, typename T>
vec<N, T> step(T edge, const vec<N, T>& x) {
    vec<N, T> r;
    for (int i = 0; i < N; i++) r[i] = x[i] < edge ? T(0) : T(1);
    return r;
}
template <int N, typename T>
vec<N, bool> greaterThanEqual(const vec<N, T>& a, const vec<N, T>& b) {
    vec<N, bool> r;
    for (int i = 0; i < N; i++) r[i] = a[i] >= b[i];
    return r;
}
template <int N, typename T>
vec<N, T> mix(const vec<N, T>& a, const vec<N, T>& b, const vec<N, bool>& t) {
    vec<N, T> r;
    for (int i = 0; i < N; i++) r[i] = t[i] ? b[i] : a[i];
    return r;
}
template <int N, typename T>
vec<N, T> mix(const vec<N, T>& a, const vec<N, T>& b, const vec<N, T>& t) {
    vec<N, T> r;
    for (int i = 0; i < N; i++) r[i] = a[i] * (T(1) - t[i]) + b[i] * t[i];
    return r;
}

// IEEE binary16 packing with round-to-nearest-even (GLM packHalf2x16: x in the low half).
inline uint16_t to_half(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    uint32_t sign = (u >> 16) & 0x8000u, e = (u >> 23) & 0xFF, m = u & 0x7FFFFFu;
    if (e == 0xFF) return (uint16_t)(sign | 0x7C00u | (m ? 0x200u : 0));
    int32_t he = (int32_t)e - 127 + 15;
    if (he >= 31) return (uint16_t)(sign | 0x7C00u);
    if (he <= 0) {
        if (he < -10) return (uint16_t)sign;
        m |= 0x800000u;
        uint32_t shift = (uint32_t)(14 - he);
        uint32_t hm = m >> shift, rem = m & ((1u << shift) - 1), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1))) hm++;
        return (uint16_t)(sign | hm);
    }
    uint32_t hm = m >> 13, rem = m & 0x1FFFu;
    uint32_t r = sign | ((uint32_t)he << 10) | hm;
    if (rem > 0x1000u || (rem == 0x1000u && (hm & 1))) r++;
    return (uint16_t)r;
}
inline uint32_t packHalf2x16(const vec2& v) { return (uint32_t)to_half(v.x) | (uint32_t)to_half(v.y) << 16; }

// Column-major 4x4 matrix.
struct mat4 {
    vec4 c[4];
    constexpr mat4() : c{vec4(1, 0, 0, 0), vec4(0, 1, 0, 0), vec4(0, 0, 1, 0), vec4(0, 0, 0, 1)} {}
    explicit mat4(float d) : c{vec4(d, 0, 0, 0), vec4(0, d, 0, 0), vec4(0, 0, d, 0), vec4(0, 0, 0, d)} {}
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline vec4 operator*(const mat4& m, const vec4& v) {
    return m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w;
}
inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r;
    for (int i = 0; i < 4; i++) r[i] = a * b[i];
    return r;
}
inline mat4 translate(const mat4& m, const vec3& v) {
    mat4 r = m;
    r[3] = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3];
    return r;
}
inline mat4 scale(const mat4& m, const vec3& v) {
    mat4 r = m;
    r[0] = m[0] * v.x;
    r[1] = m[1] * v.y;
    r[2] = m[2] * v.z;
    return r;
}
inline mat4 inverse(const mat4& m) {
    // Gauss-Jordan elimination with partial pivoting
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int col = 0; col < 4; col++) {
            a[r][col] = m[col][r];
            a[r][col + 4] = r == col ? 1.0 : 0.0;
        }
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        for (int k = 0; k < 8; k++) std::swap(a[col][k], a[piv][k]);
        double d = a[col][col];
        for (int k = 0; k < 8; k++) a[col][k] /= d;
        for (int r = 0; r < 4; r++)
            if (r != col) {
                double f = a[r][col];
                for (int k = 0; k < 8; k++) a[r][k] -= f * a[col][k];
            }
    }
    mat4 out;
    for (int r = 0; r < 4; r++)
        for (int col = 0; col < 4; col++) out[col][r] = (float)a[r][col + 4];
    return out;
}

}  // namespace glm
