// glm_host.hpp - the few glm vector types and functions the reference's host set-up code uses, so
// that code compiles here as it is written (test infrastructure: oracle/ref_host.cpp includes the
// extracted reference sources after this header). Semantics follow glm 1.x: component-wise
// arithmetic, glm::clamp/min/max/abs/floor/ceil per component, floor-then-convert constructors
// between vector types, IEEE binary16 round-to-nearest-even for packHalf2x16 (the one function
// whose rounding the reference does not pin down: glm is not available to compare against).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

namespace glm {

template <typename T, int N>
struct vec_base;

template <typename T>
struct vec_base<T, 2> {
    T x, y;
    constexpr vec_base() : x(0), y(0) {}
    constexpr explicit vec_base(T s) : x(s), y(s) {}
    constexpr vec_base(T a, T b) : x(a), y(b) {}
    T& operator[](int i) { return i == 0 ? x : y; }
    const T& operator[](int i) const { return i == 0 ? x : y; }
};
template <typename T>
struct vec_base<T, 3> {
    T x, y, z;
    constexpr vec_base() : x(0), y(0), z(0) {}
    constexpr explicit vec_base(T s) : x(s), y(s), z(s) {}
    constexpr vec_base(T a, T b, T c) : x(a), y(b), z(c) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <typename T>
struct vec_base<T, 4> {
    T x, y, z, w;
    constexpr vec_base() : x(0), y(0), z(0), w(0) {}
    constexpr explicit vec_base(T s) : x(s), y(s), z(s), w(s) {}
    constexpr vec_base(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

template <typename T, int N>
struct vec : vec_base<T, N> {
    using B = vec_base<T, N>;
    using B::B;
    constexpr vec() : B() {}
    // conversions between component types (glm's explicit converting constructors)
    template <typename U>
    explicit vec(const vec<U, N>& o) {
        for (int i = 0; i < N; ++i) (*this)[i] = static_cast<T>(o[i]);
    }
    // vec4(vec3, w)
    template <typename U, int M = N, typename = typename std::enable_if<M == 4>::type>
    vec(const vec<U, 3>& o, T w) : B(static_cast<T>(o.x), static_cast<T>(o.y), static_cast<T>(o.z), w) {}
    // vec3(vec4) drops w (glm's explicit truncating constructor)
    template <typename U, int M = N, typename = typename std::enable_if<M == 3>::type>
    explicit vec(const vec<U, 4>& o) : B(static_cast<T>(o.x), static_cast<T>(o.y), static_cast<T>(o.z)) {}
    static constexpr int length() { return N; }
};

using vec2 = vec<float, 2>;
using vec3 = vec<float, 3>;
using vec4 = vec<float, 4>;
using ivec3 = vec<int, 3>;
using ivec4 = vec<int, 4>;
using uvec3 = vec<unsigned, 3>;
using uvec4 = vec<unsigned, 4>;
using bvec3 = vec<bool, 3>;

#define GLM_HOST_BINOP(op)                                                                 \
    template <typename T, int N>                                                           \
    vec<T, N> operator op(const vec<T, N>& a, const vec<T, N>& b) {                        \
        vec<T, N> r;                                                                       \
        for (int i = 0; i < N; ++i) r[i] = a[i] op b[i];                                   \
        return r;                                                                          \
    }                                                                                      \
    template <typename T, int N>                                                           \
    vec<T, N> operator op(const vec<T, N>& a, T s) {                                       \
        vec<T, N> r;                                                                       \
        for (int i = 0; i < N; ++i) r[i] = a[i] op s;                                      \
        return r;                                                                          \
    }                                                                                      \
    template <typename T, int N>                                                           \
    vec<T, N> operator op(T s, const vec<T, N>& a) {                                       \
        vec<T, N> r;                                                                       \
        for (int i = 0; i < N; ++i) r[i] = s op a[i];                                      \
        return r;                                                                          \
    }                                                                                      \
    template <typename T, int N>                                                           \
    vec<T, N>& operator op##=(vec<T, N>& a, const vec<T, N>& b) {                          \
        for (int i = 0; i < N; ++i) a[i] = a[i] op b[i];                                   \
        return a;                                                                          \
    }
GLM_HOST_BINOP(+)
GLM_HOST_BINOP(-)
GLM_HOST_BINOP(*)
GLM_HOST_BINOP(/)
#undef GLM_HOST_BINOP

template <typename T, int N>
vec<T, N> operator-(const vec<T, N>& a) {
    vec<T, N> r;
    for (int i = 0; i < N; ++i) r[i] = -a[i];
    return r;
}
template <typename T, int N>
bool operator==(const vec<T, N>& a, const vec<T, N>& b) {
    for (int i = 0; i < N; ++i)
        if (!(a[i] == b[i])) return false;
    return true;
}
template <typename T, int N>
bool operator!=(const vec<T, N>& a, const vec<T, N>& b) {
    return !(a == b);
}

#define GLM_HOST_UNARY(name, expr)             \
    template <typename T, int N>               \
    vec<T, N> name(const vec<T, N>& a) {       \
        vec<T, N> r;                           \
        for (int i = 0; i < N; ++i) {          \
            const T v = a[i];                  \
            r[i] = (expr);                     \
        }                                      \
        return r;                              \
    }
GLM_HOST_UNARY(abs, v < T(0) ? -v : v)
GLM_HOST_UNARY(floor, std::floor(v))
GLM_HOST_UNARY(ceil, std::ceil(v))
GLM_HOST_UNARY(round, std::round(v))
#undef GLM_HOST_UNARY

template <typename T, int N>
vec<T, N> min(const vec<T, N>& a, const vec<T, N>& b) {
    vec<T, N> r;
    for (int i = 0; i < N; ++i) r[i] = b[i] < a[i] ? b[i] : a[i];
    return r;
}
template <typename T, int N>
vec<T, N> max(const vec<T, N>& a, const vec<T, N>& b) {
    vec<T, N> r;
    for (int i = 0; i < N; ++i) r[i] = a[i] < b[i] ? b[i] : a[i];
    return r;
}
template <typename T, int N>
vec<T, N> clamp(const vec<T, N>& v, const vec<T, N>& lo, const vec<T, N>& hi) {
    return min(max(v, lo), hi);
}
template <typename T>
T clamp(T v, T lo, T hi) {
    return v < lo ? lo : (hi < v ? hi : v);
}
template <typename T, int N>
T dot(const vec<T, N>& a, const vec<T, N>& b) {
    T s = a[0] * b[0];
    for (int i = 1; i < N; ++i) s = s + a[i] * b[i];
    return s;
}
template <typename T, int N>
T length(const vec<T, N>& a) {
    return std::sqrt(dot(a, a));
}
template <typename T, int N>
vec<T, N> normalize(const vec<T, N>& a) {
    return a * (T(1) / length(a));
}
template <typename T, int N>
vec<bool, N> lessThan(const vec<T, N>& a, const vec<T, N>& b) {
    vec<bool, N> r;
    for (int i = 0; i < N; ++i) r[i] = a[i] < b[i];
    return r;
}
template <typename T, int N>
vec<bool, N> greaterThan(const vec<T, N>& a, const vec<T, N>& b) {
    vec<bool, N> r;
    for (int i = 0; i < N; ++i) r[i] = a[i] > b[i];
    return r;
}
template <int N>
bool any(const vec<bool, N>& a) {
    for (int i = 0; i < N; ++i)
        if (a[i]) return true;
    return false;
}

template <typename T>
constexpr T pi() {
    return T(3.14159265358979323846264338327950288);
}
template <typename T>
constexpr T two_pi() {
    return T(6.28318530717958647692528676655900576);
}
// glm multiplies by the constant rounded to the argument type
inline float radians(float deg) { return deg * static_cast<float>(0.01745329251994329576923690768489); }
inline float degrees(float rad) { return rad * static_cast<float>(57.295779513082320876798154814105); }

// IEEE binary16, round to nearest even (overflow to infinity, subnormals kept).
inline uint16_t half_from_float(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    const uint32_t sign = (u >> 16) & 0x8000u;
    const uint32_t ax = u & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); // rounds to >= 65520: infinity
    if (ax < 0x38800000u) {                                  // below the smallest normal half
        if (ax < 0x33000000u) return (uint16_t)sign;          // below half of the smallest subnormal
        const uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        const int shift = 126 - (int)(ax >> 23);              // 14 .. 24
        uint32_t h = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1);
        if (rem > halfway || (rem == halfway && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((ax >> 13) - (112u << 10));
    const uint32_t rem = ax & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}
inline uint32_t packHalf2x16(const vec2& v) {
    return (uint32_t)half_from_float(v.x) | ((uint32_t)half_from_float(v.y) << 16);
}

}  // namespace glm
