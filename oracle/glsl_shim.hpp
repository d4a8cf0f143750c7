// glsl_shim.hpp - just enough GLSL 4.60 compute-shader semantics, in C++, to compile the reference's
// own shader files on the CPU (test infrastructure; see oracle/build_ref.py).
//
// Vector types follow the GLSL spec: component-wise arithmetic in float, swizzles .xyz/.xy/.zw (the
// build step rewrites them to calls: writable proxies on lvalues, values on rvalues), mix() as
// x * (1 - a) + y * a, step(), exp()/sin()/cos() per component, textures as flat RGBA arrays.
// exp() is emlab_expf, or libm expf when ref_driver.cpp sets g_libm_exp (the tolerance variant).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "../em_lab_gb300/csrc/emlab_math.h"

namespace glsl {

extern bool g_libm_exp;

typedef unsigned uint;

struct vec2;
struct vec3;
struct vec4;
struct ivec2;
struct ivec3;

struct vec2 {
    float x = 0, y = 0;
    vec2() = default;
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    float& operator[](int i) & { return i == 0 ? x : y; }
    float operator[](int i) const& { return i == 0 ? x : y; }
};

struct Swz2 {
    float *a, *b;
    operator vec2() const { return vec2(*a, *b); }
    Swz2& operator=(const vec2& v) { *a = v.x, *b = v.y; return *this; }
    Swz2& operator+=(const vec2& v) { *a = *a + v.x, *b = *b + v.y; return *this; }
};

struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(const ivec3& v);
    float& operator[](int i) & { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const& { return i == 0 ? x : (i == 1 ? y : z); }
};

struct Swz3 {
    float *a, *b, *c;
    operator vec3() const { return vec3(*a, *b, *c); }
    Swz3& operator=(const vec3& v) { *a = v.x, *b = v.y, *c = v.z; return *this; }
    Swz3& operator+=(const vec3& v) { *a = *a + v.x, *b = *b + v.y, *c = *c + v.z; return *this; }
    Swz3& operator-=(const vec3& v) { *a = *a - v.x, *b = *b - v.y, *c = *c - v.z; return *this; }
    Swz3& operator*=(const vec3& v) { *a = *a * v.x, *b = *b * v.y, *c = *c * v.z; return *this; }
};

struct vec4 {
    float x = 0, y = 0, z = 0, w = 0;
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec2& v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    float& operator[](int i) & { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const& { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    Swz3 xyz() & { return Swz3{&x, &y, &z}; }
    vec3 xyz() const& { return vec3(x, y, z); }
    vec3 xyz() && { return vec3(x, y, z); }
    Swz3 rgb() & { return Swz3{&x, &y, &z}; }
    vec3 rgb() const& { return vec3(x, y, z); }
    vec3 rgb() && { return vec3(x, y, z); }
    Swz2 xy() & { return Swz2{&x, &y}; }
    vec2 xy() const& { return vec2(x, y); }
    vec2 xy() && { return vec2(x, y); }
    Swz2 zw() & { return Swz2{&z, &w}; }
    vec2 zw() const& { return vec2(z, w); }
    vec2 zw() && { return vec2(z, w); }
};

struct bvec3 {
    bool x, y, z;
};

struct ivec2 {
    int x = 0, y = 0;
    ivec2() = default;
    explicit ivec2(int s) : x(s), y(s) {}
    ivec2(int a, int b) : x(a), y(b) {}
    int& operator[](int i) & { return i == 0 ? x : y; }
    int operator[](int i) const& { return i == 0 ? x : y; }
};

struct uvec3 {
    uint x = 0, y = 0, z = 0;
    ivec2 xy() const { return ivec2((int)x, (int)y); }  // used only as ivec2(gl_GlobalInvocationID.xy)
};

struct ivec3 {
    int x = 0, y = 0, z = 0;
    ivec3() = default;
    explicit ivec3(int s) : x(s), y(s), z(s) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const uvec3& u) : x((int)u.x), y((int)u.y), z((int)u.z) {}
    int& operator[](int i) & { return i == 0 ? x : (i == 1 ? y : z); }
    int operator[](int i) const& { return i == 0 ? x : (i == 1 ? y : z); }
};

struct ivec4 {
    int x = 0, y = 0, z = 0, w = 0;
    ivec4() = default;
    ivec4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
    ivec3 xyz() const { return ivec3(x, y, z); }
};

struct uvec4 {
    uint x = 0, y = 0, z = 0, w = 0;
};

inline vec3::vec3(const ivec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}

// ---- arithmetic ---------------------------------------------------------------------------------
#define GLSL_V3_OP(OP)                                                                                       \
    inline vec3 operator OP(const vec3& a, const vec3& b) { return vec3(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
    inline vec3 operator OP(const vec3& a, float s) { return vec3(a.x OP s, a.y OP s, a.z OP s); }            \
    inline vec3 operator OP(float s, const vec3& a) { return vec3(s OP a.x, s OP a.y, s OP a.z); }
GLSL_V3_OP(+)
GLSL_V3_OP(-)
GLSL_V3_OP(*)
GLSL_V3_OP(/)
#undef GLSL_V3_OP
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, const vec3& b) { a = a + b; return a; }
inline vec3& operator-=(vec3& a, const vec3& b) { a = a - b; return a; }
inline vec3& operator*=(vec3& a, const vec3& b) { a = a * b; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }
inline vec3& operator+=(vec3& a, float s) { a = a + s; return a; }

#define GLSL_V4_OP(OP)                                                                                    \
    inline vec4 operator OP(const vec4& a, const vec4& b) {                                               \
        return vec4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w);                                      \
    }                                                                                                     \
    inline vec4 operator OP(float s, const vec4& a) { return vec4(s OP a.x, s OP a.y, s OP a.z, s OP a.w); } \
    inline vec4 operator OP(const vec4& a, float s) { return vec4(a.x OP s, a.y OP s, a.z OP s, a.w OP s); }
GLSL_V4_OP(+)
GLSL_V4_OP(-)
GLSL_V4_OP(*)
#undef GLSL_V4_OP
inline vec4& operator+=(vec4& a, const vec4& b) { a = a + b; return a; }

#define GLSL_V2_OP(OP)                                                                                     \
    inline vec2 operator OP(const vec2& a, const vec2& b) { return vec2(a.x OP b.x, a.y OP b.y); }          \
    inline vec2 operator OP(float s, const vec2& a) { return vec2(s OP a.x, s OP a.y); }                     \
    inline vec2 operator OP(const vec2& a, float s) { return vec2(a.x OP s, a.y OP s); }
GLSL_V2_OP(+)
GLSL_V2_OP(-)
GLSL_V2_OP(*)
#undef GLSL_V2_OP

inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator-(const ivec3& a, const ivec3& b) { return ivec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline ivec3 operator-(const ivec3& a, int s) { return ivec3(a.x - s, a.y - s, a.z - s); }
inline ivec3 operator+(const ivec3& a, int s) { return ivec3(a.x + s, a.y + s, a.z + s); }
inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }

// ---- built-in functions -------------------------------------------------------------------------
inline float glsl_exp(float x) { return g_libm_exp ? expf(x) : emlab_expf(x); }
inline float exp(float x) { return glsl_exp(x); }
inline vec3 exp(const vec3& v) { return vec3(glsl_exp(v.x), glsl_exp(v.y), glsl_exp(v.z)); }
inline float cos(float x) { return cosf(x); }
inline float sin(float x) { return sinf(x); }
inline float max(float a, float b) { return a < b ? b : a; }  // max(x, y): y if x < y
inline float min(float a, float b) { return b < a ? b : a; }  // min(x, y): y if y < x
inline int max(int a, int b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline float abs(float a) { return fabsf(a); }
inline vec3 abs(const vec3& a) { return vec3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
inline int clamp(int v, int lo, int hi) { return min(max(v, lo), hi); }
inline ivec3 clamp(const ivec3& v, const ivec3& lo, const ivec3& hi) {
    return ivec3(clamp(v.x, lo.x, hi.x), clamp(v.y, lo.y, hi.y), clamp(v.z, lo.z, hi.z));
}
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& x, const vec3& y) {
    return vec3(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline vec3 step(const vec3& e, const vec3& x) { return vec3(step(e.x, x.x), step(e.y, x.y), step(e.z, x.z)); }
inline vec3 mix(const vec3& x, const vec3& y, const vec3& a) { return x * (1.0f - a) + y * a; }
inline bvec3 lessThan(const ivec3& a, const ivec3& b) { return {a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec3 greaterThanEqual(const ivec3& a, const ivec3& b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bvec3 lessThan(const ivec2& a, const ivec2& b) { return {a.x < b.x, a.y < b.y, true}; }
inline bvec3 equal(const vec3& a, const vec3& b) { return {a.x == b.x, a.y == b.y, a.z == b.z}; }
inline bool any(const bvec3& b) { return b.x || b.y || b.z; }
inline bool all(const bvec3& b) { return b.x && b.y && b.z; }
inline vec2 unpackHalf2x16(uint v) {
    return vec2(emlab_half_to_float((uint16_t)(v & 0xffffu)), emlab_half_to_float((uint16_t)(v >> 16)));
}
// fragment-stage built-ins used by raymarch.frag
inline float clamp(float v, float lo, float hi) { return min(max(v, lo), hi); }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float length(const vec3& v) { return sqrtf(dot(v, v)); }
inline vec3 normalize(const vec3& v) {
    const float l = length(v);
    return vec3(v.x / l, v.y / l, v.z / l);
}
inline float fract(float x) { return x - floorf(x); }
inline float smoothstep(float e0, float e1, float x) {
    const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline float pow(float x, float y) { return powf(x, y); }
inline vec3 pow(const vec3& x, const vec3& y) { return vec3(powf(x.x, y.x), powf(x.y, y.y), powf(x.z, y.z)); }
// Workgroup barrier: ref_driver.cpp runs a workgroup's invocations as fibers and installs the hook
// that suspends the calling invocation until all of them have arrived.
extern thread_local void (*g_barrier_hook)();
inline void barrier() {
    if (g_barrier_hook) g_barrier_hook();
}
inline void memoryBarrierShared() {}

// ---- resources ----------------------------------------------------------------------------------
struct sampler3D {
    const float* data = nullptr;  // RGBA per texel
    ivec3 size;
};
struct usampler3D {
    const uint32_t* data = nullptr;  // 4 uints per texel
    ivec3 size;
};
struct image3D {
    float* data = nullptr;
    ivec3 size;
};
inline long long texel_index(const ivec3& s, const ivec3& p) { return ((long long)p.z * s.y + p.y) * s.x + p.x; }
inline vec4 texelFetch(const sampler3D& t, const ivec3& p, int) {
    const float* q = t.data + 4 * texel_index(t.size, p);
    return vec4(q[0], q[1], q[2], q[3]);
}
inline uvec4 texelFetch(const usampler3D& t, const ivec3& p, int) {
    const uint32_t* r = t.data + 4 * texel_index(t.size, p);
    return uvec4{r[0], r[1], r[2], r[3]};
}
inline vec4 imageLoad(const image3D& t, const ivec3& p) {
    const float* q = t.data + 4 * texel_index(t.size, p);
    return vec4(q[0], q[1], q[2], q[3]);
}
inline void imageStore(const image3D& t, const ivec3& p, const vec4& v) {
    float* q = t.data + 4 * texel_index(t.size, p);
    q[0] = v.x, q[1] = v.y, q[2] = v.z, q[3] = v.w;
}

// texture(sampler3D, uvw) with a linear filter and clamp-to-edge: the eight texels around
// uvw * size - 0.5, weights multiplied x, y, z, accumulated z-, y-, x-major.
inline vec4 texture(const sampler3D& t, const vec3& uvw) {
    const float px = uvw.x * (float)t.size.x - 0.5f, py = uvw.y * (float)t.size.y - 0.5f,
                pz = uvw.z * (float)t.size.z - 0.5f;
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const float ax = px - fx, ay = py - fy, az = pz - fz;
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    vec4 r(0.0f);
    for (int dz = 0; dz <= 1; ++dz)
        for (int dy = 0; dy <= 1; ++dy)
            for (int dx = 0; dx <= 1; ++dx) {
                const float w = (dx ? ax : 1.0f - ax) * (dy ? ay : 1.0f - ay) * (dz ? az : 1.0f - az);
                const ivec3 p(clamp(ix + dx, 0, t.size.x - 1), clamp(iy + dy, 0, t.size.y - 1),
                              clamp(iz + dz, 0, t.size.z - 1));
                r += w * texelFetch(t, p, 0);
            }
    return r;
}

struct mat4 {
    vec4 c[4];  // columns
};
inline vec4 operator*(const mat4& m, const vec4& v) {
    return vec4(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z + m.c[3].x * v.w,
                m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z + m.c[3].y * v.w,
                m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z + m.c[3].z * v.w,
                m.c[0].w * v.x + m.c[1].w * v.y + m.c[2].w * v.z + m.c[3].w * v.w);
}

// ---- invocation ids (per OpenMP thread) -----------------------------------------------------------
extern thread_local uvec3 gl_GlobalInvocationID;
extern thread_local uvec3 gl_WorkGroupID;
extern thread_local uint gl_LocalInvocationIndex;
extern thread_local uvec3 gl_NumWorkGroups;
extern thread_local vec4 gl_FragCoord;

}  // namespace glsl
