// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// A minimal GLSL vocabulary in C++ so that the reference's traversal shaders
// (Shaders/Intersectors/Include/TraverseBVHStack.glsl and TraverseBVHStackless.glsl) compile as C++
// (oracle/Makefile pipes their traversal functions after this header; see ref_glsl_harness.cpp).
// The semantics are those the GLSL 4.50 specification gives, evaluated in IEEE binary32 without
// contraction (the recipe passes -ffp-contract=off):
//  * vector arithmetic is component-wise, one rounding per operation;
//  * min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x (spec 8.3), component-wise for vectors;
//  * dot(a, b) = (a.x b.x + a.y b.y) + a.z b.z, cross as in spec 8.5;
//  * mat4 * vec4 sums the columns left to right, ((c0 x + c1 y) + c2 z) + c3 w: the specification
//    leaves the order to the implementation, and this is the order the engine and the CPU
//    restatement define;
//  * floatBitsToInt / intBitsToFloat / floatBitsToUint / uintBitsToFloat reinterpret bits;
//  * packSnorm2x16 rounds half to even and packs NaN as 0, pow(x, 2.0) is x * x (both left open).
// `.xyz` / `.xy` are rewritten to `.xyz()` / `.xy()` by the recipe; `in` becomes empty and
// `out T` / `inout T` become `T&`.
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace glsl {

struct vec4;
struct vec2;
struct ivec3;
typedef uint32_t uint;

struct vec3 {
    float x, y, z;
    vec3() = default;
    vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& v, float c);
    explicit vec3(const vec4& v);
    explicit vec3(const ivec3& v);
    vec3 xyz() const { return *this; }
    vec2 xz() const;
};

struct vec4 {
    float x, y, z, w;
    vec4() = default;
    vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(float a, const vec3& v) : x(a), y(v.x), z(v.y), w(v.z) {}
    vec3 xyz() const { return vec3(x, y, z); }
};

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct vec2 {
    float x, y;
    vec2() = default;
    vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2 xy() const { return *this; }
};

inline vec3::vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
inline vec2 vec3::xz() const { return {x, z}; }

// int(float) truncates toward zero (GLSL 4.50 5.4.1).
struct uvec3 {
    uint32_t x, y, z;
    uvec3 xyz() const { return *this; }
};
struct ivec3 {
    int x, y, z;
    ivec3() = default;
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x(int(v.x)), y(int(v.y)), z(int(v.z)) {}
    explicit ivec3(const uvec3& v) : x(int(v.x)), y(int(v.y)), z(int(v.z)) {}
};
inline vec3::vec3(const ivec3& v) : x(float(v.x)), y(float(v.y)), z(float(v.z)) {}
struct ivec2 {
    int x, y;
    ivec2() = default;
    ivec2(int s) : x(s), y(s) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2& v) : x(int(v.x)), y(int(v.y)) {}
};

struct uvec2 {
    uint32_t x, y;
};

struct uvec4 {
    uint32_t x, y, z, w;
    uvec2 xy() const { return {x, y}; }
};

struct mat4 {
    vec4 c[4];  // columns
};

inline vec2 operator+(vec2 a, vec2 b) { return {a.x + b.x, a.y + b.y}; }
inline vec2 operator*(vec2 a, float s) { return {a.x * s, a.y * s}; }
inline vec2 operator*(vec2 a, vec2 b) { return {a.x * b.x, a.y * b.y}; }
inline vec3 operator+(vec3 a, vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(vec3 a, vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(vec3 a, vec3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator/(vec3 a, vec3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline vec3 operator*(vec3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator*(float s, vec3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline vec3 operator/(float s, vec3 a) { return {s / a.x, s / a.y, s / a.z}; }
inline vec3 operator/(vec3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline vec3 operator-(vec3 a) { return {-a.x, -a.y, -a.z}; }
inline vec3& operator-=(vec3& a, vec3 b) { return a = a - b; }
inline vec3& operator+=(vec3& a, vec3 b) { return a = a + b; }
inline vec3& operator*=(vec3& a, vec3 b) { return a = a * b; }
inline vec3& operator/=(vec3& a, float s) { return a = a / s; }
inline vec3 operator+(vec3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline bool operator==(vec3 a, vec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline vec2 operator*(float s, vec2 a) { return {s * a.x, s * a.y}; }
inline vec2 operator+(vec2 a, float s) { return {a.x + s, a.y + s}; }

inline vec4 operator*(const mat4& m, vec4 v) {
    vec4 r;
    r.x = ((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z) + m.c[3].x * v.w;
    r.y = ((m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z) + m.c[3].y * v.w;
    r.z = ((m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z) + m.c[3].z * v.w;
    r.w = ((m.c[0].w * v.x + m.c[1].w * v.y) + m.c[2].w * v.z) + m.c[3].w * v.w;
    return r;
}

inline float abs(float x) { return std::fabs(x); }
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline vec3 min(vec3 a, vec3 b) { return {min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)}; }
inline vec3 max(vec3 a, vec3 b) { return {max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)}; }
inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// sqrt, cos, sin: the C library's (GLSL leaves their precision to the implementation).
inline float sqrt(float x) { return std::sqrt(x); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
inline vec3 normalize(vec3 v) { return v / sqrt(dot(v, v)); }
inline vec3 reflect(vec3 i, vec3 n) { return i - 2.0f * dot(n, i) * n; }
inline vec3 max(vec3 a, float s) { return {max(a.x, s), max(a.y, s), max(a.z, s)}; }
inline vec3 abs(vec3 v) { return {abs(v.x), abs(v.y), abs(v.z)}; }
inline vec3 floor(vec3 v) { return {std::floor(v.x), std::floor(v.y), std::floor(v.z)}; }
inline vec3 ceil(vec3 v) { return {std::ceil(v.x), std::ceil(v.y), std::ceil(v.z)}; }
inline float length(vec3 v) { return std::sqrt(dot(v, v)); }
inline float acos(float x) { return std::acos(x); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec2 clamp(vec2 v, float lo, float hi) { return {clamp(v.x, lo, hi), clamp(v.y, lo, hi)}; }
inline vec3 clamp(vec3 v, float lo, float hi) { return {clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)}; }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec2 mix(vec2 x, vec2 y, float a) { return {mix(x.x, y.x, a), mix(x.y, y.y, a)}; }
inline vec3 mix(vec3 x, vec3 y, float a) { return {mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a)}; }
// pow: the C library's, except pow(x, 2.0) = x * x (the correctly rounded square; GLSL leaves
// pow's precision to the implementation).
inline float pow(float x, float y) { return y == 2.0f ? x * x : std::pow(x, y); }
inline vec3 pow(vec3 x, vec3 y) { return {pow(x.x, y.x), pow(x.y, y.y), pow(x.z, y.z)}; }
inline bool isnan(float x) { return std::isnan(x); }
inline bool isinf(float x) { return std::isinf(x); }
// unpackHalf2x16: binary16 halves (low half first) converted exactly.
inline float half_to_float(uint32_t h) {
    const uint32_t s = (h >> 15) & 1u, e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
    float f;
    if (e == 0) {
        f = std::ldexp(static_cast<float>(m), -24);
    } else if (e == 31) {
        uint32_t bits = 0x7F800000u | (m << 13);
        std::memcpy(&f, &bits, 4);
    } else {
        f = std::ldexp(static_cast<float>(m | 0x400u), static_cast<int>(e) - 25);
    }
    return s ? -f : f;
}
inline vec2 unpackHalf2x16(uint32_t v) { return {half_to_float(v & 0xFFFFu), half_to_float(v >> 16)}; }
// packSnorm2x16 / unpackSnorm2x16 (GLSL 4.50 8.4): round(clamp(c, -1, 1) * 32767) with rounding
// half to even and NaN packed as 0 (both left open by the specification); clamp(f / 32767, -1, 1).
inline uint32_t snorm16(float c) {
    const float s = clamp(c, -1.0f, 1.0f) * 32767.0f;
    if (s != s) return 0u;
    return uint32_t(uint16_t(int16_t(std::nearbyint(s))));
}
inline uint32_t packSnorm2x16(vec2 v) { return snorm16(v.x) | (snorm16(v.y) << 16); }
inline float unsnorm16(uint32_t h) { return clamp(float(int16_t(uint16_t(h & 0xFFFFu))) / 32767.0f, -1.0f, 1.0f); }
inline vec2 unpackSnorm2x16(uint32_t p) { return {unsnorm16(p), unsnorm16(p >> 16)}; }
inline uint32_t floatBitsToUint(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float uintBitsToFloat(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline int floatBitsToInt(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}
inline float intBitsToFloat(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

}  // namespace glsl
