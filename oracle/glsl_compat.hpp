// glsl_compat.hpp -- just enough of GLSL 4.50 for the reference's shader
// functions to compile as C++20 (TEST INFRASTRUCTURE: used only to build
// oracle/_ref, the reference's own traversal code run on the CPU).
//
// Semantics follow the GLSL spec where it is defined: component-wise IEEE
// single-precision arithmetic (built with -ffp-contract=off), float -> int
// conversion truncating toward zero, mat4 * vec4 with the matrix read
// column-major.  Where GLSL leaves a result undefined, the choices are the ones
// a GPU makes and the CPU restatement in vt_oracle.c also makes:
//   - float -> uint conversion saturates negative values to 0;
//   - normalize(v) = v / sqrt(dot(v, v)), with correctly rounded division.
#pragma once

#include <math.h>
#include <stddef.h>
#include <stdint.h>

typedef uint32_t uint;

struct bvec3 {
    bool x, y, z;
};

struct ivec3;
struct uvec3;

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
};

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(const ivec2& v) : x((float)v.x), y((float)v.y) {}
};

struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(const ivec3& v);
    explicit vec3(const uvec3& v);
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec2& v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    vec3 xyz() const { return vec3(x, y, z); }
};

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    explicit ivec3(int s) : x(s), y(s), z(s) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
    explicit ivec3(const uvec3& v);
    int& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline uint f2u(float f) { return f <= 0.0f ? 0u : (uint)f; }

struct uvec3 {
    uint x, y, z;
    uvec3() : x(0), y(0), z(0) {}
    explicit uvec3(const ivec3& v) : x((uint)v.x), y((uint)v.y), z((uint)v.z) {}
    explicit uvec3(const vec3& v) : x(f2u(v.x)), y(f2u(v.y)), z(f2u(v.z)) {}
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};

inline vec3::vec3(const ivec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
inline vec3::vec3(const uvec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
inline ivec3::ivec3(const uvec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}

// column-major 4x4: m[4*col + row]
struct mat4 {
    float m[16];
};

inline vec4 operator*(const mat4& a, const vec4& v) {
    float r[4];
    for (int i = 0; i < 4; ++i)
        r[i] = ((a.m[0 * 4 + i] * v.x + a.m[1 * 4 + i] * v.y) + a.m[2 * 4 + i] * v.z) + a.m[3 * 4 + i] * v.w;
    return vec4(r[0], r[1], r[2], r[3]);
}

// ---- vec2
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator-(const vec2& a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2& operator*=(vec2& a, float s) { a.x *= s; a.y *= s; return a; }

// ---- vec3 arithmetic
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(float s, const vec3& a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, const vec3& b) { a = a + b; return a; }
inline vec3& operator+=(vec3& a, const ivec3& b) { a = a + vec3(b); return a; }
// mixed int/float vector operands convert the int vector to float first
inline vec3 operator+(const ivec3& a, const vec3& b) { return vec3(a) + b; }
inline vec3 operator-(const ivec3& a, const vec3& b) { return vec3(a) - b; }
inline vec3 operator-(const vec3& a, const ivec3& b) { return a - vec3(b); }

// ---- ivec3 / uvec3 arithmetic
inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator-(const ivec3& a, const ivec3& b) { return ivec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline ivec3 operator+(int s, const ivec3& a) { return ivec3(s + a.x, s + a.y, s + a.z); }
inline ivec3 operator>>(const ivec3& a, int s) { return ivec3(a.x >> s, a.y >> s, a.z >> s); }
inline ivec3 operator<<(const ivec3& a, uint s) {
    return ivec3((int)((uint)a.x << s), (int)((uint)a.y << s), (int)((uint)a.z << s));
}
inline ivec3 operator%(const ivec3& a, int s) { return ivec3(a.x % s, a.y % s, a.z % s); }
inline ivec3 operator&(const ivec3& a, int s) { return ivec3(a.x & s, a.y & s, a.z & s); }
inline ivec3& operator+=(ivec3& a, const ivec3& b) { a = a + b; return a; }
inline ivec3& operator-=(ivec3& a, const ivec3& b) { a = a - b; return a; }
inline uvec3 operator+(const uvec3& a, const uvec3& b) { return uvec3(a.x + b.x, a.y + b.y, a.z + b.z); }

// ---- comparisons
inline bvec3 lessThan(const ivec3& a, const ivec3& b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec3 greaterThanEqual(const ivec3& a, const ivec3& b) { return bvec3{a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bvec3 lessThan(const vec3& a, const vec3& b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bool any(const bvec3& b) { return b.x || b.y || b.z; }

// ---- built-in functions
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline float max(float a, int b) { return max(a, (float)b); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float clamp(float x, float a, float b) { return min(max(x, a), b); }
inline float sgn1(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline vec3 sign(const vec3& v) { return vec3(sgn1(v.x), sgn1(v.y), sgn1(v.z)); }
inline vec3 fract(const vec3& v) { return vec3(v.x - floorf(v.x), v.y - floorf(v.y), v.z - floorf(v.z)); }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec3& a) { return sqrtf(dot(a, a)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec3 normalize(const vec3& a) { return a / length(a); }
inline vec4 normalize(const vec4& a) {
    const float l = sqrtf(((a.x * a.x + a.y * a.y) + a.z * a.z) + a.w * a.w);
    return vec4(a.x / l, a.y / l, a.z / l, a.w / l);
}
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// pow, tan and sqrt on floats are the single-precision overloads <math.h>
// provides in C++ (powf, tanf, sqrtf)

// ---- RGBA8 images
inline uint packUnorm4x8(const vec4& v) {
    auto q = [](float f) { return (uint)(int)rintf(clamp(f, 0.0f, 1.0f) * 255.0f); };
    return q(v.x) | (q(v.y) << 8) | (q(v.z) << 16) | (q(v.w) << 24);
}
inline vec4 unpackUnorm4x8(uint p) {
    return vec4((float)(p & 255u) / 255.0f, (float)((p >> 8) & 255u) / 255.0f, (float)((p >> 16) & 255u) / 255.0f,
                (float)((p >> 24) & 255u) / 255.0f);
}

// a read-only RGBA8 3D image (the reference's 256^3 model atlas)
struct image3D {
    const uint* texels = nullptr;  // x + 256 * (y + 256 * z)
};
inline vec4 imageLoad(const image3D& img, const ivec3& p) {
    if (!img.texels || p.x < 0 || p.y < 0 || p.z < 0 || p.x > 255 || p.y > 255 || p.z > 255) return vec4(0.0f);
    return unpackUnorm4x8(img.texels[(size_t)p.x + 256u * ((size_t)p.y + 256u * (size_t)p.z)]);
}
