// ref_shim.hpp -- the GLSL types and built-ins the reference's LBM compute
// shaders use, as plain C++, so that oracle/build_ref.py can compile those
// shader sources (mechanically lowered) on the host.  TEST INFRASTRUCTURE:
// only the reference-built checker under oracle/_ref/ includes it.
//
// Semantics chosen where GLSL leaves them to the implementation:
//  * float arithmetic is IEEE binary32, one rounding per operation (the
//    translation units are compiled with -ffp-contract=off);
//  * pow(x, 2) is x*x and pow(x, 4) is (x*x)*(x*x) (GLSL leaves pow(x<0, y)
//    undefined and the shaders square signed values);
//  * normalize(v) = v / length(v), length(v) = sqrt(dot(v, v));
//  * storage buffers behave like GL robust buffer access: out-of-range
//    reads return 0, out-of-range writes are dropped;
//  * r16f image stores round to IEEE half, nearest-even;
//  * exp(x) is the project's single-precision exponential (Cody-Waite
//    reduction, degree-7 Taylor polynomial, exact 2^k scaling; within 1.5 ulp
//    of the exact value, tested against libm): GLSL only bounds exp's error
//    (3 + 2|x| ulp) and the kernels under test evaluate it this way, so the
//    checker's remaining freedom is pinned to the same choice.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <array>
#include <vector>

namespace glsl {

typedef unsigned int uint;

struct ivec2;
struct ivec3;
struct uvec3;

struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const ivec3& v);
    vec3 xyz() const { return *this; }
};
struct vec4 {
    float x = 0, y = 0, z = 0, w = 0;
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec3 xyz() const { return vec3(x, y, z); }
};
struct vec2f;
struct ivec2 {
    int x = 0, y = 0;
    ivec2() = default;
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2f& v);
};
struct ivec3 {
    int x = 0, y = 0, z = 0;
    ivec3() = default;
    explicit ivec3(int s) : x(s), y(s), z(s) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
    explicit ivec3(const uvec3& v);
};
struct uvec3 {
    uint x = 0, y = 0, z = 0;
    uvec3() = default;
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};
inline vec3::vec3(const ivec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
inline ivec3::ivec3(const uvec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3& operator+=(vec3& a, vec3 b) { a = a + b; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }
inline ivec3 operator+(ivec3 a, ivec3 b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator-(ivec3 a, ivec3 b) { return ivec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline ivec3 operator*(ivec3 a, ivec3 b) { return ivec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline ivec3 operator%(ivec3 a, ivec3 b) { return ivec3(a.x % b.x, a.y % b.y, a.z % b.z); }
inline bool operator==(vec3 a, vec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(vec3 v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(vec3 v) { return v / length(v); }
inline float pow(float x, float y) {
    if (y == 2.0f) return x * x;
    if (y == 4.0f) return (x * x) * (x * x);
    return std::pow(x, y);
}
inline float exp(float x) {
    const float L2E = 0x1.715476p+0f, LN2_HI = 0x1.62e4p-1f, LN2_LO = 0x1.7f7d1cp-20f;
    const float kf = std::rint(x * L2E);
    const float r = (x - kf * LN2_HI) - kf * LN2_LO;
    float q = 0x1.a01a02p-13f;
    q = q * r + 0x1.6c16c2p-10f;
    q = q * r + 0x1.111112p-7f;
    q = q * r + 0x1.555556p-5f;
    q = q * r + 0x1.555556p-3f;
    q = q * r + 0x1p-1f;
    q = q * r + 1.0f;
    q = q * r + 1.0f;
    const uint32_t sb = (uint32_t)((int)kf + 127) << 23;
    float sc;
    std::memcpy(&sc, &sb, 4);
    return q * sc;
}
inline float sqrt(float x) { return std::sqrt(x); }
inline float mod(float a, float b) { return a - b * std::floor(a / b); }
inline vec3 mod(vec3 a, vec3 b) { return vec3(mod(a.x, b.x), mod(a.y, b.y), mod(a.z, b.z)); }
// the ivec2 overloads of the shaders' positive_modulo (never called by the 3D/2D paths here)
struct vec2f { float x, y; };
inline vec2f mod(ivec2 a, ivec2 b) { return {mod((float)a.x, (float)b.x), mod((float)a.y, (float)b.y)}; }
inline vec2f mod(vec2f a, ivec2 b) { return {mod(a.x, (float)b.x), mod(a.y, (float)b.y)}; }
inline vec2f operator+(vec2f a, ivec2 b) { return {a.x + (float)b.x, a.y + (float)b.y}; }
inline ivec2::ivec2(const vec2f& v) : x((int)v.x), y((int)v.y) {}
inline int max(int a, int b) { return a > b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
struct bvec3 { bool x, y, z; };
inline bvec3 greaterThanEqual(uvec3 a, ivec3 b) { return {(int)a.x >= b.x, (int)a.y >= b.y, (int)a.z >= b.z}; }
inline bvec3 greaterThanEqual(uvec3 a, uvec3 b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bool any(bvec3 b) { return b.x || b.y || b.z; }

// storage buffer with GL robust-access semantics
template <class T>
struct ssbo {
    T* p = nullptr;
    size_t n = 0;
    T sink{};
    T& operator[](size_t i) {
        if (i >= n) { sink = T{}; return sink; }
        return p[i];
    }
    T& operator[](int i) { return (*this)[(size_t)(unsigned)i]; }
    T& operator[](uint i) { return (*this)[(size_t)i]; }
};

// image3D with a single-channel (r16f / r32f) or four-channel (rgba32f) float format
struct image3D {
    std::vector<float>* data = nullptr;
    int sx = 0, sy = 0, sz = 0, channels = 1;
    bool half = false;
    vec4 load(ivec3 c) const {
        if (!data || c.x < 0 || c.y < 0 || c.z < 0 || c.x >= sx || c.y >= sy || c.z >= sz) return vec4(0.f);
        const size_t k = (((size_t)c.z * sy + c.y) * sx + c.x) * channels;
        if (channels == 1) return vec4((*data)[k], 0.f, 0.f, 1.f);
        return vec4((*data)[k], (*data)[k + 1], (*data)[k + 2], (*data)[k + 3]);
    }
    void store(ivec3 c, vec4 v) {
        if (!data || c.x < 0 || c.y < 0 || c.z < 0 || c.x >= sx || c.y >= sy || c.z >= sz) return;
        const size_t k = (((size_t)c.z * sy + c.y) * sx + c.x) * channels;
        if (channels == 1) { (*data)[k] = half ? round_half(v.x) : v.x; return; }
        (*data)[k] = v.x; (*data)[k + 1] = v.y; (*data)[k + 2] = v.z; (*data)[k + 3] = v.w;
    }
    static float round_half(float f);
};
typedef image3D image2D;
inline vec4 imageLoad(const image3D& im, ivec3 c) { return im.load(c); }
inline void imageStore(image3D& im, ivec3 c, vec4 v) { im.store(c, v); }

// IEEE binary32 -> binary16 (nearest even) -> binary32
inline float image3D::round_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = x & 0x80000000u;
    uint32_t mag = x & 0x7fffffffu;
    float out;
    if (mag >= 0x477ff000u) {  // overflow (or NaN/inf)
        uint32_t r = sign | (mag > 0x7f800000u ? 0x7fc00000u : 0x7f800000u);
        std::memcpy(&out, &r, 4);
        return out;
    }
    if (mag < 0x38800000u) {  // half subnormal range: quantum 2^-24
        const double q = std::nearbyint((double)std::fabs(f) * 16777216.0) / 16777216.0;  // ties to even
        out = (float)q;
        return sign ? -out : out;
    }
    const uint32_t rem = mag & 0x1fffu;
    mag &= ~0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (mag & 0x2000u))) mag += 0x2000u;
    uint32_t r = sign | mag;
    std::memcpy(&out, &r, 4);
    return out;
}

}  // namespace glsl
