// metal_shim.h -- the few Metal Shading Language types and functions that the reference's
// packed-site decoder and packed render weights use (backends/metal/shaders/
// sad_common.metal: the declarations up to decodePackedSite, voronoi_dmix2,
// computePackedWeights), as plain C++, so that their source compiles on the host as the
// oracle's reference for the 16-byte serving format.  Test infrastructure only.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

// address-space and argument qualifiers carry no meaning on the host
#define constant
#define thread
#define device

typedef uint32_t uint;
typedef uint16_t ushort;
typedef _Float16 half;

struct float2 {
    float x, y;
    float2() : x(0), y(0) {}
    float2(float a, float b) : x(a), y(b) {}
};
struct float3 {
    float x, y, z;
    float3() : x(0), y(0), z(0) {}
    explicit float3(float a) : x(a), y(a), z(a) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
    float3& operator+=(const float3& o) {
        x += o.x;
        y += o.y;
        z += o.z;
        return *this;
    }
};
inline float2 operator-(const float2& a, const float2& b) { return float2(a.x - b.x, a.y - b.y); }
inline float3 operator*(float s, const float3& v) { return float3(s * v.x, s * v.y, s * v.z); }
inline float dot(const float2& a, const float2& b) { return a.x * b.x + a.y * b.y; }
struct uint4 {
    uint x, y, z, w;
};
struct half4 {
    half x, y, z, w;
};

// Metal's max/min of floats return the non-NaN operand, as fmax/fmin do
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float cos(float a) { return std::cos(a); }
inline float sin(float a) { return std::sin(a); }
inline float exp(float a) { return std::exp(a); }
inline float sqrt(float a) { return std::sqrt(a); }

template <class T, class U>
inline T as_type(U v) {
    static_assert(sizeof(T) == sizeof(U), "as_type: sizes differ");
    T t;
    std::memcpy(&t, &v, sizeof(T));
    return t;
}
