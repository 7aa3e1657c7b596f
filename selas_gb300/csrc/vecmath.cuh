// Small float3 helpers for device code.
#pragma once

#include <cuda_runtime.h>

namespace sel {

#define SEL_HD __host__ __device__ __forceinline__

SEL_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
SEL_HD float3 f3(float s) { return make_float3(s, s, s); }
SEL_HD float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
SEL_HD float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
SEL_HD float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
SEL_HD float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
SEL_HD float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
SEL_HD float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
SEL_HD float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
SEL_HD float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
SEL_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SEL_HD float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
SEL_HD float length(float3 a) { return sqrtf(dot(a, a)); }
// v * (1 / |v|), the way the reference's Normalize scales (FloatFuncs.h:401-407)
SEL_HD float3 normalize(float3 a) { return a * (1.0f / length(a)); }
SEL_HD float saturate(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }
SEL_HD float clampf(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }
SEL_HD float lerpf(float a, float b, float t) { return (1.0f - t) * a + t * b; }
SEL_HD float3 lerp3(float3 a, float3 b, float t) { return (1.0f - t) * a + t * b; }
SEL_HD float sqr(float x) { return x * x; }
SEL_HD float3 sqrt3(float3 a) { return f3(sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)); }
SEL_HD float3 pow3(float3 a, float e) { return f3(powf(a.x, e), powf(a.y, e), powf(a.z, e)); }
SEL_HD float max3(float3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
SEL_HD float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }

constexpr float kPi = 3.141592653589793f;
constexpr float kTwoPi = kPi * 2.0f;
constexpr float kInvPi = 1.0f / kPi;
constexpr float kInv4Pi = 1.0f / (4.0f * kPi);

}  // namespace sel
