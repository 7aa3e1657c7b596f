// ORACLE - test infrastructure only.  Vector type and BSDF entry points shared by the oracle's BSDF
// restatement (oracle_bsdf.cpp) and its path tracers.
#pragma once

#include <cmath>
#include <cstdint>

namespace orc {

struct V3 {
    float x, y, z;
    V3() : x(0), y(0), z(0) {}
    explicit V3(float s) : x(s), y(s), z(s) {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
};
inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(V3 a, V3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 Cross(V3 a, V3 b) { return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline float Len(V3 a) { return std::sqrt(Dot(a, a)); }
inline V3 Norm(V3 a) { float il = 1.f / Len(a); return V3(a.x * il, a.y * il, a.z * il); }
inline V3 Sqrt(V3 a) { return V3(std::sqrt(a.x), std::sqrt(a.y), std::sqrt(a.z)); }

struct Surf {
    V3 t, n, b;
    V3 baseColor, transmittanceColor;
    float sheen, sheenTint, clearcoat, clearcoatGloss, metallic, specTrans, diffTrans, flatness;
    float anisotropic, relativeIOR, specularTint, roughness, scatterDistance, ior;
    int shader;
};

struct Sample {
    unsigned flags = 0;
    int phase = 0;
    V3 ext, refl, wi;
    float fwd = 0, rev = 0;
};

Surf surf_from_record(const float* r);
V3 bsdf_evaluate(const Surf& s, V3 v, V3 l, float& fwd, float& rev);
bool bsdf_sample(const Surf& s, V3 v, const float* u, int& used, Sample& o);

}  // namespace orc
