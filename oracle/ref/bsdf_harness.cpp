// ORACLE harness (test infrastructure only): links the reference's own BSDF sources, compiled where they
// lie in the reference checkout, and exposes them to the fixture generator through a C interface.
//
//   * EvaluateBsdf / SampleBsdfFunction: Source/Core/Shading/SurfaceScattering.cpp:18-60 (reference code,
//     not restated here);
//   * CSampler (Source/Core/MathLib/Sampler.h:14-29) is supplied by this file instead of Sampler.cpp so the
//     uniforms each call consumes are prescribed by the caller rather than drawn from MT19937;
//   * GeometricNormal (Source/Core/Shading/SurfaceParameters.cpp:393-396) is supplied by this file because
//     SurfaceParameters.cpp pulls in Embree and Ptex; it returns the normal row of the tangent frame.
//
// Surface records are 32 floats: t[3] n[3] b[3] baseColor[3] transmittanceColor[3] sheen sheenTint
// clearcoat clearcoatGloss metallic specTrans diffTrans flatness anisotropic relativeIOR specularTint
// roughness scatterDistance ior shader(as float) pad pad.
//
// ref_cmj exposes CorrelatedMultiJitter (Source/Core/MathLib/CorrelatedMultiJitter.cpp:53-62), reference code.

#include "MathLib/CorrelatedMultiJitter.h"
#include "MathLib/FloatFuncs.h"
#include "MathLib/Sampler.h"
#include "Shading/Scattering.h"
#include "Shading/SurfaceParameters.h"
#include "Shading/SurfaceScattering.h"

namespace {
thread_local const float* g_uniforms = nullptr;
thread_local int g_count = 0;
thread_local int g_used = 0;
}  // namespace

namespace Selas {
void CSampler::Initialize(uint32) {}
void CSampler::Shutdown() {}
void CSampler::Reseed(uint32) {}
float CSampler::UniformFloat() { return g_used < g_count ? g_uniforms[g_used++] : 0.5f; }
uint32 CSampler::UniformUInt32() { return 0; }
float3 CSampler::UniformSphere() { return float3(0.0f, 1.0f, 0.0f); }
float CSampler::UniformSpherePdf() { return 0.0f; }

float3 GeometricNormal(const SurfaceParameters& s) {
    return float3(s.worldToTangent.r0.y, s.worldToTangent.r1.y, s.worldToTangent.r2.y);
}
}  // namespace Selas

using namespace Selas;

static SurfaceParameters to_surface(const float* r) {
    SurfaceParameters s;
    memset(&s, 0, sizeof(s));
    const float3 t(r[0], r[1], r[2]), n(r[3], r[4], r[5]), b(r[6], r[7], r[8]);
    s.worldToTangent = MatrixTranspose(MakeFloat3x3(t, n, b));
    s.baseColor = float3(r[9], r[10], r[11]);
    s.transmittanceColor = float3(r[12], r[13], r[14]);
    s.sheen = r[15];
    s.sheenTint = r[16];
    s.clearcoat = r[17];
    s.clearcoatGloss = r[18];
    s.metallic = r[19];
    s.specTrans = r[20];
    s.diffTrans = r[21];
    s.flatness = r[22];
    s.anisotropic = r[23];
    s.relativeIOR = r[24];
    s.specularTint = r[25];
    s.roughness = r[26];
    s.scatterDistance = r[27];
    s.ior = r[28];
    s.shader = ShaderType(int(r[29]));
    return s;
}

extern "C" {

// out: f.x f.y f.z forwardPdfW reversePdfW per tuple
void ref_bsdf_evaluate(const float* surf, const float* wo, const float* wi, int n, float* out) {
    for (int i = 0; i < n; ++i) {
        const SurfaceParameters s = to_surface(surf + 32 * i);
        float fwd = 0.0f, rev = 0.0f;
        const float3 v(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        const float3 l(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        const float3 f = EvaluateBsdf(s, v, l, fwd, rev);
        out[5 * i + 0] = f.x;
        out[5 * i + 1] = f.y;
        out[5 * i + 2] = f.z;
        out[5 * i + 3] = fwd;
        out[5 * i + 4] = rev;
    }
}

// u: 4 uniforms per tuple (consumed in order); out (16 per tuple): success flags reflectance[3] wi[3]
// forwardPdfW reversePdfW mediumPhase extinction[3] uniformsUsed pad
void ref_bsdf_sample(const float* surf, const float* wo, const float* u, int n, float* out) {
    for (int i = 0; i < n; ++i) {
        const SurfaceParameters s = to_surface(surf + 32 * i);
        const float3 v(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        g_uniforms = u + 4 * i;
        g_count = 4;
        g_used = 0;
        CSampler sampler;
        BsdfSample bs;
        bs.flags = 0;
        const bool ok = SampleBsdfFunction(&sampler, s, v, bs);
        float* o = out + 16 * i;
        o[0] = ok ? 1.0f : 0.0f;
        o[1] = float(bs.flags);
        o[2] = bs.reflectance.x;
        o[3] = bs.reflectance.y;
        o[4] = bs.reflectance.z;
        o[5] = bs.wi.x;
        o[6] = bs.wi.y;
        o[7] = bs.wi.z;
        o[8] = bs.forwardPdfW;
        o[9] = bs.reversePdfW;
        o[10] = float(bs.medium.phaseFunction);
        o[11] = bs.medium.extinction.x;
        o[12] = bs.medium.extinction.y;
        o[13] = bs.medium.extinction.z;
        o[14] = float(g_used);
        o[15] = 0.0f;
    }
}

// xy: n points s = 0..n-1 of CorrelatedMultiJitter(s, m, m, p)
void ref_cmj(int m, int p, int n, float* xy) {
    for (int s = 0; s < n; ++s) {
        const float2 r = CorrelatedMultiJitter(s, m, m, p);
        xy[2 * s] = r.x;
        xy[2 * s + 1] = r.y;
    }
}

}  // extern "C"
