// Image-based light: importance sampling and lookups of a latitude-longitude image
// (Source/Core/SceneLib/ImageBasedLightResource.cpp:81-268, Source/Core/MathLib/Projection.cpp:109-145), used by
// the path tracer's misses and the deferred path tracer's background next-event estimation, and the environment
// emitter of VCM (ibl_env_*).
#pragma once

#include <cstdint>

#include "vecmath.cuh"

namespace sel {

// Device view of an image-based light (IblDensityFunctions + ImageBasedLightResourceData).
struct IblDev {
    const float* mdf;     // marginal CDF over rows, height entries (last = 1)
    const float* cdf;     // per-row conditional CDFs, width x height (each row's last = 1)
    const float4* light;  // width x height RGB (w unused)
    const float4* miss;   // miss_width x miss_height RGB
    uint32_t width, height, miss_width, miss_height;
    float rotation, exposure;
};

// SampleDistributionFunction (ImageBasedLightResource.cpp:81-103): the first entry >= r, and its density.
SEL_HD void ibl_search(const float* f, uint32_t count, float r, uint32_t& index, float& pdf) {
    int lo = 0, hi = int(count) - 1;
    index = count - 1;
    pdf = 0.0f;
    while (lo <= hi) {
        const int mid = (lo + hi) / 2;
        if (f[mid] >= r) {
            index = uint32_t(mid);
            pdf = mid > 0 ? f[mid] - f[mid - 1] : f[mid];
            hi = mid - 1;
        } else {
            lo = mid + 1;
        }
    }
}

// Texel (x, y) a direction looks up (SampleIbl / SampleIBlPdf / SampleIblMiss): theta = acos(y),
// phi = atan2(z, x) + pi + rotation wrapped to [0, 2 pi), truncated from (angle x size / span - 0.5).
// (wi.y is clamped to [-1, 1]: a unit vector's rounding can exceed it by an ulp, where acos has no value.)
SEL_HD void ibl_texel(float3 wi, float rotation, uint32_t width, uint32_t height, int& x, int& y, float& theta) {
    theta = acosf(fminf(fmaxf(wi.y, -1.0f), 1.0f));
    float phi = atan2f(wi.z, wi.x);
    phi = fmodf(phi + kPi + rotation, kTwoPi);
    x = int(phi * float(width) / kTwoPi - 0.5f);
    y = int(theta * float(height) / kPi - 0.5f);
    x = x < 0 ? 0 : (x > int(width) - 1 ? int(width) - 1 : x);
    y = y < 0 ? 0 : (y > int(height) - 1 ? int(height) - 1 : y);
}

SEL_HD float ibl_pdf_at(const IblDev& ibl, int x, int y, float theta) {
    const float* row = ibl.cdf + size_t(y) * ibl.width;
    const float mdf = y > 0 ? ibl.mdf[y] - ibl.mdf[y - 1] : ibl.mdf[y];
    const float cdf = x > 0 ? row[x] - row[x - 1] : row[x];
    const float inv_jacobian = (float(ibl.width) * float(ibl.height)) / kTwoPi;
    const float sin_theta = sinf(theta);
    return sin_theta > 0.0f ? mdf * cdf * inv_jacobian / sin_theta : 0.0f;
}

// SampleIBlPdf: solid-angle density of sampling direction wi.
SEL_HD float ibl_pdf(const IblDev& ibl, float3 wi) {
    int x, y;
    float theta;
    ibl_texel(wi, ibl.rotation, ibl.width, ibl.height, x, y, theta);
    return ibl_pdf_at(ibl, x, y, theta);
}

// SampleIbl(wi): the light image times the exposure (EvaluateBackground with an image).
SEL_HD float3 ibl_radiance(const IblDev& ibl, float3 wi) {
    int x, y;
    float theta;
    ibl_texel(wi, ibl.rotation, ibl.width, ibl.height, x, y, theta);
    const float4 c = ibl.light[size_t(y) * ibl.width + x];
    return ibl.exposure * f3(c.x, c.y, c.z);
}

// SampleIblMiss(wi): the miss image (EvaluateBackgroundMiss with an image).
SEL_HD float3 ibl_miss(const IblDev& ibl, float3 wi) {
    int x, y;
    float theta;
    ibl_texel(wi, ibl.rotation, ibl.miss_width, ibl.miss_height, x, y, theta);
    const float4 c = ibl.miss[size_t(y) * ibl.miss_width + x];
    return f3(c.x, c.y, c.z);
}

// Ibl + DirectIblLightSample (ImageBasedLightResource.cpp:119-155, AreaLighting.cpp:293-314): a direction from
// (r0, r1) by the marginal and conditional CDFs, its radiance and solid-angle density.
SEL_HD void ibl_sample(const IblDev& ibl, float r0, float r1, float3& dir, float3& radiance, float& pdf) {
    uint32_t x, y;
    float mdf, cdf;
    ibl_search(ibl.mdf, ibl.height, r0, y, mdf);
    ibl_search(ibl.cdf + size_t(y) * ibl.width, ibl.width, r1, x, cdf);
    const float widthf = float(ibl.width), heightf = float(ibl.height);
    const float theta = (float(y) + 0.5f) * kPi / heightf;
    const float phi = fmodf(((float(x) + 0.5f) * kTwoPi / widthf) + ibl.rotation, kTwoPi) - kPi;
    const float inv_jacobian = (widthf * heightf) / kTwoPi;
    const float sin_theta = sinf(theta);
    pdf = sin_theta > 0.0f ? mdf * cdf * inv_jacobian / sin_theta : 0.0f;
    dir = f3(sin_theta * cosf(phi), cosf(theta), sin_theta * sinf(phi));
    const float4 c = ibl.light[size_t(y) * ibl.width + x];
    radiance = ibl.exposure * f3(c.x, c.y, c.z);
}

// Environment emitter for VCM (the infinite light of the VCM technical report, sec. 5.1).  The reference samples
// texel centres with a density that integrates to pi (ibl_sample, kept by the path tracers for parity), which a
// multi-strategy estimator cannot weigh with.  Here a texel is drawn by the same CDFs and the direction jittered
// uniformly in (theta, phi) over the directions whose lookup returns that texel (ibl_texel truncates
// angle x size / span - 0.5: texel i of n covers [i + 0.5, i + 1.5) steps, the first from 0, the last up to n),
// so the solid-angle density of a direction is m c / (area x sin theta) of the texel its lookup returns.  The
// azimuth is wrapped into [0, 2 pi) (the lookup's fmod leaves it negative for a negative rotation).
SEL_HD void ibl_env_span(uint32_t i, uint32_t n, float& a, float& b) {
    a = i == 0 ? 0.0f : float(i) + 0.5f;
    b = i + 1 >= n ? float(n) : float(i) + 1.5f;
}

SEL_HD void ibl_env_texel(float3 wi, float rotation, uint32_t width, uint32_t height, int& x, int& y, float& theta) {
    theta = acosf(fminf(fmaxf(wi.y, -1.0f), 1.0f));
    float phi = atan2f(wi.z, wi.x);
    phi = fmodf(phi + kPi + rotation, kTwoPi);
    if (phi < 0.0f) phi += kTwoPi;
    x = int(phi * float(width) / kTwoPi - 0.5f);
    y = int(theta * float(height) / kPi - 0.5f);
    x = x < 0 ? 0 : (x > int(width) - 1 ? int(width) - 1 : x);
    y = y < 0 ? 0 : (y > int(height) - 1 ? int(height) - 1 : y);
}

// Solid-angle density of ibl_env_direction at wi.
SEL_HD float ibl_env_pdf(const IblDev& ibl, float3 wi) {
    int x, y;
    float theta;
    ibl_env_texel(wi, ibl.rotation, ibl.width, ibl.height, x, y, theta);
    const float m = y > 0 ? ibl.mdf[y] - ibl.mdf[y - 1] : ibl.mdf[y];
    const float* row = ibl.cdf + size_t(y) * ibl.width;
    const float c = x > 0 ? row[x] - row[x - 1] : row[x];
    float ax, bx, ay, by;
    ibl_env_span(uint32_t(x), ibl.width, ax, bx);
    ibl_env_span(uint32_t(y), ibl.height, ay, by);
    const float area = ((bx - ax) * (kTwoPi / float(ibl.width))) * ((by - ay) * (kPi / float(ibl.height)));
    const float st = sinf(theta);
    return st > 0.0f ? m * c / (area * st) : 0.0f;
}

// A direction toward the environment from four uniforms: (r0, r1) pick the texel, (r2, r3) the point in its
// region of directions.
SEL_HD float3 ibl_env_direction(const IblDev& ibl, float r0, float r1, float r2, float r3) {
    uint32_t x, y;
    float m, c;
    ibl_search(ibl.mdf, ibl.height, r0, y, m);
    ibl_search(ibl.cdf + size_t(y) * ibl.width, ibl.width, r1, x, c);
    float ax, bx, ay, by;
    ibl_env_span(x, ibl.width, ax, bx);
    ibl_env_span(y, ibl.height, ay, by);
    const float theta = (ay + r2 * (by - ay)) * (kPi / float(ibl.height));
    const float phi = (ax + r3 * (bx - ax)) * (kTwoPi / float(ibl.width)) - kPi - ibl.rotation;
    const float st = sinf(theta);
    return f3(st * cosf(phi), cosf(theta), st * sinf(phi));
}

}  // namespace sel
