// Base colour from a 2D image at the hit's uvs: the reference's non-Ptex path of CalculateSurfaceParams
// (Source/Core/Shading/SurfaceParameters.cpp:186-190,209-213: uvs interpolated from attribute slot 2, else (0, 0);
// SampleTextureFloat3 / SampleTexture, :60-119, sRGB to linear after filtering; the caller then raises it to 2.2
// as for Ptex) with TextureFiltering::Triangle at mip level 0 and Repeat wrapping (TextureFiltering.h:30-100).
// Repeat takes the remainder of the texel coordinate converted to unsigned, as the reference's `s % w` with an
// int32 s and a uint32 w does (TextureFiltering.h:32-44): a negative coordinate c reads texel (2^32 + c) mod w,
// which is the ordinary wrap w + c for the power-of-two sizes images usually have.
#pragma once

#include <cstdint>

#include "scene_types.h"
#include "shading.cuh"
#include "vecmath.cuh"

namespace sel {

// SrgbToLinearPrecise (MathLib/ColorSpace.cpp:16-23)
SEL_HD float srgb_to_linear(float x) { return x <= 0.04045f ? x / 12.92f : powf((x + 0.055f) / (1.0f + 0.055f), 2.4f); }

SEL_HD float3 tex2d_texel(const float4* tex, int w, int h, int s, int t) {
    const uint32_t ss = uint32_t(s) % uint32_t(w), tt = uint32_t(t) % uint32_t(h);
    const float4 c = tex[tt * uint32_t(w) + ss];
    return f3(c.x, c.y, c.z);
}

// The linear base colour of material m at barycentrics (bu, bv) of triangle `prim` of a mesh with attributes
// `attr` (null or without uvs: uvs (0, 0)).
SEL_HD float3 tex2d_base_colour(const MaterialDev& m, const MeshAttrDev* attr, uint32_t prim, float bu, float bv) {
    float su = 0.0f, sv = 0.0f;
    if (attr && attr->uvs) {
        const AttrCorners c = attr_corners(attr, prim, bu, bv);
        const float* a = reinterpret_cast<const float*>(attr->uvs);
        su = attr_at(c, a, 2, 0);
        sv = attr_at(c, a, 2, 1);
    }
    const float4* tex = reinterpret_cast<const float4*>(uint64_t(m.tex_lo) | (uint64_t(m.tex_hi) << 32));
    const int w = int(m.tex_width), h = int(m.tex_height);
    const float s = su * float(w) - 0.5f;
    const float t = sv * float(h) - 0.5f;
    const int s0 = int(floorf(s)), t0 = int(floorf(t));
    const float ds = s - float(s0), dt = t - float(t0);
    const float3 r = (1.0f - ds) * (1.0f - dt) * tex2d_texel(tex, w, h, s0, t0) +
                     (1.0f - ds) * dt * tex2d_texel(tex, w, h, s0, t0 + 1) +
                     ds * (1.0f - dt) * tex2d_texel(tex, w, h, s0 + 1, t0) +
                     ds * dt * tex2d_texel(tex, w, h, s0 + 1, t0 + 1);
    return f3(srgb_to_linear(r.x), srgb_to_linear(r.y), srgb_to_linear(r.z));
}

}  // namespace sel
