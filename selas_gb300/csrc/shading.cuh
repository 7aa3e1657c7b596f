// Device-side pieces of the path tracer around the BSDF: random numbers, the reference camera model,
// quad-light next-event estimation and surface setup from a hit.
#pragma once

#include <cstdint>

#include "disney.cuh"
#include "scene_types.h"
#include "vecmath.cuh"

namespace sel {

// ---------------------------------------------------------------------------------------------------
// PCG32 (O'Neill 2014, "PCG: A family of simple fast space-efficient statistically good algorithms for
// random number generation"): 64-bit LCG state, XSH-RR output; one stream per path.  Uniform floats are
// the top 24 bits scaled to [0, 1).
// ---------------------------------------------------------------------------------------------------
struct Pcg32 {
    uint64_t state, inc;
};

SEL_HD uint32_t pcg_next(Pcg32& r) {
    const uint64_t old = r.state;
    r.state = old * 6364136223846793005ull + r.inc;
    const uint32_t xs = uint32_t(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = uint32_t(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
SEL_HD Pcg32 pcg_seed(uint64_t seed, uint64_t stream) {
    Pcg32 r;
    r.state = 0;
    r.inc = (stream << 1u) | 1u;
    pcg_next(r);
    r.state += seed;
    pcg_next(r);
    return r;
}
SEL_HD float pcg_float(Pcg32& r) { return float(pcg_next(r) >> 8) * (1.0f / 16777216.0f); }

// ---------------------------------------------------------------------------------------------------
// Camera: RayCastCameraSettings (GeometryLib/Camera.h:24-42) and ImageToWorldDirection
// (GeometryLib/Camera.cpp:56-60).
// ---------------------------------------------------------------------------------------------------
struct CameraDev {
    float3 x, y, z, position;
    float width, height;
};

SEL_HD float3 camera_direction(const CameraDev& c, float px, float py) {
    const float cx = (px / c.width) * 2.0f - 1.0f;
    const float cy = 1.0f - 2.0f * py / c.height;
    return normalize(c.z - cx * c.x + cy * c.y);
}

// ---------------------------------------------------------------------------------------------------
// Quad lights: SceneLight fields as NextEventEstimation reads them (Shading/AreaLighting.cpp:113-153,
// 353-373) and the spherical-rectangle sampler of Urena, Fajardo and King (EGSR 2013) as restated in
// GeometryLib/RectangulerLightSampler.cpp:17-97.
// ---------------------------------------------------------------------------------------------------
struct RectSampler {
    float3 o, x, y, z;
    float z0, z0sq, x0, y0, y0sq, x1, y1, y1sq, b0, b1, b0sq, k, S;
};

SEL_HD void rect_init(float3 s, float3 ex, float3 ey, float3 o, RectSampler& r) {
    r.o = o;
    const float exl = length(ex), eyl = length(ey);
    r.x = ex * (1.0f / exl);
    r.y = ey * (1.0f / eyl);
    r.z = cross(r.x, r.y);
    const float3 d = s - o;
    r.z0 = dot(d, r.z);
    if (r.z0 > 0.0f) {
        r.z = -r.z;
        r.z0 *= -1.0f;
    }
    r.z0sq = r.z0 * r.z0;
    r.x0 = dot(d, r.x);
    r.y0 = dot(d, r.y);
    r.x1 = r.x0 + exl;
    r.y1 = r.y0 + eyl;
    r.y0sq = r.y0 * r.y0;
    r.y1sq = r.y1 * r.y1;
    const float3 v00 = f3(r.x0, r.y0, r.z0), v01 = f3(r.x0, r.y1, r.z0);
    const float3 v10 = f3(r.x1, r.y0, r.z0), v11 = f3(r.x1, r.y1, r.z0);
    const float3 n0 = normalize(cross(v00, v10)), n1 = normalize(cross(v10, v11));
    const float3 n2 = normalize(cross(v11, v01)), n3 = normalize(cross(v01, v00));
    const float g0 = acosf(-dot(n0, n1)), g1 = acosf(-dot(n1, n2));
    const float g2 = acosf(-dot(n2, n3)), g3 = acosf(-dot(n3, n0));
    r.b0 = n0.z;
    r.b1 = n2.z;
    r.b0sq = r.b0 * r.b0;
    r.k = 2.0f * kPi - g2 - g3;
    r.S = g0 + g1 - r.k;
}

SEL_HD float3 rect_sample(const RectSampler& r, float u, float v) {
    const float au = u * r.S + r.k;
    const float fu = (cosf(au) * r.b0 - r.b1) / sinf(au);
    float cu = 1.0f / sqrtf(fu * fu + r.b0sq) * (fu > 0.0f ? 1.0f : -1.0f);
    cu = clampf(cu, -1.0f, 1.0f);
    float xu = -(cu * r.z0) / sqrtf(1.0f - cu * cu);
    xu = clampf(xu, r.x0, r.x1);
    const float d = sqrtf(xu * xu + r.z0sq);
    const float h0 = r.y0 / sqrtf(d * d + r.y0sq);
    const float h1 = r.y1 / sqrtf(d * d + r.y1sq);
    const float hv = h0 + v * (h1 - h0), hv2 = hv * hv;
    const float yv = (hv2 < 1.0f - 1e-10f) ? (hv * d) / sqrtf(1.0f - hv2) : r.y1;  // SmallFloatEpsilon_
    return r.o + xu * r.x + yv * r.y + r.z0 * r.z;
}

struct LightSample {
    float3 direction, radiance;
    float distance, pdf;
};

// SampleRectangleLightSolidAngle (AreaLighting.cpp:113-153): radiance already carries cos(theta_light)/d^2
// and cos(theta_surface) (as the reference computes it), pdf is (1/solid angle) * cos(theta_light)/d^2.
SEL_HD void sample_quad_light(const QuadLight& L, float3 p, float3 n, float u, float v, LightSample& s) {
    const float3 corner = L.position - 0.5f * L.x - 0.5f * L.z;
    RectSampler r;
    rect_init(corner, L.x, L.z, p, r);
    const float pdf = 1.0f / r.S;
    const float3 lp = rect_sample(r, u, v);
    const float3 ul = lp - p;
    const float d2 = dot(ul, ul);
    const float d = sqrtf(d2);
    const float3 l = (1.0f / d) * ul;
    const float area = dot(L.direction, -l) / d2;
    if (area > 0.0f) {
        s.direction = l;
        s.distance = d;
        s.radiance = L.radiance * (area * dot(n, l));
        s.pdf = pdf * area;
    } else {
        s.direction = f3(0.0f);
        s.distance = 0.0f;
        s.radiance = f3(0.0f);
        s.pdf = 1.0f;
    }
}

// MakeOrthogonalCoordinateSystem (GeometryLib/CoordinateSystem.h:14-21)
SEL_HD void orthonormal_basis(float3 v1, float3& v2, float3& v3) {
    if (fabsf(v1.x) > fabsf(v1.y))
        v2 = f3(-v1.z, 0.0f, v1.x) * (1.0f / sqrtf(v1.x * v1.x + v1.z * v1.z));
    else
        v2 = f3(0.0f, v1.z, -v1.y) * (1.0f / sqrtf(v1.y * v1.y + v1.z * v1.z));
    v3 = cross(v1, v2);
}


// rtcInterpolate0 of a per-vertex attribute: (1 - u - v) a0 + u a1 + v a2 per component.
SEL_HD float attr_lerp(float a0, float a1, float a2, float u, float v) {
    const float w = 1.0f - u - v;
    return w * a0 + u * a1 + v * a2;
}

// Where a hit interpolates a mesh's vertex attributes (rtcInterpolate0).  A triangle: corners i0 i1 i2 with
// weights (1 - u - v, u, v).  A quad of a quad mesh (stored as triangles 2q = (v0, v1, v3) and 2q + 1 =
// (v2, v3, v1)): its four corners, bilinearly, t_uv = (1 - v)((1 - u) t0 + u t1) + v((1 - u) t3 + u t2)
// (RTC_GEOMETRY_TYPE_QUAD.3embree3), at the quad's (u, v): the second triangle's (u', v') corrected to
// (1 - u', 1 - v').
struct AttrCorners {
    uint32_t i[4];  // triangle: i0 i1 i2; quad: v0 v1 v2 v3
    float u, v;
    bool quad;
};

SEL_HD AttrCorners attr_corners(const MeshAttrDev* A, uint32_t prim, float u, float v) {
    AttrCorners c;
    c.quad = A->quads != 0u;
    if (!c.quad) {
        c.i[0] = A->indices[3 * prim];
        c.i[1] = A->indices[3 * prim + 1];
        c.i[2] = A->indices[3 * prim + 2];
        c.i[3] = c.i[2];
        c.u = u;
        c.v = v;
    } else {
        const uint32_t* t = A->indices + 6 * size_t(prim >> 1);  // (v0, v1, v3), (v2, v3, v1)
        c.i[0] = t[0];
        c.i[1] = t[1];
        c.i[2] = t[3];
        c.i[3] = t[2];
        c.u = (prim & 1u) ? 1.0f - u : u;
        c.v = (prim & 1u) ? 1.0f - v : v;
    }
    return c;
}

// One component of an attribute with `stride` floats per vertex at the corners.
SEL_HD float attr_at(const AttrCorners& c, const float* a, uint32_t stride, uint32_t k) {
    if (!c.quad) return attr_lerp(a[stride * c.i[0] + k], a[stride * c.i[1] + k], a[stride * c.i[2] + k], c.u, c.v);
    const float iu = 1.0f - c.u, iv = 1.0f - c.v;
    return iv * (iu * a[stride * c.i[0] + k] + c.u * a[stride * c.i[1] + k]) +
           c.v * (iu * a[stride * c.i[3] + k] + c.u * a[stride * c.i[2] + k]);
}

// Shading frame of a hit (CalculateSurfaceParams, SurfaceParameters.cpp:157-184): the normal interpolated from
// the mesh's vertex normals where it has them (else the geometric normal), the tangent from its vertex tangents
// with b = cross(n, t) x the interpolated sign (returned in `sign`), else an orthonormal basis around n (sign 1).
// `xf` carries a vector to world space (the instances' localToWorld; identity for a mesh of the rendered scene).
template <typename Xf>
SEL_HD void shading_frame(const MeshAttrDev* A, uint32_t prim, float u, float v, float3 ng, Xf xf, float3& n,
                          float3& t, float3& b, float& sign) {
    float3 nrm = ng;
    // a table entry of a mesh without normals or tangents has no index array either: read no corners then
    if (A && !A->normals && !A->tangents) A = nullptr;
    AttrCorners c;
    if (A) c = attr_corners(A, prim, u, v);
    if (A && A->normals) {
        const float* a = A->normals;
        nrm = f3(attr_at(c, a, 3, 0), attr_at(c, a, 3, 1), attr_at(c, a, 3, 2));
    }
    n = normalize(xf(nrm));
    if (A && A->tangents) {
        const float* a = reinterpret_cast<const float*>(A->tangents);
        const float3 tl = f3(attr_at(c, a, 4, 0), attr_at(c, a, 4, 1), attr_at(c, a, 4, 2));
        sign = attr_at(c, a, 4, 3);
        t = xf(tl);
        b = cross(n, t) * sign;
    } else {
        orthonormal_basis(n, t, b);
        sign = 1.0f;
    }
}

// CalculateSurfaceParams (Shading/SurfaceParameters.cpp:144-247) from a shading frame (t, n, b) and the linear
// base colour.
SEL_HD Surface make_surface_frame(const MaterialDev& m, float3 t, float3 n, float3 b, float3 view,
                                  float3 base_color_linear) {
    Surface s;
    s.t = t;
    s.n = n;
    s.b = b;
    s.base_color = base_color_linear;
    s.transmittance_color = ld3(m.transmittance_color);
    s.sheen = m.sheen;
    s.sheen_tint = m.sheen_tint;
    s.clearcoat = m.clearcoat;
    s.clearcoat_gloss = m.clearcoat_gloss;
    s.spec_trans = saturate(m.spec_trans);
    s.diff_trans = m.diffuse_trans * 0.5f;
    s.flatness = m.flatness;
    s.anisotropic = m.anisotropic;
    s.specular_tint = m.specular_tint;
    s.roughness = m.roughness;
    s.metallic = saturate(m.metallic);
    s.scatter_distance = m.scatter_distance;
    s.ior = m.ior;
    s.shader = m.shader;
    s.relative_ior = ((m.flags & kMaterialTransparent) && dot(view, n) < 0.0f) ? s.ior : 1.0f / s.ior;
    return s;
}

// The same for meshes without shading normals or tangents: the frame around the unit geometric normal n.
SEL_HD Surface make_surface_linear(const MaterialDev& m, float3 n, float3 view, float3 base_color_linear) {
    float3 t, b;
    orthonormal_basis(n, t, b);
    return make_surface_frame(m, t, n, b, view, base_color_linear);
}

// The same from a hit: frame from the normalised geometric normal, authored base colour raised to the
// power 2.2.
SEL_HD Surface make_surface(const MaterialDev& m, float3 ng, float3 view, float3 base_color_authored) {
    return make_surface_linear(m, normalize(ng), view, pow3(base_color_authored, 2.2f));
}

// ContinuationProbability (SurfaceParameters.cpp:420-424)
SEL_HD float continuation_probability(const Surface& s) {
    return saturate(fmaxf(fmaxf(s.base_color.x, s.base_color.y), s.base_color.z));
}

// OffsetRayOrigin (SurfaceParameters.cpp:403-408)
SEL_HD float3 offset_origin(float3 p, float3 n, float error, float3 dir, float scale) {
    const float side = dot(dir, n) < 0.0f ? -1.0f : 1.0f;
    return p + (side * error * scale) * n;
}

}  // namespace sel
