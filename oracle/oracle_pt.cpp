// ORACLE - test infrastructure only (see oracle_query.cpp).
//
// CPU restatement of the reference unidirectional path tracer, one path at a time:
//   EvaluatePath       Source/Applications/Selas/Source/PathTracer.cpp:142-258
//   RayPick            PathTracer.cpp:95-139 (tnear 0, error bound 32 * 1.19209e-07 * max(|p|, t))
//   OcclusionRay       PathTracer.cpp:71-92  (origin offset 0.1 * error, tnear = error)
//   JitteredCameraRay  Source/Core/GeometryLib/Camera.cpp:56-74; InitializeRayCastCamera :89-115
//   NextEventEstimation / SampleRectangleLightSolidAngle  Source/Core/Shading/AreaLighting.cpp:113-153,353-373
//   RectangleLightSampler  Source/Core/GeometryLib/RectangulerLightSampler.cpp:17-97
//   CalculateSurfaceParams Source/Core/Shading/SurfaceParameters.cpp:144-247 (no normals/tangents/uvs)
//   Isotropic media        Source/Core/Shading/IsotropicScattering.cpp, VolumetricScattering.cpp
// The deferred path tracer (Source/Applications/Selas/Source/DeferredPathTracer.cpp:61-148, 151-279,
// 349-380, 433-472) is restated by deferred_path / oracle_deferred_render: 4 x 4 correlated multi-jittered
// primary samples (Kensler 2013), quad-light next-event estimation with weight 1 and background sampling
// with the balance heuristic, shadow rays from tnear 0, no bounce limit (paths end by Russian roulette from
// 7 tracked bounces, or at a given cap), no participating media, one output layer.
// Random numbers: either PCG32 with one stream per path (stream = pass * W * H + pixel, the sampling the
// GPU path tracer uses) or MT19937 as the reference's CSampler draws them (Random.cpp:46-49), one engine
// per pixel.  Each path's two layers are summed in float as the reference's Ld[] (PathTracer.cpp:144-257)
// and the per-pixel sums are kept in double.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <thread>
#include <vector>

#include "oracle_attrs.h"
#include "oracle_env.h"
#include "oracle_bsdf.h"
#include "oracle_ptex.h"
#include "oracle_query.h"

using orc::V3;

namespace {

const float kPi = 3.141592653589793f;

struct Rng {
    bool pcg = true;
    uint64_t state = 0, inc = 1;
    std::mt19937 mt;
    uint32_t next_u32() {
        const uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        const uint32_t xs = uint32_t(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = uint32_t(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    void seed_pcg(uint64_t seed, uint64_t stream) {
        pcg = true;
        state = 0;
        inc = (stream << 1u) | 1u;
        next_u32();
        state += seed;
        next_u32();
    }
    float uniform() {
        if (pcg) return float(next_u32() >> 8) * (1.0f / 16777216.0f);
        return float(mt()) / float(0xFFFFFFFFu);
    }
};

struct Camera {
    V3 x, y, z, pos;
    float w, h;
};

Camera make_camera(const float* c, uint32_t width, uint32_t height) {
    // c: position[3] lookAt[3] up[3] fovDegrees
    Camera cam;
    const float widthf = float(width), heightf = float(height);
    const float aspect = widthf / heightf;
    const float hfov = c[9] * (kPi / 180.0f);
    const float hlen = std::tan(hfov * 0.5f);
    const float vfov = 2.0f * std::atan(hlen / aspect);
    const float vlen = std::tan(vfov * 0.5f);
    V3 pos(c[0], c[1], c[2]), look(c[3], c[4], c[5]), up(c[6], c[7], c[8]);
    V3 fwd = orc::Norm(look - pos);
    V3 right = orc::Norm(orc::Cross(up, fwd));
    cam.x = hlen * right;
    cam.y = vlen * orc::Cross(fwd, right);
    cam.z = fwd;
    cam.pos = pos;
    cam.w = widthf;
    cam.h = heightf;
    return cam;
}

struct Light {
    V3 pos, dir, x, z, radiance;
};

struct Material {
    int shader;
    uint32_t flags, light_set, ptex_base;
    float base[3], trans[3];
    float sheen, sheenTint, clearcoat, clearcoatGloss, metallic, specTrans, diffTrans, flatness;
    float anisotropic, specularTint, roughness, scatterDistance, ior;
};

Material read_material(const float* r) {
    Material m;
    int32_t sh;
    uint32_t fl, ls;
    std::memcpy(&sh, r + 0, 4);
    std::memcpy(&fl, r + 1, 4);
    std::memcpy(&ls, r + 2, 4);
    m.shader = sh;
    m.flags = fl;
    m.light_set = ls;
    std::memcpy(&m.ptex_base, r + 3, 4);
    for (int i = 0; i < 3; ++i) { m.base[i] = r[4 + i]; m.trans[i] = r[7 + i]; }
    m.sheen = r[10]; m.sheenTint = r[11]; m.clearcoat = r[12]; m.clearcoatGloss = r[13];
    m.metallic = r[14]; m.specTrans = r[15]; m.diffTrans = r[16]; m.flatness = r[17];
    m.anisotropic = r[18]; m.specularTint = r[19]; m.roughness = r[20]; m.scatterDistance = r[21]; m.ior = r[22];
    return m;
}

float Sat(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

// SampleRectangleLightSolidAngle (AreaLighting.cpp:113-153) with the sampler of RectangulerLightSampler.cpp.
void sample_light(const Light& L, V3 p, V3 n, float u, float v, V3& dir, V3& rad, float& dist, float& pdfw,
                  bool physical) {
    V3 s = L.pos - 0.5f * L.x - 0.5f * L.z;
    const float exl = orc::Len(L.x), eyl = orc::Len(L.z);
    V3 X = L.x * (1.0f / exl), Y = L.z * (1.0f / eyl), Z = orc::Cross(X, Y);
    V3 d = s - p;
    float z0 = orc::Dot(d, Z);
    if (z0 > 0) { Z = -1.0f * Z; z0 *= -1; }
    const float z0sq = z0 * z0, x0 = orc::Dot(d, X), y0 = orc::Dot(d, Y);
    const float x1 = x0 + exl, y1 = y0 + eyl, y0sq = y0 * y0, y1sq = y1 * y1;
    V3 v00(x0, y0, z0), v01(x0, y1, z0), v10(x1, y0, z0), v11(x1, y1, z0);
    V3 n0 = orc::Norm(orc::Cross(v00, v10)), n1 = orc::Norm(orc::Cross(v10, v11));
    V3 n2 = orc::Norm(orc::Cross(v11, v01)), n3 = orc::Norm(orc::Cross(v01, v00));
    const float g0 = std::acos(-orc::Dot(n0, n1)), g1 = std::acos(-orc::Dot(n1, n2));
    const float g2 = std::acos(-orc::Dot(n2, n3)), g3 = std::acos(-orc::Dot(n3, n0));
    const float b0 = n0.z, b1 = n2.z, b0sq = b0 * b0;
    const float k = 2 * kPi - g2 - g3;
    const float S = g0 + g1 - k;
    const float pdf = 1.0f / S;
    // SampleRectangleLight
    const float au = u * S + k;
    const float fu = (std::cos(au) * b0 - b1) / std::sin(au);
    float cu = 1 / std::sqrt(fu * fu + b0sq) * (fu > 0 ? +1 : -1);
    cu = std::min(std::max(cu, -1.0f), 1.0f);
    float xu = -(cu * z0) / std::sqrt(1 - cu * cu);
    xu = std::min(std::max(xu, x0), x1);
    const float dd = std::sqrt(xu * xu + z0sq);
    const float h0 = y0 / std::sqrt(dd * dd + y0sq);
    const float h1 = y1 / std::sqrt(dd * dd + y1sq);
    const float hv = h0 + v * (h1 - h0), hv2 = hv * hv;
    const float yv = (hv2 < 1 - 1e-10f) ? (hv * dd) / std::sqrt(1 - hv2) : y1;
    V3 lp = p + xu * X + yv * Y + z0 * Z;
    V3 ul = lp - p;
    const float d2 = orc::Dot(ul, ul);
    const float di = std::sqrt(d2);
    V3 l = (1.0f / di) * ul;
    const float area = orc::Dot(L.dir, -1.0f * l) / d2;
    if (area > 0) {
        dir = l;
        dist = di;
        rad = L.radiance * (physical ? area : area * orc::Dot(n, l));
        pdfw = pdf * area;
    } else {
        dir = V3(0.0f);
        dist = 0;
        rad = V3(0.0f);
        pdfw = 1.0f;
    }
}

// Image-based light (ImageBasedLightResource.cpp:81-268; densities as BuildImageBasedLight.cpp:18-107).
struct Ibl {
    uint32_t w = 0, h = 0, mw = 0, mh = 0;
    float rot = 0, exposure = 1;
    std::vector<float> mdf, cdf, light, miss;  // light / miss: RGB

    void build(const float* rgb, uint32_t width, uint32_t height, const float* miss_rgb, uint32_t miss_w,
               uint32_t miss_h, float rotation, float scale) {
        w = width; h = height; rot = rotation; exposure = scale;
        light.assign(rgb, rgb + size_t(w) * h * 3);
        if (miss_rgb) {
            mw = miss_w; mh = miss_h;
            miss.assign(miss_rgb, miss_rgb + size_t(mw) * mh * 3);
        } else {
            mw = w; mh = h;
            miss.resize(light.size());
            for (size_t i = 0; i < light.size(); ++i) miss[i] = scale * light[i];
        }
        std::vector<float> inten(size_t(w) * h);
        for (uint32_t y = 0; y < h; ++y) {
            const float sin_theta = std::sin((float(y) + 0.5f) * kPi / float(h));
            for (uint32_t x = 0; x < w; ++x) {
                const float* c = &light[(size_t(y) * w + x) * 3];
                inten[size_t(y) * w + x] = sin_theta * (c[0] * 0.299f + c[1] * 0.587f + c[2] * 0.114f);
            }
        }
        mdf.assign(h, 0.0f);
        cdf.assign(size_t(w) * h, 0.0f);
        float msum = 0.0f;
        for (uint32_t y = 0; y < h; ++y) {
            float rsum = 0.0f;
            for (uint32_t x = 0; x < w; ++x) rsum += inten[size_t(y) * w + x];
            mdf[y] = rsum;
            msum += rsum;
            if (rsum > 0.0f) {
                const float oo = 1.0f / rsum;
                float acc = 0.0f;
                for (uint32_t x = 0; x < w; ++x) {
                    acc += oo * inten[size_t(y) * w + x];
                    cdf[size_t(y) * w + x] = acc;
                }
            }
            cdf[size_t(y) * w + w - 1] = 1.0f;
        }
        if (msum > 0.0f) {
            const float oo = 1.0f / msum;
            float acc = 0.0f;
            for (uint32_t y = 0; y < h; ++y) {
                acc += mdf[y] * oo;
                mdf[y] = acc;
            }
        }
        mdf[h - 1] = 1.0f;
    }
    static void search(const float* f, uint32_t count, float r, uint32_t& index, float& pdf) {
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
    void texel(V3 wi, uint32_t width, uint32_t height, int& x, int& y, float& theta) const {
        theta = std::acos(std::min(std::max(wi.y, -1.0f), 1.0f));
        float phi = std::atan2(wi.z, wi.x);
        phi = std::fmod(phi + kPi + rot, 2.0f * kPi);
        x = int(phi * float(width) / (2.0f * kPi) - 0.5f);
        y = int(theta * float(height) / kPi - 0.5f);
        x = std::min(std::max(x, 0), int(width) - 1);
        y = std::min(std::max(y, 0), int(height) - 1);
    }
    float pdf_at(int x, int y, float theta) const {
        const float m = y > 0 ? mdf[y] - mdf[y - 1] : mdf[y];
        const float* row = &cdf[size_t(y) * w];
        const float c = x > 0 ? row[x] - row[x - 1] : row[x];
        const float inv_j = (float(w) * float(h)) / (2.0f * kPi);
        const float st = std::sin(theta);
        return st > 0.0f ? m * c * inv_j / st : 0.0f;
    }
    float pdf(V3 wi) const {
        int x, y;
        float theta;
        texel(wi, w, h, x, y, theta);
        return pdf_at(x, y, theta);
    }
    V3 radiance(V3 wi) const {
        int x, y;
        float theta;
        texel(wi, w, h, x, y, theta);
        const float* c = &light[(size_t(y) * w + x) * 3];
        return exposure * V3(c[0], c[1], c[2]);
    }
    V3 miss_radiance(V3 wi) const {
        int x, y;
        float theta;
        texel(wi, mw, mh, x, y, theta);
        const float* c = &miss[(size_t(y) * mw + x) * 3];
        return V3(c[0], c[1], c[2]);
    }
    // Environment emitter of the VCM oracle (the device's ibl_env_*): a texel from (r0, r1) by the CDFs, the
    // direction jittered by (r2, r3) uniformly in (theta, phi) over the directions that look the texel up, so
    // the solid-angle density m c / (area sin theta) belongs to the texel a direction's lookup returns.  The
    // azimuth is wrapped into [0, 2 pi) (the lookup's fmod leaves negative rotations negative).
    static void env_span(uint32_t i, uint32_t n, float& a, float& b) {
        a = i == 0 ? 0.0f : float(i) + 0.5f;
        b = i + 1 >= n ? float(n) : float(i) + 1.5f;
    }
    void env_texel(V3 wi, int& x, int& y, float& theta) const {
        theta = std::acos(std::min(std::max(wi.y, -1.0f), 1.0f));
        float phi = std::atan2(wi.z, wi.x);
        phi = std::fmod(phi + kPi + rot, 2.0f * kPi);
        if (phi < 0.0f) phi += 2.0f * kPi;
        x = int(phi * float(w) / (2.0f * kPi) - 0.5f);
        y = int(theta * float(h) / kPi - 0.5f);
        x = std::min(std::max(x, 0), int(w) - 1);
        y = std::min(std::max(y, 0), int(h) - 1);
    }
    float env_pdf(V3 wi) const {
        int x, y;
        float theta;
        env_texel(wi, x, y, theta);
        const float m = y > 0 ? mdf[y] - mdf[y - 1] : mdf[y];
        const float* row = &cdf[size_t(y) * w];
        const float c = x > 0 ? row[x] - row[x - 1] : row[x];
        float ax, bx, ay, by;
        env_span(uint32_t(x), w, ax, bx);
        env_span(uint32_t(y), h, ay, by);
        const float area = ((bx - ax) * ((2.0f * kPi) / float(w))) * ((by - ay) * (kPi / float(h)));
        const float st = std::sin(theta);
        return st > 0.0f ? m * c / (area * st) : 0.0f;
    }
    V3 env_direction(float r0, float r1, float r2, float r3) const {
        uint32_t x, y;
        float m, c;
        search(mdf.data(), h, r0, y, m);
        search(&cdf[size_t(y) * w], w, r1, x, c);
        float ax, bx, ay, by;
        env_span(x, w, ax, bx);
        env_span(y, h, ay, by);
        const float theta = (ay + r2 * (by - ay)) * (kPi / float(h));
        const float phi = (ax + r3 * (bx - ax)) * ((2.0f * kPi) / float(w)) - kPi - rot;
        const float st = std::sin(theta);
        return V3(st * std::cos(phi), std::cos(theta), st * std::sin(phi));
    }
    void sample(float r0, float r1, V3& dir, V3& rad, float& p) const {
        uint32_t x, y;
        float m, c;
        search(mdf.data(), h, r0, y, m);
        search(&cdf[size_t(y) * w], w, r1, x, c);
        const float theta = (float(y) + 0.5f) * kPi / float(h);
        const float phi = std::fmod(((float(x) + 0.5f) * (2.0f * kPi) / float(w)) + rot, 2.0f * kPi) - kPi;
        const float inv_j = (float(w) * float(h)) / (2.0f * kPi);
        const float st = std::sin(theta);
        p = st > 0.0f ? m * c * inv_j / st : 0.0f;
        dir = V3(st * std::cos(phi), std::cos(theta), st * std::sin(phi));
        const float* l = &light[(size_t(y) * w + x) * 3];
        rad = exposure * V3(l[0], l[1], l[2]);
    }
};

// Vertex attributes of the soup (oracle_set_attributes): per triangle, the three corners' shading normals and
// tangents and flags (1 normals, 2 tangents); `first` maps (scene << 32 | geomID) to the mesh's first triangle.
struct Attrs {
    std::vector<float> normals, tangents, uvs;  // uvs: (u, v) of the three corners, flag 4
    std::vector<uint8_t> flags;
    std::map<uint64_t, int64_t> first;
};

struct Scene {
    const void* bvh = nullptr;
    const Ibl* ibl = nullptr;                       // image-based light (null: the uniform background)
    const Attrs* attrs = nullptr;                   // vertex attributes (null: none)
    const void* graph = nullptr;                    // instanced scene graph (replaces bvh when set)
    std::vector<std::vector<Material>> gmats;       // graph: materials of each scene, by geomID
    std::vector<const orp::Texture*> gptex;         // graph: Ptex of each scene (null: none)
    const orp::Texture* ptex = nullptr;
    bool physical_nee = false;
    std::vector<Material> materials;
    std::vector<Light> lights;
    std::vector<uint32_t> set_first, set_count;
    V3 background;
};

bool sc_closest(const Scene& sc, const float* o, const float* d, float tnear, float tfar, orq::Hit& h) {
    return sc.graph ? orq::closest_graph(sc.graph, o, d, tnear, tfar, h) : orq::closest(sc.bvh, o, d, tnear, tfar, h);
}

bool sc_occluded(const Scene& sc, const float* o, const float* d, float tnear, float tfar) {
    return sc.graph ? orq::occluded_graph(sc.graph, o, d, tnear, tfar) : orq::occluded(sc.bvh, o, d, tnear, tfar);
}

// A vector through local-to-world rows (the device's fma chain).
V3 xvector(const float* m, V3 v) {
    return V3(std::fma(m[0], v.x, std::fma(m[1], v.y, m[2] * v.z)), std::fma(m[4], v.x, std::fma(m[5], v.y, m[6] * v.z)),
              std::fma(m[8], v.x, std::fma(m[9], v.y, m[10] * v.z)));
}

V3 offset(V3 p, V3 n, float err, V3 dir, float scale) {
    const float side = orc::Dot(dir, n) < 0.0f ? -1.0f : 1.0f;
    return p + (side * err * scale) * n;
}

// CalculateSurfaceParams (SurfaceParameters.cpp:144-247) for meshes without normals, tangents or uvs.
struct SurfHit {
    const Material* m;
    float err;
    orc::Surf s;
    V3 n, view;
};

// Shading frame of a hit (CalculateSurfaceParams, SurfaceParameters.cpp:157-184): interpolated vertex normal and
// tangent where the mesh has them, through the entered instances' localToWorld.
void shading_frame(const Scene& sc, const orq::Hit& h, V3& n, V3& t, V3& b) {
    // shading normal and tangent from vertex attributes (SurfaceParameters.cpp:157-184)
    int64_t ai = -1;
    if (sc.attrs) {
        const auto it = sc.attrs->first.find((uint64_t(h.scene) << 32) | h.geom);
        if (it != sc.attrs->first.end()) ai = it->second + h.prim;
    }
    const uint8_t aflags = ai >= 0 ? sc.attrs->flags[size_t(ai)] : 0;
    V3 ngv(h.ng[0], h.ng[1], h.ng[2]);
    if (aflags & 1u)
        ngv = V3(ora::corner_interp(sc.attrs->normals, 3, ai, aflags, h.prim, h.u, h.v, 0),
                 ora::corner_interp(sc.attrs->normals, 3, ai, aflags, h.prim, h.u, h.v, 1),
                 ora::corner_interp(sc.attrs->normals, 3, ai, aflags, h.prim, h.u, h.v, 2));
    if (h.l2w[1]) ngv = xvector(h.l2w[1], ngv);
    if (h.l2w[0]) ngv = xvector(h.l2w[0], ngv);
    n = orc::Norm(ngv);
    if (aflags & 2u) {
        V3 tl(ora::corner_interp(sc.attrs->tangents, 4, ai, aflags, h.prim, h.u, h.v, 0),
              ora::corner_interp(sc.attrs->tangents, 4, ai, aflags, h.prim, h.u, h.v, 1),
              ora::corner_interp(sc.attrs->tangents, 4, ai, aflags, h.prim, h.u, h.v, 2));
        const float sign = ora::corner_interp(sc.attrs->tangents, 4, ai, aflags, h.prim, h.u, h.v, 3);
        if (h.l2w[1]) tl = xvector(h.l2w[1], tl);
        if (h.l2w[0]) tl = xvector(h.l2w[0], tl);
        t = tl;
        b = orc::Cross(n, t) * sign;
    } else {
        if (std::fabs(n.x) > std::fabs(n.y)) t = V3(-n.z, 0, n.x) * (1.0f / std::sqrt(n.x * n.x + n.z * n.z));
        else t = V3(0, n.z, -n.y) * (1.0f / std::sqrt(n.y * n.y + n.z * n.z));
        b = orc::Cross(n, t);
    }
}

// Instanced hits (ModelDataFromRayIds, SceneResource.cpp:362-378): material and Ptex of the hit mesh's scene;
// the object-space normal through the instances' localToWorld, innermost first (SurfaceParameters.cpp:161-168).
void surface_at(const Scene& sc, const orq::Hit& h, V3 pos, V3 dir, SurfHit& o) {
    const std::vector<Material>& mats = sc.graph ? sc.gmats[h.scene] : sc.materials;
    const orp::Texture* ptex = sc.graph ? sc.gptex[h.scene] : sc.ptex;
    const Material& m = mats[h.geom < mats.size() ? h.geom : 0];
    o.m = &m;
    o.err = 32.0f * 1.19209e-07f * std::max(std::max(std::fabs(pos.x), std::fabs(pos.y)), std::max(std::fabs(pos.z), h.t));
    orc::Surf& s = o.s;
    V3 n, t, b;
    shading_frame(sc, h, n, t, b);
    s.t = t; s.n = n; s.b = b;
    float base[3] = {m.base[0], m.base[1], m.base[2]};
    if ((m.flags & 2u) && ora::quad_ptex(sc.graph ? h.scene : 0u, h.geom, h.prim, h.u, h.v, base)) {
    } else if ((m.flags & 2u) && ptex) {
        ptex->eval(int(m.ptex_base + h.prim), h.u, h.v, base);
    } else {
        ora::tex2d(sc.graph ? h.scene : 0u, h.geom, h.prim, h.u, h.v, base);
    }
    s.baseColor = V3(std::pow(base[0], 2.2f), std::pow(base[1], 2.2f), std::pow(base[2], 2.2f));
    s.transmittanceColor = V3(m.trans[0], m.trans[1], m.trans[2]);
    s.sheen = m.sheen; s.sheenTint = m.sheenTint; s.clearcoat = m.clearcoat; s.clearcoatGloss = m.clearcoatGloss;
    s.specTrans = Sat(m.specTrans); s.diffTrans = m.diffTrans * 0.5f; s.flatness = m.flatness;
    s.anisotropic = m.anisotropic; s.specularTint = m.specularTint; s.roughness = m.roughness;
    s.metallic = Sat(m.metallic); s.scatterDistance = m.scatterDistance; s.ior = m.ior; s.shader = m.shader;
    o.view = -1.0f * dir;
    s.relativeIOR = ((m.flags & 1u) && orc::Dot(o.view, n) < 0.0f) ? s.ior : 1.0f / s.ior;
    o.n = n;
}

// EvaluatePath (PathTracer.cpp:142-258); returns both layers.
void evaluate_path(const Scene& sc, Rng& rng, V3 org, V3 dir, uint32_t max_bounces, V3& ld0, V3& ld1) {
    ld0 = V3(0.0f);
    ld1 = V3(0.0f);
    V3 thr(1.0f);
    bool delta_only = true;
    int phase = 0;
    V3 ext(0.0f);
    uint32_t bounce = 0;
    while (bounce < max_bounces) {
        float tfar = 3.402823466e+38f;
        if (phase == 1) {  // Isotropic::SampleDistance
            const float ps = ext.x + ext.y + ext.z;
            const float pr = ext.x / ps, pg = ext.y / ps;
            float c;
            const float r0 = rng.uniform();
            if (r0 < pr) c = ext.x;
            else if (r0 < pr + pg) c = ext.y;
            else c = ext.z;
            tfar = -std::log(rng.uniform()) / c;
        }
        orq::Hit h;
        const float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
        const bool hit = sc_closest(sc, o, d, 0.0f, tfar, h);
        float ray_distance = tfar;
        V3 pos;
        if (hit) {
            pos = V3(org.x + h.t * dir.x, org.y + h.t * dir.y, org.z + h.t * dir.z);
            ray_distance = orc::Len(pos - org);
        }
        if (phase == 1)
            thr = thr * V3(std::exp(-ext.x * ray_distance), std::exp(-ext.y * ray_distance), std::exp(-ext.z * ray_distance));
        if (hit) {
            SurfHit sh;
            surface_at(sc, h, pos, dir, sh);
            const Material& m = *sh.m;
            const float err = sh.err;
            const orc::Surf& s = sh.s;
            const V3 n = sh.n;
            const V3 view = sh.view;
            // next-event estimation
            V3 ldir, lrad(0.0f);
            float ldist = 0, lpdf = 1;
            if (m.light_set < sc.set_count.size() && sc.set_count[m.light_set] > 0) {
                const uint32_t cnt = sc.set_count[m.light_set];
                const float p0 = rng.uniform();
                uint32_t li = uint32_t(p0 * float(cnt));
                li = std::min(li, cnt - 1);
                const float u = rng.uniform(), v = rng.uniform();
                sample_light(sc.lights[sc.set_first[m.light_set] + li], pos, n, u, v, ldir, lrad, ldist, lpdf,
                             sc.physical_nee);
                lpdf *= 1.0f / float(cnt);
            }
            if (orc::Dot(lrad, V3(1.0f)) > 0) {
                float fp, rp;
                const V3 refl = orc::bsdf_evaluate(s, view, ldir, fp, rp);
                if (orc::Dot(refl, V3(1.0f)) > 0) {
                    const V3 so = offset(pos, n, err, ldir, 0.1f);
                    const float soa[3] = {so.x, so.y, so.z}, lda[3] = {ldir.x, ldir.y, ldir.z};
                    if (!sc_occluded(sc, soa, lda, err, ldist)) ld1 = ld1 + refl * lrad * (1.0f / lpdf) * thr;
                }
            }
            // BSDF sample: uniforms drawn lazily, in order
            float u4[4];
            Rng ahead = rng;
            for (int k = 0; k < 4; ++k) u4[k] = ahead.uniform();
            int used = 0;
            orc::Sample bs;
            const bool ok = orc::bsdf_sample(s, view, u4, used, bs);
            for (int k = 0; k < used; ++k) rng.uniform();
            if (!ok) break;
            delta_only = delta_only && (bs.flags & 4u);
            if (bs.flags == 2u) {
                if (phase == 0) { phase = bs.phase; ext = bs.ext; }
                else { phase = 0; ext = V3(0.0f); }
            }
            thr = 1.0f * thr * bs.refl;
            org = offset(pos, n, err, bs.wi, 1.0f);
            dir = bs.wi;
            if (bounce == 0) ld0 = bs.refl;
        } else if (phase != 0) {
            org = org + ray_distance * dir;
            const float r0 = rng.uniform(), r1 = rng.uniform();
            const float uu = 2.0f * r1 - 1.0f;
            const float nn = std::sqrt(std::max(0.0f, 1.0f - uu * uu));
            const float th = 2.0f * kPi * r0;
            dir = V3(nn * std::cos(th), uu, nn * std::sin(th));
        } else {
            const V3 bg = sc.ibl ? (delta_only ? sc.ibl->miss_radiance(dir) : sc.ibl->radiance(dir)) : sc.background;
            ld1 = ld1 + bg * thr;
            break;
        }
        ++bounce;
        if (bounce > 8) {
            const float cp = std::max(std::max(thr.x, thr.y), thr.z);
            if (rng.uniform() > cp) break;
            thr = thr * (1.0f / cp);
        }
    }
}

// Correlated multi-jittered sampling: A. Kensler, "Correlated Multi-Jittered Sampling", Pixar Technical Memo
// 13-01 (2013), the published hash constants and steps that Source/Core/MathLib/CorrelatedMultiJitter.cpp:12-62
// uses.  cmj_permute is a bijection of [0, 2^k) walked until it lands below l (at most 2^k steps).
uint32_t cmj_permute(uint32_t i, uint32_t l, uint32_t p) {
    uint32_t w = l - 1;
    for (int sh = 1; sh <= 16; sh <<= 1) w |= w >> sh;
    do {
        i ^= p;
        i *= 0xe170893du;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3fu;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1u | p >> 27;
        i *= 0x6935fa69u;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303u;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3u;
        i ^= (i & w) >> 2;
        i *= 0xc860a3dfu;
        i &= w;
        i ^= i >> 5;
    } while (i >= l);
    return (i + p) % l;
}

float cmj_float(uint32_t i, uint32_t p) {
    i ^= p;
    i ^= i >> 17;
    i ^= i >> 10;
    i *= 0xb36534e5u;
    i ^= i >> 12;
    i ^= i >> 21;
    i *= 0x93fc4795u;
    i ^= 0xdf6e307fu;
    i ^= i >> 17;
    i *= 1u | p >> 18;
    return float(i) * (1.0f / 4294967808.0f);
}

// Sample s of an m x n pattern decorrelated by p: a point of [0,1)^2.
void cmj(int32_t s, int32_t m, int32_t n, int32_t p, float& x, float& y) {
    const uint32_t up = uint32_t(p);
    const int32_t sx = int32_t(cmj_permute(uint32_t(s % m), uint32_t(m), up * 0xa511e9b3u));
    const int32_t sy = int32_t(cmj_permute(uint32_t(s / m), uint32_t(n), up * 0x63d83595u));
    const float jx = cmj_float(uint32_t(s), up * 0xa399d265u);
    const float jy = cmj_float(uint32_t(s), up * 0x711ad6a5u);
    x = (float(s % m) + (float(sy) + jx) / float(n)) / float(m);
    y = (float(s / m) + (float(sx) + jy) / float(m)) / float(n);
}

void add(double* acc, V3 c) {
    acc[0] += c.x;
    acc[1] += c.y;
    acc[2] += c.z;
}

// One path of the deferred path tracer (DeferredPathTracer.cpp:61-148 shading, 151-230 extension rays,
// 234-279 shadow rays), contributions added to acc as the reference writes them one by one.  Per hit the
// sampler gives: light pick + 2 for the light, 2 for the background direction (drawn whatever the
// background), the BSDF's lobe + 2..3, and one for Russian roulette once 7 bounces are tracked.  The
// reference has no bounce limit; max_bounces caps the segments of a path.
void deferred_path(const Scene& sc, Rng& rng, V3 org, V3 dir, uint32_t max_bounces, double* acc) {
    const float kInv4Pi = 1.0f / (4.0f * kPi);
    V3 thr(1.0f);
    bool dirac_only = true;
    for (uint32_t bounce = 0; bounce < max_bounces; ++bounce) {
        orq::Hit h;
        const float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
        if (!sc_closest(sc, o, d, 0.0f, 3.402823466e+38f, h)) {
            const V3 bg = sc.ibl ? (dirac_only ? sc.ibl->miss_radiance(dir) : sc.ibl->radiance(dir)) : sc.background;
            add(acc, bg * thr);
            break;
        }
        const V3 pos(org.x + h.t * dir.x, org.y + h.t * dir.y, org.z + h.t * dir.z);
        SurfHit sh;
        surface_at(sc, h, pos, dir, sh);
        const Material& m = *sh.m;
        // quad light (NextEventEstimation), weight 1
        V3 ldir, lrad(0.0f);
        float ldist = 0, lpdf = 1;
        if (m.light_set < sc.set_count.size() && sc.set_count[m.light_set] > 0) {
            const uint32_t cnt = sc.set_count[m.light_set];
            const float p0 = rng.uniform();
            const uint32_t li = std::min(uint32_t(p0 * float(cnt)), cnt - 1);
            const float u = rng.uniform(), v = rng.uniform();
            sample_light(sc.lights[sc.set_first[m.light_set] + li], pos, sh.n, u, v, ldir, lrad, ldist, lpdf,
                         sc.physical_nee);
            lpdf *= 1.0f / float(cnt);
        }
        if (orc::Dot(lrad, V3(1.0f)) > 0) {
            float fp, rp;
            const V3 refl = orc::bsdf_evaluate(sh.s, sh.view, ldir, fp, rp);
            const V3 sample = 1.0f * refl * lrad * (1.0f / lpdf);
            if (orc::Dot(sample, V3(1.0f)) > 0) {
                const V3 so = offset(pos, sh.n, sh.err, ldir, 0.1f);
                const float soa[3] = {so.x, so.y, so.z}, lda[3] = {ldir.x, ldir.y, ldir.z};
                if (!sc_occluded(sc, soa, lda, 0.0f, ldist)) add(acc, sample * thr);
            }
        }
        // background (SampleBackground, AreaLighting.cpp:393-401: DirectIblLightSample with an image, else
        // BackgroundLightSample, :334-350, a uniform sphere direction with density recorded as 1), balance
        // heuristic against the BSDF's density
        const float r0 = rng.uniform(), r1 = rng.uniform();
        V3 sdir, srad;
        float spdf;
        if (sc.ibl) {
            sc.ibl->sample(r0, r1, sdir, srad, spdf);
        } else {
            const float uu = 2.0f * r1 - 1.0f;
            const float nn = std::sqrt(std::max(0.0f, 1.0f - uu * uu));
            const float th = 2.0f * kPi * r0;
            sdir = V3(nn * std::cos(th), uu, nn * std::sin(th));
            srad = sc.background;
            spdf = 1.0f;
        }
        if (orc::Dot(srad, V3(1.0f)) > 0) {
            float fp, rp;
            const V3 refl = orc::bsdf_evaluate(sh.s, sh.view, sdir, fp, rp);
            const float mis = (1.0f * spdf) / (1.0f * spdf + 1.0f * fp);
            const V3 sample = mis * refl * srad * (1.0f / spdf);
            if (orc::Dot(sample, V3(1.0f)) > 0) {
                const V3 so = offset(pos, sh.n, sh.err, sdir, 0.1f);
                const float soa[3] = {so.x, so.y, so.z}, sda[3] = {sdir.x, sdir.y, sdir.z};
                if (!sc_occluded(sc, soa, sda, 0.0f, 1e36f)) add(acc, sample * thr);
            }
        }
        // BSDF sample, weighted against the background density 1 / (4 pi)
        float u4[4];
        Rng ahead = rng;
        for (int k = 0; k < 4; ++k) u4[k] = ahead.uniform();
        int used = 0;
        orc::Sample bs;
        const bool ok = orc::bsdf_sample(sh.s, sh.view, u4, used, bs);
        for (int k = 0; k < used; ++k) rng.uniform();
        if (!ok) break;
        const float sky_pdf = sc.ibl ? sc.ibl->pdf(bs.wi) : kInv4Pi;
        const float mis = (1.0f * bs.fwd) / (1.0f * bs.fwd + 1.0f * sky_pdf);
        dirac_only = dirac_only && (bs.flags & 4u);
        V3 t = mis * thr * bs.refl;
        if (orc::Dot(t, t) == 0.0f) break;
        if (bounce >= 7) {  // Russian roulette once MaxTrackedBounces_ = 7 bounces are tracked
            const float cp = std::max(std::max(t.x, t.y), t.z);
            if (rng.uniform() >= cp) break;
            t = t * (1.0f / cp);
        }
        thr = t;
        org = offset(pos, sh.n, sh.err, bs.wi, 1.0f);
        dir = bs.wi;
    }
}

}  // namespace

// Per-pixel render loops shared by the flat and instanced entry points.
static void run_pt(const Scene& sc, const float* camera, uint32_t width, uint32_t height, uint32_t pass_begin,
            uint32_t pass_end, uint32_t max_bounces, uint64_t seed, int rng_mode, int threads, double* out) {
    const Camera cam = make_camera(camera, width, height);
    const uint32_t npix = width * height;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        for (;;) {
            const uint32_t pix0 = next.fetch_add(16);
            if (pix0 >= npix) break;
            for (uint32_t pixel = pix0; pixel < std::min(npix, pix0 + 16); ++pixel) {
                const uint32_t y = pixel / width, x = pixel - y * width;
                Rng rng;
                if (rng_mode == 1) {
                    rng.pcg = false;
                    rng.mt.seed(uint32_t(seed) + pixel);
                }
                double acc[6] = {0, 0, 0, 0, 0, 0};
                for (uint32_t pass = pass_begin; pass < pass_end; ++pass) {
                    if (rng_mode == 0) rng.seed_pcg(seed, uint64_t(pass) * npix + pixel);
                    const float vx = float(x) + rng.uniform();
                    const float vy = float(y) + rng.uniform();
                    const float cx = (vx / cam.w) * 2.0f - 1.0f;
                    const float cy = 1.0f - 2.0f * vy / cam.h;
                    const V3 d = orc::Norm(cam.z - cx * cam.x + cy * cam.y);
                    V3 l0, l1;
                    evaluate_path(sc, rng, cam.pos, d, max_bounces, l0, l1);
                    acc[0] += l0.x; acc[1] += l0.y; acc[2] += l0.z;
                    acc[3] += l1.x; acc[4] += l1.y; acc[5] += l1.z;
                }
                for (int c = 0; c < 3; ++c) {
                    out[size_t(pixel) * 3 + c] += acc[c];
                    out[(size_t(npix) + pixel) * 3 + c] += acc[3 + c];
                }
            }
        }
    };
    std::vector<std::thread> pool;
    const int nt = std::max(1, threads);
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
}

static void run_deferred(const Scene& sc, const float* camera, uint32_t width, uint32_t height, uint32_t samples_per_axis,
                  uint32_t sample_begin, uint32_t sample_end, uint32_t max_bounces, uint64_t seed, int rng_mode,
                  int threads, double* out) {
    const Camera cam = make_camera(camera, width, height);
    const uint32_t npix = width * height;
    const int32_t m = int32_t(samples_per_axis);
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        for (;;) {
            const uint32_t pix0 = next.fetch_add(16);
            if (pix0 >= npix) break;
            for (uint32_t pixel = pix0; pixel < std::min(npix, pix0 + 16); ++pixel) {
                const uint32_t y = pixel / width, x = pixel - y * width;
                double acc[3] = {0, 0, 0};
                Rng rng;
                if (rng_mode == 1) {
                    rng.pcg = false;
                    rng.mt.seed(uint32_t(seed) + pixel);
                }
                for (uint32_t smp = sample_begin; smp < sample_end; ++smp) {
                    if (rng_mode == 0) rng.seed_pcg(seed, uint64_t(smp) * npix + pixel);
                    float jx, jy;
                    cmj(int32_t(smp), m, m, int32_t(pixel), jx, jy);
                    const float vx = float(x) + jx, vy = float(y) + jy;
                    const float cx = (vx / cam.w) * 2.0f - 1.0f;
                    const float cy = 1.0f - 2.0f * vy / cam.h;
                    const V3 d = orc::Norm(cam.z - cx * cam.x + cy * cam.y);
                    deferred_path(sc, rng, cam.pos, d, max_bounces, acc);
                }
                for (int c = 0; c < 3; ++c) out[size_t(pixel) * 3 + c] += acc[c];
            }
        }
    };
    std::vector<std::thread> pool;
    const int nt = std::max(1, threads);
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
}

// The image-based light the renderers use (oracle_set_ibl; none when its width is 0).
static Ibl g_ibl;
// The vertex attributes of the next render's soup (oracle_set_attributes; none when empty).
static Attrs g_attrs;

// Maps each mesh of a soup (triangles of one (scene, geomID) are contiguous, primID counting from 0) to its first
// triangle.
struct Tex2D {
    int w = 0, h = 0;
    std::vector<float> rgba;
};
static std::map<uint64_t, Tex2D> g_tex2d;
static std::map<uint64_t, std::unique_ptr<orp::QuadTexture>> g_quad_ptex;  // (scene, geom) -> quad-mesh Ptex

static void index_attrs(const uint32_t* prim, const uint32_t* geom, const uint32_t* tri_scene, int64_t ntri) {
    g_attrs.first.clear();
    for (int64_t i = 0; i < ntri; ++i)
        if (prim[i] == 0) g_attrs.first[(uint64_t(tri_scene ? tri_scene[i] : 0) << 32) | geom[i]] = i;
}

// Scene tables of the oracle renderers' common arguments; returns the Ptex texture to delete.
static orp::Texture* load_scene(Scene& sc, const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t ntri,
                         const float* materials, int n_materials, const float* lights, int n_lights,
                         const uint32_t* sets, int n_sets, const float* background, const int32_t* ptex_rows,
                         int ptex_faces, const uint16_t* ptex_texels, int physical_nee) {
    sc.physical_nee = physical_nee != 0;
    sc.bvh = orq::build(verts, prim, geom, ntri);
    orp::Texture* tex = ptex_faces > 0 ? new orp::Texture(ptex_rows, ptex_faces, ptex_texels) : nullptr;
    sc.ptex = tex;
    for (int i = 0; i < n_materials; ++i) sc.materials.push_back(read_material(materials + 32 * i));
    for (int i = 0; i < n_lights; ++i) {
        const float* l = lights + 15 * i;
        Light L;
        L.pos = V3(l[0], l[1], l[2]);
        L.dir = V3(l[3], l[4], l[5]);
        L.x = V3(l[6], l[7], l[8]);
        L.z = V3(l[9], l[10], l[11]);
        L.radiance = V3(l[12], l[13], l[14]);
        sc.lights.push_back(L);
    }
    for (int i = 0; i < n_sets; ++i) {
        sc.set_first.push_back(sets[2 * i]);
        sc.set_count.push_back(sets[2 * i + 1]);
    }
    sc.background = V3(background[0], background[1], background[2]);
    sc.ibl = g_ibl.w ? &g_ibl : nullptr;
    if (!g_attrs.flags.empty() && ntri > 0) {
        index_attrs(prim, geom, nullptr, ntri);
        sc.attrs = &g_attrs;
    }
    return tex;
}

extern "C" {

// verts/prim/geom: triangle soup; materials: n_materials x 32 words (MaterialDev layout, indexed by geomID);
// lights: n_lights x 15 floats (position, direction, x, z, radiance); sets: n_sets x 2 (first, count);
// camera: position[3] lookAt[3] up[3] fovDegrees; ptex_rows/ptex_texels: the combined Ptex face table of
// all textured geometries (material word 3 = that geometry's first face); out: [2][height][width][3]
// doubles (sums over the paths of passes [pass_begin, pass_end)).  rng_mode 0: PCG32 streams (as the
// GPU); 1: MT19937 per pixel.  physical_nee drops the extra cos(theta_surface) factor that the reference's
// SampleRectangleLightSolidAngle puts into the NEE radiance (AreaLighting.cpp:140-146), giving the
// physically correct estimator that other integrators (VCM) converge to.
void oracle_pt_render(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t ntri,
                      const float* materials, int n_materials, const float* lights, int n_lights,
                      const uint32_t* sets, int n_sets, const float* background, const float* camera,
                      uint32_t width, uint32_t height, uint32_t pass_begin, uint32_t pass_end, uint32_t max_bounces,
                      uint64_t seed, int rng_mode, int threads, const int32_t* ptex_rows, int ptex_faces,
                      const uint16_t* ptex_texels, int physical_nee, double* out) {
    Scene sc;
    orp::Texture* tex = load_scene(sc, verts, prim, geom, ntri, materials, n_materials, lights, n_lights, sets, n_sets,
                                   background, ptex_rows, ptex_faces, ptex_texels, physical_nee);
    run_pt(sc, camera, width, height, pass_begin, pass_end, max_bounces, seed, rng_mode, threads, out);
    orq::release(const_cast<void*>(sc.bvh));
    delete tex;
}

}  // extern "C"

extern "C" {

// DeferredPathTracer::GenerateImage (DeferredPathTracer.cpp:433-472) over samples [sample_begin, sample_end) of
// each pixel's samples_per_axis^2 correlated multi-jittered samples (SamplesPerPixelX_ = SamplesPerPixelY_ = 4
// in the reference; sample s of pixel p jitters by CorrelatedMultiJitter(s, m, m, p), Camera.cpp:77-86).
// rng_mode 0: PCG32 stream s * width * height + p per path (as the GPU); 1: one MT19937 engine per pixel
// seeded seed + p, drawn as the reference's CSampler (Random.cpp:46-49) over the pixel's samples in order.
// Arguments as oracle_pt_render; out: [height][width][3]
// doubles, the un-normalised sums (the reference scales by 1 / (m * m)).
void oracle_deferred_render(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t ntri,
                            const float* materials, int n_materials, const float* lights, int n_lights,
                            const uint32_t* sets, int n_sets, const float* background, const float* camera,
                            uint32_t width, uint32_t height, uint32_t samples_per_axis, uint32_t sample_begin,
                            uint32_t sample_end, uint32_t max_bounces, uint64_t seed, int rng_mode, int threads,
                            const int32_t* ptex_rows, int ptex_faces, const uint16_t* ptex_texels, int physical_nee,
                            double* out) {
    Scene sc;
    orp::Texture* tex = load_scene(sc, verts, prim, geom, ntri, materials, n_materials, lights, n_lights, sets, n_sets,
                                   background, ptex_rows, ptex_faces, ptex_texels, physical_nee);
    run_deferred(sc, camera, width, height, samples_per_axis, sample_begin, sample_end, max_bounces, seed, rng_mode,
                 threads, out);
    orq::release(const_cast<void*>(sc.bvh));
    delete tex;
}

// Correlated multi-jittered sample points (for tests): n samples s = 0..n-1 of an m x m pattern with p.
void oracle_cmj(int32_t m, int32_t p, int32_t n, float* xy) {
    for (int32_t s = 0; s < n; ++s) cmj(s, m, m, p, xy[2 * s], xy[2 * s + 1]);
}

}  // extern "C"

extern "C" {

// The path tracer (deferred = 0; out [2][height][width][3]) or the deferred path tracer (deferred = 1; out
// [height][width][3]) over an instanced scene graph.  Triangles and instances as oracle_instanced_query (with
// local-to-world rows); scene s has materials[mat_offsets[s] .. mat_offsets[s+1]) (32-word records by geomID)
// and Ptex faces ptex_rows[row_offsets[s] ..) whose texel offsets are relative to texels + texel_offsets[s];
// lights, light sets, background and camera are the top scene's.  PCG32 sampling.
void oracle_graph_render(int n_scenes, const float* verts, const uint32_t* prim, const uint32_t* geom,
                         const uint32_t* tri_scene, int64_t ntri, const float* l2w, const uint32_t* inst_id,
                         const uint32_t* inst_scene, const uint32_t* inst_proto, int64_t ninst, int top,
                         const float* materials, const int32_t* mat_offsets, const int32_t* ptex_rows,
                         const int32_t* row_offsets, const uint16_t* texels, const int64_t* texel_offsets,
                         const float* lights, int n_lights, const uint32_t* sets, int n_sets, const float* background,
                         const float* camera, uint32_t width, uint32_t height, uint32_t begin, uint32_t end,
                         uint32_t max_bounces, uint64_t seed, int threads, int physical_nee, int deferred,
                         uint32_t samples_per_axis, double* out) {
    Scene sc;
    // lights, background and the top scene's tables through the flat loader (no triangles: the graph traces)
    orp::Texture* unused = load_scene(sc, nullptr, nullptr, nullptr, 0, materials + 32 * mat_offsets[top],
                                      mat_offsets[top + 1] - mat_offsets[top], lights, n_lights, sets, n_sets, background,
                                      nullptr, 0, nullptr, physical_nee);
    delete unused;
    if (sc.bvh) orq::release(const_cast<void*>(sc.bvh));
    sc.bvh = nullptr;
    sc.graph = orq::build_graph(n_scenes, verts, prim, geom, tri_scene, ntri, l2w, inst_id, inst_scene, inst_proto,
                                ninst, top);
    if (!g_attrs.flags.empty()) {
        index_attrs(prim, geom, tri_scene, ntri);
        sc.attrs = &g_attrs;
    }
    std::vector<orp::Texture*> owned;
    for (int s = 0; s < n_scenes; ++s) {
        std::vector<Material> mats;
        for (int i = mat_offsets[s]; i < mat_offsets[s + 1]; ++i) mats.push_back(read_material(materials + 32 * i));
        if (mats.empty()) mats.push_back(read_material(materials + 32 * mat_offsets[top]));
        sc.gmats.push_back(mats);
        const int nf = row_offsets[s + 1] - row_offsets[s];
        orp::Texture* t = nf > 0 ? new orp::Texture(ptex_rows + 8 * row_offsets[s], nf, texels + 3 * texel_offsets[s])
                                 : nullptr;
        owned.push_back(t);
        sc.gptex.push_back(t);
    }
    if (deferred)
        run_deferred(sc, camera, width, height, samples_per_axis, begin, end, max_bounces, seed, 0, threads, out);
    else
        run_pt(sc, camera, width, height, begin, end, max_bounces, seed, 0, threads, out);
    orq::release_graph(const_cast<void*>(sc.graph));
    for (orp::Texture* t : owned) delete t;
}

}  // extern "C"

extern "C" {

// Sets (width > 0) or clears the image-based light of the following oracle renders: RGB light image, optional
// miss image (null: the light image times the exposure), rotation in radians, exposure scale.
void oracle_set_ibl(const float* rgb, uint32_t width, uint32_t height, const float* miss_rgb, uint32_t miss_width,
                    uint32_t miss_height, float rotation, float exposure) {
    if (!width) {
        g_ibl = Ibl();
        return;
    }
    g_ibl.build(rgb, width, height, miss_rgb, miss_width, miss_height, rotation, exposure);
}

// IBL sampling for tests: n directions from (r0, r1) pairs (out: dir xyz, radiance rgb, pdf; 7 floats each) and
// the density and radiance the lookups give back for those directions (eval: pdf, rgb, miss rgb; 7 floats).
void oracle_ibl_sample(const float* r, int n, float* out, float* eval) {
    for (int i = 0; i < n; ++i) {
        V3 d, rad;
        float p;
        g_ibl.sample(r[2 * i], r[2 * i + 1], d, rad, p);
        float* o = out + 7 * i;
        o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = rad.x; o[4] = rad.y; o[5] = rad.z; o[6] = p;
        const V3 lr = g_ibl.radiance(d), mr = g_ibl.miss_radiance(d);
        float* e = eval + 7 * i;
        e[0] = g_ibl.pdf(d); e[1] = lr.x; e[2] = lr.y; e[3] = lr.z; e[4] = mr.x; e[5] = mr.y; e[6] = mr.z;
    }
}

// Solid-angle density of directions (n x 3 floats) under the image's sampling.
void oracle_ibl_pdf(const float* dirs, int n, float* out) {
    for (int i = 0; i < n; ++i) out[i] = g_ibl.pdf(V3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
}

}  // extern "C"

extern "C" {

// Vertex attributes of the soup of the next renders (n triangles in the soup's order): corner normals (n x 9),
// corner tangents (n x 12) and flags (1 normals, 2 tangents); n = 0 clears them.
void oracle_set_attributes(int64_t n, const float* normals, const float* tangents, const uint8_t* flags,
                           const float* uvs) {
    g_attrs = Attrs();
    if (n <= 0) return;
    g_attrs.normals.assign(normals, normals + 9 * n);
    g_attrs.tangents.assign(tangents, tangents + 12 * n);
    g_attrs.flags.assign(flags, flags + n);
    if (uvs) g_attrs.uvs.assign(uvs, uvs + 6 * n);
}

// 2D base-colour images of the following renders: n images, image k bound to (scene, geom) = keys[2k], keys[2k+1],
// dims[2k] x dims[2k+1] RGBA texels from rgba + offsets[k].
void oracle_set_textures(int n, const uint32_t* keys, const uint32_t* dims, const int64_t* offsets, const float* rgba) {
    g_tex2d.clear();
    for (int k = 0; k < n; ++k) {
        Tex2D& t = g_tex2d[(uint64_t(keys[2 * k]) << 32) | keys[2 * k + 1]];
        t.w = int(dims[2 * k]);
        t.h = int(dims[2 * k + 1]);
        t.rgba.assign(rgba + offsets[k], rgba + offsets[k] + size_t(t.w) * t.h * 4);
    }
}

// Quad-mesh Ptex textures of the following renders: n textures, texture k bound to (scene, geom) = keys[2k],
// keys[2k + 1], its face rows (10 ints each) rows[row_offsets[k] .. row_offsets[k + 1]) and half RGB texels
// texels[texel_offsets[k] .. texel_offsets[k + 1]) (in halfs).
void oracle_set_quad_ptex(int n, const uint32_t* keys, const int64_t* row_offsets, const int32_t* rows,
                          const int64_t* texel_offsets, const uint16_t* texels) {
    g_quad_ptex.clear();
    for (int k = 0; k < n; ++k)
        g_quad_ptex[(uint64_t(keys[2 * k]) << 32) | keys[2 * k + 1]] = std::make_unique<orp::QuadTexture>(
            rows + 10 * row_offsets[k], int(row_offsets[k + 1] - row_offsets[k]), texels + texel_offsets[k],
            size_t(texel_offsets[k + 1] - texel_offsets[k]));
}

}  // extern "C"

namespace ora {

bool quad_ptex(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, float rgb[3]) {
    const auto it = g_quad_ptex.find((uint64_t(scene) << 32) | geom);
    if (it == g_quad_ptex.end()) return false;
    // soup triangle 2q + half of quad q: Embree's quad (u, v) is (1 - u, 1 - v) on the second half
    const bool second = (prim & 1u) != 0u;
    it->second->eval(int(prim >> 1), second ? 1.0f - u : u, second ? 1.0f - v : v, rgb);
    return true;
}

float corner_interp(const std::vector<float>& arr, int per, int64_t tri, uint8_t flags, uint32_t prim, float u, float v,
                    int k) {
    if (!(flags & 8u)) {
        const float* c = &arr[size_t(tri) * 3 * per];
        const float w = 1.0f - u - v;
        return w * c[k] + u * c[per + k] + v * c[2 * per + k];
    }
    const int64_t first = tri - int64_t(prim & 1u);  // soup triangle 2q: (v0, v1, v3); 2q + 1: (v2, v3, v1)
    const float* c0 = &arr[size_t(first) * 3 * per];
    const float* c1 = &arr[size_t(first + 1) * 3 * per];
    const float qu = (prim & 1u) ? 1.0f - u : u, qv = (prim & 1u) ? 1.0f - v : v;
    const float iu = 1.0f - qu, iv = 1.0f - qv;
    return iv * (iu * c0[k] + qu * c0[per + k]) + qv * (iu * c0[2 * per + k] + qu * c1[k]);
}

bool tex2d(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, float rgb[3]) {
    const auto it = g_tex2d.find((uint64_t(scene) << 32) | geom);
    if (it == g_tex2d.end() || it->second.w <= 0 || it->second.h <= 0) return false;
    const Tex2D& t = it->second;
    float su = 0.0f, sv = 0.0f;
    const auto f = g_attrs.first.find((uint64_t(scene) << 32) | geom);
    if (f != g_attrs.first.end() && !g_attrs.uvs.empty()) {
        const int64_t tri = f->second + prim;
        const uint8_t fl = g_attrs.flags[size_t(tri)];
        if ((fl & 4u) != 0) {
            su = corner_interp(g_attrs.uvs, 2, tri, fl, prim, u, v, 0);
            sv = corner_interp(g_attrs.uvs, 2, tri, fl, prim, u, v, 1);
        }
    }
    // Repeat (TextureFiltering.h:32-44): `s % w` with s int32 and w uint32 takes the remainder of s converted
    // to unsigned, so a negative coordinate c reads texel (2^32 + c) mod w.
    auto texel = [&](int s, int tt, int ch) {
        const uint32_t ss = uint32_t(s) % uint32_t(t.w), ts = uint32_t(tt) % uint32_t(t.h);
        return t.rgba[(size_t(ts) * uint32_t(t.w) + ss) * 4 + ch];
    };
    const float s = su * float(t.w) - 0.5f, tt = sv * float(t.h) - 0.5f;
    const int s0 = int(std::floor(s)), t0 = int(std::floor(tt));
    const float ds = s - float(s0), dt = tt - float(t0);
    for (int c = 0; c < 3; ++c) {
        const float x = (1.0f - ds) * (1.0f - dt) * texel(s0, t0, c) + (1.0f - ds) * dt * texel(s0, t0 + 1, c) +
                        ds * (1.0f - dt) * texel(s0 + 1, t0, c) + ds * dt * texel(s0 + 1, t0 + 1, c);
        rgb[c] = x <= 0.04045f ? x / 12.92f : std::pow((x + 0.055f) / (1.0f + 0.055f), 2.4f);
    }
    return true;
}

bool env_present() { return g_ibl.w != 0; }

void env_direction(float r0, float r1, float r2, float r3, float dir[3]) {
    const V3 d = g_ibl.env_direction(r0, r1, r2, r3);
    dir[0] = d.x; dir[1] = d.y; dir[2] = d.z;
}

float env_pdf(const float dir[3]) { return g_ibl.env_pdf(V3(dir[0], dir[1], dir[2])); }

void env_radiance(const float dir[3], float rad[3]) {
    const V3 r = g_ibl.radiance(V3(dir[0], dir[1], dir[2]));
    rad[0] = r.x; rad[1] = r.y; rad[2] = r.z;
}

void env_miss(const float dir[3], float rad[3]) {
    const V3 r = g_ibl.miss_radiance(V3(dir[0], dir[1], dir[2]));
    rad[0] = r.x; rad[1] = r.y; rad[2] = r.z;
}

bool index(const uint32_t* prim, const uint32_t* geom, const uint32_t* tri_scene, int64_t ntri) {
    if (g_attrs.flags.empty() || ntri <= 0) return false;
    index_attrs(prim, geom, tri_scene, ntri);
    return true;
}

void frame(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, const float ng[3], float n[3], float t[3],
           float b[3]) {
    frame_through(scene, geom, prim, u, v, ng, nullptr, nullptr, n, t, b);
}

void frame_through(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, const float ng[3], const float* l2w0,
                   const float* l2w1, float n[3], float t[3], float b[3]) {
    orq::Hit h;
    h.l2w[0] = l2w0;
    h.l2w[1] = l2w1;
    h.u = u;
    h.v = v;
    h.prim = prim;
    h.geom = geom;
    h.scene = scene;
    for (int k = 0; k < 3; ++k) h.ng[k] = ng[k];
    Scene sc;
    sc.attrs = g_attrs.flags.empty() ? nullptr : &g_attrs;
    V3 nn, tt, bb;
    shading_frame(sc, h, nn, tt, bb);
    n[0] = nn.x; n[1] = nn.y; n[2] = nn.z;
    t[0] = tt.x; t[1] = tt.y; t[2] = tt.z;
    b[0] = bb.x; b[1] = bb.y; b[2] = bb.z;
}

}  // namespace ora
