// ORACLE - test infrastructure only (see oracle_query.cpp).
//
// CPU vertex connection and merging, the checker for the GPU VCM integrator.  The reference's VCM
// (Source/Applications/Selas/Source/VCM.cpp) is commented out, emits only from an IBL, reads fields that no
// longer exist and carries estimator errors (BSDF values that already include the cosine multiplied by it
// again, forward/reverse pdfs swapped at light vertices, Russian roulette without compensation, a surface
// density conversion without the surface cosine and distance).  This file therefore restates the published
// algorithm the reference cites (Georgiev, Krivanek, Davidovic, Slusallek, "Implementing Vertex Connection
// and Merging", 2012 technical report) on the reference's scene model, keeping the reference's structure:
//   iteration constants       VCMCommon.cpp:91-112 (radius r_i = r0 / i^((1-alpha)/2), eta = pi r^2 N)
//   light / camera sub-paths  VCMCommon.cpp:37-89, VCM.cpp:502-666
//   hash grid                 VCMHashGrid.cpp:15-155 (cells of 2r over the vertex bounds widened by r,
//                             3-prime hash, counting sort, 2x2x2 cell search)
// with the reference's lights: quad lights that NEE and light tracing use but that camera and BSDF rays
// never hit, so the strategy "camera path hits the emitter" does not exist for them and its MIS terms are
// zero (dVC = dVM = 0 at the emitter, wLight = 0 in next-event estimation), as for delta lights.  The
// image-based light, the reference VCM's only emitter (GenerateLightSample, VCMCommon.cpp:37-62), is an
// environment emitter (tech report sec. 5.1, the infinite light): light sub-paths start on a disc of the
// scene's bounding-sphere radius facing a sampled direction (EmitIblLightSample, AreaLighting.cpp:246-290),
// next-event estimation samples it, and camera paths that leave the scene take its radiance with the
// camera-hit weight (ConnectToSkyLight, VCM.cpp:171-187).  It is one more light in the uniform light pick.
// Its directions are drawn from the image's CDFs and jittered within the texel (ora::env_direction), so the
// density a strategy weighs with is the one it sampled with.  The BSDF is the reference Disney model
// (oracle_bsdf.cpp), whose evaluation returns f * |cos(l)|.  Quad lights come from light set 0; a uniform
// background is not an emitter here.  Random numbers: PCG32, stream (2 * iteration + 0) * N + p for light
// path p and (2 * iteration + 1) * N + p for camera path p.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle_attrs.h"
#include "oracle_bsdf.h"
#include "oracle_env.h"
#include "oracle_ptex.h"
#include "oracle_query.h"

using orc::V3;

namespace {

const float kPi = 3.141592653589793f;

struct Rng {
    uint64_t state, inc;
    uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        const uint32_t xs = uint32_t(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = uint32_t(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    void seed(uint64_t s, uint64_t stream) {
        state = 0;
        inc = (stream << 1u) | 1u;
        next();
        state += s;
        next();
    }
    float uniform() { return float(next() >> 8) * (1.0f / 16777216.0f); }
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
    std::memcpy(&m.shader, r + 0, 4);
    std::memcpy(&m.flags, r + 1, 4);
    std::memcpy(&m.light_set, r + 2, 4);
    std::memcpy(&m.ptex_base, r + 3, 4);
    for (int i = 0; i < 3; ++i) { m.base[i] = r[4 + i]; m.trans[i] = r[7 + i]; }
    m.sheen = r[10]; m.sheenTint = r[11]; m.clearcoat = r[12]; m.clearcoatGloss = r[13];
    m.metallic = r[14]; m.specTrans = r[15]; m.diffTrans = r[16]; m.flatness = r[17];
    m.anisotropic = r[18]; m.specularTint = r[19]; m.roughness = r[20]; m.scatterDistance = r[21]; m.ior = r[22];
    return m;
}

struct Light {
    V3 pos, dir, x, z, radiance;
};

struct Camera {
    V3 x, y, z, pos;
    float w, h;
    float image_plane;  // distance at which a pixel has unit area
};

float Sat(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

V3 offset(V3 p, V3 n, float err, V3 dir, float scale) {
    const float side = orc::Dot(dir, n) < 0.0f ? -1.0f : 1.0f;
    return p + (side * err * scale) * n;
}

struct Scene {
    const void* bvh = nullptr;
    const void* graph = nullptr;                // instanced scene graph (replaces bvh when set)
    std::vector<std::vector<Material>> gmats;   // graph: materials of each scene, by geomID
    std::vector<const orp::Texture*> gptex;     // graph: Ptex of each scene (null: none)
    const orp::Texture* ptex = nullptr;
    std::vector<Material> materials;
    std::vector<Light> lights;  // light set 0
    Camera cam;
    uint32_t max_len;
    bool env = false;          // the image-based light emits (one light after the quads)
    V3 center;                 // bounding sphere of the scene's bounding box
    float radius = 0.0f;
    float disc_pdf = 0.0f;     // ConcentricDiscPdf / radius^2: area density of the emission disc
};

// MakeOrthogonalCoordinateSystem (GeometryLib/CoordinateSystem.h:14-21)
void basis(V3 v1, V3& v2, V3& v3) {
    if (std::fabs(v1.x) > std::fabs(v1.y))
        v2 = V3(-v1.z, 0.0f, v1.x) * (1.0f / std::sqrt(v1.x * v1.x + v1.z * v1.z));
    else
        v2 = V3(0.0f, v1.z, -v1.y) * (1.0f / std::sqrt(v1.y * v1.y + v1.z * v1.z));
    v3 = orc::Cross(v1, v2);
}

// Concentric map of the unit square onto the unit disc (Shirley and Chiu, "A Low Distortion Map Between Disk
// and Square", 1997), the disc sample of EmitIblLightSample.
void concentric_disc(float r0, float r1, float& u, float& v) {
    const float a = 2.0f * r0 - 1.0f, b = 2.0f * r1 - 1.0f;
    if (a == 0.0f && b == 0.0f) {
        u = 0.0f;
        v = 0.0f;
        return;
    }
    float r, phi;
    if (std::fabs(a) > std::fabs(b)) {
        r = a;
        phi = (kPi / 4.0f) * (b / a);
    } else {
        r = b;
        phi = kPi / 2.0f - (kPi / 4.0f) * (a / b);
    }
    u = r * std::cos(phi);
    v = r * std::sin(phi);
}

// Surface at a hit (CalculateSurfaceParams without normals/tangents/uvs, as the path tracers use).
struct Hit {
    V3 pos, n, view;
    float err;
    orc::Surf s;
    float cont;  // ContinuationProbability (SurfaceParameters.cpp:420-424)
    bool delta;
    bool transparent;  // material flag eTransparent
};

// Instanced graphs (ModelDataFromRayIds, SceneResource.cpp:362-378): the hit mesh's scene gives the material,
// Ptex and vertex attributes; its object-space normal goes through the instances' localToWorld.
bool make_hit(const Scene& sc, V3 org, V3 dir, Hit& out) {
    orq::Hit h;
    const float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
    if (sc.graph ? !orq::closest_graph(sc.graph, o, d, 0.0f, 3.402823466e+38f, h)
                 : !orq::closest(sc.bvh, o, d, 0.0f, 3.402823466e+38f, h))
        return false;
    const std::vector<Material>& mats = sc.graph ? sc.gmats[h.scene] : sc.materials;
    const orp::Texture* ptex = sc.graph ? sc.gptex[h.scene] : sc.ptex;
    const Material& m = mats[h.geom < mats.size() ? h.geom : 0];
    out.pos = V3(org.x + h.t * dir.x, org.y + h.t * dir.y, org.z + h.t * dir.z);
    out.err = 32.0f * 1.19209e-07f * std::max(std::max(std::fabs(out.pos.x), std::fabs(out.pos.y)),
                                              std::max(std::fabs(out.pos.z), h.t));
    // shading frame, with vertex normals and tangents where the mesh has them (SurfaceParameters.cpp:157-184)
    float fn[3], ft[3], fb[3];
    ora::frame_through(h.scene, h.geom, h.prim, h.u, h.v, h.ng, h.l2w[0], h.l2w[1], fn, ft, fb);
    const V3 n(fn[0], fn[1], fn[2]);
    orc::Surf& s = out.s;
    s.t = V3(ft[0], ft[1], ft[2]); s.n = n; s.b = V3(fb[0], fb[1], fb[2]);
    float base[3] = {m.base[0], m.base[1], m.base[2]};
    if ((m.flags & 2u) && ora::quad_ptex(h.scene, h.geom, h.prim, h.u, h.v, base)) {
    } else if ((m.flags & 2u) && ptex) {
        ptex->eval(int(m.ptex_base + h.prim), h.u, h.v, base);
    } else {
        ora::tex2d(h.scene, h.geom, h.prim, h.u, h.v, base);
    }
    s.baseColor = V3(std::pow(base[0], 2.2f), std::pow(base[1], 2.2f), std::pow(base[2], 2.2f));
    s.transmittanceColor = V3(m.trans[0], m.trans[1], m.trans[2]);
    s.sheen = m.sheen; s.sheenTint = m.sheenTint; s.clearcoat = m.clearcoat; s.clearcoatGloss = m.clearcoatGloss;
    s.specTrans = Sat(m.specTrans); s.diffTrans = m.diffTrans * 0.5f; s.flatness = m.flatness;
    s.anisotropic = m.anisotropic; s.specularTint = m.specularTint; s.roughness = m.roughness;
    s.metallic = Sat(m.metallic); s.scatterDistance = m.scatterDistance; s.ior = m.ior; s.shader = m.shader;
    out.view = -1.0f * dir;
    s.relativeIOR = ((m.flags & 1u) && orc::Dot(out.view, n) < 0.0f) ? s.ior : 1.0f / s.ior;
    out.n = n;
    out.cont = Sat(std::max(std::max(s.baseColor.x, s.baseColor.y), s.baseColor.z));
    out.delta = s.shader == 2;
    out.transparent = (m.flags & 1u) != 0;
    return true;
}

struct PathState {
    V3 org, dir, thr;
    float dVCM, dVC, dVM;
    uint32_t len;
    bool delta_only = true;  // camera path: every vertex so far is a Dirac surface
};

struct LightVertex {
    Hit hit;
    V3 thr;
    float dVCM, dVC, dVM;
    uint32_t len;
};

struct Consts {
    float radius, radius2, vm_norm, vm_weight, vc_weight;
    float n_paths;
};

// BSDF sampling with Russian roulette and the partial-weight recursion (VCM.cpp:407-433 structure,
// tech report eq. 38-40).
//
// The reference BSDF is not reciprocal (the retro-reflection term, Disney.cpp:241-261, is not symmetric in
// v and l), and every evaluation here is oriented f(v = camera side, l = light side), as the reference's
// vertex connection and merging evaluate it (VCM.cpp:304-319,387).  A light sub-path samples its next
// direction d with the reference sampler from the incoming direction, whose weight is f(view, d) * cos / pdf;
// its throughput takes the adjoint weight, that weight times f(d, view) / f(view, d) per channel (the sampled
// value itself where either evaluation is zero or the event is a Dirac one).
bool scatter(Rng& rng, const Hit& h, const Consts& c, PathState& st, bool light_path) {
    float u4[4];
    Rng ahead = rng;
    for (int k = 0; k < 4; ++k) u4[k] = ahead.uniform();
    int used = 0;
    orc::Sample bs;
    const bool ok = orc::bsdf_sample(h.s, h.view, u4, used, bs);
    for (int k = 0; k < used; ++k) rng.uniform();
    if (!ok) return false;
    if (bs.refl.x == 0.0f && bs.refl.y == 0.0f && bs.refl.z == 0.0f) return false;
    if (rng.uniform() > h.cont) return false;
    V3 weight = bs.refl;
    if (light_path && !h.delta && !(bs.flags & 4u)) {
        float a0, a1, b0, b1;
        const V3 adj = orc::bsdf_evaluate(h.s, bs.wi, h.view, a0, a1);  // f(d, view) |cos view|
        const V3 fw = orc::bsdf_evaluate(h.s, h.view, bs.wi, b0, b1);   // f(view, d) |cos d|
        const float cv = std::fabs(orc::Dot(h.n, h.view)), cd = std::fabs(orc::Dot(h.n, bs.wi));
        const float k = cv > 0.0f ? cd / cv : 0.0f;
        weight.x = (adj.x > 0.0f && fw.x > 0.0f) ? bs.refl.x * (adj.x * k / fw.x) : bs.refl.x;
        weight.y = (adj.y > 0.0f && fw.y > 0.0f) ? bs.refl.y * (adj.y * k / fw.y) : bs.refl.y;
        weight.z = (adj.z > 0.0f && fw.z > 0.0f) ? bs.refl.z * (adj.z * k / fw.z) : bs.refl.z;
    }
    const float fwd = bs.fwd * h.cont, rev = bs.rev * h.cont;
    const float cos_out = std::fabs(orc::Dot(bs.wi, h.n));
    if (h.delta) {
        st.dVCM = 0.0f;
        st.dVC *= cos_out;
        st.dVM *= cos_out;
    } else {
        st.dVC = (cos_out / fwd) * (st.dVC * rev + st.dVCM + c.vm_weight);
        st.dVM = (cos_out / fwd) * (st.dVM * rev + st.dVCM * c.vc_weight + 1.0f);
        st.dVCM = 1.0f / fwd;
    }
    st.thr = st.thr * weight * (1.0f / h.cont);
    st.org = offset(h.pos, h.n, h.err, bs.wi, 1.0f);
    st.dir = bs.wi;
    st.len += 1;
    return true;
}

bool visible(const Scene& sc, const Hit& h, V3 dir, float tfar) {
    const V3 o = offset(h.pos, h.n, h.err, dir, 0.1f);
    const float oa[3] = {o.x, o.y, o.z}, da[3] = {dir.x, dir.y, dir.z};
    return sc.graph ? !orq::occluded_graph(sc.graph, oa, da, h.err, tfar) : !orq::occluded(sc.bvh, oa, da, h.err, tfar);
}

// World position -> pixel (inverse of ImageToWorldDirection, GeometryLib/Camera.cpp:56-60).
bool to_pixel(const Camera& cam, V3 p, int& px, int& py) {
    const V3 d = p - cam.pos;
    const float dz = orc::Dot(d, cam.z);
    if (dz <= 0.0f) return false;
    const float cx = -orc::Dot(d, cam.x) / (dz * orc::Dot(cam.x, cam.x));
    const float cy = orc::Dot(d, cam.y) / (dz * orc::Dot(cam.y, cam.y));
    const float fx = (cx + 1.0f) * 0.5f * cam.w, fy = (1.0f - cy) * 0.5f * cam.h;
    if (!(fx >= 0.0f && fx < cam.w && fy >= 0.0f && fy < cam.h)) return false;
    px = int(fx);
    py = int(fy);
    return true;
}

struct Grid {
    V3 lo, hi;
    float inv_cell, radius2;
    uint32_t cells;
    std::vector<uint32_t> ends, index;
};

uint32_t cell_hash(int x, int y, int z, uint32_t cells) {
    const uint32_t ux = uint32_t(x), uy = uint32_t(y), uz = uint32_t(z);
    return ((ux * 73856093u) ^ (uy * 19349663u) ^ (uz * 83492791u)) % cells;
}

uint32_t cell_of(const Grid& g, V3 p) {
    const V3 f = p - g.lo;
    return cell_hash(int(std::floor(g.inv_cell * f.x)), int(std::floor(g.inv_cell * f.y)),
                     int(std::floor(g.inv_cell * f.z)), g.cells);
}

// BuildHashGrid (VCMHashGrid.cpp:48-96)
void build_grid(Grid& g, const std::vector<LightVertex>& v, uint32_t cells, float radius) {
    g.radius2 = radius * radius;
    g.inv_cell = 1.0f / (2.0f * radius);
    g.cells = cells;
    g.lo = V3(INFINITY);
    g.hi = V3(-INFINITY);
    for (const LightVertex& lv : v) {
        g.lo = V3(std::min(g.lo.x, lv.hit.pos.x), std::min(g.lo.y, lv.hit.pos.y), std::min(g.lo.z, lv.hit.pos.z));
        g.hi = V3(std::max(g.hi.x, lv.hit.pos.x), std::max(g.hi.y, lv.hit.pos.y), std::max(g.hi.z, lv.hit.pos.z));
    }
    // bounds widened by the radius, the correction the reference leaves commented out
    // (VCMHashGrid.cpp:69-72): without it a camera vertex on a bounding plane of the vertex set (a wall of
    // a closed room) fails the range test about half the time and its merges are lost
    g.lo = g.lo - V3(radius);
    g.hi = g.hi + V3(radius);
    g.ends.assign(cells, 0);
    g.index.assign(v.size(), 0);
    for (const LightVertex& lv : v) ++g.ends[cell_of(g, lv.hit.pos)];
    uint32_t sum = 0;
    for (uint32_t c = 0; c < cells; ++c) {
        const uint32_t n = g.ends[c];
        g.ends[c] = sum;
        sum += n;
    }
    for (size_t i = 0; i < v.size(); ++i) g.index[g.ends[cell_of(g, v[i].hit.pos)]++] = uint32_t(i);
}

}  // namespace

// The passes of a VCM render over a set-up scene (shared by the flat and the instanced entry points).
static void vcm_passes(Scene& sc, const float* camera, uint32_t width, uint32_t height, uint32_t iter_begin,
                       uint32_t iter_end, float radius0, float alpha, uint64_t seed, int threads, int merging,
                       int strategies, double* out) {
    // strategies: bit 0 next-event estimation, 1 vertex connection, 2 vertex merging, 3 light tracing (15: all,
    // MIS-weighted, with camera paths hitting the environment); otherwise the enabled strategies are weighted 1
    // (unweighted estimators of their own paths), and bit 4 adds camera paths hitting the environment
    const bool single = (strategies & 15) != 15;
    const bool use_nee = strategies & 1, use_vc = strategies & 2, use_vm = strategies & 4, use_lt = strategies & 8;
    const bool use_hit = !single || (strategies & 16);
    const uint32_t nq = uint32_t(sc.lights.size());
    const uint32_t n_emitters = nq + (sc.env ? 1u : 0u);
    {  // InitializeRayCastCamera (GeometryLib/Camera.cpp:89-115); the pixel-area image plane uses tan(fov/2)
        const float aspect = float(width) / float(height);
        const float hfov = camera[9] * (kPi / 180.0f);
        const float hlen = std::tan(hfov * 0.5f);
        const float vlen = std::tan(2.0f * std::atan(hlen / aspect) * 0.5f);
        const V3 pos(camera[0], camera[1], camera[2]);
        const V3 fwd = orc::Norm(V3(camera[3], camera[4], camera[5]) - pos);
        const V3 right = orc::Norm(orc::Cross(V3(camera[6], camera[7], camera[8]), fwd));
        sc.cam.x = hlen * right;
        sc.cam.y = vlen * orc::Cross(fwd, right);
        sc.cam.z = fwd;
        sc.cam.pos = pos;
        sc.cam.w = float(width);
        sc.cam.h = float(height);
        sc.cam.image_plane = float(width) / (2.0f * hlen);
    }
    const uint32_t N = width * height;
    const int nt = std::max(1, threads);
    std::vector<std::vector<double>> lt_images(size_t(nt), std::vector<double>(size_t(N) * 3, 0.0));
    const float light_pick = n_emitters == 0 ? 0.0f : 1.0f / float(n_emitters);

    for (uint32_t it = iter_begin; it < iter_end; ++it) {
        Consts c;
        c.radius = radius0 / std::pow(float(it + 1), 0.5f * (1.0f - alpha));
        c.radius2 = c.radius * c.radius;
        c.n_paths = float(N);
        const float eta = kPi * c.radius2 * c.n_paths;
        c.vm_weight = merging ? eta : 0.0f;  // without merging: bidirectional path tracing weights
        c.vc_weight = 1.0f / eta;
        c.vm_norm = 1.0f / eta;

        // ---- light sub-paths
        std::vector<std::vector<LightVertex>> per_path(N);
        std::atomic<uint32_t> next{0};
        auto light_worker = [&](int tid) {
            std::vector<double>& img = lt_images[size_t(tid)];
            for (;;) {
                const uint32_t p = next.fetch_add(1);
                if (p >= N) break;
                if (n_emitters == 0) continue;
                Rng rng;
                rng.seed(seed, (uint64_t(it) * 2 + 0) * N + p);
                const float pick = rng.uniform();
                const uint32_t li = std::min(uint32_t(pick * float(n_emitters)), n_emitters - 1);
                PathState st;
                bool area_start = true;
                if (li == nq) {
                    // EmitIblLightSample (AreaLighting.cpp:246-290): a direction toward the environment, the ray
                    // entering the scene from a disc of the bounding-sphere radius facing it
                    const float r0 = rng.uniform(), r1 = rng.uniform(), r2 = rng.uniform(), r3 = rng.uniform();
                    const float r4 = rng.uniform(), r5 = rng.uniform();
                    float d[3], rad[3];
                    ora::env_direction(r0, r1, r2, r3, d);
                    const float pdf_w = ora::env_pdf(d);
                    if (!(pdf_w > 0.0f)) continue;
                    ora::env_radiance(d, rad);
                    const V3 to_env(d[0], d[1], d[2]);
                    float du, dv;
                    concentric_disc(r4, r5, du, dv);
                    V3 dx, dz;
                    basis(to_env, dx, dz);
                    const float emission_pdf = pdf_w * sc.disc_pdf * light_pick;
                    const float direct_pdfA = pdf_w * light_pick;
                    st.org = sc.center + sc.radius * (to_env + du * dx + dv * dz);
                    st.dir = -1.0f * to_env;
                    st.thr = V3(rad[0], rad[1], rad[2]) * (1.0f / emission_pdf);
                    st.dVCM = direct_pdfA / emission_pdf;
                    st.dVC = 1.0f / emission_pdf;  // cos at an infinite light: 1
                    st.dVM = st.dVC * c.vc_weight;
                    area_start = false;            // no distance term on the first segment
                } else {
                    // GenerateLightSample for a quad light: uniform point, cosine-weighted direction
                    const Light& L = sc.lights[li];
                    const float u = rng.uniform(), v = rng.uniform();
                    const V3 lp = L.pos - 0.5f * L.x - 0.5f * L.z + u * L.x + v * L.z;
                    const float pdfA = 1.0f / (orc::Len(L.x) * orc::Len(L.z));
                    const V3 ln = orc::Norm(L.dir);
                    V3 lt, lb;
                    basis(ln, lt, lb);
                    const float r0 = rng.uniform(), r1 = rng.uniform();
                    const float rr = std::sqrt(r0), ph = 2.0f * kPi * r1;
                    const float cosl = std::sqrt(std::max(0.0f, 1.0f - r0));
                    const V3 dir = orc::Norm(rr * std::cos(ph) * lt + cosl * ln + rr * std::sin(ph) * lb);
                    if (!(cosl > 0.0f)) continue;
                    const float emission_pdf = pdfA * cosl / kPi * light_pick;
                    const float direct_pdfA = pdfA * light_pick;
                    st.org = lp;
                    st.dir = dir;
                    st.thr = L.radiance * (cosl / emission_pdf);
                    st.dVCM = direct_pdfA / emission_pdf;
                    st.dVC = 0.0f;  // the emitter cannot be hit by camera or BSDF rays
                    st.dVM = 0.0f;
                }
                st.len = 1;
                while (st.len + 2 <= sc.max_len + 1) {
                    Hit h;
                    if (!make_hit(sc, st.org, st.dir, h)) break;
                    const float d2 = orc::Dot(h.pos - st.org, h.pos - st.org);
                    const float cos_in = std::fabs(orc::Dot(h.n, h.view));
                    if (st.len > 1 || area_start) st.dVCM *= d2;
                    area_start = false;
                    st.dVCM *= 1.0f / cos_in;
                    st.dVC *= 1.0f / cos_in;
                    st.dVM *= 1.0f / cos_in;
                    if (!h.delta) {
                        per_path[p].push_back({h, st.thr, st.dVCM, st.dVC, st.dVM, st.len});
                        // light tracing: connect to the camera (tech report sec. 5.3)
                        if (use_lt && st.len + 1 <= sc.max_len) {
                            int px, py;
                            if (to_pixel(sc.cam, h.pos, px, py)) {
                                V3 to_cam = sc.cam.pos - h.pos;
                                const float dist2 = orc::Dot(to_cam, to_cam);
                                const float dist = std::sqrt(dist2);
                                to_cam = to_cam * (1.0f / dist);
                                const float cos_cam = orc::Dot(sc.cam.z, -1.0f * to_cam);
                                // the reference BSDF is not reciprocal: evaluate f(wo = toward the camera, wi = toward
                                // the light) and carry the cosine on the camera side
                                float cam_side_pdf, light_side_pdf;
                                const V3 fa = orc::bsdf_evaluate(h.s, to_cam, h.view, cam_side_pdf, light_side_pdf);
                                const float cos_view = std::fabs(orc::Dot(h.n, h.view));
                                const V3 f = cos_view > 0.0f ? fa * (std::fabs(orc::Dot(h.n, to_cam)) / cos_view) : V3(0.0f);
                                float rev = cam_side_pdf;
                                if ((f.x != 0.0f || f.y != 0.0f || f.z != 0.0f) && cos_cam > 0.0f) {
                                    rev *= h.cont;
                                    const float ip = sc.cam.image_plane / cos_cam;
                                    const float img_to_solid = ip * ip / cos_cam;
                                    const float cos_surf = std::fabs(orc::Dot(h.n, to_cam));
                                    const float camera_pdfA = img_to_solid * cos_surf / dist2;
                                    const float w_light = (camera_pdfA / c.n_paths) * (c.vm_weight + st.dVCM + st.dVC * rev);
                                    const float mis = single ? 1.0f : 1.0f / (w_light + 1.0f);
                                    const V3 contrib = (mis * img_to_solid / (c.n_paths * dist2)) * (st.thr * f);
                                    if (visible(sc, h, to_cam, dist * (1.0f - 1e-4f))) {
                                        const size_t pix = size_t(py) * width + px;
                                        img[pix * 3] += contrib.x;
                                        img[pix * 3 + 1] += contrib.y;
                                        img[pix * 3 + 2] += contrib.z;
                                    }
                                }
                            }
                        }
                    }
                    if (st.len + 2 > sc.max_len) break;
                    if (!scatter(rng, h, c, st, true)) break;
                }
            }
        };
        {
            std::vector<std::thread> pool;
            for (int t = 0; t < nt; ++t) pool.emplace_back(light_worker, t);
            for (auto& th : pool) th.join();
        }
        std::vector<LightVertex> verts_all;
        std::vector<uint32_t> path_begin(N + 1, 0);
        for (uint32_t p = 0; p < N; ++p) {
            path_begin[p] = uint32_t(verts_all.size());
            verts_all.insert(verts_all.end(), per_path[p].begin(), per_path[p].end());
        }
        path_begin[N] = uint32_t(verts_all.size());
        Grid grid;
        build_grid(grid, verts_all, N, c.radius);

        // ---- camera sub-paths
        next = 0;
        auto camera_worker = [&](int tid) {
            (void)tid;
            for (;;) {
                const uint32_t p = next.fetch_add(1);
                if (p >= N) break;
                Rng rng;
                rng.seed(seed, (uint64_t(it) * 2 + 1) * N + p);
                const uint32_t y = p / width, x = p - y * width;
                const float vx = float(x) + rng.uniform(), vy = float(y) + rng.uniform();
                const float cx = (vx / sc.cam.w) * 2.0f - 1.0f, cy = 1.0f - 2.0f * vy / sc.cam.h;
                const V3 d = orc::Norm(sc.cam.z - cx * sc.cam.x + cy * sc.cam.y);
                const float cos_cam = orc::Dot(sc.cam.z, d);
                const float ip = sc.cam.image_plane / cos_cam;
                const float camera_pdfW = ip * ip / cos_cam;
                PathState st;
                st.org = sc.cam.pos;
                st.dir = d;
                st.thr = V3(1.0f);
                st.dVCM = c.n_paths / camera_pdfW;
                st.dVC = 0.0f;
                st.dVM = 0.0f;
                st.len = 1;
                V3 color(0.0f);
                for (;;) {
                    Hit h;
                    if (!make_hit(sc, st.org, st.dir, h)) {
                        // the path leaves the scene: the environment's radiance with the camera-hit weight
                        // (ConnectToSkyLight, VCM.cpp:171-187; tech report sec. 5.2); camera rays and chains of
                        // Dirac vertices see the miss image, with weight 1 (no other strategy makes them)
                        if (sc.env && use_hit) {
                            const float d[3] = {st.dir.x, st.dir.y, st.dir.z};
                            float rad[3];
                            if (st.delta_only) ora::env_miss(d, rad);
                            else ora::env_radiance(d, rad);
                            float mis = 1.0f;
                            if (st.len > 1 && !single) {
                                const float pdf_w = ora::env_pdf(d);
                                const float direct_pdfA = pdf_w * light_pick;
                                const float emission_pdf = pdf_w * sc.disc_pdf * light_pick;
                                const float w_camera = direct_pdfA * st.dVCM + emission_pdf * st.dVC;
                                mis = 1.0f / (1.0f + w_camera);
                            }
                            color = color + mis * (st.thr * V3(rad[0], rad[1], rad[2]));
                        }
                        break;
                    }
                    const float d2 = orc::Dot(h.pos - st.org, h.pos - st.org);
                    const float cos_in = std::fabs(orc::Dot(h.n, h.view));
                    st.dVCM *= d2;
                    st.dVCM *= 1.0f / cos_in;
                    st.dVC *= 1.0f / cos_in;
                    st.dVM *= 1.0f / cos_in;
                    st.delta_only = st.delta_only && h.delta;
                    if (!h.delta) {
                        // next-event estimation to light set 0 and the environment (tech report sec. 5.4; wLight
                        // = 0 for the quads, which BSDF rays cannot hit)
                        if (st.len + 1 <= sc.max_len && n_emitters > 0) {
                            const float pick = rng.uniform();
                            const uint32_t li = std::min(uint32_t(pick * float(n_emitters)), n_emitters - 1);
                            if (li == nq) {
                                const float r0 = rng.uniform(), r1 = rng.uniform(), r2 = rng.uniform(), r3 = rng.uniform();
                                float d[3], rad[3];
                                ora::env_direction(r0, r1, r2, r3, d);
                                const float pdf_w = ora::env_pdf(d);
                                const V3 to_l(d[0], d[1], d[2]);
                                if (pdf_w > 0.0f) {
                                    float fwd, rev;
                                    const V3 f = orc::bsdf_evaluate(h.s, h.view, to_l, fwd, rev);
                                    if (f.x != 0.0f || f.y != 0.0f || f.z != 0.0f) {
                                        ora::env_radiance(d, rad);
                                        fwd *= h.cont;
                                        rev *= h.cont;
                                        const float emission_pdfW = pdf_w * sc.disc_pdf;
                                        const float cos_to_light = std::fabs(orc::Dot(h.n, to_l));
                                        const float w_light = fwd / (light_pick * pdf_w);
                                        const float w_camera = (emission_pdfW * cos_to_light / pdf_w) *
                                                               (c.vm_weight + st.dVCM + st.dVC * rev);
                                        const float mis = single ? 1.0f : 1.0f / (w_light + 1.0f + w_camera);
                                        const V3 contrib = (mis / (light_pick * pdf_w)) * (V3(rad[0], rad[1], rad[2]) * f);
                                        if (use_nee && visible(sc, h, to_l, 3.402823466e+38f)) color = color + st.thr * contrib;
                                    }
                                }
                            } else {
                                const Light& L = sc.lights[li];
                                const float u = rng.uniform(), v = rng.uniform();
                                const V3 lp = L.pos - 0.5f * L.x - 0.5f * L.z + u * L.x + v * L.z;
                                const float pdfA = 1.0f / (orc::Len(L.x) * orc::Len(L.z));
                                V3 to_l = lp - h.pos;
                                const float dl2 = orc::Dot(to_l, to_l), dl = std::sqrt(dl2);
                                to_l = to_l * (1.0f / dl);
                                const float cos_light = orc::Dot(orc::Norm(L.dir), -1.0f * to_l);
                                if (cos_light > 0.0f) {
                                    float fwd, rev;
                                    const V3 f = orc::bsdf_evaluate(h.s, h.view, to_l, fwd, rev);
                                    if (f.x != 0.0f || f.y != 0.0f || f.z != 0.0f) {
                                        rev *= h.cont;
                                        const float direct_pdfW = pdfA * dl2 / cos_light;
                                        const float emission_pdfW = pdfA * cos_light / kPi;
                                        const float cos_to_light = std::fabs(orc::Dot(h.n, to_l));
                                        const float w_camera = (emission_pdfW * cos_to_light / (direct_pdfW * cos_light)) *
                                                               (c.vm_weight + st.dVCM + st.dVC * rev);
                                        const float mis = single ? 1.0f : 1.0f / (1.0f + w_camera);
                                        const V3 contrib = (mis / (light_pick * direct_pdfW)) * (L.radiance * f);
                                        if (use_nee && visible(sc, h, to_l, dl * (1.0f - 1e-4f))) color = color + st.thr * contrib;
                                    }
                                }
                            }
                        }
                        // vertex connection to the vertices of light path p (tech report sec. 5.5)
                        for (uint32_t k = path_begin[p]; use_vc && k < path_begin[p + 1]; ++k) {
                            const LightVertex& lv = verts_all[k];
                            if (lv.len + 1 + st.len > sc.max_len) break;
                            V3 dir = lv.hit.pos - h.pos;
                            const float dist2 = orc::Dot(dir, dir), dist = std::sqrt(dist2);
                            dir = dir * (1.0f / dist);
                            float cfwd, crev, lfwd, lrev;
                            const V3 cf = orc::bsdf_evaluate(h.s, h.view, dir, cfwd, crev);
                            if (cf.x == 0.0f && cf.y == 0.0f && cf.z == 0.0f) continue;
                            // light side: f(v = toward the camera vertex, l = toward the previous light vertex),
                            // with the cosine at the connection carried instead of the one toward the light
                            const V3 lfa = orc::bsdf_evaluate(lv.hit.s, -1.0f * dir, lv.hit.view, lrev, lfwd);
                            const float lcos_view = std::fabs(orc::Dot(lv.hit.n, lv.hit.view));
                            const V3 lf = lcos_view > 0.0f ? lfa * (std::fabs(orc::Dot(lv.hit.n, dir)) / lcos_view) : V3(0.0f);
                            if (lf.x == 0.0f && lf.y == 0.0f && lf.z == 0.0f) continue;
                            cfwd *= h.cont; crev *= h.cont;
                            lfwd *= lv.hit.cont; lrev *= lv.hit.cont;
                            const float cos_cam_v = std::fabs(orc::Dot(dir, h.n));
                            const float cos_light_v = std::fabs(orc::Dot(-1.0f * dir, lv.hit.n));
                            const float cam_pdfA = cfwd * cos_light_v / dist2;
                            const float light_pdfA = lfwd * cos_cam_v / dist2;
                            const float w_light = cam_pdfA * (c.vm_weight + lv.dVCM + lv.dVC * lrev);
                            const float w_camera = light_pdfA * (c.vm_weight + st.dVCM + st.dVC * crev);
                            const float mis = single ? 1.0f : 1.0f / (w_light + 1.0f + w_camera);
                            const V3 contrib = (mis / dist2) * (cf * lf);
                            const float bias = 0.1f * h.err;
                            if (visible(sc, h, dir, dist - 16.0f * bias)) color = color + st.thr * lv.thr * contrib;
                        }
                        // vertex merging over the hash grid (tech report sec. 5.6; VCMHashGrid.cpp:107-155)
                        V3 merged(0.0f);
                        const V3 dmin = h.pos - grid.lo, dmax = grid.hi - h.pos;
                        if (merging && use_vm && !verts_all.empty() && dmin.x >= 0 && dmin.y >= 0 && dmin.z >= 0 && dmax.x >= 0 && dmax.y >= 0 &&
                            dmax.z >= 0) {
                            const V3 cp = grid.inv_cell * dmin;
                            const float fx = std::floor(cp.x), fy = std::floor(cp.y), fz = std::floor(cp.z);
                            int x0 = int(fx) - (cp.x - fx < 0.5f ? 1 : 0);
                            int y0 = int(fy) - (cp.y - fy < 0.5f ? 1 : 0);
                            int z0 = int(fz) - (cp.z - fz < 0.5f ? 1 : 0);
                            for (int dz = 0; dz <= 1; ++dz)
                                for (int dy = 0; dy <= 1; ++dy)
                                    for (int dx = 0; dx <= 1; ++dx) {
                                        const uint32_t cell = cell_hash(x0 + dx, y0 + dy, z0 + dz, grid.cells);
                                        const uint32_t b = cell == 0 ? 0 : grid.ends[cell - 1], e = grid.ends[cell];
                                        for (uint32_t k = b; k < e; ++k) {
                                            const LightVertex& lv = verts_all[grid.index[k]];
                                            const V3 dd = h.pos - lv.hit.pos;
                                            if (orc::Dot(dd, dd) > grid.radius2) continue;
                                            if (st.len + lv.len > sc.max_len) continue;
                                            // the reference merges only between surfaces of the same
                                            // transparency (VCM.cpp:372-375)
                                            if (h.transparent != lv.hit.transparent) continue;
                                            const V3 ldir = lv.hit.view;
                                            float fwd, rev;
                                            const V3 fc = orc::bsdf_evaluate(h.s, h.view, ldir, fwd, rev);
                                            const float cosl = std::fabs(orc::Dot(h.n, ldir));
                                            if ((fc.x == 0.0f && fc.y == 0.0f && fc.z == 0.0f) || cosl == 0.0f) continue;
                                            fwd *= h.cont;
                                            rev *= lv.hit.cont;
                                            const float w_light = lv.dVCM * c.vc_weight + lv.dVM * fwd;
                                            const float w_camera = st.dVCM * c.vc_weight + st.dVM * rev;
                                            const float mis = single ? 1.0f : 1.0f / (w_light + 1.0f + w_camera);
                                            merged = merged + (mis / cosl) * (fc * lv.thr);
                                        }
                                    }
                        }
                        color = color + c.vm_norm * (st.thr * merged);
                    }
                    if (st.len >= sc.max_len) break;
                    if (!scatter(rng, h, c, st, false)) break;
                }
                out[size_t(p) * 3] += color.x;
                out[size_t(p) * 3 + 1] += color.y;
                out[size_t(p) * 3 + 2] += color.z;
            }
        };
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) pool.emplace_back(camera_worker, t);
        for (auto& th : pool) th.join();
    }
    for (const auto& img : lt_images)
        for (size_t i = 0; i < img.size(); ++i) out[i] += img[i];
}

// The environment's emission disc: the bounding sphere of the scene box lo..hi (SceneResource.h:77-78 keeps aaBox
// and boundingSphere), as for the default merge radius.
static void env_disc(Scene& sc, const float* lo, const float* hi) {
    float d2 = 0.0f;
    for (int a = 0; a < 3; ++a) {
        const float e = hi[a] - lo[a];
        d2 += e * e;
    }
    sc.env = true;
    sc.center = V3(0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), 0.5f * (lo[2] + hi[2]));
    sc.radius = 0.5f * std::sqrt(d2);
    sc.disc_pdf = (1.0f / kPi) * (1.0f / (sc.radius * sc.radius));
}

extern "C" {

// One VCM render: `iterations` passes, each with width*height light and camera paths.  Inputs as
// oracle_pt_render (materials: 32-word records per geomID; lights: light set 0 as n x 15 floats; camera:
// position lookAt up fovDegrees).  out: [height][width][3] doubles, the sum over iterations (divide by
// `iterations` for the image).  radius0: initial merge radius; alpha: radius reduction; merging 0 turns
// merging off (bidirectional path tracing with the same connections and weights).
void oracle_vcm_render(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t ntri,
                       const float* materials, int n_materials, const float* lights, int n_lights,
                       const float* camera, uint32_t width, uint32_t height, uint32_t iter_begin, uint32_t iter_end,
                       uint32_t max_len, float radius0, float alpha, uint64_t seed, int threads,
                       const int32_t* ptex_rows, int ptex_faces, const uint16_t* ptex_texels, int merging,
                       int strategies, double* out) {
    Scene sc;
    sc.bvh = orq::build(verts, prim, geom, ntri);
    ora::index(prim, geom, nullptr, ntri);
    orp::Texture* tex = ptex_faces > 0 ? new orp::Texture(ptex_rows, ptex_faces, ptex_texels) : nullptr;
    sc.ptex = tex;
    sc.max_len = max_len;
    for (int i = 0; i < n_materials; ++i) sc.materials.push_back(read_material(materials + 32 * i));
    for (int i = 0; i < n_lights; ++i) {
        const float* l = lights + 15 * i;
        sc.lights.push_back({V3(l[0], l[1], l[2]), V3(l[3], l[4], l[5]), V3(l[6], l[7], l[8]), V3(l[9], l[10], l[11]),
                             V3(l[12], l[13], l[14])});
    }
    if (ora::env_present() && ntri > 0) {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t k = 0; k < ntri * 3; ++k)
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], verts[k * 3 + a]);
                hi[a] = std::max(hi[a], verts[k * 3 + a]);
            }
        env_disc(sc, lo, hi);
    }
    vcm_passes(sc, camera, width, height, iter_begin, iter_end, radius0, alpha, seed, threads, merging, strategies, out);
    orq::release(const_cast<void*>(sc.bvh));
    delete tex;
}

// VCM over an instanced scene graph (two levels): triangles and instances as oracle_graph_render (local-to-world
// rows), scene s has materials[mat_offsets[s] .. mat_offsets[s+1]) and Ptex faces ptex_rows[row_offsets[s] ..)
// whose texel offsets are relative to texels + texel_offsets[s]; lights are the top scene's light set 0 and
// bounds[6] (lo, hi) its world box.  Other arguments as oracle_vcm_render.
void oracle_vcm_graph_render(int n_scenes, const float* verts, const uint32_t* prim, const uint32_t* geom,
                             const uint32_t* tri_scene, int64_t ntri, const float* l2w, const uint32_t* inst_id,
                             const uint32_t* inst_scene, const uint32_t* inst_proto, int64_t ninst, int top,
                             const float* materials, const int32_t* mat_offsets, const int32_t* ptex_rows,
                             const int32_t* row_offsets, const uint16_t* texels, const int64_t* texel_offsets,
                             const float* lights, int n_lights, const float* bounds, const float* camera,
                             uint32_t width, uint32_t height, uint32_t iter_begin, uint32_t iter_end, uint32_t max_len,
                             float radius0, float alpha, uint64_t seed, int threads, int merging, int strategies,
                             double* out) {
    Scene sc;
    sc.graph = orq::build_graph(n_scenes, verts, prim, geom, tri_scene, ntri, l2w, inst_id, inst_scene, inst_proto,
                                ninst, top);
    ora::index(prim, geom, tri_scene, ntri);
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
    sc.max_len = max_len;
    for (int i = 0; i < n_lights; ++i) {
        const float* l = lights + 15 * i;
        sc.lights.push_back({V3(l[0], l[1], l[2]), V3(l[3], l[4], l[5]), V3(l[6], l[7], l[8]), V3(l[9], l[10], l[11]),
                             V3(l[12], l[13], l[14])});
    }
    if (ora::env_present()) env_disc(sc, bounds, bounds + 3);
    vcm_passes(sc, camera, width, height, iter_begin, iter_end, radius0, alpha, seed, threads, merging, strategies, out);
    orq::release_graph(const_cast<void*>(sc.graph));
    for (orp::Texture* t : owned) delete t;
}


}  // extern "C"
