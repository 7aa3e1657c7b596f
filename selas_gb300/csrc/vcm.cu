// Vertex connection and merging (Georgiev, Krivanek, Davidovic, Slusallek, "Implementing Vertex
// Connection and Merging", 2012 technical report), the integrator of the reference's VCM.cpp:171-666 with
// VCMCommon.cpp:37-112 and VCMHashGrid.cpp:15-155, on the reference's scene model: quad lights of light
// set 0 that light sub-paths start from and next-event estimation samples, and that camera and BSDF rays do
// not hit (so the emitter-hit strategy has weight zero: dVC = dVM = 0 at the emitter).
//
// One pass = N = width * height light paths and N camera paths:
//   k_light     one thread per light path: emission, closest hits, a stored vertex per non-Dirac hit (fixed
//               slots, max_len - 1 per path), light tracing to the camera (occlusion ray, FP64 splat), BSDF
//               scattering.  The reference BSDF is not reciprocal, so every evaluation is oriented
//               f(v = camera side, l = light side) and a light sub-path's sampled weight is corrected by
//               f(d, view) / f(view, d) (VCM.cpp:304-319,387 orient the connections the same way).
//   grid        bounds of the stored vertices (widened by the radius), compaction in path order, a stable
//               LSD radix sort of (cell, slot) pairs by cell and per-cell ranges: the vertices of a cell
//               are visited in path order, as a sequential counting sort (VCMHashGrid.cpp:48-96) leaves them.
//   k_camera    one thread per camera path: closest hits; per non-Dirac vertex next-event estimation, a
//               connection to every vertex of the light path with the same index, and merging with the
//               vertices in the 2x2x2 cells around it (VCMHashGrid.cpp:107-155); BSDF scattering.
//
// Random numbers: PCG32, stream (2 * pass) * N + p for light path p and (2 * pass + 1) * N + p for
// camera path p, consumed as: light [light pick, u, v, r0, r1], per bounce [4 drawn ahead for the BSDF
// sample, advanced by the number used, Russian roulette]; camera [jitter x, y], per vertex [light pick, u,
// v], [BSDF sample], [Russian roulette].
#include "vcm.h"

#include <algorithm>
#include <cstring>

#include "capi_internal.h"
#include "graph.h"
#include "hitref.cuh"
#include "ibl.cuh"
#include "ptex.cuh"
#include "ptex_quad.cuh"
#include "radix.cuh"
#include "scan.cuh"
#include "shading.cuh"
#include "tex2d.cuh"
#include "traverse.cuh"

namespace sel {

namespace {

constexpr int kBlock = 128;
constexpr float kFloatMax = 3.402823466e+38f;
constexpr int kBoundsBlocks = 256;

struct VcmParams {
    const void* nodes;
    const float4* tris;
    const MaterialDev* materials;
    uint32_t material_count;
    const QuadLight* lights;  // light set 0
    uint32_t light_count;
    const IblDev* ibl;        // the image-based light as an environment emitter (null: none), picked after the quads
    float3 env_center;        // bounding sphere of the scene's bounding box: the environment's emission disc
    float env_radius, env_disc_pdf;
    const PtexFace* ptex_faces;
    const __half* ptex_texels;
    uint32_t ptex_face_count;
    const MeshAttrDev* attrs;
    uint32_t attr_count;
    const InstanceRecord* insts;  // the scene's instance table (null: no instances)
    CameraDev cam;
    float image_plane;
    uint32_t width, height, npaths, max_len, slots;
    uint64_t seed;
    int merging;
    double* accum;
    VcmState st;
    const uint32_t* sorted_index;  // vertex slots sorted by cell (the last radix pass's output)
    uint32_t* err;
};

// A shading point of a sub-path.
struct VHit {
    float3 pos, n, view;
    float err, cont, bsign;  // bsign: the shading frame's bitangent sign (b = cross(n, t) x bsign)
    Surface s;
    const MaterialDev* mat;  // the hit mesh's material record (its scene's table: the rendered one or an instance's)
    bool delta, transparent;
};

struct PathState {
    float3 org, dir, thr;
    float dvcm, dvc, dvm;
    uint32_t len;
    uint32_t flags;  // kPathEnvStart, kPathNonDelta (stored in the top bits of the length word)
};
constexpr uint32_t kPathEnvStart = 1u;  // light path from the environment: no distance term on its first segment
constexpr uint32_t kPathNonDelta = 2u;  // camera path: a non-Dirac vertex seen (else a miss sees the miss image)

// Stored light vertex: 96 bytes (kVertF4 float4s); the tangent and bitangent sign rebuild the shading frame.
constexpr int kVertF4 = 6;
struct LightVertex {
    float3 pos, n, view, thr, base, t;
    float dvcm, dvc, dvm, bsign;
    uint32_t len;
    const MaterialDev* mat;
};

// A stored vertex's path length (at most 32) and the address of its material record share two words: the length
// in bits 0..7 of one with address bits 32..55 above it, address bits 0..31 in the other (device addresses
// lie below 2^56; the render checks the material tables it hands out).
__device__ __forceinline__ uint32_t pack_len(uint32_t len, const MaterialDev* m) {
    return len | (uint32_t(reinterpret_cast<uint64_t>(m) >> 32) << 8);
}
__device__ __forceinline__ uint32_t mat_lo(const MaterialDev* m) { return uint32_t(reinterpret_cast<uint64_t>(m)); }
__device__ __forceinline__ uint32_t unpack_len(uint32_t w) { return w & 0xffu; }
__device__ __forceinline__ const MaterialDev* unpack_mat(uint32_t len_word, uint32_t lo) {
    return reinterpret_cast<const MaterialDev*>((uint64_t(len_word >> 8) << 32) | lo);
}



__device__ __forceinline__ void store_vertex(float4* v, const VHit& h, const PathState& st) {
    v[0] = make_float4(h.pos.x, h.pos.y, h.pos.z, __uint_as_float(pack_len(st.len, h.mat)));
    v[1] = make_float4(h.n.x, h.n.y, h.n.z, __uint_as_float(mat_lo(h.mat)));
    v[2] = make_float4(h.view.x, h.view.y, h.view.z, st.dvcm);
    v[3] = make_float4(st.thr.x, st.thr.y, st.thr.z, st.dvc);
    v[4] = make_float4(h.s.base_color.x, h.s.base_color.y, h.s.base_color.z, st.dvm);
    v[5] = make_float4(h.s.t.x, h.s.t.y, h.s.t.z, h.bsign);
}

__device__ __forceinline__ LightVertex load_vertex(const float4* v) {
    const float4 a = v[0], b = v[1], c = v[2], d = v[3], e = v[4], g = v[5];
    LightVertex lv;
    lv.pos = f3(a.x, a.y, a.z);
    lv.len = unpack_len(__float_as_uint(a.w));
    lv.n = f3(b.x, b.y, b.z);
    lv.mat = unpack_mat(__float_as_uint(a.w), __float_as_uint(b.w));
    lv.view = f3(c.x, c.y, c.z);
    lv.dvcm = c.w;
    lv.thr = f3(d.x, d.y, d.z);
    lv.dvc = d.w;
    lv.base = f3(e.x, e.y, e.z);
    lv.dvm = e.w;
    lv.t = f3(g.x, g.y, g.z);
    lv.bsign = g.w;
    return lv;
}

__device__ __forceinline__ bool nonzero(float3 a) { return a.x != 0.0f || a.y != 0.0f || a.z != 0.0f; }

// BSDF sampling, Russian roulette and the partial MIS weights (VCM.cpp:412-444; tech report eq. 38-40).
__device__ bool scatter(Pcg32& rng, const VHit& h, const VcmConsts& c, PathState& st, bool light_path) {
    float u4[4];
    Pcg32 ahead = rng;
    for (int k = 0; k < 4; ++k) u4[k] = pcg_float(ahead);
    int used = 0;
    BsdfSampleOut bs;
    const bool ok = bsdf_sample(h.s, h.view, u4, used, bs);
    for (int k = 0; k < used; ++k) pcg_next(rng);
    if (!ok) return false;
    if (!nonzero(bs.reflectance)) return false;
    if (pcg_float(rng) > h.cont) return false;
    float3 weight = bs.reflectance;
    if (light_path && !h.delta && !(bs.flags & kDiracEvent)) {
        float a0, a1, b0, b1;
        const float3 adj = bsdf_evaluate(h.s, bs.wi, h.view, a0, a1);  // f(d, view) |cos view|
        const float3 fw = bsdf_evaluate(h.s, h.view, bs.wi, b0, b1);   // f(view, d) |cos d|
        const float cv = fabsf(dot(h.n, h.view)), cd = fabsf(dot(h.n, bs.wi));
        const float k = cv > 0.0f ? cd / cv : 0.0f;
        weight.x = (adj.x > 0.0f && fw.x > 0.0f) ? bs.reflectance.x * (adj.x * k / fw.x) : bs.reflectance.x;
        weight.y = (adj.y > 0.0f && fw.y > 0.0f) ? bs.reflectance.y * (adj.y * k / fw.y) : bs.reflectance.y;
        weight.z = (adj.z > 0.0f && fw.z > 0.0f) ? bs.reflectance.z * (adj.z * k / fw.z) : bs.reflectance.z;
    }
    const float fwd = bs.forward_pdf * h.cont, rev = bs.reverse_pdf * h.cont;
    const float cos_out = fabsf(dot(bs.wi, h.n));
    if (h.delta) {
        st.dvcm = 0.0f;
        st.dvc *= cos_out;
        st.dvm *= cos_out;
    } else {
        st.dvc = (cos_out / fwd) * (st.dvc * rev + st.dvcm + c.vm_weight);
        st.dvm = (cos_out / fwd) * (st.dvm * rev + st.dvcm * c.vc_weight + 1.0f);
        st.dvcm = 1.0f / fwd;
    }
    st.thr = st.thr * weight * (1.0f / h.cont);
    st.org = offset_origin(h.pos, h.n, h.err, bs.wi, 1.0f);
    st.dir = bs.wi;
    st.len += 1;
    return true;
}

// World position -> pixel, the inverse of ImageToWorldDirection (GeometryLib/Camera.cpp:56-60).
__device__ __forceinline__ bool to_pixel(const CameraDev& cam, float3 p, int& px, int& py) {
    const float3 d = p - cam.position;
    const float dz = dot(d, cam.z);
    if (dz <= 0.0f) return false;
    const float cx = -dot(d, cam.x) / (dz * dot(cam.x, cam.x));
    const float cy = dot(d, cam.y) / (dz * dot(cam.y, cam.y));
    const float fx = (cx + 1.0f) * 0.5f * cam.width, fy = (1.0f - cy) * 0.5f * cam.height;
    if (!(fx >= 0.0f && fx < cam.width && fy >= 0.0f && fy < cam.height)) return false;
    px = int(fx);
    py = int(fy);
    return true;
}

__device__ __forceinline__ void splat(double* accum, uint32_t pixel, float3 c) {
    double* p = accum + size_t(pixel) * 3;
    atomicAdd(p, double(c.x));
    atomicAdd(p + 1, double(c.y));
    atomicAdd(p + 2, double(c.z));
}

// Warp-aggregated append of one entry per willing lane (full warps only).
__device__ __forceinline__ uint32_t warp_append(uint32_t* count, bool want) {
    const uint32_t mask = __ballot_sync(0xffffffffu, want);
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0;
    if (lane == 0 && mask) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// Warp-aggregated reservation of n entries per lane (full warps only): returns this lane's first entry.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* count, uint32_t n) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t incl = n;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= uint32_t(o)) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(count, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + incl - n;
}

__device__ __forceinline__ Pcg32 load_rng(const VcmParams& P, uint32_t s, uint64_t stream) {
    Pcg32 r;
    r.state = P.st.prng[s];
    r.inc = (stream << 1u) | 1u;
    return r;
}

__device__ __forceinline__ PathState load_path(const VcmParams& P, uint32_t s) {
    const float4 o = P.st.po[s], d = P.st.pd[s], t = P.st.pt[s];
    PathState st;
    st.org = f3(o.x, o.y, o.z);
    st.dvcm = o.w;
    st.dir = f3(d.x, d.y, d.z);
    st.dvc = d.w;
    st.thr = f3(t.x, t.y, t.z);
    st.dvm = t.w;
    const uint32_t pl = P.st.plen[s];
    st.len = pl & 0x3fffffffu;
    st.flags = pl >> 30;
    return st;
}

__device__ __forceinline__ void store_path(const VcmParams& P, uint32_t s, const PathState& st) {
    P.st.po[s] = make_float4(st.org.x, st.org.y, st.org.z, st.dvcm);
    P.st.pd[s] = make_float4(st.dir.x, st.dir.y, st.dir.z, st.dvc);
    P.st.pt[s] = make_float4(st.thr.x, st.thr.y, st.thr.z, st.dvm);
    P.st.plen[s] = st.len | (st.flags << 30);
}

// Surface at a stored closest hit of the ray (org, dir) (CalculateSurfaceParams as the path tracer uses it).
// kPretex: the base colour of textured hits was filtered or sampled by k_vtexture into P.st.base[s] (every bounce
// of a material-sorted pass or of a scene with quad-mesh Ptex); otherwise the shading kernel filters triangle Ptex
// and samples 2D images itself (the plain form: SEL_OPTION_MATERIAL_SORT 0).
template <bool kPretex, bool kInst>
__device__ void make_vhit(const VcmParams& P, uint32_t s, float3 org, float3 dir, float4 hit, VHit& h,
                          uint32_t& status) {
    const uint32_t tri = __float_as_uint(hit.w);
    const HitRef hr = hit_ref_of<kInst>(P, kInst ? P.st.phinst[s] : make_uint2(0u, 0u), tri);
    const float4 p0 = __ldg(hr.tp), p1 = __ldg(hr.tp + 1), p2 = __ldg(hr.tp + 2);
    const uint32_t geom = __float_as_uint(p1.w);
    const uint32_t mi = geom < hr.mat_count ? geom : 0;
    const MaterialDev& m = hr.mats[mi];
    h.pos = f3(org.x + hit.x * dir.x, org.y + hit.x * dir.y, org.z + hit.x * dir.z);
    h.err = 32.0f * 1.19209e-07f * fmaxf(fmaxf(fabsf(h.pos.x), fabsf(h.pos.y)), fmaxf(fabsf(h.pos.z), hit.x));
    float3 base = ld3(m.base_color);
    const MeshAttrDev* attr = geom < hr.attr_count ? hr.attrs + geom : nullptr;
    if (m.flags & kMaterialTextured) {
        if constexpr (kPretex) {
            const float4 b = P.st.base[s];
            base = f3(b.x, b.y, b.z);
        } else if (m.flags & kMaterialUsesPtex) {
            uint32_t pstatus = 0;
            ptex_eval(static_cast<const PtexFace*>(hr.ptex_faces), int(hr.ptex_count),
                      static_cast<const __half*>(hr.ptex_texels), int(m.ptex_base + __float_as_uint(p0.w)), hit.y,
                      hit.z, base, pstatus);
            status |= pstatus;
        } else {
            base = tex2d_base_colour(m, attr, __float_as_uint(p0.w), hit.y, hit.z);
        }
    }
    h.view = -dir;
    float3 fn, ft, fb;
    const float3 ng = kInst ? record_ng(hr.tp, p0, p1, p2, hr.rec0, hr.rec1, org, dir, hit.x, hit.y)
                            : triangle_ng(p0, p1, p2);
    shading_frame(attr, __float_as_uint(p0.w), hit.y, hit.z, ng,
                  [&](float3 x) { return kInst ? world_normal(hr, x) : x; }, fn, ft, fb, h.bsign);
    h.s = make_surface_frame(m, ft, fn, fb, h.view, pow3(base, 2.2f));
    h.n = h.s.n;
    h.cont = continuation_probability(h.s);
    h.mat = &m;
    h.delta = m.shader == kDiracTransparent;
    h.transparent = (m.flags & kMaterialTransparent) != 0u;
}

// Shadow-ray record for a segment leaving a hit: origin offset 0.1 x the hit's error bound, tnear = the
// error bound (OcclusionRay, PathTracer.cpp:71-92); contribution and pixel ride along.
__device__ __forceinline__ void push_shadow(const VcmParams& P, uint32_t slot, const VHit& h, float3 dir, float tfar,
                                            float3 c, uint32_t pixel) {
    const float3 o = offset_origin(h.pos, h.n, h.err, dir, 0.1f);
    P.st.so[slot] = make_float4(o.x, o.y, o.z, h.err);
    P.st.sd[slot] = make_float4(dir.x, dir.y, dir.z, tfar);
    P.st.sc[slot] = make_float4(c.x, c.y, c.z, __uint_as_float(pixel));
}

__global__ void k_reset(uint32_t* counters) {
    if (threadIdx.x < 8) counters[threadIdx.x] = 0u;
}

__global__ void k_bounce_reset(uint32_t* counters, int next) {
    if (threadIdx.x == 0) {
        counters[next] = 0u;
        counters[2] = 0u;  // shadow entries
        counters[3] = 0u;  // extend cursor
        counters[4] = 0u;  // shadow cursor
        counters[5] = 0u;  // camera-vertex records
        counters[6] = 0u;  // connection pairs
    }
}

// Concentric map of the unit square onto the unit disc (Shirley and Chiu, "A Low Distortion Map Between Disk and
// Square", 1997): the disc sample of EmitIblLightSample (AreaLighting.cpp:268-272).
__device__ __forceinline__ void concentric_disc(float r0, float r1, float& u, float& v) {
    const float a = 2.0f * r0 - 1.0f, b = 2.0f * r1 - 1.0f;
    if (a == 0.0f && b == 0.0f) {
        u = 0.0f;
        v = 0.0f;
        return;
    }
    float r, phi;
    if (fabsf(a) > fabsf(b)) {
        r = a;
        phi = (kPi / 4.0f) * (b / a);
    } else {
        r = b;
        phi = kPi / 2.0f - (kPi / 4.0f) * (a / b);
    }
    u = r * cosf(phi);
    v = r * sinf(phi);
}

// GenerateLightSample (VCMCommon.cpp:37-62): a light picked uniformly among the quads of light set 0 and the
// environment.  A quad emits from a uniform point, cosine-weighted about its facing direction; the environment
// (EmitIblLightSample, AreaLighting.cpp:246-290; tech report sec. 5.1) along a sampled direction from a disc of
// the bounding-sphere radius facing it, as an infinite light (cos 1, hit by camera and BSDF rays).
__global__ void __launch_bounds__(kBlock) k_l_generate(VcmParams P) {
    const VcmConsts c = P.st.consts[*P.st.iter];
    const uint32_t N = P.npaths;
    const uint32_t n_emitters = P.light_count + (P.ibl ? 1u : 0u);
    for (uint32_t base = blockIdx.x * blockDim.x; base < N; base += gridDim.x * blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        bool alive = false;
        if (p < N) {
            P.st.vcount[p] = 0;
            if (n_emitters > 0) {
                const uint64_t stream = (uint64_t(c.pass) * 2 + 0) * N + p;
                Pcg32 rng = pcg_seed(P.seed, stream);
                const float pick = pcg_float(rng);
                uint32_t li = uint32_t(pick * float(n_emitters));
                li = li < n_emitters - 1 ? li : n_emitters - 1;
                const float light_pick = 1.0f / float(n_emitters);
                PathState st;
                st.len = 1;
                st.flags = 0;
                if (li == P.light_count) {
                    const float r0 = pcg_float(rng), r1 = pcg_float(rng), r2 = pcg_float(rng), r3 = pcg_float(rng);
                    const float r4 = pcg_float(rng), r5 = pcg_float(rng);
                    const IblDev& ibl = *P.ibl;
                    const float3 to_env = ibl_env_direction(ibl, r0, r1, r2, r3);
                    const float pdf_w = ibl_env_pdf(ibl, to_env);
                    if (pdf_w > 0.0f) {
                        const float3 rad = ibl_radiance(ibl, to_env);
                        float du, dv;
                        concentric_disc(r4, r5, du, dv);
                        float3 dx, dz;
                        orthonormal_basis(to_env, dx, dz);
                        const float emission_pdf = pdf_w * P.env_disc_pdf * light_pick;
                        const float direct_pdf_a = pdf_w * light_pick;
                        st.org = P.env_center + P.env_radius * (to_env + du * dx + dv * dz);
                        st.dir = -to_env;
                        st.thr = rad * (1.0f / emission_pdf);
                        st.dvcm = direct_pdf_a / emission_pdf;
                        st.dvc = 1.0f / emission_pdf;  // cos at an infinite light: 1
                        st.dvm = st.dvc * c.vc_weight;
                        st.flags = kPathEnvStart;
                        alive = true;
                    }
                } else {
                    const QuadLight L = P.lights[li];
                    const float u = pcg_float(rng), v = pcg_float(rng);
                    const float3 lp = L.position - 0.5f * L.x - 0.5f * L.z + u * L.x + v * L.z;
                    const float pdf_a = 1.0f / (length(L.x) * length(L.z));
                    const float3 ln = normalize(L.direction);
                    float3 lt, lb;
                    orthonormal_basis(ln, lt, lb);
                    const float r0 = pcg_float(rng), r1 = pcg_float(rng);
                    const float rr = sqrtf(r0), ph = 2.0f * kPi * r1;
                    const float cosl = sqrtf(fmaxf(0.0f, 1.0f - r0));
                    const float3 dir = normalize(rr * cosf(ph) * lt + cosl * ln + rr * sinf(ph) * lb);
                    if (cosl > 0.0f) {
                        const float emission_pdf = pdf_a * cosl / kPi * light_pick;
                        const float direct_pdf_a = pdf_a * light_pick;
                        st.org = lp;
                        st.dir = dir;
                        st.thr = L.radiance * (cosl / emission_pdf);
                        st.dvcm = direct_pdf_a / emission_pdf;
                        st.dvc = 0.0f;  // the emitter cannot be hit by camera or BSDF rays
                        st.dvm = 0.0f;
                        alive = true;
                    }
                }
                if (alive) {
                    store_path(P, p, st);
                    P.st.prng[p] = rng.state;
                }
            }
        }
        const uint32_t q = warp_append(&P.st.counters[0], alive);
        if (alive) P.st.queue[0][q] = p;
    }
}

// Camera rays (GenerateCameraPaths, VCM.cpp:563-574, with x = p - y * width): one jittered sample per pixel.
__global__ void __launch_bounds__(kBlock) k_c_generate(VcmParams P) {
    const VcmConsts c = P.st.consts[*P.st.iter];
    const uint32_t N = P.npaths;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
        Pcg32 rng = pcg_seed(P.seed, (uint64_t(c.pass) * 2 + 1) * N + p);
        const uint32_t y = p / P.width, x = p - y * P.width;
        const float vx = float(x) + pcg_float(rng), vy = float(y) + pcg_float(rng);
        const float3 d = camera_direction(P.cam, vx, vy);
        const float cos_cam = dot(P.cam.z, d);
        const float ip = P.image_plane / cos_cam;
        const float camera_pdf_w = ip * ip / cos_cam;
        PathState st;
        st.org = P.cam.position;
        st.dir = d;
        st.thr = f3(1.0f);
        st.dvcm = c.n_paths / camera_pdf_w;
        st.dvc = 0.0f;
        st.dvm = 0.0f;
        st.len = 1;
        st.flags = 0;
        store_path(P, p, st);
        P.st.prng[p] = rng.state;
        P.st.queue[0][p] = p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) P.st.counters[0] = N;
}

// Closest hits of the queued paths: persistent blocks, warps take 32-entry packets through an atomic cursor.
template <int K, int B>
__global__ void __launch_bounds__(B, 1024 / B) k_extend(VcmParams P, int cur) {
    __shared__ typename Tracer<K>::Entry stack_mem[Tracer<K>::kDepth * B];
    const uint32_t n = P.st.counters[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(P.st.rays, (unsigned long long)n);
    const uint32_t* queue = P.st.queue[cur];
    uint32_t status = 0;
    for (;;) {
        uint32_t base = 0;
        if ((threadIdx.x & 31u) == 0) base = atomicAdd(&P.st.counters[3], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t e = base + (threadIdx.x & 31u);
        if (e < n) {
            const uint32_t s = queue[e];
            const float4 o = P.st.po[s], d = P.st.pd[s];
            QueryRay q;
            q.ox = o.x; q.oy = o.y; q.oz = o.z; q.tnear = 0.0f;
            q.dx = d.x; q.dy = d.y; q.dz = d.z; q.tfar = kFloatMax;
            if constexpr (K == 2) {
                InstHit h;
                const bool found = trace_instanced<false>(static_cast<const uint4*>(P.nodes), P.tris, P.insts, q, h,
                                                          stack_mem + threadIdx.x, B, status);
                P.st.phit[s] = found ? make_float4(h.t, h.u, h.v, __uint_as_float(h.tri))
                                     : make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xffffffffu));
                P.st.phinst[s] = found ? inst_indices(P.insts, h) : make_uint2(0u, 0u);
            } else {
                QueryHit h;
                const bool found = Tracer<K>::template trace<false>(P.nodes, P.tris, q, h, stack_mem + threadIdx.x, B,
                                                                    status);
                P.st.phit[s] = found ? make_float4(h.t, h.u, h.v, __uint_as_float(h.tri))
                                     : make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xffffffffu));
            }
        }
    }
    if (status) atomicOr(P.err, status);
}

// Any-hit of the queued shadow rays; unoccluded ones add their contribution to their pixel.
template <int K, int B>
__global__ void __launch_bounds__(B, 1024 / B) k_shadow(VcmParams P) {
    __shared__ typename Tracer<K>::Entry stack_mem[Tracer<K>::kDepth * B];
    const uint32_t n = P.st.counters[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(P.st.rays + 1, (unsigned long long)n);
    uint32_t status = 0;
    for (;;) {
        uint32_t base = 0;
        if ((threadIdx.x & 31u) == 0) base = atomicAdd(&P.st.counters[4], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t e = base + (threadIdx.x & 31u);
        // 8-wide layout: the packet's lanes test their leaf triangles together (trace_wide_warp): passes 1.2 % faster
        // on the room at 1280 x 720 (20.54 against 20.79 ms).  The path tracer's shadow kernel, whose packets can mix
        // jobs' scenes, measured 3 % slower this way on the Cornell box and keeps one lane per ray.
        if constexpr (K == 0) {
            float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (e < n) c = P.st.sc[e];
            const bool live = c.x != 0.0f || c.y != 0.0f || c.z != 0.0f;
            QueryRay q{};
            if (live) {
                const float4 o = P.st.so[e], d = P.st.sd[e];
                q.ox = o.x; q.oy = o.y; q.oz = o.z; q.tnear = o.w;
                q.dx = d.x; q.dy = d.y; q.dz = d.z; q.tfar = d.w;
            }
            QueryHit h;
            const bool hit = trace_wide_warp<true>(static_cast<const uint4*>(P.nodes), P.tris, live, q, h,
                                                   stack_mem + threadIdx.x, B, nullptr, status);
            if (live && !hit) splat(P.accum, __float_as_uint(c.w), f3(c.x, c.y, c.z));
            continue;
        }
        if (e < n) {
            const float4 c = P.st.sc[e];
            if (c.x != 0.0f || c.y != 0.0f || c.z != 0.0f) {
                const float4 o = P.st.so[e], d = P.st.sd[e];
                QueryRay q;
                q.ox = o.x; q.oy = o.y; q.oz = o.z; q.tnear = o.w;
                q.dx = d.x; q.dy = d.y; q.dz = d.z; q.tfar = d.w;
                bool hit;
                if constexpr (K == 2) {
                    InstHit h;
                    hit = trace_instanced<true>(static_cast<const uint4*>(P.nodes), P.tris, P.insts, q, h,
                                                stack_mem + threadIdx.x, B, status);
                } else {
                    QueryHit h;
                    hit = Tracer<K>::template trace<true>(P.nodes, P.tris, q, h, stack_mem + threadIdx.x, B, status);
                }
                if (!hit) splat(P.accum, __float_as_uint(c.w), f3(c.x, c.y, c.z));
            }
        }
    }
    if (status) atomicOr(P.err, status);
}

// Light sub-path vertices (EvaluateLightPaths, VCM.cpp:502-561): MIS update, stored vertex, connection to
// the camera (ConnectLightPathToCamera, VCM.cpp:190-233; tech report sec. 5.3) and scattering.
template <bool kSorted, bool kInst>
__global__ void __launch_bounds__(kBlock) k_l_shade(VcmParams P, int cur, const uint32_t* in_queue) {
    const VcmConsts c = P.st.consts[*P.st.iter];
    const uint32_t n = P.st.counters[cur];
    const uint32_t N = P.npaths;
    const int next = cur ^ 1;
    uint32_t status = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        bool cont = false, shadow = false;
        uint32_t s = 0, pixel = 0;
        VHit h;
        float3 to_cam = f3(0.0f), contrib = f3(0.0f);
        float sh_tfar = 0.0f;
        if (e < n) {
            s = in_queue[e];
            const float4 hit = P.st.phit[s];
            if (__float_as_uint(hit.w) != 0xffffffffu) {
                PathState st = load_path(P, s);
                make_vhit<kSorted, kInst>(P, s, st.org, st.dir, hit, h, status);
                const float3 seg = h.pos - st.org;
                const float d2 = dot(seg, seg);
                const float cos_in = fabsf(dot(h.n, h.view));
                if (st.len > 1 || !(st.flags & kPathEnvStart)) st.dvcm *= d2;
                st.dvcm *= 1.0f / cos_in;
                st.dvc *= 1.0f / cos_in;
                st.dvm *= 1.0f / cos_in;
                if (!h.delta) {
                    const uint32_t k = P.st.vcount[s];
                    store_vertex(P.st.verts + (size_t(s) * P.slots + k) * kVertF4, h, st);
                    P.st.vcount[s] = k + 1;
                    int px, py;
                    if (st.len + 1 <= P.max_len && to_pixel(P.cam, h.pos, px, py)) {
                        to_cam = P.cam.position - h.pos;
                        const float dist2 = dot(to_cam, to_cam);
                        const float dist = sqrtf(dist2);
                        to_cam = to_cam * (1.0f / dist);
                        const float cos_cam = dot(P.cam.z, -to_cam);
                        float cam_side_pdf, light_side_pdf;
                        const float3 fa = bsdf_evaluate(h.s, to_cam, h.view, cam_side_pdf, light_side_pdf);
                        const float cos_view = fabsf(dot(h.n, h.view));
                        const float3 f = cos_view > 0.0f ? fa * (fabsf(dot(h.n, to_cam)) / cos_view) : f3(0.0f);
                        float rev = cam_side_pdf;
                        if (nonzero(f) && cos_cam > 0.0f) {
                            rev *= h.cont;
                            const float ip = P.image_plane / cos_cam;
                            const float img_to_solid = ip * ip / cos_cam;
                            const float cos_surf = fabsf(dot(h.n, to_cam));
                            const float camera_pdf_a = img_to_solid * cos_surf / dist2;
                            const float w_light = (camera_pdf_a / c.n_paths) * (c.vm_weight + st.dvcm + st.dvc * rev);
                            const float mis = 1.0f / (w_light + 1.0f);
                            contrib = (mis * img_to_solid / (c.n_paths * dist2)) * (st.thr * f);
                            sh_tfar = dist * (1.0f - 1e-4f);
                            pixel = uint32_t(py) * P.width + uint32_t(px);
                            shadow = nonzero(contrib);
                        }
                    }
                }
                if (st.len + 2 <= P.max_len) {
                    Pcg32 rng = load_rng(P, s, (uint64_t(c.pass) * 2 + 0) * N + s);
                    cont = scatter(rng, h, c, st, true);
                    P.st.prng[s] = rng.state;
                    if (cont) store_path(P, s, st);
                }
            }
        }
        const uint32_t q = warp_append(&P.st.counters[next], cont);
        if (cont) P.st.queue[next][q] = s;
        const uint32_t sq = warp_append(&P.st.counters[2], shadow);
        if (shadow) push_shadow(P, sq, h, to_cam, sh_tfar, contrib, pixel);
    }
    if (status) atomicOr(P.err, status);
}

// ---------------------------------------------------------------------------------------------------
// Material-class sort of a bounce's hits (as the path tracer's): counting sort by class (0 miss; else
// 1 + shader * 4 + 2 (Ptex) + 1 (transparent)), then the Ptex filter of the sorted hits in a kernel of its own,
// so the shading kernels run one kind of surface per warp and carry no filter code.
// ---------------------------------------------------------------------------------------------------
template <bool kInst>
__device__ __forceinline__ uint32_t vmaterial_class(const VcmParams& P, uint32_t s) {
    const uint32_t tri = __float_as_uint(P.st.phit[s].w);
    if (tri == 0xffffffffu) return 0u;
    const HitRef hr = hit_ref_of<kInst>(P, kInst ? P.st.phinst[s] : make_uint2(0u, 0u), tri);
    const uint32_t geom = __float_as_uint(__ldg(hr.tp + 1).w);
    const MaterialDev& m = hr.mats[geom < hr.mat_count ? geom : 0];
    const uint32_t shader = uint32_t(m.shader) < 3u ? uint32_t(m.shader) : 0u;
    return 1u + shader * 4u + ((m.flags & kMaterialTextured) ? 2u : 0u) + ((m.flags & kMaterialTransparent) ? 1u : 0u);
}

__global__ void k_vclass_reset(uint32_t* counters) {
    if (threadIdx.x < 32) counters[32 + threadIdx.x] = 0u;
}

template <bool kInst>
__global__ void __launch_bounds__(kBlock) k_vclassify(VcmParams P, int cur) {
    const uint32_t n = P.st.counters[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        const bool valid = e < n;
        const uint32_t c = valid ? vmaterial_class<kInst>(P, P.st.queue[cur][e]) : 0xffu;
        if (valid) P.st.cls[e] = c;
        const uint32_t peers = __match_any_sync(0xffffffffu, c);
        const uint32_t lane = threadIdx.x & 31u;
        if (valid && (__ffs(peers) - 1) == int(lane)) atomicAdd(&P.st.counters[32 + c], __popc(peers));
    }
}

__global__ void k_vclass_offsets(uint32_t* counters) {
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int c = 0; c < 16; ++c) {
            counters[48 + c] = run;
            run += counters[32 + c];
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_vclass_scatter(VcmParams P, int cur) {
    const uint32_t n = P.st.counters[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        const bool valid = e < n;
        const uint32_t c = valid ? P.st.cls[e] : 0xffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, c);
        const uint32_t lane = threadIdx.x & 31u;
        const int leader = __ffs(peers) - 1;
        uint32_t at = 0;
        if (valid && leader == int(lane)) at = atomicAdd(&P.st.counters[48 + c], __popc(peers));
        at = __shfl_sync(0xffffffffu, at, leader);
        if (valid) P.st.queue_sorted[at + __popc(peers & ((1u << lane) - 1u))] = P.st.queue[cur][e];
    }
}

template <bool kInst, bool kQuad>
__global__ void __launch_bounds__(kBlock) k_vtexture(VcmParams P, int cur, const uint32_t* queue) {
    const uint32_t n = P.st.counters[cur];
    uint32_t status = 0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const uint32_t s = queue[e];
        const float4 hit = P.st.phit[s];
        const uint32_t tri = __float_as_uint(hit.w);
        if (tri == 0xffffffffu) continue;
        const HitRef hr = hit_ref_of<kInst>(P, kInst ? P.st.phinst[s] : make_uint2(0u, 0u), tri);
        const float4 p0 = __ldg(hr.tp), p1 = __ldg(hr.tp + 1);
        const uint32_t geom = __float_as_uint(p1.w);
        const MaterialDev& m = hr.mats[geom < hr.mat_count ? geom : 0];
        if (!(m.flags & kMaterialTextured)) continue;
        float3 base = ld3(m.base_color);
        if (m.flags & kMaterialUsesPtex) {
            uint32_t pstatus = 0;
            if (kQuad && (m.flags & kMaterialPtexQuad))
                ptex_material_eval(m, hr.ptex_faces, int(hr.ptex_count), static_cast<const __half*>(hr.ptex_texels),
                                   __float_as_uint(p0.w), hit.y, hit.z, base, pstatus);
            else
                ptex_eval(static_cast<const PtexFace*>(hr.ptex_faces), int(hr.ptex_count),
                          static_cast<const __half*>(hr.ptex_texels), int(m.ptex_base + __float_as_uint(p0.w)), hit.y,
                          hit.z, base, pstatus);
            status |= pstatus;
        } else {
            base = tex2d_base_colour(m, geom < hr.attr_count ? hr.attrs + geom : nullptr, __float_as_uint(p0.w), hit.y,
                                     hit.z);
        }
        P.st.base[s] = make_float4(base.x, base.y, base.z, 0.0f);
    }
    if (status) atomicOr(P.err, status);
}

// ---------------------------------------------------------------------------------------------------
// Hash grid (VCMHashGrid.cpp:48-96): bounds, compaction, radix sort by cell, cell ranges.
// ---------------------------------------------------------------------------------------------------

__device__ __forceinline__ uint32_t cell_hash(int x, int y, int z, uint32_t cells) {
    const uint32_t ux = uint32_t(x), uy = uint32_t(y), uz = uint32_t(z);
    return ((ux * 73856093u) ^ (uy * 19349663u) ^ (uz * 83492791u)) % cells;
}

// Bounds of all stored vertices: per-block partials (min x y z, max x y z), then one block reduces them,
// widens the box by the radius (the correction VCMHashGrid.cpp:69-72 leaves commented out: without it a
// vertex on a bounding plane of the vertex set fails the range test about half the time) and writes the
// grid header.
__global__ void __launch_bounds__(256) k_bounds(VcmParams P) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.npaths; p += gridDim.x * blockDim.x) {
        const uint32_t n = P.st.vcount[p];
        const float4* v = P.st.verts + size_t(p) * P.slots * kVertF4;
        for (uint32_t k = 0; k < n; ++k) {
            const float4 a = v[size_t(k) * kVertF4];
            mn[0] = fminf(mn[0], a.x); mn[1] = fminf(mn[1], a.y); mn[2] = fminf(mn[2], a.z);
            mx[0] = fmaxf(mx[0], a.x); mx[1] = fmaxf(mx[1], a.y); mx[2] = fmaxf(mx[2], a.z);
        }
    }
    __shared__ float red[6][8];
    for (int i = 0; i < 3; ++i) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[i] = fminf(mn[i], __shfl_xor_sync(0xffffffffu, mn[i], o));
            mx[i] = fmaxf(mx[i], __shfl_xor_sync(0xffffffffu, mx[i], o));
        }
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int i = 0; i < 3; ++i) { red[i][w] = mn[i]; red[3 + i][w] = mx[i]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        float r = red[threadIdx.x][0];
        for (int k = 1; k < 8; ++k) r = threadIdx.x < 3 ? fminf(r, red[threadIdx.x][k]) : fmaxf(r, red[threadIdx.x][k]);
        P.st.bounds_part[blockIdx.x * 6 + threadIdx.x] = r;
    }
}

__global__ void k_bounds_final(VcmParams P, int parts) {
    const VcmConsts c = P.st.consts[*P.st.iter];
    if (threadIdx.x < 6) {
        float r = P.st.bounds_part[threadIdx.x];
        for (int k = 1; k < parts; ++k) {
            const float x = P.st.bounds_part[k * 6 + threadIdx.x];
            r = threadIdx.x < 3 ? fminf(r, x) : fmaxf(r, x);
        }
        P.st.grid[threadIdx.x] = threadIdx.x < 3 ? r - c.radius : r + c.radius;
    }
    if (threadIdx.x == 0) {
        P.st.grid[6] = 1.0f / (2.0f * c.radius);
        P.st.grid[7] = c.radius * c.radius;
        P.st.grid[9] = __uint_as_float(P.npaths);
    }
}

__device__ __forceinline__ uint32_t cell_of(const float* grid, float3 p, uint32_t cells) {
    const float inv = grid[6];
    const float3 f = p - f3(grid[0], grid[1], grid[2]);
    return cell_hash(int(floorf(inv * f.x)), int(floorf(inv * f.y)), int(floorf(inv * f.z)), cells);
}

// Compacted (cell, slot) pairs in path order, and the number of vertices per cell.
__global__ void __launch_bounds__(256) k_keys(VcmParams P) {
    const uint32_t cells = P.npaths;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.npaths; p += gridDim.x * blockDim.x) {
        const uint32_t n = P.st.vcount[p], at = P.st.vpos[p];
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t slot = p * P.slots + k;
            const float4 a = P.st.verts[size_t(slot) * kVertF4];
            const uint32_t cell = cell_of(P.st.grid, f3(a.x, a.y, a.z), cells);
            P.st.keys[0][at + k] = cell;
            P.st.vals[0][at + k] = slot;
            atomicAdd(&P.st.cell_count[cell], 1u);
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// Camera sub-path vertices (EvaluateCameraPaths, VCM.cpp:576-666), in three kernels so that lanes of a warp
// do the same work: k_c_shade (MIS update, next-event estimation, a camera-vertex record, one connection
// entry per eligible light vertex, scattering), k_c_connect (one thread per camera-vertex / light-vertex
// pair: ConnectPathVertices, VCM.cpp:293-359) and k_c_merge (one warp per camera vertex over the light
// vertices of the 2x2x2 cells around it: MergeVertices + SearchHashGrid, VCM.cpp:362-409,
// VCMHashGrid.cpp:107-155).  Next-event and connection segments go to the shadow queue; merged radiance
// goes straight to the pixel.
// ---------------------------------------------------------------------------------------------------

// Camera vertex record: 112 bytes (kCamF4 float4s).
constexpr int kCamF4 = 7;
struct CameraVertex {
    float3 pos, n, view, base, thr, t;
    float err, cont, dvcm, dvc, dvm, bsign;
    uint32_t pixel, len, transparent;
    const MaterialDev* mat;
};

__device__ __forceinline__ void store_camera_vertex(float4* v, const VHit& h, const PathState& st, uint32_t pixel) {
    v[0] = make_float4(h.pos.x, h.pos.y, h.pos.z, h.err);
    v[1] = make_float4(h.n.x, h.n.y, h.n.z, __uint_as_float(mat_lo(h.mat)));
    v[2] = make_float4(h.view.x, h.view.y, h.view.z, h.cont);
    v[3] = make_float4(h.s.base_color.x, h.s.base_color.y, h.s.base_color.z, __uint_as_float(pixel));
    v[4] = make_float4(st.thr.x, st.thr.y, st.thr.z, __uint_as_float(pack_len(st.len, h.mat)));
    v[5] = make_float4(st.dvcm, st.dvc, st.dvm, __uint_as_float(h.transparent ? 1u : 0u));
    v[6] = make_float4(h.s.t.x, h.s.t.y, h.s.t.z, h.bsign);
}

__device__ __forceinline__ CameraVertex load_camera_vertex(const float4* v) {
    const float4 a = v[0], b = v[1], c = v[2], d = v[3], e = v[4], f = v[5], g = v[6];
    CameraVertex cv;
    cv.pos = f3(a.x, a.y, a.z);
    cv.err = a.w;
    cv.n = f3(b.x, b.y, b.z);
    cv.mat = unpack_mat(__float_as_uint(e.w), __float_as_uint(b.w));
    cv.view = f3(c.x, c.y, c.z);
    cv.cont = c.w;
    cv.base = f3(d.x, d.y, d.z);
    cv.pixel = __float_as_uint(d.w);
    cv.thr = f3(e.x, e.y, e.z);
    cv.len = unpack_len(__float_as_uint(e.w));
    cv.dvcm = f.x;
    cv.dvc = f.y;
    cv.dvm = f.z;
    cv.transparent = __float_as_uint(f.w);
    cv.t = f3(g.x, g.y, g.z);
    cv.bsign = g.w;
    return cv;
}

template <bool kSorted, bool kInst>
__global__ void __launch_bounds__(kBlock) k_c_shade(VcmParams P, int cur, const uint32_t* in_queue) {
    const VcmConsts c = P.st.consts[*P.st.iter];
    const uint32_t n = P.st.counters[cur];
    const uint32_t N = P.npaths;
    const int next = cur ^ 1;
    uint32_t status = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        bool cont = false, hit_ok = false, nee_ray = false, record = false;
        uint32_t s = 0, nvc = 0;
        VHit h;
        PathState st;
        Pcg32 rng;
        rng.state = 0;
        rng.inc = 1;
        float3 to_l = f3(0.0f), contrib = f3(0.0f);
        float tfar = 0.0f;
        if (e < n) {
            s = in_queue[e];
            const float4 hit = P.st.phit[s];
            if (__float_as_uint(hit.w) != 0xffffffffu) {
                hit_ok = true;
                st = load_path(P, s);
                make_vhit<kSorted, kInst>(P, s, st.org, st.dir, hit, h, status);
                const float3 seg = h.pos - st.org;
                const float d2 = dot(seg, seg);
                const float cos_in = fabsf(dot(h.n, h.view));
                st.dvcm *= d2;
                st.dvcm *= 1.0f / cos_in;
                st.dvc *= 1.0f / cos_in;
                st.dvm *= 1.0f / cos_in;
                rng = load_rng(P, s, (uint64_t(c.pass) * 2 + 1) * N + s);
                if (!h.delta) st.flags |= kPathNonDelta;
                const uint32_t n_emitters = P.light_count + (P.ibl ? 1u : 0u);
                const float light_pick = n_emitters ? 1.0f / float(n_emitters) : 0.0f;
                if (!h.delta) {
                    record = true;
                    // next-event estimation to light set 0 and the environment (tech report sec. 5.4; wLight = 0
                    // for the quads, which BSDF rays cannot hit)
                    if (st.len + 1 <= P.max_len && n_emitters > 0) {
                        const float pick = pcg_float(rng);
                        uint32_t li = uint32_t(pick * float(n_emitters));
                        li = li < n_emitters - 1 ? li : n_emitters - 1;
                        if (li == P.light_count) {
                            const float r0 = pcg_float(rng), r1 = pcg_float(rng), r2 = pcg_float(rng);
                            const float r3 = pcg_float(rng);
                            const IblDev& ibl = *P.ibl;
                            to_l = ibl_env_direction(ibl, r0, r1, r2, r3);
                            const float pdf_w = ibl_env_pdf(ibl, to_l);
                            if (pdf_w > 0.0f) {
                                float fwd, rev;
                                const float3 f = bsdf_evaluate(h.s, h.view, to_l, fwd, rev);
                                if (nonzero(f)) {
                                    const float3 rad = ibl_radiance(ibl, to_l);
                                    fwd *= h.cont;
                                    rev *= h.cont;
                                    const float emission_pdf_w = pdf_w * P.env_disc_pdf;
                                    const float cos_to_light = fabsf(dot(h.n, to_l));
                                    const float w_light = fwd / (light_pick * pdf_w);
                                    const float w_camera = (emission_pdf_w * cos_to_light / pdf_w) *
                                                           (c.vm_weight + st.dvcm + st.dvc * rev);
                                    const float mis = 1.0f / (w_light + 1.0f + w_camera);
                                    contrib = st.thr * ((mis / (light_pick * pdf_w)) * (rad * f));
                                    tfar = kFloatMax;
                                    nee_ray = nonzero(contrib);
                                }
                            }
                        } else {
                            const QuadLight L = P.lights[li];
                            const float u = pcg_float(rng), v = pcg_float(rng);
                            const float3 lp = L.position - 0.5f * L.x - 0.5f * L.z + u * L.x + v * L.z;
                            const float pdf_a = 1.0f / (length(L.x) * length(L.z));
                            to_l = lp - h.pos;
                            const float dl2 = dot(to_l, to_l), dl = sqrtf(dl2);
                            to_l = to_l * (1.0f / dl);
                            const float cos_light = dot(normalize(L.direction), -to_l);
                            if (cos_light > 0.0f) {
                                float fwd, rev;
                                const float3 f = bsdf_evaluate(h.s, h.view, to_l, fwd, rev);
                                if (nonzero(f)) {
                                    rev *= h.cont;
                                    const float direct_pdf_w = pdf_a * dl2 / cos_light;
                                    const float emission_pdf_w = pdf_a * cos_light / kPi;
                                    const float cos_to_light = fabsf(dot(h.n, to_l));
                                    const float w_camera = (emission_pdf_w * cos_to_light / (direct_pdf_w * cos_light)) *
                                                           (c.vm_weight + st.dvcm + st.dvc * rev);
                                    const float mis = 1.0f / (1.0f + w_camera);
                                    contrib = st.thr * ((mis / (light_pick * direct_pdf_w)) * (L.radiance * f));
                                    tfar = dl * (1.0f - 1e-4f);
                                    nee_ray = nonzero(contrib);
                                }
                            }
                        }
                    }
                    // light vertices of path s that a connection may join (path length bound)
                    const uint32_t lcount = P.st.vcount[s];
                    const float4* lslots = P.st.verts + size_t(s) * P.slots * kVertF4;
                    while (nvc < lcount &&
                           unpack_len(__float_as_uint(lslots[size_t(nvc) * kVertF4].w)) + 1 + st.len <= P.max_len)
                        ++nvc;
                }
            } else if (P.ibl) {
                // the path leaves the scene: the environment's radiance with the camera-hit weight (ConnectToSkyLight,
                // VCM.cpp:171-187; tech report sec. 5.2); camera rays and chains of Dirac vertices see the miss
                // image, with weight 1 (no other strategy makes them)
                const PathState ms = load_path(P, s);
                const IblDev& ibl = *P.ibl;
                const float3 rad = (ms.flags & kPathNonDelta) ? ibl_radiance(ibl, ms.dir) : ibl_miss(ibl, ms.dir);
                float mis = 1.0f;
                if (ms.len > 1) {
                    const float pdf_w = ibl_env_pdf(ibl, ms.dir);
                    const float light_pick = 1.0f / float(P.light_count + 1u);
                    const float direct_pdf_a = pdf_w * light_pick;
                    const float emission_pdf = pdf_w * P.env_disc_pdf * light_pick;
                    const float w_camera = direct_pdf_a * ms.dvcm + emission_pdf * ms.dvc;
                    mis = 1.0f / (1.0f + w_camera);
                }
                const float3 env = mis * (ms.thr * rad);
                if (nonzero(env)) splat(P.accum, s, env);
            }
        }
        // camera-vertex record with the state at the vertex, its connection pairs, the next-event segment
        const uint32_t vi = warp_append(&P.st.counters[5], record);
        if (record) store_camera_vertex(P.st.cverts + size_t(vi) * kCamF4, h, st, s);
        const uint32_t pair0 = warp_reserve(&P.st.counters[6], nvc);
        for (uint32_t k = 0; k < nvc; ++k) P.st.pairs[pair0 + k] = make_uint2(vi, k);
        const uint32_t sq = warp_append(&P.st.counters[2], nee_ray);
        if (nee_ray) push_shadow(P, sq, h, to_l, tfar, contrib, s);
        if (hit_ok) {
            if (st.len < P.max_len) {
                cont = scatter(rng, h, c, st, false);
                if (cont) store_path(P, s, st);
            }
            P.st.prng[s] = rng.state;
        }
        const uint32_t q = warp_append(&P.st.counters[next], cont);
        if (cont) P.st.queue[next][q] = s;
    }
    if (status) atomicOr(P.err, status);
}

// One thread per (camera vertex, light vertex) pair: ConnectPathVertices (VCM.cpp:293-359), with the light
// side oriented f(v = toward the camera vertex, l = toward the previous light vertex) and the cosine at the
// connection carried.
__global__ void __launch_bounds__(kBlock) k_c_connect(VcmParams P) {
    const VcmConsts c = P.st.consts[*P.st.iter];
    const uint32_t n = P.st.counters[6];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        bool ray = false;
        float3 dir = f3(0.0f), contrib = f3(0.0f);
        float tfar = 0.0f;
        CameraVertex cv;
        cv.pixel = 0;
        if (e < n) {
            const uint2 pr = P.st.pairs[e];
            cv = load_camera_vertex(P.st.cverts + size_t(pr.x) * kCamF4);
            const LightVertex lv = load_vertex(P.st.verts + (size_t(cv.pixel) * P.slots + pr.y) * kVertF4);
            dir = lv.pos - cv.pos;
            const float dist2 = dot(dir, dir), dist = sqrtf(dist2);
            dir = dir * (1.0f / dist);
            const Surface cs = make_surface_frame(*cv.mat, cv.t, cv.n, cross(cv.n, cv.t) * cv.bsign, cv.view,
                                                  cv.base);
            float cfwd, crev, lfwd, lrev;
            const float3 cf = bsdf_evaluate(cs, cv.view, dir, cfwd, crev);
            if (nonzero(cf)) {
                const Surface ls = make_surface_frame(*lv.mat, lv.t, lv.n, cross(lv.n, lv.t) * lv.bsign,
                                                      lv.view, lv.base);
                const float lcont = continuation_probability(ls);
                const float3 lfa = bsdf_evaluate(ls, -dir, lv.view, lrev, lfwd);
                const float lcos_view = fabsf(dot(lv.n, lv.view));
                const float3 lf = lcos_view > 0.0f ? lfa * (fabsf(dot(lv.n, dir)) / lcos_view) : f3(0.0f);
                if (nonzero(lf)) {
                    cfwd *= cv.cont; crev *= cv.cont;
                    lfwd *= lcont; lrev *= lcont;
                    const float cos_cam_v = fabsf(dot(dir, cv.n));
                    const float cos_light_v = fabsf(dot(-dir, lv.n));
                    const float cam_pdf_a = cfwd * cos_light_v / dist2;
                    const float light_pdf_a = lfwd * cos_cam_v / dist2;
                    const float w_light = cam_pdf_a * (c.vm_weight + lv.dvcm + lv.dvc * lrev);
                    const float w_camera = light_pdf_a * (c.vm_weight + cv.dvcm + cv.dvc * crev);
                    const float mis = 1.0f / (w_light + 1.0f + w_camera);
                    contrib = cv.thr * lv.thr * ((mis / dist2) * (cf * lf));
                    const float bias = 0.1f * cv.err;
                    tfar = dist - 16.0f * bias;
                    ray = nonzero(contrib);
                }
            }
        }
        const uint32_t sq = warp_append(&P.st.counters[2], ray);
        if (ray) {
            const float3 o = offset_origin(cv.pos, cv.n, cv.err, dir, 0.1f);
            P.st.so[sq] = make_float4(o.x, o.y, o.z, cv.err);
            P.st.sd[sq] = make_float4(dir.x, dir.y, dir.z, tfar);
            P.st.sc[sq] = make_float4(contrib.x, contrib.y, contrib.z, __uint_as_float(cv.pixel));
        }
    }
}

// Positions of the stored vertices in cell order (position, slot bits): the merge's distance test reads
// consecutive entries.
__global__ void __launch_bounds__(256) k_gather_positions(VcmParams P) {
    const uint32_t total = P.st.vpos[P.npaths];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        const uint32_t slot = P.sorted_index[k];
        const float4 a = P.st.verts[size_t(slot) * kVertF4];
        P.st.spos[k] = make_float4(a.x, a.y, a.z, __uint_as_float(slot));
    }
}

// One warp per camera vertex (MergeVertices + SearchHashGrid, VCM.cpp:362-409, VCMHashGrid.cpp:107-155;
// tech report sec. 5.6): the ranges of the 2x2x2 cells around it are concatenated (a cell visited twice
// when two of the eight cells hash to one bucket, as the sequential search visits it), lanes test the
// concatenation against the radius and compact the hits, all lanes evaluate the compacted candidates,
// each keeps a partial sum and a fixed xor-tree reduction adds them.
// Five blocks per SM (96 registers, about 150 bytes of spills a thread): passes 2 % faster on the room at 1280 x 720
// than four blocks at 128 registers (20.70 against 21.12 ms), which were 7 % faster than the 143-register build.
__global__ void __launch_bounds__(kBlock, 5) k_c_merge(VcmParams P) {
    __shared__ uint32_t mbuf[kBlock / 32][64];  // per warp: candidates inside the radius, awaiting evaluation
    const VcmConsts c = P.st.consts[*P.st.iter];
    const uint32_t n = P.st.counters[5];
    const uint32_t N = P.npaths;
    const float* grid = P.st.grid;
    if (!P.merging || P.st.vpos[N] == 0) return;
    const float3 glo = f3(grid[0], grid[1], grid[2]), ghi = f3(grid[3], grid[4], grid[5]);
    const float ginv = grid[6], gr2 = grid[7];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        const float4* rec = P.st.cverts + size_t(i) * kCamF4;
        const float4 r0 = rec[0];
        const float3 pos = f3(r0.x, r0.y, r0.z);
        const float3 dmin = pos - glo, dmax = ghi - pos;
        if (!(dmin.x >= 0.0f && dmin.y >= 0.0f && dmin.z >= 0.0f && dmax.x >= 0.0f && dmax.y >= 0.0f &&
              dmax.z >= 0.0f))
            continue;  // uniform across the warp
        const float3 cp = ginv * dmin;
        const float fx = floorf(cp.x), fy = floorf(cp.y), fz = floorf(cp.z);
        const int x0 = int(fx) - (cp.x - fx < 0.5f ? 1 : 0);
        const int y0 = int(fy) - (cp.y - fy < 0.5f ? 1 : 0);
        const int z0 = int(fz) - (cp.z - fz < 0.5f ? 1 : 0);
        // lane j < 8 owns cell j = (dx, dy, dz) in the search order dz, dy, dx
        uint32_t cb = 0, cn = 0;
        if (lane < 8) {
            const int dx = int(lane & 1u), dy = int((lane >> 1) & 1u), dz = int(lane >> 2);
            const uint32_t cell = cell_hash(x0 + dx, y0 + dy, z0 + dz, N);
            cb = P.st.cell_start[cell];
            cn = P.st.cell_start[cell + 1] - cb;
        }
        uint32_t incl = cn;  // inclusive prefix of the counts over lanes 0..7
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= uint32_t(o)) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 7);
        if (total == 0) continue;
        const CameraVertex cv = load_camera_vertex(rec);
        const Surface cs = make_surface_frame(*cv.mat, cv.t, cv.n, cross(cv.n, cv.t) * cv.bsign, cv.view,
                                              cv.base);
        float3 merged = f3(0.0f);
        // two phases so that the BSDF work runs on full warps: lanes test 32 candidates at a time against
        // the radius and append the ones inside to the warp's buffer; every 32 buffered candidates are
        // evaluated by all lanes together
        uint32_t* buf = mbuf[threadIdx.x >> 5];
        uint32_t pending = 0;
        const uint32_t below = (1u << lane) - 1u;
        auto evaluate = [&](uint32_t vslot) {
            const LightVertex lv = load_vertex(P.st.verts + size_t(vslot) * kVertF4);
            if (cv.len + lv.len > P.max_len) return;
            // the reference merges only between surfaces of the same transparency (VCM.cpp:372-375)
            const uint32_t lt = (lv.mat->flags & kMaterialTransparent) ? 1u : 0u;
            if (cv.transparent != lt) return;
            float fwd, rev;
            const float3 fc = bsdf_evaluate(cs, cv.view, lv.view, fwd, rev);
            const float cosl = fabsf(dot(cv.n, lv.view));
            if (!nonzero(fc) || cosl == 0.0f) return;
            const float lcont = saturate(max3(lv.base));
            fwd *= cv.cont;
            rev *= lcont;
            const float w_light = lv.dvcm * c.vc_weight + lv.dvm * fwd;
            const float w_camera = cv.dvcm * c.vc_weight + cv.dvm * rev;
            const float mis = 1.0f / (w_light + 1.0f + w_camera);
            merged = merged + (mis / cosl) * (fc * lv.thr);
        };
        for (uint32_t t0 = 0; t0 < total; t0 += 32) {
            const uint32_t t = t0 + lane;
            bool in = false;
            uint32_t vslot = 0;
            // the cell whose range of the concatenation holds t: lanes 0..7 hold each cell's start (cb) and
            // inclusive end (incl); shuffled per round rather than held in registers across the loop
            uint32_t start = 0, b = 0, prev = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const uint32_t eq = __shfl_sync(0xffffffffu, incl, q);
                const uint32_t bq = __shfl_sync(0xffffffffu, cb, q);
                if (t >= prev && t < eq) { b = bq; start = prev; }
                prev = eq;
            }
            if (t < total) {
                const float4 sp = P.st.spos[b + (t - start)];
                const float3 dd = pos - f3(sp.x, sp.y, sp.z);
                in = dot(dd, dd) <= gr2;
                vslot = __float_as_uint(sp.w);
            }
            const uint32_t m = __ballot_sync(0xffffffffu, in);
            if (in) buf[pending + __popc(m & below)] = vslot;
            pending += __popc(m);
            __syncwarp();
            if (pending >= 32) {
                evaluate(buf[lane]);
                __syncwarp();
                const uint32_t rest = pending - 32;
                const uint32_t v = lane < rest ? buf[32 + lane] : 0u;
                __syncwarp();
                if (lane < rest) buf[lane] = v;
                __syncwarp();
                pending = rest;
            }
        }
        if (lane < pending) evaluate(buf[lane]);
        __syncwarp();
        for (int o = 16; o > 0; o >>= 1) {
            merged.x += __shfl_xor_sync(0xffffffffu, merged.x, o);
            merged.y += __shfl_xor_sync(0xffffffffu, merged.y, o);
            merged.z += __shfl_xor_sync(0xffffffffu, merged.z, o);
        }
        if (lane == 0) {
            const float4 e = rec[4];  // throughput, reloaded rather than held across the loop
            const float3 mc = c.vm_norm * (f3(e.x, e.y, e.z) * merged);
            if (nonzero(mc)) splat(P.accum, __float_as_uint(rec[3].w), mc);
        }
    }
}

__global__ void k_pass_end(uint32_t* iter) {
    if (threadIdx.x == 0) *iter += 1u;
}

}  // namespace

namespace {

// One layout walk for both sizing and carving.
template <typename Take>
void vcm_layout(VcmState& st, Take take, uint32_t paths, uint32_t max_len, uint32_t passes) {
    const uint32_t slots = max_len - 1;
    const size_t nv = size_t(paths) * slots;
    const size_t ntiles = (nv + kSortTile - 1) / kSortTile;
    const size_t scan_n = std::max<size_t>(std::max<size_t>(size_t(paths) + 1, 256 * ntiles), 1);
    const size_t shadow = size_t(paths) * max_len;  // per bounce: one next-event + up to max_len - 1 connections
    st.verts = reinterpret_cast<float4*>(take(16 * kVertF4 * nv));
    st.vcount = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.vpos = reinterpret_cast<uint32_t*>(take(4ull * (paths + 1)));
    st.po = reinterpret_cast<float4*>(take(16ull * paths));
    st.pd = reinterpret_cast<float4*>(take(16ull * paths));
    st.pt = reinterpret_cast<float4*>(take(16ull * paths));
    st.plen = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.prng = reinterpret_cast<uint64_t*>(take(8ull * paths));
    st.phit = reinterpret_cast<float4*>(take(16ull * paths));
    st.phinst = reinterpret_cast<uint2*>(take(8ull * paths));
    st.queue[0] = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.queue[1] = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.queue_sorted = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.cls = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.base = reinterpret_cast<float4*>(take(16ull * paths));
    st.so = reinterpret_cast<float4*>(take(16 * shadow));
    st.sd = reinterpret_cast<float4*>(take(16 * shadow));
    st.sc = reinterpret_cast<float4*>(take(16 * shadow));
    st.shadow_capacity = uint32_t(shadow);
    st.counters = reinterpret_cast<uint32_t*>(take(4 * 64));
    st.rays = reinterpret_cast<unsigned long long*>(take(16));
    st.cverts = reinterpret_cast<float4*>(take(16ull * kCamF4 * paths));
    st.pairs = reinterpret_cast<uint2*>(take(8 * nv));
    st.spos = reinterpret_cast<float4*>(take(16 * nv));
    for (int k = 0; k < 2; ++k) {
        st.keys[k] = reinterpret_cast<uint32_t*>(take(4 * nv));
        st.vals[k] = reinterpret_cast<uint32_t*>(take(4 * nv));
    }
    st.cell_count = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.cell_start = reinterpret_cast<uint32_t*>(take(4ull * (paths + 1)));
    st.hist = reinterpret_cast<uint32_t*>(take(4 * 256 * ntiles));
    st.hist_off = reinterpret_cast<uint32_t*>(take(4 * (256 * ntiles + 1)));
    st.scan_tmp = reinterpret_cast<uint32_t*>(take(4 * ((scan_n + kScanTile - 1) / kScanTile + 1)));
    st.bounds_part = reinterpret_cast<float*>(take(4 * 6 * kBoundsBlocks));
    st.grid = reinterpret_cast<float*>(take(4 * 16));
    st.iter = reinterpret_cast<uint32_t*>(take(4 * 4));
    st.consts = reinterpret_cast<VcmConsts*>(take(sizeof(VcmConsts) * passes));
    st.paths = paths;
    st.slots_per_path = slots;
    st.consts_capacity = passes;
}

}  // namespace

VcmState vcm_state_carve(void* block, uint32_t paths, uint32_t max_len, uint32_t passes) {
    char* p = static_cast<char*>(block);
    VcmState st;
    vcm_layout(st, [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    }, paths, max_len, passes);
    return st;
}

size_t vcm_state_block_bytes(uint32_t paths, uint32_t max_len, uint32_t passes) {
    size_t total = 0;
    VcmState st;
    vcm_layout(st, [&](size_t bytes) {
        total += (bytes + 255) & ~size_t(255);
        return static_cast<char*>(nullptr);
    }, paths, max_len, passes);
    return total;
}

cudaError_t vcm_upload_constants(const VcmState& st, const VcmConsts* host_consts, uint32_t passes,
                                 cudaStream_t stream) {
    if (passes > st.consts_capacity) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemcpyAsync(st.consts, host_consts, sizeof(VcmConsts) * passes, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(st.iter, 0, sizeof(uint32_t), stream);
    return e;
}

cudaError_t vcm_run_passes(const PtScene& sc, const VcmCamera& cam, const VcmSettings& set, uint32_t passes,
                           const VcmState& st, double* d_accum, uint32_t* d_err, cudaStream_t stream,
                           GraphCache* graphs) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    VcmParams P;
    std::memset(&P, 0, sizeof(P));
    P.nodes = sc.nodes;
    P.tris = sc.tris;
    P.materials = sc.materials;
    P.material_count = sc.material_count;
    P.lights = sc.lights;
    P.light_count = 0;
    P.ptex_faces = static_cast<const PtexFace*>(sc.ptex_faces);
    P.ptex_texels = static_cast<const __half*>(sc.ptex_texels);
    P.ptex_face_count = sc.ptex_face_count;
    P.attrs = sc.attrs;
    P.attr_count = sc.attr_count;
    P.insts = sc.insts;
    P.cam.x = make_float3(cam.cam.x[0], cam.cam.x[1], cam.cam.x[2]);
    P.cam.y = make_float3(cam.cam.y[0], cam.cam.y[1], cam.cam.y[2]);
    P.cam.z = make_float3(cam.cam.z[0], cam.cam.z[1], cam.cam.z[2]);
    P.cam.position = make_float3(cam.cam.position[0], cam.cam.position[1], cam.cam.position[2]);
    P.cam.width = float(cam.cam.width);
    P.cam.height = float(cam.cam.height);
    P.image_plane = cam.image_plane;
    P.width = cam.cam.width;
    P.height = cam.cam.height;
    P.npaths = st.paths;
    P.max_len = set.max_len;
    P.slots = st.slots_per_path;
    P.seed = set.seed;
    P.merging = set.merging;
    P.accum = d_accum;
    P.st = st;
    P.err = d_err;
    P.lights = sc.lights + set.light_first;
    P.light_count = set.light_count;
    if (sc.ibl) {
        // the environment's emission disc: the bounding sphere of the scene's bounding box, radius half its diagonal
        float d2 = 0.0f;
        for (int a = 0; a < 3; ++a) {
            const float e = sc.hi[a] - sc.lo[a];
            d2 += e * e;
        }
        P.ibl = sc.ibl;
        P.env_center = make_float3(0.5f * (sc.lo[0] + sc.hi[0]), 0.5f * (sc.lo[1] + sc.hi[1]), 0.5f * (sc.lo[2] + sc.hi[2]));
        P.env_radius = 0.5f * std::sqrt(d2);
        P.env_disc_pdf = (1.0f / kPi) * (1.0f / (P.env_radius * P.env_radius));
    }

    const uint32_t N = st.paths;
    const size_t nv = size_t(N) * st.slots_per_path;
    const uint32_t ntiles = uint32_t((nv + kSortTile - 1) / kSortTile);
    int bits = 0;
    while (bits < 32 && (uint64_t(N - 1) >> bits) != 0) ++bits;  // cells = N: keys below N
    const int radix_passes = (bits + 7) / 8;
    const uint32_t list_grid = std::min<uint32_t>((N + 255) / 256, uint32_t(sms) * 16);
    int cur = 0;
    for (int r = 0; r < radix_passes; ++r) cur ^= 1;
    P.sorted_index = st.vals[cur];
    // traversal blocks of 256 or 128 threads, 1024 threads per SM either way (the scene's tuned block size)
    const int tb = (set.trace_block == 256 && sc.bvh_kind == 0) ? 256 : 128;
    const int trace_grid = sms * (1024 / tb);
    const int shade_grid = sms * 8;
    // the register-heavy shading, connection and merge kernels run one resident wave of grid-striding blocks (a
    // second partial wave left SMs idle at its tail: VCM room passes 2.4 % faster)
    auto wave = [&](const void* kernel) {
        int blocks = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, kBlock, 0);
        return sms * std::max(blocks, 1);
    };
    // scenes with instances: the instanced traversal (128-thread blocks, 4 per SM: its 40-entry stacks) and the
    // shading kernels that read a hit's scene through its instances
    const bool inst = sc.insts != nullptr;
    const int inst_grid = sms * 4;
    auto extend = [&](cudaStream_t stream, int cur) {
        if (inst) k_extend<2, 128><<<inst_grid, 128, 0, stream>>>(P, cur);
        else if (sc.bvh_kind != 0) k_extend<1, 128><<<trace_grid, 128, 0, stream>>>(P, cur);
        else if (tb == 256) k_extend<0, 256><<<trace_grid, 256, 0, stream>>>(P, cur);
        else k_extend<0, 128><<<trace_grid, 128, 0, stream>>>(P, cur);
    };
    auto shadow = [&](cudaStream_t stream) {
        if (inst) k_shadow<2, 128><<<inst_grid, 128, 0, stream>>>(P);
        else if (sc.bvh_kind != 0) k_shadow<1, 128><<<trace_grid, 128, 0, stream>>>(P);
        else if (tb == 256) k_shadow<0, 256><<<trace_grid, 256, 0, stream>>>(P);
        else k_shadow<0, 128><<<trace_grid, 128, 0, stream>>>(P);
    };
    // Textures are filtered by the texture pass (k_vtexture) over the sorted queue when the hits are sorted; the
    // plain form (SEL_OPTION_MATERIAL_SORT 0) filters triangle Ptex inline in queue order, and quad-mesh Ptex, which
    // only the texture pass evaluates, over the queue in its own order
    const bool sort = sc.sort_hint != 0 || inst;
    const bool quads = sc.ptex_quads != 0;
    const bool pretex = sort || quads;
    const void* l_fn = inst ? reinterpret_cast<const void*>(&k_l_shade<true, true>)
                            : pretex ? reinterpret_cast<const void*>(&k_l_shade<true, false>)
                                     : reinterpret_cast<const void*>(&k_l_shade<false, false>);
    const void* c_fn = inst ? reinterpret_cast<const void*>(&k_c_shade<true, true>)
                            : pretex ? reinterpret_cast<const void*>(&k_c_shade<true, false>)
                                     : reinterpret_cast<const void*>(&k_c_shade<false, false>);
    const int l_grid = wave(l_fn);
    const int c_grid = wave(c_fn);
    const int connect_grid = wave(reinterpret_cast<const void*>(&k_c_connect));
    const int merge_grid = wave(reinterpret_cast<const void*>(&k_c_merge));
    // material-class sort and Ptex of a bounce's hits; returns the queue the shading kernel reads
    auto sort_hits = [&](cudaStream_t stream, int cur) -> const uint32_t* {
        if (!pretex) return st.queue[cur];
        const uint32_t* q = st.queue[cur];
        if (sort) {
            k_vclass_reset<<<1, 32, 0, stream>>>(st.counters);
            if (inst) k_vclassify<true><<<shade_grid, kBlock, 0, stream>>>(P, cur);
            else k_vclassify<false><<<shade_grid, kBlock, 0, stream>>>(P, cur);
            k_vclass_offsets<<<1, 32, 0, stream>>>(st.counters);
            k_vclass_scatter<<<shade_grid, kBlock, 0, stream>>>(P, cur);
            q = st.queue_sorted;
        }
        if (inst && quads) k_vtexture<true, true><<<shade_grid, kBlock, 0, stream>>>(P, cur, q);
        else if (inst) k_vtexture<true, false><<<shade_grid, kBlock, 0, stream>>>(P, cur, q);
        else if (quads) k_vtexture<false, true><<<shade_grid, kBlock, 0, stream>>>(P, cur, q);
        else k_vtexture<false, false><<<shade_grid, kBlock, 0, stream>>>(P, cur, q);
        return q;
    };
    // one pass; identical launches every pass (the pass reads its constants through st.iter)
    auto enqueue = [&](cudaStream_t stream) {
        // light sub-paths: vertices and light tracing
        k_reset<<<1, 32, 0, stream>>>(st.counters);
        k_l_generate<<<shade_grid, kBlock, 0, stream>>>(P);
        for (uint32_t b = 0; b + 1 < set.max_len; ++b) {
            const int cur = int(b & 1u);
            k_bounce_reset<<<1, 32, 0, stream>>>(st.counters, cur ^ 1);
            extend(stream, cur);
            const uint32_t* q = sort_hits(stream, cur);
            if (inst) k_l_shade<true, true><<<l_grid, kBlock, 0, stream>>>(P, cur, q);
            else if (pretex) k_l_shade<true, false><<<l_grid, kBlock, 0, stream>>>(P, cur, q);
            else k_l_shade<false, false><<<l_grid, kBlock, 0, stream>>>(P, cur, q);
            shadow(stream);
        }
        // hash grid over the stored vertices
        k_bounds<<<kBoundsBlocks, 256, 0, stream>>>(P);
        k_bounds_final<<<1, 32, 0, stream>>>(P, kBoundsBlocks);
        scan_exclusive(st.vcount, N, st.vpos, st.scan_tmp, stream);
        cudaMemsetAsync(st.cell_count, 0, sizeof(uint32_t) * N, stream);
        k_keys<<<list_grid, 256, 0, stream>>>(P);
        scan_exclusive(st.cell_count, N, st.cell_start, st.scan_tmp, stream);
        int from = 0;
        for (int r = 0; r < radix_passes; ++r) {
            k_radix_hist<<<ntiles, 256, 0, stream>>>(st.keys[from], st.vpos + N, 8 * r, st.hist, ntiles);
            scan_exclusive(st.hist, 256 * ntiles, st.hist_off, st.scan_tmp, stream);
            k_radix_scatter<<<ntiles, 256, 0, stream>>>(st.keys[from], st.vals[from], st.keys[from ^ 1], st.vals[from ^ 1],
                                                        st.vpos + N, 8 * r, st.hist_off, ntiles);
            from ^= 1;
        }
        k_gather_positions<<<list_grid, 256, 0, stream>>>(P);
        // camera sub-paths: next-event estimation, connections, merging
        k_reset<<<1, 32, 0, stream>>>(st.counters);
        k_c_generate<<<shade_grid, kBlock, 0, stream>>>(P);
        for (uint32_t b = 0; b < set.max_len; ++b) {
            const int cur = int(b & 1u);
            k_bounce_reset<<<1, 32, 0, stream>>>(st.counters, cur ^ 1);
            extend(stream, cur);
            const uint32_t* q = sort_hits(stream, cur);
            if (inst) k_c_shade<true, true><<<c_grid, kBlock, 0, stream>>>(P, cur, q);
            else if (pretex) k_c_shade<true, false><<<c_grid, kBlock, 0, stream>>>(P, cur, q);
            else k_c_shade<false, false><<<c_grid, kBlock, 0, stream>>>(P, cur, q);
            k_c_connect<<<connect_grid, kBlock, 0, stream>>>(P);
            k_c_merge<<<merge_grid, kBlock, 0, stream>>>(P);
            shadow(stream);
        }
        k_pass_end<<<1, 32, 0, stream>>>(st.iter);
    };
    struct Key {
        VcmParams P;
        int kind, sms, radix_passes, sort, tb, quads;
    } key;
    std::memset(&key, 0, sizeof(key));
    std::memcpy(&key.P, &P, sizeof(P));
    key.kind = sc.bvh_kind;
    key.tb = tb;
    key.sms = sms;
    key.radix_passes = radix_passes;
    key.sort = sort ? 1 : 0;
    key.quads = quads ? 1 : 0;
    return replay(graphs, &key, sizeof(key), stream, passes, enqueue);
}

cudaError_t vcm_render(const PtScene& sc, const VcmCamera& cam, const VcmSettings& set, const VcmConsts* host_consts,
                       uint32_t passes, const VcmState& st, double* d_accum, uint32_t* d_err, cudaStream_t stream,
                       GraphCache* graphs) {
    cudaError_t e = vcm_upload_constants(st, host_consts, passes, stream);
    if (e != cudaSuccess) return e;
    return vcm_run_passes(sc, cam, set, passes, st, d_accum, d_err, stream, graphs);
}

}  // namespace sel
