// ORACLE harness (test infrastructure only): runs the reference's own path tracer and the functions around it,
// compiled from the reference checkout where they lie (oracle/ref/build_ref.py), to produce golden images and
// golden scalar tables under tests/golden/.  The product never loads anything built from this file.
//
// Reference code run here, unmodified:
//   * EvaluatePath / RayPick / OcclusionRay   Source/Applications/Selas/Source/PathTracer.cpp:71-258 (static
//     functions: the file is compiled as part of this translation unit so that the harness can call them);
//   * ShadeHitPosition / ShadeHitBatch / TraceRayBatch / TraceOcclusionBatch, and GeneratePrimaryRays' ray set-up
//     Source/Applications/Selas/Source/DeferredPathTracer.cpp:61-346 (static too: compiled in this unit), the
//     integrator main.cpp:121 runs, with JitteredCameraRay's correlated multi-jittered form (Camera.cpp:77-86);
//   * CalculateSurfaceParams, OffsetRayOrigin  Source/Core/Shading/SurfaceParameters.cpp:144-247,393-408;
//   * ModelDataFromRayIds                      Source/Core/SceneLib/SceneResource.cpp:362-378,
//                                              Source/Core/SceneLib/SubsceneResource.cpp:186-195;
//   * NextEventEstimation, LightingPdf, EvaluateBackground(Miss)  Source/Core/Shading/AreaLighting.cpp:113-153,
//     353-436, with Source/Core/GeometryLib/RectangulerLightSampler.cpp:17-97;
//   * JitteredCameraRay, InitializeRayCastCamera  Source/Core/GeometryLib/Camera.cpp:62-115;
//   * Ibl, SampleIbl, SampleIblMiss, SampleIBlPdf  Source/Core/SceneLib/ImageBasedLightResource.cpp:81-268, with
//     the densities of Source/Core/BuildCommon/BuildImageBasedLight.cpp:24-101 (static functions: that file is
//     compiled as part of this translation unit too);
//   * the BSDF (Shading/Disney.cpp etc.), media (Shading/VolumetricScattering.cpp, IsotropicScattering.cpp),
//     2D texture filtering (TextureLib/TextureFiltering.h) and Ptex 2.2 (Middleware/ptex/Include).
//   * CalculateIterationConstants              Source/Applications/Selas/Source/VCMCommon.cpp:91-112.
//
// Supplied by this file in place of code that needs Embree, the asset pipeline or the threading layer:
//   * Embree 3.2's rtcIntersect1 / rtcOccluded1 / rtcInterpolate (the reference binds only their binary
//     release): the oracle's watertight BVH traversal (oracle/oracle_query.cpp) with instID = {0, 0} (one subscene
//     instance holding one model instance, the two table levels ModelDataFromRayIds walks), and the interpolation
//     (1 - u - v) a0 + u a1 + v a2 over the triangle's three corner values.  Every other Embree entry point the
//     compiled files reference is an aborting stub (embree_stubs.c): scenes are put together here, not cooked.
//   * CSampler (MathLib/Sampler.h:14-29): PCG32 with one stream per path (stream = pass * W * H + pixel, the
//     sampling the GPU path tracer uses), the reference's own MT19937 (MathLib/Random.cpp, one engine per pixel
//     seeded seed + pixel), or uniforms prescribed by the caller (scalar probes).
//   * TextureCache / GeometryCache members (lookups into this file's tables), FramebufferWriter_Write (adds the
//     path's two layers to a per-pixel FP64 sum), and aborting stubs for file reading.
//   * PathTracingBatcher (Shading/PathTracingBatcher.h; its .cpp needs <windows.h> file mappings): per-thread
//     queues, so that the deferred tracer's batch functions process one path at a time (its ray, its hit, its
//     shadow rays, its bounce ray) and each path draws its own PCG32 stream in the order the reference draws it;
//     rtcIntersect8 / rtcOccluded8 over the oracle's BVH lane by lane.

#include "PathTracer.cpp"
#include "DeferredPathTracer.cpp"
#include "BuildCommon/BuildImageBasedLight.cpp"
#include "VCMCommon.h"

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "Ptexture.h"
#include "oracle_query.h"

using namespace Selas;

// ---------------------------------------------------------------------------------------------------
// Sampler
// ---------------------------------------------------------------------------------------------------
namespace {

enum SamplerMode { kPcg = 0, kMt = 1, kPrescribed = 2 };

struct Pcg {
    uint64_t state = 0, inc = 1;
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
};

thread_local int tl_mode = kPcg;
thread_local Pcg tl_pcg;
thread_local const float* tl_uniforms = nullptr;
thread_local int tl_count = 0;
thread_local int tl_used = 0;

}  // namespace

namespace Selas {
void CSampler::Initialize(uint32 seed) {
    twister.data = nullptr;
    if (tl_mode == kMt) Random::MersenneTwisterInitialize(&twister, seed);
}
void CSampler::Shutdown() {
    if (twister.data) Random::MersenneTwisterShutdown(&twister);
}
void CSampler::Reseed(uint32 seed) {
    if (tl_mode == kMt) Random::MersenneTwisterReseed(&twister, seed);
}
float CSampler::UniformFloat() {
    if (tl_mode == kMt) return Random::MersenneTwisterFloat(&twister);
    if (tl_mode == kPrescribed) return tl_used < tl_count ? tl_uniforms[tl_used++] : 0.5f;
    return float(tl_pcg.next() >> 8) * (1.0f / 16777216.0f);
}
uint32 CSampler::UniformUInt32() { return tl_mode == kMt ? Random::MersenneTwisterUint32(&twister) : tl_pcg.next(); }
float3 CSampler::UniformSphere() {
    const float r0 = UniformFloat();
    const float r1 = UniformFloat();
    const float u = 2.0f * r1 - 1.0f;
    const float norm = Math::Sqrtf(Max(0.0f, 1.0f - u * u));
    const float theta = Math::TwoPi_ * r0;
    return float3(norm * Math::Cosf(theta), u, norm * Math::Sinf(theta));
}
float CSampler::UniformSpherePdf() { return Math::Inv4Pi_; }
}  // namespace Selas

// ---------------------------------------------------------------------------------------------------
// Embree 3.2 queries over the oracle's BVH
// ---------------------------------------------------------------------------------------------------
namespace {

struct ShimScene {
    void* bvh = nullptr;
};

// A triangle mesh's vertex attributes: corner values of its triangles in the soup (normals 9, tangents 12,
// uvs 6 floats per triangle), `first` = the soup index of its primID 0.
struct ShimGeometry {
    int64_t first = 0;
    const float* normals = nullptr;
    const float* tangents = nullptr;
    const float* uvs = nullptr;
};

}  // namespace

extern "C" {

void rtcIntersect1(RTCScene scene, struct RTCIntersectContext*, struct RTCRayHit* rh) {
    const ShimScene* s = reinterpret_cast<const ShimScene*>(scene);
    const float o[3] = {rh->ray.org_x, rh->ray.org_y, rh->ray.org_z};
    const float d[3] = {rh->ray.dir_x, rh->ray.dir_y, rh->ray.dir_z};
    orq::Hit h;
    if (!orq::closest(s->bvh, o, d, rh->ray.tnear, rh->ray.tfar, h)) return;
    rh->ray.tfar = h.t;
    rh->hit.Ng_x = h.ng[0];
    rh->hit.Ng_y = h.ng[1];
    rh->hit.Ng_z = h.ng[2];
    rh->hit.u = h.u;
    rh->hit.v = h.v;
    rh->hit.primID = h.prim;
    rh->hit.geomID = h.geom;
    rh->hit.instID[0] = 0;
    rh->hit.instID[1] = 0;
}

void rtcOccluded1(RTCScene scene, struct RTCIntersectContext*, struct RTCRay* ray) {
    const ShimScene* s = reinterpret_cast<const ShimScene*>(scene);
    const float o[3] = {ray->org_x, ray->org_y, ray->org_z};
    const float d[3] = {ray->dir_x, ray->dir_y, ray->dir_z};
    if (orq::occluded(s->bvh, o, d, ray->tnear, ray->tfar)) ray->tfar = -std::numeric_limits<float>::infinity();
}

void rtcIntersect8(const int* valid, RTCScene scene, struct RTCIntersectContext*, struct RTCRayHit8* rh) {
    const ShimScene* s = reinterpret_cast<const ShimScene*>(scene);
    for (int k = 0; k < 8; ++k) {
        if (valid[k] != -1) continue;
        const float o[3] = {rh->ray.org_x[k], rh->ray.org_y[k], rh->ray.org_z[k]};
        const float d[3] = {rh->ray.dir_x[k], rh->ray.dir_y[k], rh->ray.dir_z[k]};
        orq::Hit h;
        if (!orq::closest(s->bvh, o, d, rh->ray.tnear[k], rh->ray.tfar[k], h)) continue;
        rh->ray.tfar[k] = h.t;
        rh->hit.Ng_x[k] = h.ng[0];
        rh->hit.Ng_y[k] = h.ng[1];
        rh->hit.Ng_z[k] = h.ng[2];
        rh->hit.u[k] = h.u;
        rh->hit.v[k] = h.v;
        rh->hit.primID[k] = h.prim;
        rh->hit.geomID[k] = h.geom;
        rh->hit.instID[0][k] = 0;
        rh->hit.instID[1][k] = 0;
    }
}

void rtcOccluded8(const int* valid, RTCScene scene, struct RTCIntersectContext*, struct RTCRay8* ray) {
    const ShimScene* s = reinterpret_cast<const ShimScene*>(scene);
    for (int k = 0; k < 8; ++k) {
        if (valid[k] != -1) continue;
        const float o[3] = {ray->org_x[k], ray->org_y[k], ray->org_z[k]};
        const float d[3] = {ray->dir_x[k], ray->dir_y[k], ray->dir_z[k]};
        if (orq::occluded(s->bvh, o, d, ray->tnear[k], ray->tfar[k]))
            ray->tfar[k] = -std::numeric_limits<float>::infinity();
    }
}

void rtcInterpolate(const struct RTCInterpolateArguments* a) {
    const ShimGeometry* g = reinterpret_cast<const ShimGeometry*>(a->geometry);
    const int64_t t = g->first + int64_t(a->primID);
    const float* c = nullptr;
    unsigned stride = 0;
    if (a->bufferSlot == 0) { c = g->normals; stride = 3; }
    else if (a->bufferSlot == 1) { c = g->tangents; stride = 4; }
    else { c = g->uvs; stride = 2; }
    c += t * 3 * stride;
    const float w = 1.0f - a->u - a->v;
    for (unsigned i = 0; i < a->valueCount; ++i) a->P[i] = w * c[i] + a->u * c[stride + i] + a->v * c[2 * stride + i];
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------
// Texture and geometry caches, framebuffer, file access
// ---------------------------------------------------------------------------------------------------
namespace {

struct TextureTable {
    Ptex::PtexCache* cache = nullptr;
    std::vector<std::string> ptex_paths;          // handle hash k + 1 -> Ptex file (k < ptex_paths.size())
    std::vector<TextureResource*> images;         // handle hash 1 + 0x10000 + k -> 2D image
};
TextureTable g_textures;

thread_local double* tl_frame = nullptr;  // [2][H][W][3] sums
thread_local uint32_t tl_frame_w = 0, tl_frame_h = 0;

}  // namespace

namespace Selas {

TextureCache::TextureCache() : cacheData(nullptr) {}
TextureCache::~TextureCache() {}
void TextureCache::Initialize(uint64) {}
void TextureCache::Shutdown() {}
Error TextureCache::LoadTextureResource(const FilePathString&, TextureHandle&) { std::abort(); }
Error TextureCache::LoadTexturePtex(const FilePathString& filepath, TextureHandle& handle) {
    g_textures.ptex_paths.push_back(filepath.Ascii());
    handle.hash = Hash32(g_textures.ptex_paths.size());
    return Success_;
}
void TextureCache::UnloadTexture(TextureHandle) {}
const TextureResource* TextureCache::FetchTexture(TextureHandle handle) {
    if (handle.hash == InvalidTextureHandle_) return nullptr;
    return g_textures.images[handle.hash - 1 - 0x10000];
}
Ptex::PtexTexture* TextureCache::FetchPtex(TextureHandle handle) {
    Ptex::String err;
    return g_textures.cache->get(g_textures.ptex_paths[handle.hash - 1].c_str(), err);
}
void TextureCache::ReleaseTexture(TextureHandle) {}

void GeometryCache::EnsureSubsceneGeometryLoaded(SubsceneResource*) {}
void GeometryCache::FinishUsingSubceneGeometry(SubsceneResource*) {}

void FramebufferWriter_Initialize(FramebufferWriter* writer, Framebuffer* frame, uint32, uint32) {
    std::memset(writer, 0, sizeof(*writer));
    writer->framebuffer = frame;
}
void FramebufferWriter_Write(FramebufferWriter*, float3* samples, uint32 layerCount, uint32 x, uint32 y) {
    const size_t npix = size_t(tl_frame_w) * tl_frame_h, p = size_t(y) * tl_frame_w + x;
    for (uint32 l = 0; l < layerCount && l < 2; ++l) {
        double* o = tl_frame + (l * npix + p) * 3;
        o[0] += samples[l].x;
        o[1] += samples[l].y;
        o[2] += samples[l].z;
    }
}
void FramebufferWriter_Write(FramebufferWriter*, float3* samples, uint32 layerCount, uint32 index) {
    FramebufferWriter_Write(nullptr, samples, layerCount, index % tl_frame_w, index / tl_frame_w);
}
void FramebufferWriter_Shutdown(FramebufferWriter*) {}

}  // namespace Selas

namespace {
// The deferred tracer's queues: one path at a time per thread.
thread_local std::vector<DeferredRay> tl_rays;
thread_local std::vector<OcclusionRay> tl_occlusion;
thread_local std::vector<HitParameters> tl_hits;
}  // namespace

namespace Selas {

PathTracingBatcher::PathTracingBatcher() {}
PathTracingBatcher::~PathTracingBatcher() {}
void PathTracingBatcher::Initialize(uint, uint) {}
void PathTracingBatcher::Shutdown() {}
void PathTracingBatcher::AddUnsortedDeferredRay(const DeferredRay& ray) { tl_rays.push_back(ray); }
void PathTracingBatcher::AddUnsortedOcclusionRay(const OcclusionRay& ray) { tl_occlusion.push_back(ray); }
void PathTracingBatcher::AddUnsortedHit(const HitParameters& hit) { tl_hits.push_back(hit); }
void PathTracingBatcher::Flush() {}
bool PathTracingBatcher::Empty() { return tl_rays.empty() && tl_occlusion.empty() && tl_hits.empty(); }
bool PathTracingBatcher::GetSortedBatch(DeferredRay*&, uint&) { std::abort(); }
void PathTracingBatcher::FreeRays(DeferredRay*) { std::abort(); }
bool PathTracingBatcher::GetSortedBatch(OcclusionRay*&, uint&) { std::abort(); }
void PathTracingBatcher::FreeRays(OcclusionRay*) { std::abort(); }
bool PathTracingBatcher::GetSortedHits(HitParameters*&, uint&) { std::abort(); }
void PathTracingBatcher::FreeHits(HitParameters*) { std::abort(); }
void FrameBuffer_Initialize(Framebuffer*, uint32, uint32, uint32) { std::abort(); }
void FrameBuffer_Shutdown(Framebuffer*) { std::abort(); }
void FrameBuffer_Save(Framebuffer*, cpointer) { std::abort(); }
void FrameBuffer_Scale(Framebuffer*, float) { std::abort(); }

namespace AssetFileUtils {
void AssetFilePath(cpointer, uint64, cpointer, FilePathString&) { std::abort(); }
void ContentFilePath(cpointer, FilePathString&) { std::abort(); }
}  // namespace AssetFileUtils
namespace File {
Error ReadWholeFile(cpointer, void**, uint64*) { std::abort(); }
Error Size(cpointer, uint64&) { std::abort(); }
}  // namespace File
Error BuildProcessorContext::AddFileDependency(cpointer) { std::abort(); }
Error StbImageRead(cpointer, uint, uint, uint&, uint&, uint&, bool&, void*&) { std::abort(); }
Error StbImageWrite(cpointer, uint, uint, uint, StbImageFormats, void*) { std::abort(); }
namespace Directory {
void EnsureDirectoryExists(const char*) { std::abort(); }
}  // namespace Directory

// The densities the reference's IBL build step stores in a cooked ImageBasedLightResource
// (BuildImageBasedLight.cpp:24-101, static there): used by cooked_harness.cpp.
void HarnessIblDensities(Selas::uint width, Selas::uint height, float3* light, IblDensityFunctions* out) {
    float* intensities = CalculateIntensityMap(width, height, light);
    CalculateStrataDistributionFunctions(width, height, intensities, out);
    FreeAligned_(intensities);
}

}  // namespace Selas

// ---------------------------------------------------------------------------------------------------
// Scenes in the reference's structures
// ---------------------------------------------------------------------------------------------------
namespace {

struct RefScene {
    ShimScene rtc;
    std::vector<ShimGeometry> geoms;
    std::vector<float> normals, tangents, uvs;  // soup-order corner attributes (copies)
    std::vector<MaterialResourceData> materials;
    std::vector<SceneLight> lights;
    SceneResourceData data;
    SceneResource scene;
    SubsceneResourceData subdata;
    SubsceneResource subscene;
    ModelResource model;
    SubsceneResource* subscenes[1];
    ModelResource* models[1];
    ImageBasedLightResourceData ibl_data;
    ImageBasedLightResource ibl;
    std::vector<float3> ibl_light, ibl_miss;
    std::vector<TextureResourceData> image_data;
    std::vector<TextureResource> images;
    std::vector<std::vector<float>> image_texels;
    TextureCache textures;
    GeometryCache geometry;
};

float3 f3(const float* p) { return float3(p[0], p[1], p[2]); }

// 32-word material records (shader, flags, light set, Ptex base, baseColor, transmittanceColor, sheen, sheenTint,
// clearcoat, clearcoatGloss, metallic, specTrans, diffTrans, flatness, anisotropic, specularTint, roughness,
// scatterDistance, ior) to MaterialResourceData.
MaterialResourceData to_material(const float* r, uint32_t& light_set) {
    MaterialResourceData m;
    int32_t shader;
    uint32_t flags;
    std::memcpy(&shader, r + 0, 4);
    std::memcpy(&flags, r + 1, 4);
    std::memcpy(&light_set, r + 2, 4);
    m.shader = ShaderType(shader);
    m.flags = ((flags & 1u) ? eTransparent : 0u) | ((flags & 2u) ? eUsesPtex : 0u);
    m.baseColor = f3(r + 4);
    m.transmittanceColor = f3(r + 7);
    m.scalarAttributeValues[eSheen] = r[10];
    m.scalarAttributeValues[eSheenTint] = r[11];
    m.scalarAttributeValues[eClearcoat] = r[12];
    m.scalarAttributeValues[eClearcoatGloss] = r[13];
    m.scalarAttributeValues[eMetallic] = r[14];
    m.scalarAttributeValues[eSpecTrans] = r[15];
    m.scalarAttributeValues[eDiffuseTrans] = r[16];
    m.scalarAttributeValues[eFlatness] = r[17];
    m.scalarAttributeValues[eAnisotropic] = r[18];
    m.scalarAttributeValues[eSpecularTint] = r[19];
    m.scalarAttributeValues[eRoughness] = r[20];
    m.scalarAttributeValues[eScatterDistance] = r[21];
    m.scalarAttributeValues[eIor] = r[22];
    return m;
}

void make_camera(const float* c, uint32_t width, uint32_t height, RayCastCameraSettings& out) {
    CameraSettings cs;
    cs.position = f3(c);
    cs.lookAt = f3(c + 3);
    cs.up = f3(c + 6);
    cs.fovDegrees = c[9];
    cs.znear = 0.1f;
    cs.zfar = 1e6f;
    InitializeRayCastCamera(cs, width, height, out);
}

void init_context(RefScene* s, GIIntegratorContext& ctx, uint32_t max_bounces) {
    ctx.rtcScene = s->scene.rtcScene;
    ctx.scene = &s->scene;
    ctx.geometryCache = &s->geometry;
    ctx.textureCache = &s->textures;
    ctx.camera = nullptr;
    ctx.maxPathLength = max_bounces;
    FramebufferWriter_Initialize(&ctx.frameWriter, nullptr, 0, 0);
}

}  // namespace

extern "C" {

// Builds a scene in the reference's structures.  verts/prim/geom: triangle soup (meshes contiguous, primID from
// 0); materials: n_materials x 32 words by geomID; lights: n_lights x 15 floats (position, direction, x, z,
// radiance) grouped by light set, sets: n_sets x (first, count); background: RGB.  normals/tangents/uvs/aflags:
// per soup triangle corner attributes and flags (1 normals, 2 tangents, 4 uvs), or null.  ptex_paths:
// n_materials entries, the Ptex file of each geometry (null: none).  tex_desc: n_tex x (geomID, width, height,
// float offset) into tex_rgba (RGBA floats, mip 0 only as the reference samples).  ibl_rgb: W x H RGB light
// image (null: none) with an optional miss image (null: the light image times the exposure).
void* ref_scene_new(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t ntri,
                    const float* materials, int n_materials, const float* lights, int n_lights, const uint32_t* sets,
                    int n_sets, const float* background, const float* normals, const float* tangents,
                    const float* uvs, const uint8_t* aflags, const char* const* ptex_paths, const uint32_t* tex_desc,
                    int n_tex, const float* tex_rgba, const float* ibl_rgb, uint32_t ibl_w, uint32_t ibl_h,
                    const float* miss_rgb, uint32_t miss_w, uint32_t miss_h, float rotation, float exposure) {
    if (!g_textures.cache) g_textures.cache = Ptex::PtexCache::create(64, 1 << 28, true, nullptr, nullptr);
    RefScene* s = new RefScene();
    s->rtc.bvh = orq::build(verts, prim, geom, ntri);
    // geometry tables: first soup triangle of every geomID
    s->geoms.resize(size_t(n_materials));
    std::vector<uint8_t> gflags(size_t(n_materials), 0);
    if (normals) s->normals.assign(normals, normals + ntri * 9);
    if (tangents) s->tangents.assign(tangents, tangents + ntri * 12);
    if (uvs) s->uvs.assign(uvs, uvs + ntri * 6);
    for (int64_t t = ntri - 1; t >= 0; --t) {
        if (geom[t] >= uint32_t(n_materials)) continue;
        ShimGeometry& g = s->geoms[geom[t]];
        g.first = t - int64_t(prim[t]);
        if (aflags) gflags[geom[t]] |= aflags[t];
    }
    for (ShimGeometry& g : s->geoms) {
        g.normals = s->normals.empty() ? nullptr : s->normals.data();
        g.tangents = s->tangents.empty() ? nullptr : s->tangents.data();
        g.uvs = s->uvs.empty() ? nullptr : s->uvs.data();
    }
    // 2D images
    s->image_data.resize(size_t(n_tex));
    s->images.resize(size_t(n_tex));
    s->image_texels.resize(size_t(n_tex));
    std::map<uint32_t, int> image_of;
    for (int k = 0; k < n_tex; ++k) {
        const uint32_t* d = tex_desc + 4 * k;
        TextureResourceData& td = s->image_data[k];
        std::memset(&td, 0, sizeof(td));
        td.mipCount = 1;
        td.mipWidths[0] = d[1];
        td.mipHeights[0] = d[2];
        td.mipOffsets[0] = 0;
        td.format = TextureResourceData::Float4;
        td.dataSize = d[1] * d[2] * 16;
        s->image_texels[k].assign(tex_rgba + d[3], tex_rgba + d[3] + size_t(d[1]) * d[2] * 4);
        td.texture = reinterpret_cast<uint8*>(s->image_texels[k].data());
        s->images[k].data = &td;
        image_of[d[0]] = k;
    }
    // materials and the model's per-geometry user data (ModelResource.cpp:236-297 fills the same fields)
    s->materials.resize(size_t(n_materials));
    s->model.userDatas.Resize(uint64(n_materials));
    for (int gid = 0; gid < n_materials; ++gid) {
        uint32_t light_set = 0;
        s->materials[gid] = to_material(materials + 32 * gid, light_set);
        ModelGeometryUserData& u = s->model.userDatas[gid];
        std::memset(&u, 0, sizeof(u));
        u.material = &s->materials[gid];
        u.subscene = &s->subscene;
        u.rtcGeometry = reinterpret_cast<RTCGeometry>(&s->geoms[gid]);
        u.baseColorTextureHandle = TextureHandle();
        u.flags = uint16((gflags[gid] & 1u ? HasNormals : 0) | (gflags[gid] & 2u ? HasTangents : 0) |
                         (gflags[gid] & 4u ? HasUvs : 0));
        u.lightSetIndex = uint16(light_set);
        if ((s->materials[gid].flags & eUsesPtex) && ptex_paths && ptex_paths[gid]) {
            FilePathString p;
            p.Copy(ptex_paths[gid]);
            s->textures.LoadTexturePtex(p, u.baseColorTextureHandle);
        } else if (image_of.count(uint32_t(gid))) {
            // TextureHandle holds only its (private) hash: handle 1 + 0x10000 + k names image k
            g_textures.images.push_back(&s->images[image_of[uint32_t(gid)]]);
            const Hash32 v = Hash32(1 + 0x10000 + g_textures.images.size() - 1);
            static_assert(sizeof(TextureHandle) == sizeof(Hash32), "TextureHandle layout");
            std::memcpy(&u.baseColorTextureHandle, &v, sizeof(v));
        }
    }
    s->models[0] = &s->model;
    s->subscenes[0] = &s->subscene;
    Instance inst;
    inst.index = 0;
    s->subdata.modelInstances.Add(inst);
    s->subscene.data = &s->subdata;
    s->subscene.models = s->models;
    s->data.subsceneInstances.Add(inst);
    s->data.backgroundIntensity = float4(background[0], background[1], background[2], 1.0f);
    // lights and light sets (SceneResource.cpp builds lightSets the same way from lightSetRanges)
    for (int i = 0; i < n_lights; ++i) {
        const float* l = lights + 15 * i;
        SceneLight L;
        L.type = QuadLight;
        L.position = f3(l);
        L.direction = f3(l + 3);
        L.x = f3(l + 6);
        L.z = f3(l + 9);
        L.radiance = f3(l + 12);
        s->lights.push_back(L);
    }
    for (int i = 0; i < n_sets; ++i) {
        SceneLightSet set;
        set.count = sets[2 * i + 1];
        set.lights = s->lights.data() + sets[2 * i];
        s->scene.lightSets.Add(set);
    }
    s->scene.data = &s->data;
    s->scene.rtcScene = reinterpret_cast<RTCScene>(&s->rtc);
    s->scene.subscenes = s->subscenes;
    s->scene.iblResource = nullptr;
    if (ibl_rgb && ibl_w && ibl_h) {
        s->ibl_light.resize(size_t(ibl_w) * ibl_h);
        for (size_t i = 0; i < s->ibl_light.size(); ++i) s->ibl_light[i] = f3(ibl_rgb + 3 * i);
        float* intensities = CalculateIntensityMap(ibl_w, ibl_h, s->ibl_light.data());
        CalculateStrataDistributionFunctions(ibl_w, ibl_h, intensities, &s->ibl_data.densityfunctions);
        FreeAligned_(intensities);
        if (miss_rgb && miss_w && miss_h) {
            s->ibl_miss.resize(size_t(miss_w) * miss_h);
            for (size_t i = 0; i < s->ibl_miss.size(); ++i) s->ibl_miss[i] = f3(miss_rgb + 3 * i);
        } else {
            miss_w = ibl_w;
            miss_h = ibl_h;
            s->ibl_miss.resize(s->ibl_light.size());
            for (size_t i = 0; i < s->ibl_miss.size(); ++i) s->ibl_miss[i] = exposure * s->ibl_light[i];
        }
        s->ibl_data.missWidth = miss_w;
        s->ibl_data.missHeight = miss_h;
        s->ibl_data.rotationRadians = rotation;
        s->ibl_data.exposureScale = exposure;
        s->ibl_data.lightData = s->ibl_light.data();
        s->ibl_data.missData = s->ibl_miss.data();
        s->ibl.data = &s->ibl_data;
        s->scene.iblResource = &s->ibl;
    }
    return s;
}

void ref_scene_release(void* handle) {
    RefScene* s = static_cast<RefScene*>(handle);
    orq::release(s->rtc.bvh);
    if (s->scene.iblResource) ShutdownDensityFunctions(&s->ibl_data.densityfunctions);
    s->scene.iblResource = nullptr;
    s->ibl.data = nullptr;
    // the structures below own nothing the harness did not allocate itself
    s->scene.data = nullptr;
    s->scene.subscenes = nullptr;
    s->subscene.data = nullptr;
    s->subscene.models = nullptr;
    s->model.data = nullptr;
    s->model.geometry = nullptr;
    s->model.rtcScene = nullptr;
    s->model.defaultMaterial = nullptr;
    delete s;
}

// PathTracer::GenerateImage's loop (PathTracer.cpp:262-347) over passes [pass_begin, pass_end) of every pixel:
// JitteredCameraRay then EvaluatePath, the reference's own code, with max_bounces as maxPathLength.
// camera: position[3] lookAt[3] up[3] fovDegrees.  rng_mode 0: PCG32 stream pass * W * H + pixel per path;
// 1: the reference's MT19937, one engine per pixel seeded seed + pixel.  out: [2][H][W][3] FP64 sums.
void ref_pt_render(void* handle, const float* camera, uint32_t width, uint32_t height, uint32_t pass_begin,
                   uint32_t pass_end, uint32_t max_bounces, uint64_t seed, int rng_mode, int threads, double* out) {
    RefScene* s = static_cast<RefScene*>(handle);
    RayCastCameraSettings cam;
    make_camera(camera, width, height, cam);
    const uint32_t npix = width * height;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        tl_mode = rng_mode == 1 ? kMt : kPcg;
        tl_frame = out;
        tl_frame_w = width;
        tl_frame_h = height;
        GIIntegratorContext ctx;
        init_context(s, ctx, max_bounces);
        ctx.camera = &cam;
        for (;;) {
            const uint32_t pix0 = next.fetch_add(16);
            if (pix0 >= npix) break;
            for (uint32_t pixel = pix0; pixel < std::min(npix, pix0 + 16); ++pixel) {
                const uint32_t y = pixel / width, x = pixel - y * width;
                if (rng_mode == 1) ctx.sampler.Initialize(uint32_t(seed) + pixel);
                for (uint32_t pass = pass_begin; pass < pass_end; ++pass) {
                    if (rng_mode == 0) tl_pcg.seed(seed, uint64_t(pass) * npix + pixel);
                    Ray ray = JitteredCameraRay(ctx.camera, &ctx.sampler, float(x), float(y));
                    PathTracer::EvaluatePath(&ctx, ray, x, y);
                }
                if (rng_mode == 1) ctx.sampler.Shutdown();
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < std::max(1, threads); ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
}

// DeferredPathTracer::GenerateImage's work (DeferredPathTracer.cpp:283-472) over samples [sample_begin,
// sample_end) of each pixel's m x m correlated multi-jittered samples, one path at a time: the primary ray as
// GeneratePrimaryRays makes it, then TraceRayBatch / ShadeHitBatch / TraceOcclusionBatch on that path's queues
// until it ends or max_bounces rays have been traced (the reference has no cap; Russian roulette ends paths).
// PCG32 stream s * W * H + pixel per path.  out: [H][W][3] FP64 sums.
void ref_deferred_render(void* handle, const float* camera, uint32_t width, uint32_t height, uint32_t m,
                         uint32_t sample_begin, uint32_t sample_end, uint32_t max_bounces, uint64_t seed, int threads,
                         double* out) {
    RefScene* s = static_cast<RefScene*>(handle);
    RayCastCameraSettings cam;
    make_camera(camera, width, height, cam);
    const uint32_t npix = width * height;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        tl_mode = kPcg;
        tl_frame = out;
        tl_frame_w = width;
        tl_frame_h = height;
        GIIntegratorContext ctx;
        init_context(s, ctx, 1);
        ctx.camera = &cam;
        PathTracingBatcher batcher;
        for (;;) {
            const uint32_t pix0 = next.fetch_add(16);
            if (pix0 >= npix) break;
            for (uint32_t pixel = pix0; pixel < std::min(npix, pix0 + 16); ++pixel) {
                const uint32_t y = pixel / width, x = pixel - y * width;
                for (uint32_t smp = sample_begin; smp < sample_end; ++smp) {
                    tl_pcg.seed(seed, uint64_t(smp) * npix + pixel);
                    tl_rays.clear();
                    tl_hits.clear();
                    tl_occlusion.clear();
                    DeferredRay dr;
                    dr.ray = JitteredCameraRay(&cam, int32(x), int32(y), int32(smp), int32(m), int32(m), int32(pixel));
                    dr.error = 0.0f;
                    dr.index = pixel;
                    dr.diracScatterOnly = 1;
                    dr.throughput = float3::One_;
                    dr.trackedBounces = 0;
                    tl_rays.push_back(dr);
                    for (uint32_t traced = 0; !tl_rays.empty() && traced < max_bounces; ++traced) {
                        std::vector<DeferredRay> rays;
                        rays.swap(tl_rays);
                        const size_t count = rays.size();
                        // TraceRayBatch reads all 8 lanes of its last packet, also those past rayCount (their
                        // misses go to the framebuffer, DeferredPathTracer.cpp:194-205): pad with rays that carry
                        // no throughput, so that those lanes add nothing
                        DeferredRay pad = rays.back();
                        pad.throughput = float3::Zero_;
                        rays.resize((count + 7) / 8 * 8, pad);
                        DeferredPathTracer::TraceRayBatch(&ctx, &batcher, rays.data(), count);
                        std::vector<HitParameters> hits;
                        hits.swap(tl_hits);
                        if (!hits.empty()) DeferredPathTracer::ShadeHitBatch(&ctx, &batcher, hits.data(), hits.size());
                        std::vector<OcclusionRay> occ;
                        occ.swap(tl_occlusion);
                        if (!occ.empty()) DeferredPathTracer::TraceOcclusionBatch(&ctx, occ.data(), occ.size());
                    }
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < std::max(1, threads); ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
}

// CalculateSurfaceParams on given hits.  hits: n x 12 floats (position, geometric normal Ng as Embree reports it,
// ray direction, u, v, t); ids: n x 2 (geomID, primID).  out: n x 32 floats: worldToTangent rows r0 r1 r2 (9),
// baseColor (3), transmittanceColor (3), sheen, sheenTint, clearcoat, clearcoatGloss, metallic, specTrans,
// diffTrans, flatness, anisotropic, specularTint, roughness, scatterDistance, ior, relativeIOR, error,
// shader, materialFlags (as float), lightSetIndex (as float).  (HitParameters as RayPick fills it,
// PathTracer.cpp:122-136.)
void ref_surface_params(void* handle, const float* hits, const uint32_t* ids, int n, float* out) {
    RefScene* s = static_cast<RefScene*>(handle);
    GIIntegratorContext ctx;
    init_context(s, ctx, 8);
    for (int i = 0; i < n; ++i) {
        const float* h = hits + 12 * i;
        HitParameters hit;
        std::memset(&hit, 0, sizeof(hit));
        hit.position = f3(h);
        hit.normal = f3(h + 3);
        hit.view = -f3(h + 6);
        hit.baryCoords = float2(h[9], h[10]);
        hit.geomId = int32(ids[2 * i]);
        hit.primId = int32(ids[2 * i + 1]);
        hit.instId[0] = 0;
        hit.instId[1] = 0;
        const float kErr = 32.0f * 1.19209e-07f;
        hit.error = kErr * Max(Max(Math::Absf(hit.position.x), Math::Absf(hit.position.y)),
                               Max(Math::Absf(hit.position.z), h[11]));
        SurfaceParameters sp;
        std::memset(&sp, 0, sizeof(sp));
        CalculateSurfaceParams(&ctx, &hit, sp);
        float* o = out + 40 * i;
        const float3x3& m = sp.worldToTangent;
        const float rows[9] = {m.r0.x, m.r0.y, m.r0.z, m.r1.x, m.r1.y, m.r1.z, m.r2.x, m.r2.y, m.r2.z};
        for (int k = 0; k < 9; ++k) o[k] = rows[k];
        o[9] = sp.baseColor.x; o[10] = sp.baseColor.y; o[11] = sp.baseColor.z;
        o[12] = sp.transmittanceColor.x; o[13] = sp.transmittanceColor.y; o[14] = sp.transmittanceColor.z;
        o[15] = sp.sheen; o[16] = sp.sheenTint; o[17] = sp.clearcoat; o[18] = sp.clearcoatGloss;
        o[19] = sp.metallic; o[20] = sp.specTrans; o[21] = sp.diffTrans; o[22] = sp.flatness;
        o[23] = sp.anisotropic; o[24] = sp.specularTint; o[25] = sp.roughness; o[26] = sp.scatterDistance;
        o[27] = sp.ior; o[28] = sp.relativeIOR; o[29] = sp.error; o[30] = float(sp.shader);
        o[31] = float(sp.materialFlags); o[32] = float(sp.lightSetIndex);
        // OffsetRayOrigin for the bounce (scale 1) and shadow (scale 0.1) rays along the view direction
        const float3 b = OffsetRayOrigin(sp, -f3(h + 6), 1.0f);
        o[33] = b.x; o[34] = b.y; o[35] = b.z;
        const float3 sh = OffsetRayOrigin(sp, -f3(h + 6), 0.1f);
        o[36] = sh.x; o[37] = sh.y; o[38] = sh.z;
        o[39] = 0.0f;
    }
}

// NextEventEstimation + LightingPdf with prescribed uniforms.  q: n x 6 floats (position, normal); light_sets:
// n; u: n x 3 uniforms (light pick, then the two of the spherical-rectangle sample); wi: n x 3 directions for
// LightingPdf.  out: n x 10: direction (3), radiance (3), distance, pdfW, index (as float), LightingPdf(wi).
void ref_nee(void* handle, const float* q, const uint32_t* light_sets, const float* u, const float* wi, int n,
             float* out) {
    RefScene* s = static_cast<RefScene*>(handle);
    GIIntegratorContext ctx;
    init_context(s, ctx, 8);
    tl_mode = kPrescribed;
    for (int i = 0; i < n; ++i) {
        tl_uniforms = u + 3 * i;
        tl_count = 3;
        tl_used = 0;
        LightDirectSample ls;
        std::memset(&ls, 0, sizeof(ls));
        NextEventEstimation(&ctx, light_sets[i], f3(q + 6 * i), f3(q + 6 * i + 3), ls);
        float* o = out + 10 * i;
        o[0] = ls.direction.x; o[1] = ls.direction.y; o[2] = ls.direction.z;
        o[3] = ls.radiance.x; o[4] = ls.radiance.y; o[5] = ls.radiance.z;
        o[6] = ls.distance; o[7] = ls.pdfW; o[8] = float(ls.index);
        o[9] = LightingPdf(&ctx, light_sets[i], ls, f3(q + 6 * i), f3(wi + 3 * i));
    }
    tl_mode = kPcg;
}

// JitteredCameraRay with prescribed uniforms: q: n x 4 (pixel x, pixel y, u0, u1); out: n x 6 (origin, direction);
// info: cameraX, cameraY, cameraZ, forward (12 floats), virtualImagePlaneDistance.
void ref_camera_rays(const float* camera, uint32_t width, uint32_t height, const float* q, int n, float* out,
                     float* info) {
    RayCastCameraSettings cam;
    make_camera(camera, width, height, cam);
    CSampler sampler;
    tl_mode = kPrescribed;
    for (int i = 0; i < n; ++i) {
        tl_uniforms = q + 4 * i + 2;
        tl_count = 2;
        tl_used = 0;
        const Ray r = JitteredCameraRay(&cam, &sampler, q[4 * i], q[4 * i + 1]);
        out[6 * i + 0] = r.origin.x; out[6 * i + 1] = r.origin.y; out[6 * i + 2] = r.origin.z;
        out[6 * i + 3] = r.direction.x; out[6 * i + 4] = r.direction.y; out[6 * i + 5] = r.direction.z;
    }
    tl_mode = kPcg;
    const float3 v[4] = {cam.cameraX, cam.cameraY, cam.cameraZ, cam.forward};
    for (int k = 0; k < 4; ++k) {
        info[3 * k] = v[k].x;
        info[3 * k + 1] = v[k].y;
        info[3 * k + 2] = v[k].z;
    }
    info[12] = cam.virtualImagePlaneDistance;
}

// The scene's image-based light: Ibl() for n (r0, r1) pairs -> out n x 10 (theta, phi, x, y, pdf, direction
// SphericalToCartesian(theta, phi) (3), unused (2)), SampleIbl(x, y) -> rgb n x 3; for m directions dirs:
// eval m x 7 (SampleIBlPdf, SampleIbl(wi) rgb, SampleIblMiss(wi) rgb).  Also the densities' first
// element counts (marginal: H floats, conditional: W x H floats) copied to mdf / cdf when not null.
void ref_ibl(void* handle, const float* r, int n, float* out, float* rgb, const float* dirs, int m, float* eval,
             float* mdf, float* cdf) {
    RefScene* s = static_cast<RefScene*>(handle);
    const ImageBasedLightResourceData* ibl = &s->ibl_data;
    for (int i = 0; i < n; ++i) {
        float theta, phi, pdf;
        Selas::uint x, y;
        Ibl(ibl, r[2 * i], r[2 * i + 1], theta, phi, x, y, pdf);
        const float3 d = Math::SphericalToCartesian(theta, phi);
        const float3 c = SampleIbl(ibl, x, y);
        float* o = out + 10 * i;
        o[0] = theta; o[1] = phi; o[2] = float(x); o[3] = float(y); o[4] = pdf;
        o[5] = d.x; o[6] = d.y; o[7] = d.z; o[8] = 0.0f; o[9] = 0.0f;
        rgb[3 * i] = c.x; rgb[3 * i + 1] = c.y; rgb[3 * i + 2] = c.z;
    }
    for (int i = 0; i < m; ++i) {
        const float3 w = f3(dirs + 3 * i);
        float p0, p1;
        const float3 a = SampleIbl(ibl, w, p0);
        const float3 b = SampleIblMiss(ibl, w, p1);
        float* e = eval + 7 * i;
        e[0] = SampleIBlPdf(ibl, w);
        e[1] = a.x; e[2] = a.y; e[3] = a.z;
        e[4] = b.x; e[5] = b.y; e[6] = b.z;
    }
    const uint64 w = ibl->densityfunctions.width, h = ibl->densityfunctions.height;
    if (mdf) std::memcpy(mdf, ibl->densityfunctions.marginalDensityFunction, h * sizeof(float));
    if (cdf) std::memcpy(cdf, ibl->densityfunctions.conditionalDensityFunctions, w * h * sizeof(float));
}

// VCMCommon::CalculateIterationConstants -> out: vmSearchRadius, vmSearchRadiusSqr, vmNormalization, vmWeight,
// vcWeight.
void ref_vcm_constants(uint32_t vm_count, uint32_t vc_count, float base_radius, float alpha, float iteration,
                       float* out) {
    const VCMIterationConstants c =
        VCMCommon::CalculateIterationConstants(vm_count, vc_count, base_radius, alpha, iteration);
    out[0] = c.vmSearchRadius;
    out[1] = c.vmSearchRadiusSqr;
    out[2] = c.vmNormalization;
    out[3] = c.vmWeight;
    out[4] = c.vcWeight;
}

}  // extern "C"
