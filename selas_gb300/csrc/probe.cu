// Shading probes: the steps the integrators' kernels run per hit (k_texture's base colour, k_shade's surface
// set-up, ray offsets and quad-light next-event estimation, the image-based light's sampling and lookups),
// applied to hits, points and directions given by the caller.  They let the device code be compared value by
// value with the reference's CalculateSurfaceParams (Shading/SurfaceParameters.cpp:144-247,403-408),
// NextEventEstimation (Shading/AreaLighting.cpp:113-153,353-373) and Ibl / SampleIbl / SampleIblMiss /
// SampleIBlPdf (SceneLib/ImageBasedLightResource.cpp:118-268) on identical inputs.  The device functions are
// the integrators' own (shading.cuh, ptex.cuh, tex2d.cuh, ibl.cuh); only the loops around them are here.
#include "capi_internal.h"
#include "ibl.cuh"
#include "pt.h"
#include "ptex.cuh"
#include "ptex_quad.cuh"
#include "shading.cuh"
#include "tex2d.cuh"

namespace sel {
namespace {

// hits: n x 12 (position, Ng, ray direction, u, v, t); ids: n x 2 (geomID, primID).  out: n x 40 as the
// reference's SurfaceParameters: worldToTangent rows (t.x n.x b.x / t.y n.y b.y / t.z n.z b.z), baseColor,
// transmittanceColor, sheen, sheenTint, clearcoat, clearcoatGloss, metallic, specTrans, diffTrans, flatness,
// anisotropic, specularTint, roughness, scatterDistance, ior, relativeIOR, error, shader, material flags in the
// reference's encoding (eTransparent 1, eUsesPtex 16), light set, then OffsetRayOrigin toward -d with scale 1
// and 0.1, and a zero.
__global__ void k_surface_probe(PtScene S, const float* __restrict__ hits, const uint32_t* __restrict__ ids,
                                uint32_t n, float* __restrict__ out, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* h = hits + 12 * size_t(i);
    const uint32_t geom = ids[2 * size_t(i)], prim = ids[2 * size_t(i) + 1];
    const float3 pos = f3(h[0], h[1], h[2]), ng = f3(h[3], h[4], h[5]), d = f3(h[6], h[7], h[8]);
    const float u = h[9], v = h[10], t = h[11];
    const MaterialDev& m = S.materials[geom < S.material_count ? geom : 0];
    const MeshAttrDev* attr = geom < S.attr_count ? S.attrs + geom : nullptr;
    float3 fn, ft, fb;
    float fsign;
    shading_frame(attr, prim, u, v, ng, [](float3 x) { return x; }, fn, ft, fb, fsign);
    const float e = 32.0f * 1.19209e-07f * fmaxf(fmaxf(fabsf(pos.x), fabsf(pos.y)), fmaxf(fabsf(pos.z), t));
    float3 base = ld3(m.base_color);
    if (m.flags & kMaterialUsesPtex) {
        uint32_t status = 0;
        ptex_material_eval(m, S.ptex_faces, int(S.ptex_face_count), static_cast<const __half*>(S.ptex_texels), prim, u,
                           v, base, status);
        if (status) atomicOr(err, status);
    } else if (m.flags & kMaterialUsesTexture) {
        base = tex2d_base_colour(m, attr, prim, u, v);
    }
    const Surface sf = make_surface_frame(m, ft, fn, fb, -d, pow3(base, 2.2f));
    float* o = out + 40 * size_t(i);
    o[0] = sf.t.x; o[1] = sf.n.x; o[2] = sf.b.x;
    o[3] = sf.t.y; o[4] = sf.n.y; o[5] = sf.b.y;
    o[6] = sf.t.z; o[7] = sf.n.z; o[8] = sf.b.z;
    o[9] = sf.base_color.x; o[10] = sf.base_color.y; o[11] = sf.base_color.z;
    o[12] = sf.transmittance_color.x; o[13] = sf.transmittance_color.y; o[14] = sf.transmittance_color.z;
    o[15] = sf.sheen; o[16] = sf.sheen_tint; o[17] = sf.clearcoat; o[18] = sf.clearcoat_gloss;
    o[19] = sf.metallic; o[20] = sf.spec_trans; o[21] = sf.diff_trans; o[22] = sf.flatness;
    o[23] = sf.anisotropic; o[24] = sf.specular_tint; o[25] = sf.roughness; o[26] = sf.scatter_distance;
    o[27] = sf.ior; o[28] = sf.relative_ior; o[29] = e; o[30] = float(sf.shader);
    o[31] = float(((m.flags & kMaterialTransparent) ? 1u : 0u) | ((m.flags & kMaterialUsesPtex) ? 16u : 0u));
    o[32] = float(m.light_set);
    const float3 b1 = offset_origin(pos, sf.n, e, -d, 1.0f), b01 = offset_origin(pos, sf.n, e, -d, 0.1f);
    o[33] = b1.x; o[34] = b1.y; o[35] = b1.z;
    o[36] = b01.x; o[37] = b01.y; o[38] = b01.z;
    o[39] = 0.0f;
}

// q: n x 6 (position, normal); sets: light set per point; u: n x 3 uniforms (light pick, two for the
// spherical-rectangle sample).  out: n x 9: direction, radiance, distance, pdf, light index within the set (as
// float); zeros when the set does not exist or is empty.
__global__ void k_light_probe(PtScene S, const float* __restrict__ q, const uint32_t* __restrict__ sets,
                              const float* __restrict__ uu, uint32_t n, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 p = f3(q[6 * size_t(i)], q[6 * size_t(i) + 1], q[6 * size_t(i) + 2]);
    const float3 nrm = f3(q[6 * size_t(i) + 3], q[6 * size_t(i) + 4], q[6 * size_t(i) + 5]);
    LightSample ls;
    ls.direction = f3(0.0f);
    ls.radiance = f3(0.0f);
    ls.distance = 0.0f;
    ls.pdf = 0.0f;
    uint32_t li = 0;
    const uint32_t set_index = sets[i];
    if (set_index < S.light_set_count) {
        const uint2 set = S.light_sets[set_index];
        if (set.y > 0) {
            li = uint32_t(uu[3 * size_t(i)] * float(set.y));
            li = li < set.y ? li : set.y - 1;
            sample_quad_light(S.lights[set.x + li], p, nrm, uu[3 * size_t(i) + 1], uu[3 * size_t(i) + 2], ls);
            ls.pdf *= 1.0f / float(set.y);
        }
    }
    float* o = out + 9 * size_t(i);
    o[0] = ls.direction.x; o[1] = ls.direction.y; o[2] = ls.direction.z;
    o[3] = ls.radiance.x; o[4] = ls.radiance.y; o[5] = ls.radiance.z;
    o[6] = ls.distance; o[7] = ls.pdf; o[8] = float(li);
}

// r: n x 2 uniforms -> samples n x 7 (direction, radiance, density) of ibl_sample; dirs: m x 3 -> eval m x 7
// (ibl_pdf, ibl_radiance, ibl_miss).
__global__ void k_ibl_probe(const IblDev* __restrict__ ibl, const float* __restrict__ r, uint32_t n,
                            float* __restrict__ samples, const float* __restrict__ dirs, uint32_t m,
                            float* __restrict__ eval) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float3 dir, rad;
        float pdf;
        ibl_sample(*ibl, r[2 * size_t(i)], r[2 * size_t(i) + 1], dir, rad, pdf);
        float* o = samples + 7 * size_t(i);
        o[0] = dir.x; o[1] = dir.y; o[2] = dir.z;
        o[3] = rad.x; o[4] = rad.y; o[5] = rad.z;
        o[6] = pdf;
    }
    if (i < m) {
        const float3 w = f3(dirs[3 * size_t(i)], dirs[3 * size_t(i) + 1], dirs[3 * size_t(i) + 2]);
        const float3 a = ibl_radiance(*ibl, w), b = ibl_miss(*ibl, w);
        float* e = eval + 7 * size_t(i);
        e[0] = ibl_pdf(*ibl, w);
        e[1] = a.x; e[2] = a.y; e[3] = a.z;
        e[4] = b.x; e[5] = b.y; e[6] = b.z;
    }
}

// The scene's device view for a probe: committed, flat (instanced hits carry transforms the probe does not
// take), shading data uploaded.
int probe_scene(SelScene scene, PtScene& view) {
    if (!scene->committed) return fail(SEL_ERR_INVALID_OPERATION, "scene not committed");
    if (!scene->instances.empty()) return fail(SEL_ERR_INVALID_OPERATION, "probes take scenes without instances");
    if (int rc = set_device(scene->dev)) return rc;
    if (int rc = sync_shading(scene)) return rc;
    view = scene_view(scene);
    return SEL_OK;
}

}  // namespace
}  // namespace sel

using namespace sel;

extern "C" int sel_surface_probe_device(SelScene scene, const float* d_hits, const unsigned int* d_ids, unsigned int n,
                                        float* d_out, void* stream) {
    if (n && (!d_hits || !d_ids || !d_out)) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    PtScene view;
    if (int rc = probe_scene(scene, view)) return rc;
    if (n == 0) return SEL_OK;
    k_surface_probe<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(view, d_hits, d_ids, n, d_out,
                                                                                  scene->dev->d_err);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "surface probe launch");
}

extern "C" int sel_light_probe_device(SelScene scene, const float* d_points, const unsigned int* d_light_sets,
                                      const float* d_u, unsigned int n, float* d_out, void* stream) {
    if (n && (!d_points || !d_light_sets || !d_u || !d_out)) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    PtScene view;
    if (int rc = probe_scene(scene, view)) return rc;
    if (n == 0) return SEL_OK;
    k_light_probe<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(view, d_points, d_light_sets, d_u, n,
                                                                                d_out);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "light probe launch");
}

extern "C" int sel_ibl_probe_device(SelScene scene, const float* d_r, unsigned int n, float* d_samples,
                                    const float* d_dirs, unsigned int m, float* d_eval, void* stream) {
    if ((n && (!d_r || !d_samples)) || (m && (!d_dirs || !d_eval))) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    PtScene view;
    if (int rc = probe_scene(scene, view)) return rc;
    if (!view.ibl) return fail(SEL_ERR_INVALID_OPERATION, "the scene has no image-based light");
    const unsigned int count = n > m ? n : m;
    if (count == 0) return SEL_OK;
    k_ibl_probe<<<(count + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(view.ibl, d_r, n, d_samples, d_dirs,
                                                                                  m, d_eval);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "image-based light probe launch");
}
