// Shading data of a closest hit in a scene that may have instances, shared by the integrators' kernels.
// ModelDataFromRayIds (Source/Core/SceneLib/SceneResource.cpp:362-378): a hit's material, Ptex and vertex
// attributes are those of the scene whose mesh was hit (the innermost instance entered), and its object-space
// normal goes to world space through the entered instances' localToWorld (SurfaceParameters.cpp:161-168).
#pragma once

#include <cstdint>

#include "instance.cuh"
#include "scene_types.h"
#include "sel_internal.h"

namespace sel {

// Instances entered to a hit, as 1 + index in the parent's instance table (0: none).
__device__ __forceinline__ uint2 inst_indices(const InstanceRecord* top, const InstHit& h) {
    const uint32_t a = h.rec[0] ? uint32_t(h.rec[0] - top) + 1u : 0u;
    const uint32_t b = h.rec[1] ? uint32_t(h.rec[1] - h.rec[0]->insts) + 1u : 0u;
    return make_uint2(a, b);
}

// A hit's leaf record and the shading data of the scene whose mesh was hit: the rendered scene's, or that of
// the innermost instance entered.
struct HitRef {
    const float4* tp;
    const MaterialDev* mats;
    uint32_t mat_count;
    uint32_t ptex_count;
    const void* ptex_faces;
    const void* ptex_texels;
    const MeshAttrDev* attrs;
    uint32_t attr_count;
    const InstanceRecord* rec0;
    const InstanceRecord* rec1;
};

// S: a scene view with the rendered scene's tris, materials, material_count, ptex_faces, ptex_texels,
// ptex_face_count, attrs, attr_count and insts; hi: the instance indices of the hit (inst_indices).
template <bool kInst, typename S>
__device__ __forceinline__ HitRef hit_ref_of(const S& sc, uint2 hi, uint32_t tri) {
    HitRef r;
    r.rec0 = r.rec1 = nullptr;
    const float4* tris = sc.tris;
    r.mats = sc.materials;
    r.mat_count = sc.material_count;
    r.ptex_faces = sc.ptex_faces;
    r.ptex_texels = sc.ptex_texels;
    r.ptex_count = sc.ptex_face_count;
    r.attrs = sc.attrs;
    r.attr_count = sc.attr_count;
    if (kInst && hi.x) {
        r.rec0 = sc.insts + (hi.x - 1u);
        const InstanceRecord* in = r.rec0;
        if (hi.y) {
            r.rec1 = r.rec0->insts + (hi.y - 1u);
            in = r.rec1;
        }
        tris = static_cast<const float4*>(in->tris);
        const ShadeView* v = static_cast<const ShadeView*>(in->shading);
        r.mats = v->materials;
        r.mat_count = v->material_count;
        r.ptex_faces = v->ptex_faces;
        r.ptex_texels = v->ptex_texels;
        r.ptex_count = v->ptex_face_count;
        r.attrs = v->attrs;
        r.attr_count = v->attr_count;
    }
    r.tp = tris + size_t(tri) * 3;
    return r;
}

// World normal of a hit: the object-space normal through the entered instances' local-to-world rows,
// innermost first (CalculateSurfaceParams transforms Ng by the composed localToWorld,
// SurfaceParameters.cpp:161-168; not the inverse transpose).
__device__ __forceinline__ float3 world_normal(const HitRef& r, float3 ng) {
    const InstanceRecord* recs[2] = {r.rec1, r.rec0};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (!recs[k]) continue;
        const float4* m = reinterpret_cast<const float4*>(recs[k]->l2w);
        const float4 r0 = __ldg(m), r1 = __ldg(m + 1), r2 = __ldg(m + 2);
        float x, y, z;
        xform_vector(r0, r1, r2, ng.x, ng.y, ng.z, x, y, z);
        ng = make_float3(x, y, z);
    }
    return ng;
}

// Object-space geometric normal of a hit on leaf record tp (words p0, p1, p2): the triangle's, or for a curve
// segment the normal at (t, u) of the world ray (o, d) taken into the hit mesh's space through the entered
// instances, outermost first, as the instanced traversal takes it (curve.cuh).
__device__ __forceinline__ float3 record_ng(const float4* tp, const float4& p0, const float4& p1, const float4& p2,
                                            const InstanceRecord* rec0, const InstanceRecord* rec1, float3 o, float3 d,
                                            float t, float u) {
    if (__float_as_uint(p2.w) != kTriCurve) return triangle_ng(p0, p1, p2);
    float ox = o.x, oy = o.y, oz = o.z, dx = d.x, dy = d.y, dz = d.z;
    if (rec0) inst_apply(rec0, ox, oy, oz, dx, dy, dz);
    if (rec1) inst_apply(rec1, ox, oy, oz, dx, dy, dz);
    return curve_ng(curve_points(tp, p0), ox, oy, oz, dx, dy, dz, t, u);
}

}  // namespace sel
