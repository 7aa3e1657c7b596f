// Two-level instanced traversal of 8-wide BVHs: the GB300 form of the reference's instancing, where a scene
// holds subscene instances (user geometry whose callbacks transform the ray and call rtcIntersect1 /
// rtcOccluded1 on the subscene, Source/Core/SceneLib/SceneResource.cpp:73-187) and a subscene holds Embree
// instances of model scenes (SubsceneResource.cpp:63-79).  Hits report instID[0] = the outer instance's id and
// instID[1] = the inner one's (SceneResource.cpp:134-136), the geometric normal in the object space of the
// hit mesh (which CalculateSurfaceParams transforms by localToWorld, SurfaceParameters.cpp:161-168) and t in
// the world ray's parametrisation (the transform is affine and the direction is not renormalised).
//
// One ray walks all levels in one loop.  An instance is a leaf record of its parent's BVH (geomID word
// kInstanceGeom, primID word = index into the parent's instance table); meeting it pushes what is left of the
// current node and leaf plus a level marker, transforms the ray into the instance and continues at the
// instanced BVH's root.  Popping the marker restores the parent level's ray, recomputed from the world ray.
// The closest-hit rule is the flat one extended to instances: smallest t, then smallest
// (instID[0], instID[1], geomID, primID), so the result does not depend on the tree shapes.
#pragma once

#include "curve.cuh"
#include "traverse.cuh"

namespace sel {

constexpr uint32_t kErrInstanceDepth = 16u;  // an instance below the second level (commit prevents it)

// Affine transforms with every rounding fixed (fmaf chains), so that the CPU oracle's std::fma restatement
// transforms rays bit for bit alike.  Rows r0..r2 of a 3 x 4 matrix.
__device__ __forceinline__ void xform_point(const float4& r0, const float4& r1, const float4& r2, float x, float y,
                                            float z, float& ox, float& oy, float& oz) {
    ox = fmaf(r0.x, x, fmaf(r0.y, y, fmaf(r0.z, z, r0.w)));
    oy = fmaf(r1.x, x, fmaf(r1.y, y, fmaf(r1.z, z, r1.w)));
    oz = fmaf(r2.x, x, fmaf(r2.y, y, fmaf(r2.z, z, r2.w)));
}

__device__ __forceinline__ void xform_vector(const float4& r0, const float4& r1, const float4& r2, float x, float y,
                                             float z, float& ox, float& oy, float& oz) {
    ox = fmaf(r0.x, x, fmaf(r0.y, y, __fmul_rn(r0.z, z)));
    oy = fmaf(r1.x, x, fmaf(r1.y, y, __fmul_rn(r1.z, z)));
    oz = fmaf(r2.x, x, fmaf(r2.y, y, __fmul_rn(r2.z, z)));
}

struct InstHit {
    float t, u, v;
    uint32_t tri;                      // record index in `tris` (0xffffffff: no hit)
    const float4* tris;                // leaf records of the hit mesh's scene
    uint32_t inst[2];                  // instIDs, outermost first (SEL_INVALID_GEOMETRY_ID: none)
    const InstanceRecord* rec[2];      // the entered instance records (null: none)
};

struct InstState {
    WideState w;                       // the current level's ray and traversal (tfar shared by all levels)
    float wox, woy, woz, wdx, wdy, wdz;  // world ray
    const uint4* nodes;                // current level
    const float4* tris;
    const InstanceRecord* insts;
    const uint4* top_nodes;
    const float4* top_tris;
    const InstanceRecord* top_insts;
    const InstanceRecord* chain0;      // entered instances (kept in named fields so that the state
    const InstanceRecord* chain1;      // stays in registers)
    int level;
    uint2 pend;                        // leaf records still to test at this level (y = bit mask; 0: none)
    uint64_t cur_inst, best_inst;      // (instID[0] << 32 | instID[1]) of the current level / the best hit
    InstHit hit;
};

__device__ __forceinline__ void inst_apply(const InstanceRecord* rec, float& ox, float& oy, float& oz, float& dx,
                                           float& dy, float& dz) {
    const float4* m = reinterpret_cast<const float4*>(rec->w2l);
    const float4 r0 = __ldg(m), r1 = __ldg(m + 1), r2 = __ldg(m + 2);
    float a, b, c;
    xform_point(r0, r1, r2, ox, oy, oz, a, b, c);
    ox = a; oy = b; oz = c;
    xform_vector(r0, r1, r2, dx, dy, dz, a, b, c);
    dx = a; dy = b; dz = c;
}

__device__ __forceinline__ void inst_level_ray(InstState& s) {
    float ox = s.wox, oy = s.woy, oz = s.woz, dx = s.wdx, dy = s.wdy, dz = s.wdz;
    if (s.level >= 1) inst_apply(s.chain0, ox, oy, oz, dx, dy, dz);
    if (s.level >= 2) inst_apply(s.chain1, ox, oy, oz, dx, dy, dz);
    s.w.ox = ox; s.w.oy = oy; s.w.oz = oz;
    s.w.dx = dx; s.w.dy = dy; s.w.dz = dz;
    s.w.wt = watertight_setup(dx, dy, dz);
    s.w.ix = safe_rcp(dx); s.w.iy = safe_rcp(dy); s.w.iz = safe_rcp(dz);
    s.w.oct = (s.w.ix < 0.0f ? 4u : 0u) | (s.w.iy < 0.0f ? 2u : 0u) | (s.w.iz < 0.0f ? 1u : 0u);
}

__device__ __forceinline__ void inst_level_pointers(InstState& s) {
    if (s.level == 0) {
        s.nodes = s.top_nodes;
        s.tris = s.top_tris;
        s.insts = s.top_insts;
        s.cur_inst = ~0ull;
    } else {
        const InstanceRecord* r = s.level == 1 ? s.chain0 : s.chain1;
        s.nodes = static_cast<const uint4*>(r->nodes);
        s.tris = static_cast<const float4*>(r->tris);
        s.insts = r->insts;
        const uint64_t id0 = s.chain0->instID;
        const uint64_t id1 = s.level == 2 ? s.chain1->instID : 0xffffffffull;
        s.cur_inst = (id0 << 32) | id1;
    }
}

__device__ __forceinline__ void inst_init(InstState& s, const QueryRay& r, const uint4* nodes, const float4* tris,
                                          const InstanceRecord* insts) {
    wide_init(s.w, r);
    s.wox = r.ox; s.woy = r.oy; s.woz = r.oz;
    s.wdx = r.dx; s.wdy = r.dy; s.wdz = r.dz;
    s.top_nodes = nodes;
    s.top_tris = tris;
    s.top_insts = insts;
    s.chain0 = s.chain1 = nullptr;
    s.level = 0;
    inst_level_pointers(s);
    s.pend = make_uint2(0u, 0u);
    s.best_inst = ~0ull;
    s.hit.tri = 0xffffffffu;
    s.hit.tris = nullptr;
    s.hit.inst[0] = s.hit.inst[1] = SEL_INVALID_GEOMETRY_ID;
    s.hit.rec[0] = s.hit.rec[1] = nullptr;
}

__device__ __forceinline__ void inst_record_hit(InstState& s, float t, float u, float v, uint32_t ti) {
    s.hit.t = t; s.hit.u = u; s.hit.v = v; s.hit.tri = ti;
    s.hit.tris = s.tris;
    s.hit.rec[0] = s.level > 0 ? s.chain0 : nullptr;
    s.hit.rec[1] = s.level > 1 ? s.chain1 : nullptr;
    s.hit.inst[0] = uint32_t(s.cur_inst >> 32);
    s.hit.inst[1] = uint32_t(s.cur_inst);
}

// One step: a node visit (or a pending leaf) and the leaf records it exposes.  Returns true when the ray is
// finished (any-hit: on the first hit).
template <bool kAnyHit>
__device__ __forceinline__ bool inst_step(InstState& s, uint2* stack, int stride, uint32_t& status) {
    uint32_t tmask = 0, tbase = 0;
    if (s.pend.y) {
        tbase = s.pend.x;
        tmask = s.pend.y;
        s.pend = make_uint2(0u, 0u);
    } else if (s.w.group.y & 0xff000000u) {
        if (!wide_visit<kInstStack>(s.w, s.nodes, stack, stride, status, tmask, tbase)) return true;
    }
    while (tmask) {
        const int b = __ffs(tmask) - 1;
        tmask &= tmask - 1u;
        const uint32_t ti = tbase + uint32_t(b);
        const float4* tp = s.tris + size_t(ti) * 3;
        const float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
        if (__float_as_uint(p1.w) == kInstanceGeom) {
            if (s.level >= 2) {
                status |= kErrInstanceDepth;
                continue;
            }
            const bool more = (s.w.group.y & 0xff000000u) != 0u;
            const int need = (more ? 1 : 0) + (tmask ? 1 : 0) + 1;
            if (s.w.sp + need > kInstStack) {
                status |= kErrStackOverflow;
                return true;
            }
            if (more) stack[(s.w.sp++) * stride] = s.w.group;
            if (tmask) stack[(s.w.sp++) * stride] = make_uint2(tbase, tmask);
            stack[(s.w.sp++) * stride] = make_uint2(0u, 0u);  // level marker
            if (s.level == 0) s.chain0 = s.insts + __float_as_uint(p0.w);
            else s.chain1 = s.insts + __float_as_uint(p0.w);
            ++s.level;
            inst_level_pointers(s);
            inst_level_ray(s);
            QueryRay lr;
            lr.ox = s.w.ox; lr.oy = s.w.oy; lr.oz = s.w.oz;
            lr.dx = s.w.dx; lr.dy = s.w.dy; lr.dz = s.w.dz;
            // the instanced BVH's root; nothing to do in an instance the transformed ray cannot hit
            s.w.group = ray_untraceable(lr) ? make_uint2(0u, 0u) : make_uint2(0u, (1u << (24 + s.w.oct)) | 1u);
            tmask = 0;
            break;
        }
        float t, u, v;
        bool hit;
        if (__float_as_uint(p2.w) == kTriCurve) {  // a round B-spline curve segment (curve.cuh)
            v = 0.0f;
            hit = curve_intersect(curve_points(tp, p0), s.w.ox, s.w.oy, s.w.oz, s.w.dx, s.w.dy, s.w.dz, s.w.tnear,
                                  s.w.tfar, t, u);
        } else {
            hit = watertight_intersect(s.w.wt, s.w.ox, s.w.oy, s.w.oz, p0, p1, p2, s.w.tnear, s.w.tfar, t, u, v);
        }
        if (hit) {
            if (kAnyHit) {
                inst_record_hit(s, t, u, v, ti);
                return true;
            }
            const uint64_t key = tri_key(p0, p1);
            if (t < s.w.tfar || s.cur_inst < s.best_inst || (s.cur_inst == s.best_inst && key < s.w.best_key)) {
                s.w.tfar = t;
                s.w.best_key = key;
                s.best_inst = s.cur_inst;
                inst_record_hit(s, t, u, v, ti);
            }
        }
    }
    if (++s.w.iters > kIterationCap) {
        status |= kErrIterationCap;
        return true;
    }
    while (!(s.w.group.y & 0xff000000u) && !s.pend.y) {
        if (s.w.sp == 0) return true;
        const uint2 e = stack[(--s.w.sp) * stride];
        if (e.y == 0u) {  // level marker: back to the parent level
            --s.level;
            inst_level_pointers(s);
            inst_level_ray(s);
        } else if ((e.y >> 24) == 0u) {
            s.pend = e;
        } else {
            s.w.group = e;
        }
    }
    return false;
}

// Render-kernel policy of the instanced traversal (the flat layouts are Tracer<0> and Tracer<1>).
template <>
struct Tracer<2> {
    using Entry = uint2;
    static constexpr int kDepth = kInstStack;
};

// Whole-ray form (one thread, one ray) over a scene with instances.
template <bool kAnyHit>
__device__ __forceinline__ bool trace_instanced(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                                const InstanceRecord* insts, const QueryRay& r, InstHit& hit,
                                                uint2* stack, int stride, uint32_t& status) {
    if (ray_untraceable(r)) {
        hit.tri = 0xffffffffu;
        return false;
    }
    InstState s;
    inst_init(s, r, nodes, tris, insts);
    while (!inst_step<kAnyHit>(s, stack, stride, status)) {}
    hit = s.hit;
    return s.hit.tri != 0xffffffffu;
}

}  // namespace sel
