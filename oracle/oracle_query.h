// ORACLE - test infrastructure only.  Ray queries of the oracle BVH for the oracle integrators.
#pragma once

#include <cstdint>

namespace orq {

struct Hit {
    float t, u, v;
    float ng[3];  // object space of the hit mesh
    uint32_t prim, geom;
    uint32_t scene = 0;                        // scene of the hit mesh (instanced graphs; 0 otherwise)
    const float* l2w[2] = {nullptr, nullptr};  // local-to-world rows of the entered instances, outer first
};

void* build(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t n);
bool closest(const void* bvh, const float* org, const float* dir, float tnear, float tfar, Hit& out);
bool occluded(const void* bvh, const float* org, const float* dir, float tnear, float tfar);
void release(void* bvh);

// Instanced scene graphs (two levels): per-scene BVHs, instances carried by their world-to-local rows.
// Triangles: verts (ntri x 9), prim, geom and owning scene; instances: local-to-world rows (ninst x 12), id,
// owning scene and instanced scene.
void* build_graph(int n_scenes, const float* verts, const uint32_t* prim, const uint32_t* geom,
                  const uint32_t* tri_scene, int64_t ntri, const float* l2w, const uint32_t* inst_id,
                  const uint32_t* inst_scene, const uint32_t* inst_proto, int64_t ninst, int top);
bool closest_graph(const void* g, const float* org, const float* dir, float tnear, float tfar, Hit& out);
bool occluded_graph(const void* g, const float* org, const float* dir, float tnear, float tfar);
void release_graph(void* g);

}  // namespace orq
