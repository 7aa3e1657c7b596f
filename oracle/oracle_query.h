// ORACLE - test infrastructure only.  Ray queries of the oracle BVH for the oracle integrators.
#pragma once

#include <cstdint>

namespace orq {

struct Hit {
    float t, u, v;
    float ng[3];
    uint32_t prim, geom;
};

void* build(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t n);
bool closest(const void* bvh, const float* org, const float* dir, float tnear, float tfar, Hit& out);
bool occluded(const void* bvh, const float* org, const float* dir, float tnear, float tfar);
void release(void* bvh);

}  // namespace orq
