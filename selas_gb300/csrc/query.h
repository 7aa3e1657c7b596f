// Launchers for the ray-query kernels (query.cu).
#pragma once

#include <cuda_runtime.h>

#include "sel_internal.h"

namespace sel {

// A committed acceleration structure resident in HBM.
struct DeviceBvh {
    int kind = SEL_BVH_WIDE8_Q8;
    const void* nodes = nullptr;   // WideNode[] or BinaryNode[]
    const float4* tris = nullptr;  // TriRecord[] as 3 x float4
    uint32_t tri_count = 0;
    const InstanceRecord* insts = nullptr;  // instance table of a scene with instances (8-wide layout only)
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // scene bounds (ray ordering keys)
    bool order_rays = false;  // SEL_OPTION_RAY_SORT: large incoherent batches in HBM are traced in key order
    cudaMemPool_t pool = nullptr;  // the device's pool for the ordering scratch
};

cudaError_t launch_intersect(const DeviceBvh& bvh, SelRayHit* d_rays, uint32_t n, uint32_t* d_err, cudaStream_t s);
cudaError_t launch_occluded(const DeviceBvh& bvh, SelRay* d_rays, uint32_t n, uint32_t* d_err, cudaStream_t s);
// The same over records `record_bytes` apart (a multiple of 16, at least the record's size), 16-byte aligned,
// in any memory the device can address (HBM, or page-locked host memory mapped into its address space).
cudaError_t launch_query_strided(bool any_hit, const DeviceBvh& bvh, void* recs, size_t record_bytes, uint32_t n,
                                 uint32_t* d_err, cudaStream_t s);

}  // namespace sel
