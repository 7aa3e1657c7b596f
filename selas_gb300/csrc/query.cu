// Ray-query kernels over SelRay / SelRayHit records (Embree's RTCRay / RTCRayHit layouts) and their
// launchers.  One thread per ray; each thread keeps its traversal stack in shared memory.
#include "query.h"

#include "traverse.cuh"

namespace sel {

namespace {

constexpr int kQueryBlock = 128;

__device__ __forceinline__ QueryRay load_ray(const float4* rp) {
    const float4 a = rp[0], b = rp[1], c = rp[2];
    QueryRay r;
    r.ox = a.x; r.oy = a.y; r.oz = a.z; r.tnear = a.w;
    r.dx = b.x; r.dy = b.y; r.dz = b.z;
    r.tfar = c.x;
    return r;
}

__device__ __forceinline__ void store_hit(SelRayHit* rh, const float4* __restrict__ tris, const QueryHit& h) {
    const float4* tp = tris + size_t(h.tri) * 3;
    const float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
    const float3 ng = triangle_ng(p0, p1, p2);
    float* base = reinterpret_cast<float*>(rh);
    base[8] = h.t;  // ray.tfar
    float4* hp = reinterpret_cast<float4*>(base + 12);
    hp[0] = make_float4(ng.x, ng.y, ng.z, h.u);
    hp[1] = make_float4(h.v, p0.w, p1.w, __uint_as_float(SEL_INVALID_GEOMETRY_ID));
    reinterpret_cast<uint32_t*>(base)[20] = SEL_INVALID_GEOMETRY_ID;
}

template <int kKind>
__global__ void __launch_bounds__(kQueryBlock) k_intersect(const void* __restrict__ nodes,
                                                           const float4* __restrict__ tris, SelRayHit* rays,
                                                           uint32_t n, uint32_t* err) {
    __shared__ uint2 stack_mem[kKind == SEL_BVH_WIDE8_Q8 ? kWideStack * kQueryBlock : kBinaryStack * kQueryBlock / 2];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const QueryRay r = load_ray(reinterpret_cast<const float4*>(rays + i));
    QueryHit h;
    uint32_t status = 0;
    bool found;
    if (kKind == SEL_BVH_WIDE8_Q8) {
        found = trace_wide<false>(static_cast<const uint4*>(nodes), tris, r, h, stack_mem + threadIdx.x, kQueryBlock,
                                  status);
    } else {
        found = trace_binary<false>(static_cast<const float4*>(nodes), tris, r, h,
                                    reinterpret_cast<int*>(stack_mem) + threadIdx.x, kQueryBlock, status);
    }
    if (status) atomicOr(err, status);
    if (found) store_hit(rays + i, tris, h);
}

template <int kKind>
__global__ void __launch_bounds__(kQueryBlock) k_occluded(const void* __restrict__ nodes,
                                                          const float4* __restrict__ tris, SelRay* rays, uint32_t n,
                                                          uint32_t* err) {
    __shared__ uint2 stack_mem[kKind == SEL_BVH_WIDE8_Q8 ? kWideStack * kQueryBlock : kBinaryStack * kQueryBlock / 2];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const QueryRay r = load_ray(reinterpret_cast<const float4*>(rays + i));
    QueryHit h;
    uint32_t status = 0;
    bool found;
    if (kKind == SEL_BVH_WIDE8_Q8) {
        found = trace_wide<true>(static_cast<const uint4*>(nodes), tris, r, h, stack_mem + threadIdx.x, kQueryBlock,
                                 status);
    } else {
        found = trace_binary<true>(static_cast<const float4*>(nodes), tris, r, h,
                                   reinterpret_cast<int*>(stack_mem) + threadIdx.x, kQueryBlock, status);
    }
    if (status) atomicOr(err, status);
    if (found) rays[i].tfar = -__int_as_float(0x7f800000);
}

}  // namespace

cudaError_t launch_intersect(const DeviceBvh& bvh, SelRayHit* d_rays, uint32_t n, uint32_t* d_err, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const dim3 grid((n + kQueryBlock - 1) / kQueryBlock);
    if (bvh.kind == SEL_BVH_WIDE8_Q8)
        k_intersect<SEL_BVH_WIDE8_Q8><<<grid, kQueryBlock, 0, s>>>(bvh.nodes, bvh.tris, d_rays, n, d_err);
    else
        k_intersect<SEL_BVH_BINARY_FP32><<<grid, kQueryBlock, 0, s>>>(bvh.nodes, bvh.tris, d_rays, n, d_err);
    return cudaGetLastError();
}

cudaError_t launch_occluded(const DeviceBvh& bvh, SelRay* d_rays, uint32_t n, uint32_t* d_err, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const dim3 grid((n + kQueryBlock - 1) / kQueryBlock);
    if (bvh.kind == SEL_BVH_WIDE8_Q8)
        k_occluded<SEL_BVH_WIDE8_Q8><<<grid, kQueryBlock, 0, s>>>(bvh.nodes, bvh.tris, d_rays, n, d_err);
    else
        k_occluded<SEL_BVH_BINARY_FP32><<<grid, kQueryBlock, 0, s>>>(bvh.nodes, bvh.tris, d_rays, n, d_err);
    return cudaGetLastError();
}

}  // namespace sel
