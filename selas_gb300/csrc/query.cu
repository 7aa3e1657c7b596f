// Ray-query kernels over SelRay / SelRayHit records (Embree's RTCRay / RTCRayHit layouts) and their
// launchers.  One thread per ray; each thread keeps its traversal stack in shared memory.
#include "query.h"

#include "hitref.cuh"
#include "instance.cuh"
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

// The hit as Embree reports it.  A quad's triangles are stored as records 2q (v0, v1, v3) and 2q + 1
// (v2, v3, v1) with kind kTriQuadHalf: primID is q and the second triangle's (u', v') become (1 - u', 1 - v')
// (RTC_GEOMETRY_TYPE_QUAD.3embree3); Ng is the hit triangle's.
__device__ __forceinline__ void embree_hit(const float4& p0, const float4& p2, float& u, float& v, uint32_t& prim) {
    prim = __float_as_uint(p0.w);
    if (__float_as_uint(p2.w) == kTriQuadHalf) {
        if (prim & 1u) {
            u = __fsub_rn(1.0f, u);
            v = __fsub_rn(1.0f, v);
        }
        prim >>= 1;
    }
}

__device__ __forceinline__ void store_hit(SelRayHit* rh, const float4* __restrict__ tris, const QueryHit& h) {
    const float4* tp = tris + size_t(h.tri) * 3;
    const float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
    const float3 ng = triangle_ng(p0, p1, p2);
    float u = h.u, v = h.v;
    uint32_t prim;
    embree_hit(p0, p2, u, v, prim);
    float* base = reinterpret_cast<float*>(rh);
    base[8] = h.t;  // ray.tfar
    float4* hp = reinterpret_cast<float4*>(base + 12);
    hp[0] = make_float4(ng.x, ng.y, ng.z, u);
    hp[1] = make_float4(v, __uint_as_float(prim), p1.w, __uint_as_float(SEL_INVALID_GEOMETRY_ID));
    reinterpret_cast<uint32_t*>(base)[20] = SEL_INVALID_GEOMETRY_ID;
}

__device__ __forceinline__ void store_hit_instanced(SelRayHit* rh, const InstHit& h) {
    const float4* tp = h.tris + size_t(h.tri) * 3;
    const float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
    // object space of the hit mesh (a curve segment's from the ray, curve.cuh)
    float3 ng;
    if (__float_as_uint(p2.w) == kTriCurve) {
        const float* ray = reinterpret_cast<const float*>(rh);
        ng = record_ng(tp, p0, p1, p2, h.rec[0], h.rec[1], make_float3(ray[0], ray[1], ray[2]),
                       make_float3(ray[4], ray[5], ray[6]), h.t, h.u);
    } else {
        ng = triangle_ng(p0, p1, p2);
    }
    float u = h.u, v = h.v;
    uint32_t prim;
    embree_hit(p0, p2, u, v, prim);
    float* base = reinterpret_cast<float*>(rh);
    base[8] = h.t;
    float4* hp = reinterpret_cast<float4*>(base + 12);
    hp[0] = make_float4(ng.x, ng.y, ng.z, u);
    hp[1] = make_float4(v, __uint_as_float(prim), p1.w, __uint_as_float(h.inst[0]));
    reinterpret_cast<uint32_t*>(base)[20] = h.inst[1];
}

// Scenes with instances: one thread per ray, the instanced traversal with its deeper shared-memory stack.
template <bool kAnyHit>
__global__ void __launch_bounds__(kQueryBlock)
    k_query_instanced(const uint4* __restrict__ nodes, const float4* __restrict__ tris, const InstanceRecord* insts,
                      float4* rays, uint32_t record_float4s, uint32_t n, uint32_t* err) {
    __shared__ uint2 stack_mem[kInstStack * kQueryBlock];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    InstHit h;
    uint32_t status = 0;
    const bool found = trace_instanced<kAnyHit>(nodes, tris, insts, load_ray(rays + size_t(i) * record_float4s), h,
                                                stack_mem + threadIdx.x, kQueryBlock, status);
    if (status) atomicOr(err, status);
    if (found) {
        if (kAnyHit)
            reinterpret_cast<float*>(rays + size_t(i) * record_float4s)[8] = -__int_as_float(0x7f800000);
        else
            store_hit_instanced(reinterpret_cast<SelRayHit*>(rays + size_t(i) * record_float4s), h);
    }
}

// 8-wide traversal: one thread per ray over the whole batch, 8 resident 128-thread blocks per SM
// (64 registers, 24 KB of shared-memory stacks per block).  A sweep of persistent variants that refill
// finished lanes from per-warp ray blocks was slower on both coherent and incoherent rays (lanes lose
// the lockstep that makes node fetches shared), so the hardware block scheduler does the balancing.
// Postponing a lane's leaf triangles while few lanes of its warp test triangles (Ylitie, Karras, Laine 2017)
// was slower too at every threshold tried (6, 10, 16 lanes: incoherent closest hit 1,382 / 1,376 / 1,356
// against 1,418 Mrays/s without), with identical hits.  So was prefetching, before each step's leaf tests, the
// lines of its leaf records and of the node the next step visits (prefetch.global.L1 / .L2): incoherent closest
// hit 1,417 against 1,431 Mrays/s, and the Cornell box's path tracer 11 % slower.  Node loads marked L2
// evict_last (createpolicy + ld.global.nc.L2::cache_hint) left every set unchanged (1,432 against 1,431).
constexpr int kWideBlocksPerSm = 8;

template <bool kAnyHit>
__global__ void __launch_bounds__(kQueryBlock, kWideBlocksPerSm)
    k_query_wide(const uint4* __restrict__ nodes, const float4* __restrict__ tris, float4* rays,
                 uint32_t record_float4s, uint32_t n, uint32_t* err) {
    __shared__ uint2 stack_mem[kWideStack * kQueryBlock];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    QueryHit h;
    uint32_t status = 0;
    const bool found = trace_wide<kAnyHit>(nodes, tris, load_ray(rays + size_t(i) * record_float4s), h,
                                           stack_mem + threadIdx.x, kQueryBlock, status);
    if (status) atomicOr(err, status);
    if (found) {
        if (kAnyHit)
            reinterpret_cast<float*>(rays + size_t(i) * record_float4s)[8] = -__int_as_float(0x7f800000);
        else
            store_hit(reinterpret_cast<SelRayHit*>(rays + size_t(i) * record_float4s), tris, h);
    }
}

// Plain binary FP32 path: one thread per ray, launched over the whole batch.
template <bool kAnyHit>
__global__ void __launch_bounds__(kQueryBlock) k_query_binary(const float4* __restrict__ nodes,
                                                              const float4* __restrict__ tris, float4* rays,
                                                              uint32_t record_float4s, uint32_t n, uint32_t* err) {
    __shared__ int stack_mem[kBinaryStack * kQueryBlock];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const QueryRay r = load_ray(rays + size_t(i) * record_float4s);
    QueryHit h;
    uint32_t status = 0;
    const bool found = trace_binary<kAnyHit>(nodes, tris, r, h, stack_mem + threadIdx.x, kQueryBlock, status);
    if (status) atomicOr(err, status);
    if (found) {
        if (kAnyHit)
            reinterpret_cast<float*>(rays + size_t(i) * record_float4s)[8] = -__int_as_float(0x7f800000);
        else
            store_hit(reinterpret_cast<SelRayHit*>(rays + size_t(i) * record_float4s), tris, h);
    }
}

template <bool kAnyHit>
cudaError_t launch_query(const DeviceBvh& bvh, float4* d_rays, uint32_t record_float4s, uint32_t n, uint32_t* d_err,
                         cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const dim3 grid((n + kQueryBlock - 1) / kQueryBlock);
    if (bvh.insts) {
        k_query_instanced<kAnyHit><<<grid, kQueryBlock, 0, s>>>(static_cast<const uint4*>(bvh.nodes), bvh.tris,
                                                                bvh.insts, d_rays, record_float4s, n, d_err);
    } else if (bvh.kind == SEL_BVH_WIDE8_Q8) {
        k_query_wide<kAnyHit><<<grid, kQueryBlock, 0, s>>>(static_cast<const uint4*>(bvh.nodes), bvh.tris, d_rays,
                                                           record_float4s, n, d_err);
    } else {
        k_query_binary<kAnyHit><<<grid, kQueryBlock, 0, s>>>(static_cast<const float4*>(bvh.nodes), bvh.tris, d_rays,
                                                             record_float4s, n, d_err);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_intersect(const DeviceBvh& bvh, SelRayHit* d_rays, uint32_t n, uint32_t* d_err, cudaStream_t s) {
    return launch_query<false>(bvh, reinterpret_cast<float4*>(d_rays), sizeof(SelRayHit) / 16, n, d_err, s);
}

cudaError_t launch_occluded(const DeviceBvh& bvh, SelRay* d_rays, uint32_t n, uint32_t* d_err, cudaStream_t s) {
    return launch_query<true>(bvh, reinterpret_cast<float4*>(d_rays), sizeof(SelRay) / 16, n, d_err, s);
}

cudaError_t launch_query_strided(bool any_hit, const DeviceBvh& bvh, void* recs, size_t record_bytes, uint32_t n,
                                 uint32_t* d_err, cudaStream_t s) {
    float4* r = static_cast<float4*>(recs);
    const uint32_t stride = uint32_t(record_bytes / 16);
    return any_hit ? launch_query<true>(bvh, r, stride, n, d_err, s) : launch_query<false>(bvh, r, stride, n, d_err, s);
}

}  // namespace sel
