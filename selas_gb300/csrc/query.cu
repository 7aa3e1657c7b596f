// Ray-query kernels over SelRay / SelRayHit records (Embree's RTCRay / RTCRayHit layouts) and their
// launchers.  One thread per ray; each thread keeps its traversal stack in shared memory.
#include "query.h"

#include "hitref.cuh"
#include "instance.cuh"
#include "radix.cuh"
#include "scan.cuh"
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

// 8-wide traversal: one thread per ray over the whole batch, 8 resident 128-thread blocks per SM for closest
// hit (64 registers, 24 KB of shared-memory stacks per block).  A sweep of persistent variants that refill
// finished lanes from per-warp ray blocks was slower on both coherent and incoherent rays (lanes lose
// the lockstep that makes node fetches shared), so the hardware block scheduler does the balancing.
// Postponing a lane's leaf triangles while few lanes of its warp test triangles (Ylitie, Karras, Laine 2017)
// was slower too at every threshold tried (6, 10, 16 lanes: incoherent closest hit 1,382 / 1,376 / 1,356
// against 1,418 Mrays/s without), with identical hits.  So was prefetching, before each step's leaf tests, the
// lines of its leaf records and of the node the next step visits (prefetch.global.L1 / .L2): incoherent closest
// hit 1,417 against 1,431 Mrays/s, and the Cornell box's path tracer 11 % slower.  Node loads marked L2
// evict_last (createpolicy + ld.global.nc.L2::cache_hint) left every set unchanged (1,432 against 1,431).
// Nine blocks per SM (56 registers, a few bytes spilled) help the any-hit kernel (incoherent 2,069 against
// 2,026 Mrays/s) and slow the closest-hit one (1,363 against 1,433), so each takes its own.  The any-hit kernel
// tests each step's leaf triangles with the whole warp (trace_wide_warp: incoherent 2,147 against 2,068, coherent
// 14,660 against 14,200); for closest hit the shuffles, slots and key loads cost what the fuller warps save
// (incoherent 1,416 against 1,434, coherent 7,780 against 8,240), so it keeps one lane per ray.  Choosing per
// step (each lane its own triangles unless one lane holds 1.5x more pairs than the warp's rounds) was slower
// still (1,402 and 7,780): the warp-synchronous loop itself costs the closest-hit kernel.
template <bool kAnyHit>
constexpr int kWideBlocksPerSm = kAnyHit ? 9 : 8;

template <bool kAnyHit>
__global__ void __launch_bounds__(kQueryBlock, kWideBlocksPerSm<kAnyHit>)
    k_query_wide(const uint4* __restrict__ nodes, const float4* __restrict__ tris, float4* rays,
                 uint32_t record_float4s, uint32_t n, uint32_t* err) {
    __shared__ uint2 stack_mem[kWideStack * kQueryBlock];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    QueryHit h;
    uint32_t status = 0;
    bool found;
    if constexpr (kAnyHit) {  // the warp tests its leaf triangles together; lanes past the batch stay to help
        QueryRay r{};
        if (valid) r = load_ray(rays + size_t(i) * record_float4s);
        found = trace_wide_warp<true>(nodes, tris, valid, r, h, stack_mem + threadIdx.x, kQueryBlock, nullptr,
                                      status);
    } else {
        if (!valid) return;
        found = trace_wide<false>(nodes, tris, load_ray(rays + size_t(i) * record_float4s), h,
                                  stack_mem + threadIdx.x, kQueryBlock, status);
    }
    if (status) atomicOr(err, status);
    if (found) {
        if (kAnyHit)
            reinterpret_cast<float*>(rays + size_t(i) * record_float4s)[8] = -__int_as_float(0x7f800000);
        else
            store_hit(reinterpret_cast<SelRayHit*>(rays + size_t(i) * record_float4s), tris, h);
    }
}

// ---------------------------------------------------------------------------------------------------
// Ray order.  A large batch of incoherent rays in HBM is traced in the order of a 24-bit key (the direction's
// octant above a 21-bit Morton code of the origin in the scene bounds), so that the rays of a warp start near
// one another and fetch the same nodes and triangles: a stable radix sort of (key, index) pairs, then the query
// kernel reads ray order[i] and writes its hit in place.  Results do not depend on the order.  A batch whose
// sampled neighbouring rays run nearly parallel (camera rays in pixel order) is coherent already: k_order_gate
// sets the count to sort to 0 and the sort and the indirection drop out on the device, without a host round trip.
// ---------------------------------------------------------------------------------------------------
constexpr uint32_t kOrderMin = 1u << 20;  // smaller batches keep their order
constexpr int kGatePairs = 1024;

__global__ void __launch_bounds__(256) k_order_gate(const float4* rays, uint32_t record_float4s, uint32_t n,
                                                    uint32_t* ctl) {
    __shared__ uint32_t close;
    if (threadIdx.x == 0) close = 0;
    __syncthreads();
    uint32_t c = 0;
    for (int k = 0; k < kGatePairs / 256; ++k) {
        const size_t i = size_t(threadIdx.x * (kGatePairs / 256) + k) * (n - 2) / (kGatePairs - 1);
        const float4 a = rays[i * record_float4s + 1], b = rays[(i + 1) * record_float4s + 1];
        const float d = a.x * b.x + a.y * b.y + a.z * b.z;
        const float nn = (a.x * a.x + a.y * a.y + a.z * a.z) * (b.x * b.x + b.y * b.y + b.z * b.z);
        if (nn > 0.0f && d > 0.0f && d * d > 0.998f * nn) ++c;  // within about 2.5 degrees
    }
    atomicAdd(&close, c);
    __syncthreads();
    if (threadIdx.x == 0) ctl[0] = 2 * close > uint32_t(kGatePairs) ? 0u : n;
}

__device__ __forceinline__ uint32_t spread7(uint32_t x) {  // bits 0..6 of x to bits 0, 3, .., 18
    x &= 0x7fu;
    x = (x | (x << 8)) & 0x0000f00fu;
    x = (x | (x << 4)) & 0x000c30c3u;
    x = (x | (x << 2)) & 0x00249249u;
    return x;
}

__global__ void __launch_bounds__(256) k_order_keys(const float4* rays, uint32_t record_float4s, const uint32_t* ctl,
                                                    float3 lo, float3 scale, uint32_t* keys, uint32_t* order) {
    const uint32_t n = ctl[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 o = rays[size_t(i) * record_float4s], d = rays[size_t(i) * record_float4s + 1];
        const uint32_t qx = uint32_t(fminf(fmaxf((o.x - lo.x) * scale.x, 0.0f), 127.0f));
        const uint32_t qy = uint32_t(fminf(fmaxf((o.y - lo.y) * scale.y, 0.0f), 127.0f));
        const uint32_t qz = uint32_t(fminf(fmaxf((o.z - lo.z) * scale.z, 0.0f), 127.0f));
        const uint32_t oct = (d.x < 0.0f ? 4u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 1u : 0u);
        keys[i] = (oct << 21) | (spread7(qx) << 2) | (spread7(qy) << 1) | spread7(qz);
        order[i] = i;
    }
}

// The 8-wide traversal over rays taken in `order` when ctl[0] (the sorted count) is non-zero.
template <bool kAnyHit>
__global__ void __launch_bounds__(kQueryBlock, kWideBlocksPerSm<kAnyHit>)
    k_query_wide_ordered(const uint4* __restrict__ nodes, const float4* __restrict__ tris, float4* rays,
                         uint32_t record_float4s, uint32_t n, const uint32_t* __restrict__ order,
                         const uint32_t* ctl, uint32_t* err) {
    __shared__ uint2 stack_mem[kWideStack * kQueryBlock];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const uint32_t r = !valid ? 0u : (ctl[0] ? order[i] : i);
    QueryHit h;
    uint32_t status = 0;
    bool found;
    if constexpr (kAnyHit) {
        QueryRay ray{};
        if (valid) ray = load_ray(rays + size_t(r) * record_float4s);
        found = trace_wide_warp<true>(nodes, tris, valid, ray, h, stack_mem + threadIdx.x, kQueryBlock, nullptr,
                                      status);
    } else {
        if (!valid) return;
        found = trace_wide<false>(nodes, tris, load_ray(rays + size_t(r) * record_float4s), h,
                                  stack_mem + threadIdx.x, kQueryBlock, status);
    }
    if (status) atomicOr(err, status);
    if (found) {
        if (kAnyHit)
            reinterpret_cast<float*>(rays + size_t(r) * record_float4s)[8] = -__int_as_float(0x7f800000);
        else
            store_hit(reinterpret_cast<SelRayHit*>(rays + size_t(r) * record_float4s), tris, h);
    }
}

// Gate, keys, three radix passes and the ordered traversal on stream s, with stream-ordered scratch.
template <bool kAnyHit>
cudaError_t launch_query_ordered(const DeviceBvh& bvh, float4* d_rays, uint32_t record_float4s, uint32_t n,
                                 uint32_t* d_err, cudaStream_t s) {
    const uint32_t ntiles = (n + kSortTile - 1) / kSortTile;
    const size_t hist = size_t(256) * ntiles;
    const size_t words = 4 * size_t(n) + hist + (hist + 1) + scan_scratch_words(hist + 1) + 1;
    uint32_t* mem = nullptr;
    cudaError_t e = bvh.pool ? cudaMallocFromPoolAsync(reinterpret_cast<void**>(&mem), words * 4, bvh.pool, s)
                             : cudaMallocAsync(reinterpret_cast<void**>(&mem), words * 4, s);
    if (e != cudaSuccess) return e;
    uint32_t* keys[2] = {mem, mem + n};
    uint32_t* vals[2] = {mem + 2 * size_t(n), mem + 3 * size_t(n)};
    uint32_t* h = mem + 4 * size_t(n);
    uint32_t* h_off = h + hist;
    uint32_t* scan_tmp = h_off + hist + 1;
    uint32_t* ctl = scan_tmp + scan_scratch_words(hist + 1);
    k_order_gate<<<1, 256, 0, s>>>(d_rays, record_float4s, n, ctl);
    float3 lo, scale;
    const float* b[2] = {bvh.lo, bvh.hi};
    float sc[3];
    for (int a = 0; a < 3; ++a) {
        const float ext = b[1][a] - b[0][a];
        sc[a] = ext > 0.0f ? 128.0f / ext : 0.0f;
    }
    lo = make_float3(bvh.lo[0], bvh.lo[1], bvh.lo[2]);
    scale = make_float3(sc[0], sc[1], sc[2]);
    k_order_keys<<<1024, 256, 0, s>>>(d_rays, record_float4s, ctl, lo, scale, keys[0], vals[0]);
    int in = 0;
    for (int pass = 0; pass < 3; ++pass) {
        k_radix_hist<<<ntiles, 256, 0, s>>>(keys[in], ctl, 8 * pass, h, ntiles);
        scan_exclusive(h, uint32_t(hist), h_off, scan_tmp, s);
        k_radix_scatter<<<ntiles, 256, 0, s>>>(keys[in], vals[in], keys[in ^ 1], vals[in ^ 1], ctl, 8 * pass, h_off,
                                               ntiles);
        in ^= 1;
    }
    const dim3 grid((n + kQueryBlock - 1) / kQueryBlock);
    k_query_wide_ordered<kAnyHit><<<grid, kQueryBlock, 0, s>>>(static_cast<const uint4*>(bvh.nodes), bvh.tris,
                                                                d_rays, record_float4s, n, vals[in], ctl, d_err);
    e = cudaGetLastError();
    const cudaError_t ef = cudaFreeAsync(mem, s);
    return e != cudaSuccess ? e : ef;
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
    if (bvh.order_rays && n >= kOrderMin && !bvh.insts && bvh.kind == SEL_BVH_WIDE8_Q8)
        return launch_query_ordered<false>(bvh, reinterpret_cast<float4*>(d_rays), sizeof(SelRayHit) / 16, n, d_err, s);
    return launch_query<false>(bvh, reinterpret_cast<float4*>(d_rays), sizeof(SelRayHit) / 16, n, d_err, s);
}

cudaError_t launch_occluded(const DeviceBvh& bvh, SelRay* d_rays, uint32_t n, uint32_t* d_err, cudaStream_t s) {
    if (bvh.order_rays && n >= kOrderMin && !bvh.insts && bvh.kind == SEL_BVH_WIDE8_Q8)
        return launch_query_ordered<true>(bvh, reinterpret_cast<float4*>(d_rays), sizeof(SelRay) / 16, n, d_err, s);
    return launch_query<true>(bvh, reinterpret_cast<float4*>(d_rays), sizeof(SelRay) / 16, n, d_err, s);
}

cudaError_t launch_query_strided(bool any_hit, const DeviceBvh& bvh, void* recs, size_t record_bytes, uint32_t n,
                                 uint32_t* d_err, cudaStream_t s) {
    float4* r = static_cast<float4*>(recs);
    const uint32_t stride = uint32_t(record_bytes / 16);
    return any_hit ? launch_query<true>(bvh, r, stride, n, d_err, s) : launch_query<false>(bvh, r, stride, n, d_err, s);
}

}  // namespace sel
