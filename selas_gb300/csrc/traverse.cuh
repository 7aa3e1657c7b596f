// Device-side ray queries: watertight ray/triangle test and traversal of the two BVH layouts.
//
// The query contract is the one Embree gives rtcIntersect1 / rtcOccluded1
// (Middleware/embree-latest/include/embree3/rtcore_scene.h:94,118; used by
// Source/Applications/Selas/Source/PathTracer.cpp:71-139).  Intersection follows Woop, Benthin and
// Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1) 2013, with every rounding step written out
// (fmaf / __fmul_rn / __fadd_rn) so that the CPU oracle, written independently with the same rounding
// steps, reproduces t, u, v bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sel_internal.h"

namespace sel {

constexpr uint32_t kIterationCap = 1u << 22;  // node visits + triangle tests per ray before giving up
constexpr uint32_t kErrIterationCap = 1u;
constexpr uint32_t kErrStackOverflow = 2u;
constexpr float kBoxMargin = 1.0f / 1048576.0f;  // relative widening of the ray interval for box tests

__device__ __forceinline__ float pick3(int k, float x, float y, float z) { return k == 0 ? x : (k == 1 ? y : z); }

struct Watertight {
    int kx, ky, kz;
    float sx, sy, sz;
};

// kz = dominant axis of |d| (ties resolved x, then y, then z); kx, ky follow cyclically and are swapped
// when d[kz] < 0 to keep the winding.
__device__ __forceinline__ Watertight watertight_setup(float dx, float dy, float dz) {
    Watertight w;
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    w.kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    w.kx = w.kz == 2 ? 0 : w.kz + 1;
    w.ky = w.kx == 2 ? 0 : w.kx + 1;
    const float dkz = pick3(w.kz, dx, dy, dz);
    if (dkz < 0.0f) { int t = w.kx; w.kx = w.ky; w.ky = t; }
    const float dkx = pick3(w.kx, dx, dy, dz), dky = pick3(w.ky, dx, dy, dz);
    w.sx = __fdiv_rn(dkx, dkz);
    w.sy = __fdiv_rn(dky, dkz);
    w.sz = __frcp_rn(dkz);
    return w;
}

// Returns true and t/u/v when the triangle is hit with tnear <= t <= tfar.
__device__ __forceinline__ bool watertight_intersect(const Watertight& w, float ox, float oy, float oz, const float4& p0,
                                                     const float4& p1, const float4& p2, float tnear, float tfar,
                                                     float& t, float& u, float& v) {
    const float a0 = __fsub_rn(p0.x, ox), a1 = __fsub_rn(p0.y, oy), a2 = __fsub_rn(p0.z, oz);
    const float b0 = __fsub_rn(p1.x, ox), b1 = __fsub_rn(p1.y, oy), b2 = __fsub_rn(p1.z, oz);
    const float c0 = __fsub_rn(p2.x, ox), c1 = __fsub_rn(p2.y, oy), c2 = __fsub_rn(p2.z, oz);
    const float Akz = pick3(w.kz, a0, a1, a2), Bkz = pick3(w.kz, b0, b1, b2), Ckz = pick3(w.kz, c0, c1, c2);
    const float Ax = fmaf(-w.sx, Akz, pick3(w.kx, a0, a1, a2));
    const float Ay = fmaf(-w.sy, Akz, pick3(w.ky, a0, a1, a2));
    const float Bx = fmaf(-w.sx, Bkz, pick3(w.kx, b0, b1, b2));
    const float By = fmaf(-w.sy, Bkz, pick3(w.ky, b0, b1, b2));
    const float Cx = fmaf(-w.sx, Ckz, pick3(w.kx, c0, c1, c2));
    const float Cy = fmaf(-w.sy, Ckz, pick3(w.ky, c0, c1, c2));
    float U = fmaf(Cx, By, -__fmul_rn(Cy, Bx));
    float V = fmaf(Ax, Cy, -__fmul_rn(Ay, Cx));
    float W = fmaf(Bx, Ay, -__fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // Edge case: redo the 2D edge functions exactly (products of floats are exact in double).
        U = (float)__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx));
        V = (float)__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx));
        W = (float)__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(w.sz, Akz), Bz = __fmul_rn(w.sz, Bkz), Cz = __fmul_rn(w.sz, Ckz);
    const float T = fmaf(U, Az, fmaf(V, Bz, __fmul_rn(W, Cz)));
    const float rcp = __frcp_rn(det);
    const float tt = __fmul_rn(T, rcp);
    if (!(tt >= tnear && tt <= tfar)) return false;
    t = tt;
    u = __fmul_rn(V, rcp);
    v = __fmul_rn(W, rcp);
    return true;
}

// Geometric normal (v1 - v0) x (v2 - v0) with explicit rounding.
__device__ __forceinline__ float3 triangle_ng(const float4& p0, const float4& p1, const float4& p2) {
    const float e1x = __fsub_rn(p1.x, p0.x), e1y = __fsub_rn(p1.y, p0.y), e1z = __fsub_rn(p1.z, p0.z);
    const float e2x = __fsub_rn(p2.x, p0.x), e2y = __fsub_rn(p2.y, p0.y), e2z = __fsub_rn(p2.z, p0.z);
    return make_float3(fmaf(e1y, e2z, -__fmul_rn(e1z, e2y)), fmaf(e1z, e2x, -__fmul_rn(e1x, e2z)),
                       fmaf(e1x, e2y, -__fmul_rn(e1y, e2x)));
}

__device__ __forceinline__ float safe_rcp(float d) {
    return __frcp_rn(fabsf(d) > 1e-30f ? d : copysignf(1e-30f, d));
}

struct QueryRay {
    float ox, oy, oz, dx, dy, dz, tnear, tfar;
};

struct QueryHit {
    float t, u, v;
    uint32_t tri;  // index into the triangle array in leaf order (0xffffffff: no hit)
};

__device__ __forceinline__ uint64_t tri_key(const float4& p0, const float4& p1) {
    return (uint64_t(__float_as_uint(p1.w)) << 32) | uint64_t(__float_as_uint(p0.w));
}

__device__ __forceinline__ float byte_as_float(uint32_t word, int byte) {
    return __uint2float_rn((word >> (8 * byte)) & 0xffu);
}

// ---------------------------------------------------------------------------------------------------
// 8-wide quantised BVH.  Node groups on the stack are (child_base, hit bits 24..31 | imask bits 0..7);
// hit bit 24 + (slot ^ octant) so that the lowest set bit is the nearest child for this ray octant.
// The traversal is written as a resumable per-ray state plus one step (one node visit and the triangles
// it exposes), so that persistent kernels can refill finished lanes with new rays between steps.
// ---------------------------------------------------------------------------------------------------
struct WideState {
    float ox, oy, oz, dx, dy, dz;
    float tnear, tfar;  // tfar shrinks to the closest hit found so far
    float ix, iy, iz;
    Watertight wt;
    uint32_t oct;
    uint2 group;
    int sp;
    uint32_t iters;
    uint64_t best_key;
    QueryHit hit;
};

// A ray that no triangle can hit under the watertight test: a non-finite origin or direction component
// (NaN arithmetic rejects every triangle) or a zero direction (no dominant axis).  Traversing it would be
// worse than useless: with NaN slab distances fminf/fmaxf keep the interval bounds and every box is
// entered, so one such ray walks the whole tree.  The traversals return "no hit" for it at once, which is
// what the full walk returns.
__device__ __forceinline__ bool ray_untraceable(const QueryRay& r) {
    const bool finite = isfinite(r.ox) && isfinite(r.oy) && isfinite(r.oz) && isfinite(r.dx) && isfinite(r.dy) &&
                        isfinite(r.dz);
    return !finite || (r.dx == 0.0f && r.dy == 0.0f && r.dz == 0.0f);
}

__device__ __forceinline__ void wide_init(WideState& s, const QueryRay& r) {
    s.ox = r.ox; s.oy = r.oy; s.oz = r.oz;
    s.dx = r.dx; s.dy = r.dy; s.dz = r.dz;
    s.tnear = r.tnear;
    s.tfar = r.tfar;
    s.wt = watertight_setup(r.dx, r.dy, r.dz);
    s.ix = safe_rcp(r.dx); s.iy = safe_rcp(r.dy); s.iz = safe_rcp(r.dz);
    s.oct = (s.ix < 0.0f ? 4u : 0u) | (s.iy < 0.0f ? 2u : 0u) | (s.iz < 0.0f ? 1u : 0u);
    s.group = make_uint2(0u, (1u << (24 + s.oct)) | 1u);
    s.sp = 0;
    s.iters = 0;
    s.best_key = ~0ull;
    s.hit.tri = 0xffffffffu;
}

// q as float: 0x4B0000qq is 2^23 + q exactly, the subtraction is exact as well.
__device__ __forceinline__ float qbyte(uint32_t word, uint32_t byte) {
    return __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7540u | byte)) - 8388608.0f;
}

// Visits the nearest pending node of s.group (which must have one): pushes the rest of the group, tests the
// node's eight child boxes, makes its hit internal children the new group and returns the triangles of its
// hit leaf children as a bit mask over records tbase..tbase+31.  Returns false on stack overflow.
template <int kDepth>
__device__ __forceinline__ bool wide_visit(WideState& s, const uint4* __restrict__ nodes, uint2* stack, int stride,
                                           uint32_t& status, uint32_t& tmask, uint32_t& tbase) {
    const int b = __ffs(s.group.y >> 24) - 1;
    s.group.y &= ~(1u << (24 + b));
    const uint32_t slot = uint32_t(b) ^ s.oct;
    const uint32_t idx = s.group.x + __popc(s.group.y & ((1u << slot) - 1u));
    if (s.group.y & 0xff000000u) {
        if (s.sp >= kDepth) { status |= kErrStackOverflow; return false; }
        stack[s.sp * stride] = s.group;
        ++s.sp;
    }
    const uint4* np = nodes + size_t(idx) * 5;
    const uint4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3), n4 = __ldg(np + 4);
    const float sxs = __fmul_rn(__uint_as_float((n0.w & 0xffu) << 23), s.ix);
    const float sys = __fmul_rn(__uint_as_float(((n0.w >> 8) & 0xffu) << 23), s.iy);
    const float szs = __fmul_rn(__uint_as_float(((n0.w >> 16) & 0xffu) << 23), s.iz);
    const float oxa = __fmul_rn(__fsub_rn(__uint_as_float(n0.x), s.ox), s.ix);
    const float oya = __fmul_rn(__fsub_rn(__uint_as_float(n0.y), s.oy), s.iy);
    const float oza = __fmul_rn(__fsub_rn(__uint_as_float(n0.z), s.oz), s.iz);
    const uint32_t imask = n0.w >> 24;
    const float tnear_box = s.tnear - fabsf(s.tnear) * kBoxMargin;
    const float tfar_box = s.tfar + fabsf(s.tfar) * kBoxMargin;
    const bool px = s.ix >= 0.0f, py = s.iy >= 0.0f, pz = s.iz >= 0.0f;
    const uint32_t nx0 = px ? n2.x : n3.z, nx1 = px ? n2.y : n3.w, fx0 = px ? n3.z : n2.x, fx1 = px ? n3.w : n2.y;
    const uint32_t ny0 = py ? n2.z : n4.x, ny1 = py ? n2.w : n4.y, fy0 = py ? n4.x : n2.z, fy1 = py ? n4.y : n2.w;
    const uint32_t nz0 = pz ? n3.x : n4.z, nz1 = pz ? n3.y : n4.w, fz0 = pz ? n4.z : n3.x, fz1 = pz ? n4.w : n3.y;
    uint32_t new_hits = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t byte = uint32_t(c & 3);
        const float tnx = fmaf(qbyte(c < 4 ? nx0 : nx1, byte), sxs, oxa);
        const float tfx = fmaf(qbyte(c < 4 ? fx0 : fx1, byte), sxs, oxa);
        const float tny = fmaf(qbyte(c < 4 ? ny0 : ny1, byte), sys, oya);
        const float tfy = fmaf(qbyte(c < 4 ? fy0 : fy1, byte), sys, oya);
        const float tnz = fmaf(qbyte(c < 4 ? nz0 : nz1, byte), szs, oza);
        const float tfz = fmaf(qbyte(c < 4 ? fz0 : fz1, byte), szs, oza);
        const float tmin = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tnear_box));
        const float tmax = fminf(fminf(tfx, tfy), fminf(tfz, tfar_box));
        if (tmin <= tmax) {
            if ((imask >> c) & 1u) {
                new_hits |= 1u << (uint32_t(c) ^ s.oct);
            } else {
                const uint32_t meta = ((c < 4 ? n1.z : n1.w) >> (8 * byte)) & 0xffu;
                if (meta != kLeafNone) tmask |= (0xffu >> (7u - (meta >> 5))) << (meta & 31u);
            }
        }
    }
    s.group = make_uint2(n1.x, (new_hits << 24) | imask);
    tbase = n1.y;
    return true;
}

// One traversal step.  Returns true when the ray is finished (any-hit: on the first hit).
template <bool kAnyHit>
__device__ __forceinline__ bool wide_step(WideState& s, const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                          uint2* stack, int stride, uint32_t& status) {
    uint32_t tmask = 0, tbase = 0;
    if (s.group.y & 0xff000000u) {
        if (!wide_visit<kWideStack>(s, nodes, stack, stride, status, tmask, tbase)) return true;
    }
    while (tmask) {
        const int b = __ffs(tmask) - 1;
        tmask &= tmask - 1u;
        const uint32_t ti = tbase + uint32_t(b);
        const float4* tp = tris + size_t(ti) * 3;
        const float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
        float t, u, v;
        if (watertight_intersect(s.wt, s.ox, s.oy, s.oz, p0, p1, p2, s.tnear, s.tfar, t, u, v)) {
            if (kAnyHit) {
                s.hit.t = t; s.hit.u = u; s.hit.v = v; s.hit.tri = ti;
                return true;
            }
            const uint64_t key = tri_key(p0, p1);
            if (t < s.tfar || key < s.best_key) {
                s.tfar = t;
                s.best_key = key;
                s.hit.t = t; s.hit.u = u; s.hit.v = v; s.hit.tri = ti;
            }
        }
    }
    if (++s.iters > kIterationCap) { status |= kErrIterationCap; return true; }
    if (!(s.group.y & 0xff000000u)) {
        if (s.sp == 0) return true;
        --s.sp;
        s.group = stack[s.sp * stride];
    }
    return false;
}

// Whole-ray form (one thread, one ray).
template <bool kAnyHit>
__device__ __forceinline__ bool trace_wide(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                           const QueryRay& r, QueryHit& hit, uint2* stack, int stride,
                                           uint32_t& status) {
    if (ray_untraceable(r)) {
        hit.tri = 0xffffffffu;
        return false;
    }
    WideState s;
    wide_init(s, r);
    while (!wide_step<kAnyHit>(s, nodes, tris, stack, stride, status)) {}
    hit = s.hit;
    return s.hit.tri != 0xffffffffu;
}

// Warp-cooperative form (one ray per lane, all 32 lanes of the warp together, finished and idle lanes included):
// each step every lane with a pending node visits it, then the warp tests the leaf triangles those visits exposed
// together, 32 (ray, triangle) pairs a round, each lane testing one pair with its owner's ray taken by shuffles.
// Incoherent rays leave most lanes of the one-lane form idle during leaf tests (9 of 32 active per instruction);
// here the tests run on full warps.  The owner takes its candidates in the one-lane form's order (ascending
// record index within a step) under the same rule (t < tfar, or t == tfar and a smaller (geomID, primID)), and a
// candidate's t, u, v do not depend on the tfar it was tested against, so the hits are the same bits.
// slots: this warp's 32 result slots in shared memory (closest hit only; any hit needs none).  The query kernels
// use this form for any hit only: for closest hit it measured no faster than the one-lane form.
struct CoopSlot {
    float t, u, v;
    uint32_t ti;
};

template <bool kAnyHit>
__device__ __forceinline__ bool trace_wide_warp(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                                bool valid, const QueryRay& r, QueryHit& hit, uint2* stack,
                                                int stride, CoopSlot* slots, uint32_t& status) {
    const uint32_t lane = threadIdx.x & 31u;
    WideState s;
    wide_init(s, r);
    bool done = !valid || ray_untraceable(r);
    while (__any_sync(0xffffffffu, !done)) {
        uint32_t tmask = 0, tbase = 0;
        if (!done && (s.group.y & 0xff000000u)) {
            if (!wide_visit<kWideStack>(s, nodes, stack, stride, status, tmask, tbase)) {
                done = true;
                tmask = 0;
            }
        }
        // pairs: lane L owns pairs [excl, incl) of the warp's concatenation, its set tmask bits in ascending order
        const uint32_t cnt = __popc(tmask);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= uint32_t(o)) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        const uint32_t excl = incl - cnt;
        const uint32_t kpack = uint32_t(s.wt.kx) | (uint32_t(s.wt.ky) << 2) | (uint32_t(s.wt.kz) << 4);
        for (uint32_t r0 = 0; r0 < total; r0 += 32) {
            const uint32_t j = r0 + lane;
            uint32_t owner = 0;  // the first lane whose inclusive end exceeds j
#pragma unroll
            for (uint32_t step = 16; step >= 1; step >>= 1) {
                const uint32_t e = __shfl_sync(0xffffffffu, incl, owner + step - 1);
                if (e <= j) owner += step;
            }
            const uint32_t o_mask = __shfl_sync(0xffffffffu, tmask, owner);
            const uint32_t o_base = __shfl_sync(0xffffffffu, tbase, owner);
            const uint32_t o_excl = __shfl_sync(0xffffffffu, excl, owner);
            const uint32_t kp = __shfl_sync(0xffffffffu, kpack, owner);
            Watertight w;
            w.kx = int(kp & 3u);
            w.ky = int((kp >> 2) & 3u);
            w.kz = int((kp >> 4) & 3u);
            w.sx = __shfl_sync(0xffffffffu, s.wt.sx, owner);
            w.sy = __shfl_sync(0xffffffffu, s.wt.sy, owner);
            w.sz = __shfl_sync(0xffffffffu, s.wt.sz, owner);
            const float rox = __shfl_sync(0xffffffffu, s.ox, owner);
            const float roy = __shfl_sync(0xffffffffu, s.oy, owner);
            const float roz = __shfl_sync(0xffffffffu, s.oz, owner);
            const float rtn = __shfl_sync(0xffffffffu, s.tnear, owner);
            const float rtf = __shfl_sync(0xffffffffu, s.tfar, owner);
            bool got = false;
            float t = 0.0f, u = 0.0f, v = 0.0f;
            uint32_t ti = 0xffffffffu;
            const uint32_t bit = j < total ? __fns(o_mask, 0u, int(j - o_excl) + 1) : 0xffffffffu;
            if (bit < 32u) {
                ti = o_base + bit;
                const float4* tp = tris + size_t(ti) * 3;
                const float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
                got = watertight_intersect(w, rox, roy, roz, p0, p1, p2, rtn, rtf, t, u, v);
            }
            // this lane's own pairs in the round: [a, b) of the concatenation
            const uint32_t a = excl > r0 ? excl : r0;
            const uint32_t b = incl < r0 + 32 ? incl : r0 + 32;
            if constexpr (kAnyHit) {
                const uint32_t hits = __ballot_sync(0xffffffffu, got);
                if (!done && a < b) {
                    const uint32_t span = b - a;
                    const uint32_t mine = (hits >> (a - r0)) & (span >= 32 ? 0xffffffffu : ((1u << span) - 1u));
                    if (mine) {
                        s.hit.tri = 0u;  // occluded: only the fact of a hit is reported
                        done = true;
                    }
                }
            } else {
                slots[lane] = CoopSlot{t, u, v, got ? ti : 0xffffffffu};
                __syncwarp();
                for (uint32_t q = a; q < b; ++q) {
                    const CoopSlot c = slots[q - r0];
                    if (c.ti == 0xffffffffu || c.t > s.tfar) continue;
                    const float4* cp = tris + size_t(c.ti) * 3;
                    const uint64_t key = (uint64_t(__float_as_uint(__ldg(&cp[1].w))) << 32) |
                                         uint64_t(__float_as_uint(__ldg(&cp[0].w)));
                    if (c.t < s.tfar || key < s.best_key) {
                        s.tfar = c.t;
                        s.best_key = key;
                        s.hit.t = c.t;
                        s.hit.u = c.u;
                        s.hit.v = c.v;
                        s.hit.tri = c.ti;
                    }
                }
                __syncwarp();
            }
        }
        if (!done) {
            if (++s.iters > kIterationCap) {
                status |= kErrIterationCap;
                done = true;
            } else if (!(s.group.y & 0xff000000u)) {
                if (s.sp == 0) {
                    done = true;
                } else {
                    --s.sp;
                    s.group = stack[s.sp * stride];
                }
            }
        }
    }
    hit = s.hit;
    return valid && s.hit.tri != 0xffffffffu;
}

// ---------------------------------------------------------------------------------------------------
// Binary FP32 BVH (the plain GPU path): classic stack traversal, nearer child first.
// `stack` points at this thread's first int entry; entries are `stride` ints apart.
// ---------------------------------------------------------------------------------------------------
template <bool kAnyHit>
__device__ __forceinline__ bool trace_binary(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                             const QueryRay& r, QueryHit& hit, int* stack, int stride,
                                             uint32_t& status) {
    if (ray_untraceable(r)) {
        hit.tri = 0xffffffffu;
        return false;
    }
    const Watertight wt = watertight_setup(r.dx, r.dy, r.dz);
    const float ix = safe_rcp(r.dx), iy = safe_rcp(r.dy), iz = safe_rcp(r.dz);
    const float oix = __fmul_rn(r.ox, ix), oiy = __fmul_rn(r.oy, iy), oiz = __fmul_rn(r.oz, iz);
    const float tnear_box = r.tnear - fabsf(r.tnear) * kBoxMargin;
    float tfar = r.tfar;
    float tfar_box = tfar + fabsf(tfar) * kBoxMargin;
    uint64_t best_key = ~0ull;
    bool found = false;
    hit.tri = 0xffffffffu;
    const bool nx = ix < 0.0f, ny = iy < 0.0f, nz = iz < 0.0f;

    int node = 0;
    int sp = 0;
    uint32_t iters = 0;
    for (;;) {
        if (++iters > kIterationCap) { status |= kErrIterationCap; break; }
        const float4* np = nodes + size_t(node) * 4;
        const float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
        const int4 refs = __ldg(reinterpret_cast<const int4*>(np + 3));
        // child 0
        const float t0nx = fmaf(nx ? a.y : a.x, ix, -oix), t0fx = fmaf(nx ? a.x : a.y, ix, -oix);
        const float t0ny = fmaf(ny ? a.w : a.z, iy, -oiy), t0fy = fmaf(ny ? a.z : a.w, iy, -oiy);
        const float t0nz = fmaf(nz ? c.y : c.x, iz, -oiz), t0fz = fmaf(nz ? c.x : c.y, iz, -oiz);
        const float t1nx = fmaf(nx ? b.y : b.x, ix, -oix), t1fx = fmaf(nx ? b.x : b.y, ix, -oix);
        const float t1ny = fmaf(ny ? b.w : b.z, iy, -oiy), t1fy = fmaf(ny ? b.z : b.w, iy, -oiy);
        const float t1nz = fmaf(nz ? c.w : c.z, iz, -oiz), t1fz = fmaf(nz ? c.z : c.w, iz, -oiz);
        const float tmin0 = fmaxf(fmaxf(t0nx, t0ny), fmaxf(t0nz, tnear_box));
        const float tmax0 = fminf(fminf(t0fx, t0fy), fminf(t0fz, tfar_box));
        const float tmin1 = fmaxf(fmaxf(t1nx, t1ny), fmaxf(t1nz, tnear_box));
        const float tmax1 = fminf(fminf(t1fx, t1fy), fminf(t1fz, tfar_box));
        bool h0 = tmin0 <= tmax0 && refs.z >= 0;
        bool h1 = tmin1 <= tmax1 && refs.w >= 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const bool hk = k == 0 ? h0 : h1;
            const int cnt = k == 0 ? refs.z : refs.w;
            if (!hk || cnt <= 0) continue;
            const int first = k == 0 ? refs.x : refs.y;
            for (int i = 0; i < cnt; ++i) {
                const float4* tp = tris + size_t(first + i) * 3;
                const float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
                float t, u, v;
                if (watertight_intersect(wt, r.ox, r.oy, r.oz, p0, p1, p2, r.tnear, tfar, t, u, v)) {
                    if (kAnyHit) {
                        hit.t = t; hit.u = u; hit.v = v; hit.tri = uint32_t(first + i);
                        return true;
                    }
                    const uint64_t key = tri_key(p0, p1);
                    if (t < tfar || key < best_key) {
                        tfar = t;
                        tfar_box = tfar + fabsf(tfar) * kBoxMargin;
                        best_key = key;
                        hit.t = t; hit.u = u; hit.v = v; hit.tri = uint32_t(first + i);
                        found = true;
                    }
                }
            }
            if (k == 0) h0 = false; else h1 = false;
        }
        if (h0 && h1) {
            const bool first0 = tmin0 <= tmin1;
            if (sp >= kBinaryStack) { status |= kErrStackOverflow; break; }
            stack[sp * stride] = first0 ? refs.y : refs.x;
            ++sp;
            node = first0 ? refs.x : refs.y;
        } else if (h0) {
            node = refs.x;
        } else if (h1) {
            node = refs.y;
        } else {
            if (sp == 0) break;
            --sp;
            node = stack[sp * stride];
        }
    }
    return found;
}

// ---------------------------------------------------------------------------------------------------
// Traversal policies for the render kernels, which are instantiated for both BVH layouts: the 8-wide
// quantised one and the plain binary FP32 one (the comparison path).  Stack entries live in shared memory,
// `stride` entries apart per thread.
// ---------------------------------------------------------------------------------------------------
template <int kKind>
struct Tracer;

template <>
struct Tracer<0> {  // SEL_BVH_WIDE8_Q8
    using Entry = uint2;
    static constexpr int kDepth = kWideStack;
    template <bool kAnyHit>
    static __device__ __forceinline__ bool trace(const void* nodes, const float4* tris, const QueryRay& r, QueryHit& h,
                                                 Entry* stack, int stride, uint32_t& status) {
        return trace_wide<kAnyHit>(static_cast<const uint4*>(nodes), tris, r, h, stack, stride, status);
    }
};

template <>
struct Tracer<1> {  // SEL_BVH_BINARY_FP32
    using Entry = int;
    static constexpr int kDepth = kBinaryStack;
    template <bool kAnyHit>
    static __device__ __forceinline__ bool trace(const void* nodes, const float4* tris, const QueryRay& r, QueryHit& h,
                                                 Entry* stack, int stride, uint32_t& status) {
        return trace_binary<kAnyHit>(static_cast<const float4*>(nodes), tris, r, h, stack, stride, status);
    }
};

}  // namespace sel
