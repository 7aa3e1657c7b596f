// Device-side Ptex triangle filter over packed per-face texel arrays.
//
// Restates PtexTriangleFilter::eval as Selas calls it (Source/Core/Shading/SurfaceParameters.cpp:196-206:
// getFilter(f_bspline) on a triangle mesh, eval(faceid = primId, u, v, widths 0)) -- buildKernel,
// splitAndApply, applyAcrossEdge and apply of Middleware/ptex/Include/PtexTriangleFilter.cpp:50-218 with
// the kernel algebra of PtexTriangleKernel.h:60-231 and the Gaussian walk of PtexTriangleKernel.cpp:44-75.
// The reference recursion across face edges becomes an explicit frame stack that visits faces in the same
// depth-first order, so texel weights are summed in the same order.
//
// HBM layout: a face table of PtexFace records (32 bytes each, the SelPtexFace layout: log2 resolution,
// texel offset, three neighbours, three neighbour edge ids) and one array of half-float RGB texels, each
// face's texels row-major at its offset.  All faces of a mesh share one resolution (no mip reductions are
// stored).
#pragma once

#include <cstdint>
#include <cuda_fp16.h>

#include "vecmath.cuh"

namespace sel {

struct PtexFace {
    int32_t log2;        // square resolution 2^log2
    uint32_t offset;     // texel offset of this face (in texels)
    int32_t adj[3];      // neighbouring face across edge i (-1 on a boundary); edge i: vertex i -> i+1
    int32_t adjedge[3];  // the neighbour's edge id for the shared edge
};

constexpr int kPtexStack = 24;
constexpr uint32_t kErrPtexStack = 4u;

struct PtexKernel {
    float u, v, u1, v1, w1, u2, v2, w2, A, B, C;
    int reslog2;
};

__device__ __forceinline__ void pk_set(PtexKernel& k, float uu, float vv, float a1, float b1, float c1, float a2,
                                       float b2, float c2) {
    k.u = uu; k.v = vv; k.u1 = a1; k.v1 = b1; k.w1 = c1; k.u2 = a2; k.v2 = b2; k.w2 = c2;
}
__device__ __forceinline__ void pk_rotate1(PtexKernel& k) {
    const float A = k.A, B = k.B, C = k.C;
    k.A = C; k.B = 2.0f * C - B; k.C = A + C - B;
}
__device__ __forceinline__ void pk_rotate2(PtexKernel& k) {
    const float A = k.A, B = k.B, C = k.C;
    k.A = A + C - B; k.B = 2.0f * A - B; k.C = A;
}
// PtexTriangleKernel::reorient: express the kernel in the neighbour's coordinates
__device__ __forceinline__ void pk_reorient(PtexKernel& k, int eid, int aeid) {
    const float u = k.u, v = k.v, w = 1.0f - k.u - k.v;
    const float u1 = k.u1, v1 = k.v1, w1 = k.w1, u2 = k.u2, v2 = k.v2, w2 = k.w2;
    switch (eid * 3 + aeid) {
        case 0: pk_set(k, 1.0f - u, -v, 1.0f - u2, -v2, 1.0f - w2, 1.0f - u1, -v1, 1.0f - w1); break;
        case 1: pk_set(k, 1.0f - w, 1.0f - u, 1.0f - w2, 1.0f - u2, -v2, 1.0f - w1, 1.0f - u1, -v1); pk_rotate1(k); break;
        case 2: pk_set(k, -v, 1.0f - w, -v2, 1.0f - w2, 1.0f - u2, -v1, 1.0f - w1, 1.0f - u1); pk_rotate2(k); break;
        case 3: pk_set(k, 1.0f - v, -w, 1.0f - v2, -w2, 1.0f - u2, 1.0f - v1, -w1, 1.0f - u1); pk_rotate2(k); break;
        case 4: pk_set(k, 1.0f - u, 1.0f - v, 1.0f - u2, 1.0f - v2, -w2, 1.0f - u1, 1.0f - v1, -w1); break;
        case 5: pk_set(k, -w, 1.0f - u, -w2, 1.0f - u2, 1.0f - v2, -w1, 1.0f - u1, 1.0f - v1); pk_rotate1(k); break;
        case 6: pk_set(k, 1.0f - w, -u, 1.0f - w2, -u2, 1.0f - v2, 1.0f - w1, -u1, 1.0f - v1); pk_rotate1(k); break;
        case 7: pk_set(k, 1.0f - v, 1.0f - w, 1.0f - v2, 1.0f - w2, -u2, 1.0f - v1, 1.0f - w1, -u1); pk_rotate2(k); break;
        default: pk_set(k, -u, 1.0f - v, -u2, 1.0f - v2, 1.0f - w2, -u1, 1.0f - v1, 1.0f - w1); break;
    }
}

// One iterator of PtexTriangleKernelIter over a face's texels (finite-difference ellipse walk).
__device__ __forceinline__ void ptex_walk(int rowlen, float ku, float kv, int u1, int v1, int w1, int u2, int v2,
                                          int w2, float A, float B, float C, float wscale,
                                          const __half* __restrict__ data, float3& acc, float& weight) {
    const float gscale = -0.5f * (3.5f * 3.5f);  // PtexTriangleKernelWidth = 3.5
    const float DDQ = 2.0f * A;
    for (int vi = v1; vi != v2; ++vi) {
        const int xw = rowlen - vi;
        const int x1 = max(u1, xw - w2);
        const int x2 = min(u2, xw - w1);
        const float U = (float)x1 - ku;
        const float V = (float)vi - kv;
        float DQ = A * (2.0f * U + 1.0f) + B * V;
        float Q = A * U * U + (B * U + C * V) * V;
        for (int x = x1; x < x2; ++x) {
            if (Q < 1.0f) {
                const float w = expf(gscale * Q) * wscale;
                weight += w;
                const __half* p = data + (size_t(vi) * rowlen + x) * 3;
                acc.x += __half2float(p[0]) * w;
                acc.y += __half2float(p[1]) * w;
                acc.z += __half2float(p[2]) * w;
            }
            Q += DQ;
            DQ += DDQ;
        }
    }
}

// PtexTriangleFilter::apply: clamp, build the even and odd iterators, walk both over the face whose
// resolution is 2^flog2 and whose texels start at `data`.
__device__ __forceinline__ void ptex_apply(PtexKernel k, int flog2, const __half* __restrict__ data, float3& acc,
                                           float& weight) {
    k.reslog2 = min(k.reslog2, flog2);
    k.u1 = fmaxf(k.u1, 0.0f);
    k.v1 = fmaxf(k.v1, 0.0f);
    k.w1 = fmaxf(k.w1, 0.0f);
    k.u2 = fminf(k.u2, 1.0f - (k.v1 + k.w1));
    k.v2 = fminf(k.v2, 1.0f - (k.w1 + k.u1));
    k.w2 = fminf(k.w2, 1.0f - (k.u1 + k.v1));
    const int resu = 1 << k.reslog2;
    const float Finv = 1.0f / ((float)resu * (float)resu * (k.A * k.C - 0.25f * k.B * k.B));
    const float Ak = k.A * Finv, Bk = k.B * Finv, Ck = k.C * Finv;
    const float third = float(1 / 3.0);
    const float scale = (float)resu;
    const float wscale = 1.0f / ((float)resu * (float)resu);
    // even iterator
    const int eu1 = int(ceilf(k.u1 * scale - third)), ev1 = int(ceilf(k.v1 * scale - third));
    const int ew1 = int(ceilf(k.w1 * scale - third)), eu2 = int(ceilf(k.u2 * scale - third));
    const int ev2 = int(ceilf(k.v2 * scale - third)), ew2 = int(ceilf(k.w2 * scale - third));
    const bool even = eu2 > eu1 && ev2 > ev1 && ew2 > ew1;
    // odd iterator: flipped across the diagonal
    const int ou1 = int(ceilf((1.0f - k.v2) * scale - third)), ov1 = int(ceilf((1.0f - k.u2) * scale - third));
    const int ow1 = int(ceilf((-k.w2) * scale - third)), ou2 = int(ceilf((1.0f - k.v1) * scale - third));
    const int ov2 = int(ceilf((1.0f - k.u1) * scale - third)), ow2 = int(ceilf((-k.w1) * scale - third));
    const bool odd = ou2 > ou1 && ov2 > ov1 && ow2 > ow1;
    if (!even && !odd) return;
    if (even) {
        float we = 0.0f;
        ptex_walk(resu, k.u * scale - third, k.v * scale - third, eu1, ev1, ew1, eu2, ev2, ew2, Ak, Bk, Ck, wscale,
                  data, acc, we);
        weight += we;
    }
    if (odd) {
        float wo = 0.0f;
        ptex_walk(resu, (1.0f - k.v) * scale - third, (1.0f - k.u) * scale - third, ou1, ov1, ow1, ou2, ov2, ow2, Ck,
                  Bk, Ak, wscale, data, acc, wo);
        weight += wo;
    }
}

// One application of the filter: the kernel in one face's coordinates (before apply's clamping), the face's
// resolution and its first texel.
struct PtexApp {
    PtexKernel k;
    int log2;
    const __half* data;
};

// splitAndApply (PtexTriangleFilter.cpp:96-167) as a resumable depth-first walk over an explicit frame stack:
// each call of ptex_split_next runs to the next application, in the order of the reference's recursion.
struct PtexSplit {
    struct Frame {
        PtexKernel k;
        int face;
        int phase;  // 0/1/2: split across edges 2 (u), 0 (v), 1 (w) next; 3: apply
    };
    Frame st[kPtexStack];
    int sp;
};

// buildKernel for a zero-size footprint (PtexTriangleFilter.cpp:50-94) on a face of resolution 2^log2: only the
// texel-size term of the blur survives.  u and v are clamped to [0, 1].
__device__ __forceinline__ void ptex_root_kernel(int log2, float u, float v, PtexKernel& k) {
    u = clampf(u, 0.0f, 1.0f);
    v = clampf(v, 0.0f, 1.0f);
    const float res = (float)(1 << log2);
    const float b = (0.5f / res) * (0.5f / res);
    const float Ac = 0.0f + b, Cc = 0.0f + b, Bc = 0.0f, X = 0.0f;
    const float m = sqrtf(2.0f * (Ac * Cc - 0.25f * Bc * Bc) / (Ac + Cc + X));
    const int reslog2 = max(0, 127 - int((__float_as_uint(2.0f * m) >> 23) & 0xffu));
    float A = float(4 / 3.0) * Ac;
    float B = (2.0f / 1.7320508075688772f) * Bc + A;
    float C = -0.25f * A + 0.5f * B + Cc;
    const float sc = 3.5f * 3.5f;
    A *= sc;
    B *= sc;
    C *= sc;
    const float uw = fminf(sqrtf(C), 1.0f), vw = fminf(sqrtf(A), 1.0f), ww = fminf(sqrtf(A - B + C), 1.0f);
    const float w = 1.0f - u - v;
    k.u = u; k.v = v;
    k.u1 = u - uw; k.v1 = v - vw; k.w1 = w - ww;
    k.u2 = u + uw; k.v2 = v + vw; k.w2 = w + ww;
    k.A = A; k.B = B; k.C = C;
    k.reslog2 = reslog2;
}

// `face` must be a valid face index.
__device__ __forceinline__ void ptex_split_init(PtexSplit& w, const PtexFace* __restrict__ faces, int face, float u,
                                                float v) {
    PtexSplit::Frame& fr = w.st[0];
    ptex_root_kernel(faces[face].log2, u, v, fr.k);
    fr.face = face;
    fr.phase = 0;
    w.sp = 0;
}

// The edges that the footprint of a query at (face, u, v) crosses (bit 0: u, bit 1: v, bit 2: w below 0): the
// first branches of the split walk.  Queries with the same face and region mostly walk the same faces, so a
// queue ordered by (face, region) keeps a warp's filter walks in step.  0 for a face outside [0, nfaces).
__device__ __forceinline__ uint32_t ptex_region(const PtexFace* __restrict__ faces, int nfaces, int face, float u,
                                                float v) {
    if (face < 0 || face >= nfaces) return 0u;
    PtexKernel k;
    ptex_root_kernel(faces[face].log2, u, v, k);
    return (k.u1 < 0.0f ? 1u : 0u) | (k.v1 < 0.0f ? 2u : 0u) | (k.w1 < 0.0f ? 4u : 0u);
}

// The next application of the walk into `app`; false when the walk is over (or its stack overflowed, which
// sets kErrPtexStack and ends it as the reference's filter would have run out of stack).
__device__ __forceinline__ bool ptex_split_next(PtexSplit& w, const PtexFace* __restrict__ faces,
                                                const __half* __restrict__ texels, PtexApp& app, uint32_t& status) {
    while (w.sp >= 0) {
        PtexSplit::Frame& fr = w.st[w.sp];
        const PtexFace f = faces[fr.face];
        int eid = -1;
        while (fr.phase < 3 && eid < 0) {
            const int ph = fr.phase++;
            if (ph == 0 && fr.k.u1 < 0.0f && f.adj[2] >= 0) eid = 2;
            else if (ph == 1 && fr.k.v1 < 0.0f && f.adj[0] >= 0) eid = 0;
            else if (ph == 2 && fr.k.w1 < 0.0f && f.adj[1] >= 0) eid = 1;
        }
        if (eid >= 0) {
            if (w.sp + 1 >= kPtexStack) {
                status |= kErrPtexStack;
                w.sp = -1;
                return false;
            }
            PtexKernel ka = fr.k;
            if (eid == 2) { fr.k.u1 = 0.0f; ka.u2 = 0.0f; }
            else if (eid == 0) { fr.k.v1 = 0.0f; ka.v2 = 0.0f; }
            else { fr.k.w1 = 0.0f; ka.w2 = 0.0f; }
            const int aeid = f.adjedge[eid];
            pk_reorient(ka, eid, aeid);
            PtexSplit::Frame& nx = w.st[w.sp + 1];
            nx.k = ka;
            nx.face = f.adj[eid];
            nx.phase = 0;
            ++w.sp;
            continue;
        }
        app.k = fr.k;
        app.log2 = f.log2;
        app.data = texels + size_t(f.offset) * 3;
        --w.sp;
        return true;
    }
    return false;
}

// Filtered RGB at (face, u, v), one query per thread.  Returns false (and leaves `out`) for a face outside
// [0, nfaces).
__device__ __forceinline__ bool ptex_eval(const PtexFace* __restrict__ faces, int nfaces,
                                          const __half* __restrict__ texels, int face, float u, float v,
                                          float3& out, uint32_t& status) {
    if (face < 0 || face >= nfaces) return false;
    PtexSplit w;
    ptex_split_init(w, faces, face, u, v);
    float3 acc = f3(0.0f);
    float weight = 0.0f;
    PtexApp a;
    while (ptex_split_next(w, faces, texels, a, status)) ptex_apply(a.k, a.log2, a.data, acc, weight);
    const float s = 1.0f / (weight * 1.0f);
    out = f3(acc.x * s, acc.y * s, acc.z * s);
    return true;
}

}  // namespace sel
