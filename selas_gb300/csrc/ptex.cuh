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

// PtexTriangleFilter::apply: clamp, build the even and odd iterators, walk both.
__device__ __forceinline__ void ptex_apply(PtexKernel k, const PtexFace& f, const __half* __restrict__ texels,
                                           float3& acc, float& weight) {
    const int flog2 = f.log2;
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
    const __half* data = texels + size_t(f.offset) * 3;
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

// Filtered RGB at (face, u, v).  Returns false (and leaves `out`) for a face outside [0, nfaces).
__device__ __forceinline__ bool ptex_eval(const PtexFace* __restrict__ faces, int nfaces,
                                          const __half* __restrict__ texels, int face, float u, float v,
                                          float3& out, uint32_t& status) {
    if (face < 0 || face >= nfaces) return false;
    const PtexFace f0 = faces[face];
    u = clampf(u, 0.0f, 1.0f);
    v = clampf(v, 0.0f, 1.0f);
    // buildKernel for a zero-size footprint: only the texel-size term of the blur survives
    const float res = (float)(1 << f0.log2);
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

    struct Frame {
        PtexKernel k;
        int face;
        int phase;
    };
    Frame st[kPtexStack];
    int sp = 0;
    st[0].k.u = u; st[0].k.v = v;
    st[0].k.u1 = u - uw; st[0].k.v1 = v - vw; st[0].k.w1 = w - ww;
    st[0].k.u2 = u + uw; st[0].k.v2 = v + vw; st[0].k.w2 = w + ww;
    st[0].k.A = A; st[0].k.B = B; st[0].k.C = C;
    st[0].k.reslog2 = reslog2;
    st[0].face = face;
    st[0].phase = 0;
    float3 acc = f3(0.0f);
    float weight = 0.0f;
    // splitAndApply as a loop: phases 0/1/2 split across edges 2 (u), 0 (v), 1 (w); phase 3 applies
    while (sp >= 0) {
        Frame& fr = st[sp];
        const PtexFace f = faces[fr.face];
        int eid = -1;
        while (fr.phase < 3 && eid < 0) {
            const int ph = fr.phase++;
            if (ph == 0 && fr.k.u1 < 0.0f && f.adj[2] >= 0) eid = 2;
            else if (ph == 1 && fr.k.v1 < 0.0f && f.adj[0] >= 0) eid = 0;
            else if (ph == 2 && fr.k.w1 < 0.0f && f.adj[1] >= 0) eid = 1;
        }
        if (eid >= 0) {
            if (sp + 1 >= kPtexStack) {
                status |= kErrPtexStack;
                break;
            }
            PtexKernel ka = fr.k;
            if (eid == 2) { fr.k.u1 = 0.0f; ka.u2 = 0.0f; }
            else if (eid == 0) { fr.k.v1 = 0.0f; ka.v2 = 0.0f; }
            else { fr.k.w1 = 0.0f; ka.w2 = 0.0f; }
            const int aeid = f.adjedge[eid];
            pk_reorient(ka, eid, aeid);
            Frame& nx = st[sp + 1];
            nx.k = ka;
            nx.face = f.adj[eid];
            nx.phase = 0;
            ++sp;
            continue;
        }
        ptex_apply(fr.k, f, texels, acc, weight);
        --sp;
    }
    const float s = 1.0f / (weight * 1.0f);
    out = f3(acc.x * s, acc.y * s, acc.z * s);
    return true;
}

}  // namespace sel
