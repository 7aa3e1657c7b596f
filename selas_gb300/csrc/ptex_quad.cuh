// Device-side Ptex filter of quad meshes: the separable bicubic filter with B-spline weights that
// PtexFilter::getFilter(f_bspline) returns for an mt_quad texture, evaluated as Selas calls it
// (Source/Core/Shading/SurfaceParameters.cpp:196-206: eval(faceid = primId, u, v, widths 0)).
//
// Restates Middleware/ptex/Include:
//   PtexBicubicFilter (sharpness 0: B = 1, C = 0) and PtexWidth4Filter::buildKernelAxis   PtexFilters.cpp:116-285
//     (lerp off, the Options default; faces of 1, 2 and 4 texels a side take its wide-kernel branches)
//   PtexSeparableFilter::eval / splitAndApply / applyAcrossEdge / applyToCorner / applyToCornerFace / apply
//                                                                                        PtexSeparableFilter.cpp:47-359
//   PtexSeparableKernel's strip, weight, merge, split, flip, swap, rotate and makeSymmetric
//                                                                                        PtexSeparableKernel.h:60-420
//   the row-by-row application (PtexSeparableKernel.cpp:40-66, PtexUtils.h:200-233) and the constant-face
//   forms: a face whose texels are all one value is applied through its kernel weight, and a constant face
//   whose neighbourhood is constant returns its value (the writer's flags, PtexWriter.cpp:814-816,996-1075,
//   computed when the texture is bound).
// Every multiply and add is rounded on its own (no fused multiply-add), as the vendored library computes them,
// so the filter reproduces it bit for bit.
//
// Texture model: every face has the same square resolution 2^log2 (so no kernel is ever reduced or enlarged
// across an edge), no subfaces, clamp borders (the writer's default), half RGB texels row-major per face.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>

#include "ptex.cuh"
#include "scene_types.h"
#include "vecmath.cuh"

namespace sel {

// 32 bytes, stored in the same face table as the triangle faces (PtexFace): word 0 = log2 | flags << 8.
struct PtexQuadFace {
    uint32_t log2_flags;  // bits 0-7: square resolution 2^log2; bit 8: constant face; bit 9: constant neighbourhood
    uint32_t offset;      // texel offset of this face (in texels)
    int32_t adj[4];       // neighbouring face across edge i (bottom, right, top, left; -1 on a boundary)
    uint32_t adjedge;     // the neighbour's edge id for edge i in bits 8i..8i+7
    uint32_t pad;
};
static_assert(sizeof(PtexQuadFace) == sizeof(PtexFace), "quad and triangle faces share one table");
constexpr uint32_t kQuadConstant = 1u << 8, kQuadNbConstant = 1u << 9;

namespace pq {

constexpr int kMax = 10;
enum { kBottom = 0, kRight = 1, kTop = 2, kLeft = 3 };

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

// The bicubic family at B = 1, C = 0 (the cubic B-spline), coefficients as PtexBicubicFilter computes them.
struct Coeffs {
    float c0, c1, c2, c3, c4, c5, c6;
};
__device__ __forceinline__ Coeffs bspline_coeffs() {
    const float B = 1.0f;
    Coeffs c;
    c.c0 = fs(1.5f, B);
    c.c1 = fs(fm(1.5f, B), 2.5f);
    c.c2 = fs(1.0f, fm(float(1.0 / 3.0), B));
    c.c3 = fs(fm(float(1.0 / 3.0), B), 0.5f);
    c.c4 = fs(2.5f, fm(1.5f, B));
    c.c5 = fs(fm(2.0f, B), 4.0f);
    c.c6 = fs(2.0f, fm(float(2.0 / 3.0), B));
    return c;
}
__device__ __forceinline__ float bspline(float x, const Coeffs& c) {
    x = fabsf(x);
    if (x < 1.0f) return fa(fm(fm(fa(fm(c.c0, x), c.c1), x), x), c.c2);
    if (x < 2.0f) return fa(fm(fa(fm(fa(fm(c.c3, x), c.c4), x), c.c5), x), c.c6);
    return 0.0f;
}
__device__ __forceinline__ float blur(float x) {
    x = fabsf(x);
    return x < 1.0f ? fa(fm(fm(fs(fm(2.0f, x), 3.0f), x), x), 1.0f) : 0.0f;
}
__device__ __forceinline__ float sum(const float* p, int n) {
    float r = 0.0f;
    for (int i = 0; i < n; ++i) r = fa(r, p[i]);
    return r;
}

// A separable kernel over one face: weights ku[ko .. ko + uw) and kv[vo .. vo + vw) of fixed buffers.
struct Kernel {
    int log2u, log2v, u, v, uw, vw, ko, vo, rot;
    float ku[kMax], kv[kMax];

    __device__ int resu() const { return 1 << log2u; }
    __device__ int resv() const { return 1 << log2v; }

    __device__ void set(int lu, int lv, int uu, int vv, int uww, int vww, const float* su, const float* sv, int r) {
        float tu[kMax], tv[kMax];
        for (int i = 0; i < uww; ++i) tu[i] = su[i];
        for (int i = 0; i < vww; ++i) tv[i] = sv[i];
        log2u = lu; log2v = lv; u = uu; v = vv; uw = uww; vw = vww; ko = 0; vo = 0; rot = r;
        for (int i = 0; i < uww; ++i) ku[i] = tu[i];
        for (int i = 0; i < vww; ++i) kv[i] = tv[i];
    }
    __device__ void copy_from(const Kernel& k) { set(k.log2u, k.log2v, k.u, k.v, k.uw, k.vw, k.ku + k.ko, k.kv + k.vo, k.rot); }

    __device__ void strip_zeros() {
        while (ku[ko] == 0.0f && uw > 1) { ++ko; ++u; --uw; }
        while (ku[ko + uw - 1] == 0.0f && uw > 1) --uw;
        while (kv[vo] == 0.0f && vw > 1) { ++vo; ++v; --vw; }
        while (kv[vo + vw - 1] == 0.0f && vw > 1) --vw;
    }
    __device__ float weight() const { return fm(sum(ku + ko, uw), sum(kv + vo, vw)); }

    __device__ void mergeL() { const int w = -u; ku[ko + w] = fa(ku[ko + w], sum(ku + ko, w)); ko += w; uw -= w; u = 0; }
    __device__ void mergeR() {
        const int w = uw + u - resu();
        float* kp = ku + ko + uw - w;
        kp[-1] = fa(kp[-1], sum(kp, w));
        uw -= w;
    }
    __device__ void mergeB() { const int w = -v; kv[vo + w] = fa(kv[vo + w], sum(kv + vo, w)); vo += w; vw -= w; v = 0; }
    __device__ void mergeT() {
        const int w = vw + v - resv();
        float* kp = kv + vo + vw - w;
        kp[-1] = fa(kp[-1], sum(kp, w));
        vw -= w;
    }
    __device__ void splitL(Kernel& k) {
        const int w = -u;
        if (w < uw) {
            k.set(log2u, log2v, resu() - w, v, w, vw, ku + ko, kv + vo, 0);
            u = 0; uw -= w; ko += w;
        } else {
            k.copy_from(*this);
            k.u += resu();
            u = 0; uw = 0;
        }
    }
    __device__ void splitR(Kernel& k) {
        const int w = u + uw - resu();
        if (w < uw) {
            k.set(log2u, log2v, 0, v, w, vw, ku + ko + uw - w, kv + vo, 0);
            uw -= w;
        } else {
            k.copy_from(*this);
            k.u -= resu();
            u = 0; uw = 0;
        }
    }
    __device__ void splitB(Kernel& k) {
        const int w = -v;
        if (w < vw) {
            k.set(log2u, log2v, u, resv() - w, uw, w, ku + ko, kv + vo, 0);
            v = 0; vw -= w; vo += w;
        } else {
            k.copy_from(*this);
            k.v += resv();
            v = 0; vw = 0;
        }
    }
    __device__ void splitT(Kernel& k) {
        const int w = v + vw - resv();
        if (w < vw) {
            k.set(log2u, log2v, u, 0, uw, w, ku + ko, kv + vo + vw - w, 0);
            vw -= w;
        } else {
            k.copy_from(*this);
            k.v -= resv();
            v = 0; vw = 0;
        }
    }
    __device__ void flipU() {
        u = resu() - u - uw;
        for (int i = 0, j = uw - 1; i < j; ++i, --j) { const float t = ku[ko + i]; ku[ko + i] = ku[ko + j]; ku[ko + j] = t; }
    }
    __device__ void flipV() {
        v = resv() - v - vw;
        for (int i = 0, j = vw - 1; i < j; ++i, --j) { const float t = kv[vo + i]; kv[vo + i] = kv[vo + j]; kv[vo + j] = t; }
    }
    __device__ void swapUV() {
        int t = log2u; log2u = log2v; log2v = t;
        t = u; u = v; v = t;
        t = uw; uw = vw; vw = t;
        t = ko; ko = vo; vo = t;
        for (int i = 0; i < kMax; ++i) { const float x = ku[i]; ku[i] = kv[i]; kv[i] = x; }
    }
    __device__ void rotate(int r) {
        switch (r & 3) {
            default: return;
            case 1: flipU(); swapUV(); break;
            case 2: flipU(); flipV(); break;
            case 3: flipV(); swapUV(); break;
        }
        rot = (rot + r) & 3;
    }
    // square faces of one resolution: neither axis needs reducing first
    __device__ float make_symmetric(float initial) {
        uw = vw = uw < vw ? uw : vw;
        float nw = 0.0f;
        for (int i = 0; i < uw; ++i) {
            const float s = fa(ku[ko + i], kv[vo + i]);
            ku[ko + i] = kv[vo + i] = s;
            nw = fa(nw, s);
        }
        nw = fm(nw, nw);
        const float scale = nw == 0.0f ? 1.0f : __fdiv_rn(initial, nw);
        if (scale >= 1.0f) {
        } else if (scale < -1.0f) {
            for (int i = 0; i < uw; ++i) ku[ko + i] = fm(ku[ko + i], -1.0f);
            nw = -nw;
        } else {
            for (int i = 0; i < uw; ++i) ku[ko + i] = fm(ku[ko + i], scale);
            nw = initial;
        }
        return nw;
    }
};

// PtexWidth4Filter::buildKernelAxis for filter width 0 (clamped to one texel) with lerp off.
__device__ __forceinline__ void build_axis(int& klog2, int& ku, int& kw, float* w, float u, int flog2,
                                           const Coeffs& c) {
    const float uw = __uint_as_float(uint32_t(127 - flog2) << 23);  // max(0, reciprocalPow2(f_ureslog2))
    klog2 = 127 - int((__float_as_uint(uw) >> 23) & 0xffu);           // calcResFromWidth
    const int resu = 1 << klog2;
    if (uw >= .25f) {
        if (uw < .5f) {
            klog2 = 2;
            const float upix = fs(fm(u, 4.0f), 0.5f);
            int u1 = int(ceilf(fs(upix, 2.0f))), u2 = int(ceilf(fa(upix, 2.0f)));
            u1 = u1 & ~1;
            u2 = (u2 + 1) & ~1;
            ku = u1;
            kw = u2 - u1;
            const float x1 = fs(float(u1), upix);
            for (int i = 0; i < kw; i += 2) {
                const float xa = fa(x1, float(i)), xb = fa(xa, 1.0f), xc = fm(fa(xa, xb), 0.25f);
                const float s = __fdiv_rn(1.0f, fa(uw, .75f));
                const float ka = bspline(xa, c), kb = bspline(xb, c), kc = blur(fm(xc, s));
                w[i] = fa(fm(ka, 1.0f), fm(kc, 0.0f));
                w[i + 1] = fa(fm(kb, 1.0f), fm(kc, 0.0f));
            }
            return;
        }
        if (uw < 1.0f) {
            klog2 = 1;
            const float upix = fs(fm(u, 2.0f), 0.5f);
            ku = int(floorf(fs(u, .5f))) * 2;
            kw = 4;
            const float x1 = fs(float(ku), upix);
            for (int i = 0; i < kw; i += 2) {
                const float xa = fa(x1, float(i)), xb = fa(xa, 1.0f), xc = fm(fa(xa, xb), 0.5f);
                const float s = __fdiv_rn(1.0f, fa(fm(uw, 1.5f), .5f));
                const float ka = blur(fm(xa, s)), kb = blur(fm(xb, s)), kc = blur(fm(xc, s));
                w[i] = fa(fm(ka, 1.0f), fm(kc, 0.0f));
                w[i + 1] = fa(fm(kb, 1.0f), fm(kc, 0.0f));
            }
            return;
        }
        klog2 = 0;
        const float upix = fs(u, .5f);
        kw = 2;
        const float ui = floorf(upix);
        ku = int(ui);
        w[0] = blur(fs(upix, ui));
        w[1] = fs(1.0f, w[0]);
        return;
    }
    const float upix = fs(fm(u, float(resu)), 0.5f);
    const float uwpix = fm(uw, float(resu));
    const float dupix = fm(2.0f, uwpix);
    const int u1 = int(ceilf(fs(upix, dupix))), u2 = int(ceilf(fa(upix, dupix)));
    ku = u1;
    kw = u2 - u1;
    const float x1 = __fdiv_rn(fs(float(u1), upix), uwpix), step = __fdiv_rn(1.0f, uwpix);
    for (int i = 0; i < kw && i < kMax; ++i) w[i] = bspline(fa(x1, fm(float(i), step)), c);
}

struct Filter {
    const PtexQuadFace* __restrict__ faces;
    const __half* __restrict__ texels;
    float3 acc;
    float weight;

    __device__ void apply(const Kernel& k, int faceid) {
        if (k.uw <= 0 || k.vw <= 0) return;
        const PtexQuadFace f = faces[faceid];
        const __half* d = texels + size_t(f.offset) * 3;
        if (f.log2_flags & kQuadConstant) {
            const float w = k.weight();
            acc.x = fa(acc.x, fm(__half2float(d[0]), w));
            acc.y = fa(acc.y, fm(__half2float(d[1]), w));
            acc.z = fa(acc.z, fm(__half2float(d[2]), w));
            return;
        }
        const int resu = k.resu();
        for (int j = 0; j < k.vw; ++j) {
            const __half* p = d + (size_t(k.v + j) * resu + k.u) * 3;
            const float k0 = k.ku[k.ko];
            float rx = fm(__half2float(p[0]), k0), ry = fm(__half2float(p[1]), k0), rz = fm(__half2float(p[2]), k0);
            for (int i = 1; i < k.uw; ++i) {
                const float ki = k.ku[k.ko + i];
                rx = fa(rx, fm(__half2float(p[3 * i]), ki));
                ry = fa(ry, fm(__half2float(p[3 * i + 1]), ki));
                rz = fa(rz, fm(__half2float(p[3 * i + 2]), ki));
            }
            const float kvj = k.kv[k.vo + j];
            acc.x = fa(acc.x, fm(rx, kvj));
            acc.y = fa(acc.y, fm(ry, kvj));
            acc.z = fa(acc.z, fm(rz, kvj));
        }
    }
    __device__ void across_edge(Kernel& k, int faceid, int eid) {
        const PtexQuadFace& f = faces[faceid];
        const int afid = f.adj[eid], aeid = int((f.adjedge >> (8 * eid)) & 3u);
        k.rotate(eid - aeid + 2);
        apply(k, afid);
    }
    __device__ void corner_face(Kernel& k, int eid, int cfid, int ceid) {
        k.rotate(eid - ceid + 2);
        apply(k, cfid);
    }
    __device__ void to_corner(Kernel& k, int faceid, int eid) {
        int afid = faceid, aeid = eid;
        int cface[10], cedge[10];
        int num = 0;
        for (int i = 0; i < 10; ++i) {
            const PtexQuadFace& af = faces[afid];
            const int a = af.adj[aeid];
            aeid = int(((af.adjedge >> (8 * aeid)) + 1u) & 3u);
            afid = a;
            if (afid < 0 || (afid == faceid && aeid == eid)) {
                num = i - 2;
                break;
            }
            cface[i] = afid;
            cedge[i] = aeid;
        }
        if (num == 1) {
            corner_face(k, eid, cface[1], cedge[1]);
        } else if (num > 1) {
            k.rotate(eid + 2);
            const float initial = k.weight();
            const float nw = k.make_symmetric(initial);
            for (int i = 1; i <= num; ++i) {
                Kernel kc;
                kc.copy_from(k);
                corner_face(kc, 2, cface[i], cedge[i]);
            }
            weight = fa(weight, fs(fm(nw, float(num)), initial));
        } else {
            weight = fs(weight, k.weight());
        }
    }
    __device__ void split_and_apply(Kernel& k, int faceid) {
        const PtexQuadFace& f = faces[faceid];
        const bool splitR = k.u + k.uw > k.resu(), splitL = k.u < 0;
        const bool splitT = k.v + k.vw > k.resv(), splitB = k.v < 0;
        if (splitR || splitL || splitT || splitB) {
            Kernel ka, kc;
            if (splitR) {
                if (f.adj[kRight] >= 0) {
                    k.splitR(ka);
                    if (splitT) {
                        if (f.adj[kTop] >= 0) { ka.splitT(kc); to_corner(kc, faceid, kTop); }
                        else ka.mergeT();
                    }
                    if (splitB) {
                        if (f.adj[kBottom] >= 0) { ka.splitB(kc); to_corner(kc, faceid, kRight); }
                        else ka.mergeB();
                    }
                    across_edge(ka, faceid, kRight);
                } else {
                    k.mergeR();
                }
            }
            if (splitL) {
                if (f.adj[kLeft] >= 0) {
                    k.splitL(ka);
                    if (splitT) {
                        if (f.adj[kTop] >= 0) { ka.splitT(kc); to_corner(kc, faceid, kLeft); }
                        else ka.mergeT();
                    }
                    if (splitB) {
                        if (f.adj[kBottom] >= 0) { ka.splitB(kc); to_corner(kc, faceid, kBottom); }
                        else ka.mergeB();
                    }
                    across_edge(ka, faceid, kLeft);
                } else {
                    k.mergeL();
                }
            }
            if (splitT) {
                if (f.adj[kTop] >= 0) { k.splitT(ka); across_edge(ka, faceid, kTop); }
                else k.mergeT();
            }
            if (splitB) {
                if (f.adj[kBottom] >= 0) { k.splitB(ka); across_edge(ka, faceid, kBottom); }
                else k.mergeB();
            }
        }
        apply(k, faceid);
    }
};

}  // namespace pq

// PtexSeparableFilter::eval at (face, u, v) with zero filter widths; false (out untouched) for an invalid face.
// Not inlined: the shading kernels that call it keep one copy of its code.
static __device__ __noinline__ bool ptex_quad_eval(const PtexQuadFace* __restrict__ faces, int nfaces,
                                               const __half* __restrict__ texels, int face, float u, float v,
                                               float3& out) {
    if (face < 0 || face >= nfaces) return false;
    const PtexQuadFace f = faces[face];
    if (f.log2_flags & kQuadNbConstant) {
        const __half* d = texels + size_t(f.offset) * 3;
        out = make_float3(__half2float(d[0]), __half2float(d[1]), __half2float(d[2]));
        return true;
    }
    u = fminf(fmaxf(u, 0.0f), 1.0f);
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    const pq::Coeffs c = pq::bspline_coeffs();
    const int flog2 = int(f.log2_flags & 0xffu);
    pq::Kernel k;
    k.ko = k.vo = 0;
    k.rot = 0;
    pq::build_axis(k.log2u, k.u, k.uw, k.ku, u, flog2, c);
    pq::build_axis(k.log2v, k.v, k.vw, k.kv, v, flog2, c);
    k.strip_zeros();
    pq::Filter flt;
    flt.faces = faces;
    flt.texels = texels;
    flt.acc = make_float3(0.0f, 0.0f, 0.0f);
    flt.weight = k.weight();
    flt.split_and_apply(k, face);
    const float scale = __fdiv_rn(1.0f, pq::fm(flt.weight, 1.0f));
    out = make_float3(pq::fm(flt.acc.x, scale), pq::fm(flt.acc.y, scale), pq::fm(flt.acc.z, scale));
    return true;
}

// Base colour of a Ptex material at a hit: `prim` is the hit record's primitive word (a quad mesh: 2 * quad +
// half, with (u, v) the half-triangle's barycentrics, which Embree reports for the quad as (1 - u, 1 - v) on the
// second half); the quad filter for materials bound to a quad-mesh texture, else the triangle filter.
__device__ __forceinline__ void ptex_material_eval(const MaterialDev& m, const void* faces, int nfaces,
                                                   const __half* texels, uint32_t prim, float u, float v,
                                                   float3& base, uint32_t& status) {
    if (m.flags & kMaterialPtexQuad) {
        const bool second = (prim & 1u) != 0u;
        ptex_quad_eval(static_cast<const PtexQuadFace*>(faces), nfaces, texels, int(m.ptex_base + (prim >> 1)),
                       second ? 1.0f - u : u, second ? 1.0f - v : v, base);
    } else {
        ptex_eval(static_cast<const PtexFace*>(faces), nfaces, texels, int(m.ptex_base + prim), u, v, base, status);
    }
}

}  // namespace sel
