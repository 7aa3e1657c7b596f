// ORACLE - test infrastructure only (see oracle_query.cpp).
//
// CPU restatement of the Ptex triangle filter as Selas calls it (SurfaceParameters.cpp:196-208:
// getFilter(f_bspline) on a triangle mesh -> PtexTriangleFilter, eval(faceid = primId, u, v, all widths 0)),
// pinned against tests/golden/ptex_golden.npz generated by the vendored Ptex 2.2 source:
//   PtexTriangleFilter::eval / buildKernel / splitAndApply / applyAcrossEdge / apply
//                                        Middleware/ptex/Include/PtexTriangleFilter.cpp:50-218
//   PtexTriangleKernel (split, rotate, reorient, clamp, iterators)  PtexTriangleKernel.h:60-231
//   Gaussian weights, finite-difference ellipse walk               PtexTriangleKernel.cpp:44-75
//   calcResFromWidth                                               PtexUtils.h:102-113
// Texture model: every face of a mesh has the same square resolution 2^log2 (the synthetic textures),
// half-float RGB texels stored per face row-major, adjacency as Ptex FaceInfo (edge i runs from vertex i
// to vertex i+1; edge 0 is v = 0, edge 1 is w = 0, edge 2 is u = 0).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

float half_to_float(uint16_t h) {
    const uint32_t sign = uint32_t(h >> 15) << 31;
    const uint32_t exp = (h >> 10) & 0x1f;
    const uint32_t man = h & 0x3ff;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {  // subnormal: renormalise
            int e = -1;
            uint32_t m = man;
            do { m <<= 1; ++e; } while (!(m & 0x400));
            bits = sign | uint32_t(127 - 15 - e) << 23 | (m & 0x3ff) << 13;
        }
    } else if (exp == 31) {
        bits = sign | 0x7f800000u | man << 13;
    } else {
        bits = sign | (exp + 112) << 23 | man << 13;
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

struct Face {
    int log2;
    uint32_t offset;  // in texels
    int adj[3];
    int adjedge[3];
};

const float kWidth = 3.5f;  // PtexTriangleKernelWidth

struct Iter {
    int rowlen;
    float u, v;
    int u1, v1, w1, u2, v2, w2;
    float A, B, C;
    bool valid;
    float wscale, weight;
};

struct Kernel {
    int reslog2;
    float u, v, u1, v1, w1, u2, v2, w2, A, B, C;

    void set(float uu, float vv, float a1, float b1, float c1, float a2, float b2, float c2) {
        u = uu; v = vv; u1 = a1; v1 = b1; w1 = c1; u2 = a2; v2 = b2; w2 = c2;
    }
    void setABC(float a, float b, float c) { A = a; B = b; C = c; }
    void rotate1() { setABC(C, 2.0f * C - B, A + C - B); }
    void rotate2() { setABC(A + C - B, 2.0f * A - B, A); }
    void reorient(int eid, int aeid) {
        const float w = 1.0f - u - v;
        switch (eid * 3 + aeid) {
            case 0: set(1.0f - u, -v, 1.0f - u2, -v2, 1.0f - w2, 1.0f - u1, -v1, 1.0f - w1); break;
            case 1: set(1.0f - w, 1.0f - u, 1.0f - w2, 1.0f - u2, -v2, 1.0f - w1, 1.0f - u1, -v1); rotate1(); break;
            case 2: set(-v, 1.0f - w, -v2, 1.0f - w2, 1.0f - u2, -v1, 1.0f - w1, 1.0f - u1); rotate2(); break;
            case 3: set(1.0f - v, -w, 1.0f - v2, -w2, 1.0f - u2, 1.0f - v1, -w1, 1.0f - u1); rotate2(); break;
            case 4: set(1.0f - u, 1.0f - v, 1.0f - u2, 1.0f - v2, -w2, 1.0f - u1, 1.0f - v1, -w1); break;
            case 5: set(-w, 1.0f - u, -w2, 1.0f - u2, 1.0f - v2, -w1, 1.0f - u1, 1.0f - v1); rotate1(); break;
            case 6: set(1.0f - w, -u, 1.0f - w2, -u2, 1.0f - v2, 1.0f - w1, -u1, 1.0f - v1); rotate1(); break;
            case 7: set(1.0f - v, 1.0f - w, 1.0f - v2, 1.0f - w2, -u2, 1.0f - v1, 1.0f - w1, -u1); rotate2(); break;
            case 8: set(-u, 1.0f - v, -u2, 1.0f - v2, 1.0f - w2, -u1, 1.0f - v1, 1.0f - w1); break;
        }
    }
    void clamp_extent() {
        u1 = std::max(u1, 0.0f);
        v1 = std::max(v1, 0.0f);
        w1 = std::max(w1, 0.0f);
        u2 = std::min(u2, 1.0f - (v1 + w1));
        v2 = std::min(v2, 1.0f - (w1 + u1));
        w2 = std::min(w2, 1.0f - (u1 + v1));
    }
    void iterators(Iter& ke, Iter& ko) const {
        const int resu = 1 << reslog2;
        const float Finv = 1.0f / ((float)resu * (float)resu * (A * C - 0.25f * B * B));
        const float Ak = A * Finv, Bk = B * Finv, Ck = C * Finv;
        const float third = float(1 / 3.0);
        const float scale = (float)resu;
        ke.rowlen = resu;
        ke.wscale = 1.0f / ((float)resu * (float)resu);
        ke.u = u * scale - third;
        ke.v = v * scale - third;
        ke.u1 = int(std::ceil(u1 * scale - third));
        ke.v1 = int(std::ceil(v1 * scale - third));
        ke.w1 = int(std::ceil(w1 * scale - third));
        ke.u2 = int(std::ceil(u2 * scale - third));
        ke.v2 = int(std::ceil(v2 * scale - third));
        ke.w2 = int(std::ceil(w2 * scale - third));
        ke.A = Ak; ke.B = Bk; ke.C = Ck;
        ke.valid = ke.u2 > ke.u1 && ke.v2 > ke.v1 && ke.w2 > ke.w1;
        ke.weight = 0;
        ko.rowlen = ke.rowlen;
        ko.wscale = ke.wscale;
        ko.u = (1.0f - v) * scale - third;
        ko.v = (1.0f - u) * scale - third;
        ko.u1 = int(std::ceil((1.0f - v2) * scale - third));
        ko.v1 = int(std::ceil((1.0f - u2) * scale - third));
        ko.w1 = int(std::ceil((-w2) * scale - third));
        ko.u2 = int(std::ceil((1.0f - v1) * scale - third));
        ko.v2 = int(std::ceil((1.0f - u1) * scale - third));
        ko.w2 = int(std::ceil((-w1) * scale - third));
        ko.A = Ck; ko.B = Bk; ko.C = Ak;
        ko.valid = ko.u2 > ko.u1 && ko.v2 > ko.v1 && ko.w2 > ko.w1;
        ko.weight = 0;
    }
};

struct Filter {
    const Face* faces;
    int nfaces;
    const uint16_t* texels;
    float result[3];
    float weight;

    void apply_iter(Iter& k, const uint16_t* data) {
        const float scale = -0.5f * (kWidth * kWidth);
        const float DDQ = 2.0f * k.A;
        for (int vi = k.v1; vi != k.v2; vi++) {
            const int xw = k.rowlen - vi;
            const int x1 = std::max(k.u1, xw - k.w2);
            const int x2 = std::min(k.u2, xw - k.w1);
            const float U = (float)x1 - k.u;
            const float V = (float)vi - k.v;
            float DQ = k.A * (2.0f * U + 1.0f) + k.B * V;
            float Q = k.A * U * U + (k.B * U + k.C * V) * V;
            for (int x = x1; x < x2; ++x) {
                if (Q < 1.0f) {
                    const float w = (float)std::exp(scale * Q) * k.wscale;
                    k.weight += w;
                    const uint16_t* p = data + (size_t(vi) * k.rowlen + x) * 3;
                    for (int c = 0; c < 3; ++c) result[c] += half_to_float(p[c]) * w;
                }
                Q += DQ;
                DQ += DDQ;
            }
        }
    }

    void apply(Kernel& k, int faceid) {
        const Face& f = faces[faceid];
        k.reslog2 = std::min(k.reslog2, f.log2);  // clampRes
        k.clamp_extent();
        Iter ke, ko;
        k.iterators(ke, ko);
        if (!ke.valid && !ko.valid) return;
        const uint16_t* data = texels + size_t(f.offset) * 3;
        if (ke.valid) { apply_iter(ke, data); weight += ke.weight; }
        if (ko.valid) { apply_iter(ko, data); weight += ko.weight; }
    }

    void across(Kernel k, int faceid, int eid) {
        const Face& f = faces[faceid];
        const int afid = f.adj[eid], aeid = f.adjedge[eid];
        k.reorient(eid, aeid);
        split_and_apply(k, afid);
    }

    void split_and_apply(Kernel& k, int faceid) {
        const Face& f = faces[faceid];
        if (k.u1 < 0 && f.adj[2] >= 0) {
            Kernel ka = k;
            k.u1 = 0;
            ka.u2 = 0;
            across(ka, faceid, 2);
        }
        if (k.v1 < 0 && f.adj[0] >= 0) {
            Kernel ka = k;
            k.v1 = 0;
            ka.v2 = 0;
            across(ka, faceid, 0);
        }
        if (k.w1 < 0 && f.adj[1] >= 0) {
            Kernel ka = k;
            k.w1 = 0;
            ka.w2 = 0;
            across(ka, faceid, 1);
        }
        apply(k, faceid);
    }

    // PtexTriangleFilter::eval with uw1 = vw1 = uw2 = vw2 = 0, width 1, blur 0
    bool eval(int faceid, float u, float v, float* out) {
        if (faceid < 0 || faceid >= nfaces) return false;
        const Face& f = faces[faceid];
        u = std::min(std::max(u, 0.0f), 1.0f);
        v = std::min(std::max(v, 0.0f), 1.0f);
        // buildKernel (PtexTriangleFilter.cpp:105-164) for a zero-size footprint
        const float sqrt3 = 1.7320508075688772f;
        const float uw1 = 0, vw1 = 0, uw2 = 0, vw2 = 0, width = 1.0f, blur = 0.0f;
        const float scaleAC = 0.25f * width * width;
        const float scaleB = -2.0f * scaleAC;
        float A = (vw1 * vw1 + vw2 * vw2) * scaleAC;
        float B = (uw1 * vw1 + uw2 * vw2) * scaleB;
        float C = (uw1 * uw1 + uw2 * uw2) * scaleAC;
        float Ac = 0.75f * A;
        float Bc = float(sqrt3 / 2) * (B - A);
        float Cc = 0.25f * A - 0.5f * B + C;
        const float maxEcc = 15.0f;
        const float eccRatio = (maxEcc * maxEcc + 1.0f) / (maxEcc * maxEcc - 1.0f);
        const float X = std::sqrt((Ac - Cc) * (Ac - Cc) + Bc * Bc);
        const float b_e = 0.5f * (eccRatio * X - (Ac + Cc));
        const float b_t = (0.5f / (float)(1 << f.log2)) * (0.5f / (float)(1 << f.log2));
        const float b_b = 0.25f * blur * blur;
        const float b = std::max(b_b, std::max(b_e, b_t));
        Ac += b;
        Cc += b;
        const float m = std::sqrt(2.0f * (Ac * Cc - 0.25f * Bc * Bc) / (Ac + Cc + X));
        const float w2m = 2.0f * m;
        uint32_t bits;
        std::memcpy(&bits, &w2m, 4);
        const int reslog2 = std::max(0, 127 - int((bits >> 23) & 0xff));
        A = float(4 / 3.0) * Ac;
        B = float(2 / sqrt3) * Bc + A;
        C = -0.25f * A + 0.5f * B + Cc;
        const float sc = kWidth * kWidth;
        A *= sc;
        B *= sc;
        C *= sc;
        const float uw = std::min(std::sqrt(C), 1.0f);
        const float vw = std::min(std::sqrt(A), 1.0f);
        const float ww = std::min(std::sqrt(A - B + C), 1.0f);
        const float w = 1.0f - u - v;
        Kernel k;
        k.reslog2 = reslog2;
        k.set(u, v, u - uw, v - vw, w - ww, u + uw, v + vw, w + ww);
        k.setABC(A, B, C);
        weight = 0;
        result[0] = result[1] = result[2] = 0;
        split_and_apply(k, faceid);
        const float s = 1.0f / (weight * 1.0f);
        for (int c = 0; c < 3; ++c) out[c] = float(result[c] * s);
        return true;
    }
};

}  // namespace

#include "oracle_ptex.h"

namespace orp {

Texture::Texture(const int32_t* rows, int n, const uint16_t* tex) : nfaces(n), texels(tex) {
    Face* fs = new Face[size_t(n > 0 ? n : 1)];
    for (int i = 0; i < n; ++i) {
        const int32_t* r = rows + 8 * i;
        fs[i].log2 = r[0];
        fs[i].offset = uint32_t(r[1]);
        for (int e = 0; e < 3; ++e) {
            fs[i].adj[e] = r[2 + e];
            fs[i].adjedge[e] = r[5 + e];
        }
    }
    faces = fs;
}

Texture::~Texture() { delete[] static_cast<Face*>(faces); }

bool Texture::eval(int face, float u, float v, float* out) const {
    Filter flt;
    flt.faces = static_cast<const Face*>(faces);
    flt.nfaces = nfaces;
    flt.texels = texels;
    return flt.eval(face, u, v, out);
}

}  // namespace orp

extern "C" {

// faces: nfaces x 8 ints (log2, texel offset, adj0, adj1, adj2, adjedge0, adjedge1, adjedge2);
// texels: half RGB; queries: n x (face as int bits, u, v); out: n x 3 (untouched for invalid faces).
void oracle_ptex_eval(const int32_t* faces, int nfaces, const uint16_t* texels, const float* queries, int64_t n,
                      float* out) {
    Face* fs = new Face[size_t(nfaces > 0 ? nfaces : 1)];
    for (int i = 0; i < nfaces; ++i) {
        const int32_t* r = faces + 8 * i;
        fs[i].log2 = r[0];
        fs[i].offset = uint32_t(r[1]);
        for (int e = 0; e < 3; ++e) {
            fs[i].adj[e] = r[2 + e];
            fs[i].adjedge[e] = r[5 + e];
        }
    }
    Filter flt;
    flt.faces = fs;
    flt.nfaces = nfaces;
    flt.texels = texels;
    for (int64_t i = 0; i < n; ++i) {
        int32_t face;
        std::memcpy(&face, &queries[3 * i], 4);
        flt.eval(face, queries[3 * i + 1], queries[3 * i + 2], out + 3 * i);
    }
    delete[] fs;
}

}  // extern "C"
