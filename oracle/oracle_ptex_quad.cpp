// ORACLE - test infrastructure only (see oracle_query.cpp).
//
// CPU restatement of the Ptex filter Selas applies to a quad mesh (SurfaceParameters.cpp:196-206:
// getFilter(f_bspline) on an mt_quad texture -> PtexBicubicFilter with sharpness 0, eval(faceid = primId, u, v,
// widths 0)), pinned bit for bit against tests/golden/ptex_quad_golden.npz written and filtered by the vendored
// Ptex 2.2 source:
//   PtexBicubicFilter coefficients and kernel         Middleware/ptex/Include/PtexFilters.cpp:248-285
//   PtexWidth4Filter::buildKernelAxis                  PtexFilters.cpp:116-241 (lerp off, as Options' default)
//   PtexSeparableFilter::eval / splitAndApply / applyAcrossEdge / applyToCorner / applyToCornerFace / apply
//                                                      PtexSeparableFilter.cpp:47-359
//   PtexSeparableKernel (strip, weight, merge, split, flip, swap, rotate, makeSymmetric)
//                                                      PtexSeparableKernel.h:60-420, the row-by-row apply of
//                                                      PtexSeparableKernel.cpp:40-66 and PtexUtils.h:200-233
//   constant faces and neighbourhoods                  PtexWriter.cpp:814-816,996-1075 (the writer's flags)
// Texture model: every face has the same square resolution 2^log2 (no reductions are read), no subfaces, clamp
// borders (the writer's default), half RGB texels row-major per face; a face whose texels are all the same bits
// is constant (applied through its kernel weight), and a constant face whose neighbourhood holds only constant
// faces of the same value returns that value.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

float half_bits_to_float(uint16_t h) {
    const uint32_t sign = uint32_t(h >> 15) << 31;
    const uint32_t exp = (h >> 10) & 0x1f;
    const uint32_t man = h & 0x3ff;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {
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

struct QFace {
    int log2;
    uint32_t offset;
    int adj[4];
    int adjedge[4];
    bool constant, nbconstant;
};

enum { kBottom = 0, kRight = 1, kTop = 2, kLeft = 3 };
constexpr int kMax = 10;

// The B-spline member of the bicubic family (B = 1, C = 0), coefficients as PtexBicubicFilter computes them.
struct Coeffs {
    float c[7];
    Coeffs() {
        const float B = 1.0f - 0.0f;
        c[0] = 1.5f - B;
        c[1] = 1.5f * B - 2.5f;
        c[2] = 1.0f - float(1.0 / 3.0) * B;
        c[3] = float(1.0 / 3.0) * B - 0.5f;
        c[4] = 2.5f - 1.5f * B;
        c[5] = 2.0f * B - 4.0f;
        c[6] = 2.0f - float(2.0 / 3.0) * B;
    }
};

float bspline(float x, const float* c) {
    x = std::fabs(x);
    if (x < 1.0f) return (c[0] * x + c[1]) * x * x + c[2];
    if (x < 2.0f) return ((c[3] * x + c[4]) * x + c[5]) * x + c[6];
    return 0.0f;
}

float blur(float x) {
    x = std::fabs(x);
    return x < 1.0f ? (2.0f * x - 3.0f) * x * x + 1.0f : 0.0f;
}

float sum(const float* p, int n) {
    float r = 0.0f;
    for (int i = 0; i < n; ++i) r += p[i];
    return r;
}

// A separable kernel: weights live in fixed buffers, `ku` / `kv` index the first one in use.
struct Kernel {
    int ulog2 = 0, vlog2 = 0;
    int u = 0, v = 0, uw = 0, vw = 0;
    float kub[kMax] = {}, kvb[kMax] = {};
    int ku = 0, kv = 0;
    int rot = 0;

    int resu() const { return 1 << ulog2; }
    int resv() const { return 1 << vlog2; }
    float* KU() { return kub + ku; }
    float* KV() { return kvb + kv; }
    const float* KU() const { return kub + ku; }
    const float* KV() const { return kvb + kv; }

    // set(): the weights copied to the start of fresh buffers
    void set(int ul, int vl, int uu, int vv, int uww, int vww, const float* kuv, const float* kvv, int r = 0) {
        float tu[kMax], tv[kMax];
        std::memcpy(tu, kuv, sizeof(float) * uww);
        std::memcpy(tv, kvv, sizeof(float) * vww);
        ulog2 = ul; vlog2 = vl; u = uu; v = vv; uw = uww; vw = vww;
        std::memcpy(kub, tu, sizeof(float) * uww);
        std::memcpy(kvb, tv, sizeof(float) * vww);
        ku = 0; kv = 0; rot = r;
    }
    void copy_from(const Kernel& k) { set(k.ulog2, k.vlog2, k.u, k.v, k.uw, k.vw, k.KU(), k.KV(), k.rot); }

    void strip_zeros() {
        while (KU()[0] == 0) { ++ku; ++u; --uw; }
        while (KU()[uw - 1] == 0) { --uw; }
        while (KV()[0] == 0) { ++kv; ++v; --vw; }
        while (KV()[vw - 1] == 0) { --vw; }
    }
    float weight() const { return sum(KU(), uw) * sum(KV(), vw); }

    void mergeL() { const int w = -u; KU()[w] += sum(KU(), w); ku += w; uw -= w; u = 0; }
    void mergeR() { const int w = uw + u - resu(); float* kp = KU() + uw - w; kp[-1] += sum(kp, w); uw -= w; }
    void mergeB() { const int w = -v; KV()[w] += sum(KV(), w); kv += w; vw -= w; v = 0; }
    void mergeT() { const int w = vw + v - resv(); float* kp = KV() + vw - w; kp[-1] += sum(kp, w); vw -= w; }

    void splitL(Kernel& k) {
        const int w = -u;
        if (w < uw) {
            k.set(ulog2, vlog2, resu() - w, v, w, vw, KU(), KV());
            u = 0; uw -= w; ku += w;
        } else {
            k.copy_from(*this);
            k.u += resu();
            u = 0; uw = 0;
        }
    }
    void splitR(Kernel& k) {
        const int w = u + uw - resu();
        if (w < uw) {
            k.set(ulog2, vlog2, 0, v, w, vw, KU() + uw - w, KV());
            uw -= w;
        } else {
            k.copy_from(*this);
            k.u -= resu();
            u = 0; uw = 0;
        }
    }
    void splitB(Kernel& k) {
        const int w = -v;
        if (w < vw) {
            k.set(ulog2, vlog2, u, resv() - w, uw, w, KU(), KV());
            v = 0; vw -= w; kv += w;
        } else {
            k.copy_from(*this);
            k.v += resv();
            v = 0; vw = 0;
        }
    }
    void splitT(Kernel& k) {
        const int w = v + vw - resv();
        if (w < vw) {
            k.set(ulog2, vlog2, u, 0, uw, w, KU(), KV() + vw - w);
            vw -= w;
        } else {
            k.copy_from(*this);
            k.v -= resv();
            v = 0; vw = 0;
        }
    }
    void flipU() { u = resu() - u - uw; std::reverse(KU(), KU() + uw); }
    void flipV() { v = resv() - v - vw; std::reverse(KV(), KV() + vw); }
    void swapUV() {
        std::swap(ulog2, vlog2);
        std::swap(u, v);
        std::swap(uw, vw);
        // the weight buffers swap roles with their offsets
        float t[kMax];
        std::memcpy(t, kub, sizeof(t));
        std::memcpy(kub, kvb, sizeof(t));
        std::memcpy(kvb, t, sizeof(t));
        std::swap(ku, kv);
    }
    void rotate(int r) {
        switch (r & 3) {
            default: return;
            case 1: flipU(); swapUV(); break;
            case 2: flipU(); flipV(); break;
            case 3: flipV(); swapUV(); break;
        }
        rot = (rot + r) & 3;
    }
    float make_symmetric(float initial) {
        // square faces of one resolution: no reduction of either axis is needed
        uw = vw = std::min(uw, vw);
        float nw = 0.0f;
        for (int i = 0; i < uw; ++i) {
            const float s = KU()[i] + KV()[i];
            KU()[i] = KV()[i] = s;
            nw += s;
        }
        nw *= nw;
        const float scale = nw == 0 ? 1.0f : initial / nw;
        if (scale >= 1) {
        } else if (scale < -1) {
            for (int i = 0; i < uw; ++i) KU()[i] *= -1;
            nw = -nw;
        } else {
            for (int i = 0; i < uw; ++i) KU()[i] *= scale;
            nw = initial;
        }
        return nw;
    }
};

// PtexWidth4Filter::buildKernelAxis with lerp off (lerp1 = 1, lerp2 = 0).
void build_axis(int& klog2, int& ku, int& kw, float* w, float u, float uw, int flog2, const float* c) {
    uw = std::max(uw, [] (int p) { uint32_t bits = uint32_t(127 - p) << 23; float f; std::memcpy(&f, &bits, 4); return f; }(flog2));
    {
        uint32_t bits;
        std::memcpy(&bits, &uw, 4);
        klog2 = 127 - int((bits >> 23) & 0xff);
    }
    const int resu = 1 << klog2;
    const float lerp2 = 0.0f, lerp1 = 1.0f - lerp2;
    if (uw >= .25f) {
        if (uw < .5f) {
            klog2 = 2;
            const float upix = u * 4.0f - 0.5f;
            int u1 = int(std::ceil(upix - 2)), u2 = int(std::ceil(upix + 2));
            u1 = u1 & ~1;
            u2 = (u2 + 1) & ~1;
            ku = u1;
            kw = u2 - u1;
            const float x1 = float(u1) - upix;
            for (int i = 0; i < kw; i += 2) {
                const float xa = x1 + float(i), xb = xa + 1.0f, xc = (xa + xb) * 0.25f;
                const float s = 1.0f / (uw + .75f);
                const float ka = bspline(xa, c), kb = bspline(xb, c), kc = blur(xc * s);
                w[i] = ka * lerp1 + kc * lerp2;
                w[i + 1] = kb * lerp1 + kc * lerp2;
            }
            return;
        } else if (uw < 1) {
            klog2 = 1;
            const float upix = u * 2.0f - 0.5f;
            ku = int(std::floor(u - .5f)) * 2;
            kw = 4;
            const float x1 = float(ku) - upix;
            for (int i = 0; i < kw; i += 2) {
                const float xa = x1 + float(i), xb = xa + 1.0f, xc = (xa + xb) * 0.5f;
                const float s = 1.0f / (uw * 1.5f + .5f);
                const float ka = blur(xa * s), kb = blur(xb * s), kc = blur(xc * s);
                w[i] = ka * lerp1 + kc * lerp2;
                w[i + 1] = kb * lerp1 + kc * lerp2;
            }
            return;
        } else {
            klog2 = 0;
            const float upix = u - .5f;
            kw = 2;
            const float ui = std::floor(upix);
            ku = int(ui);
            w[0] = blur(upix - ui);
            w[1] = 1 - w[0];
            return;
        }
    }
    const float upix = u * float(resu) - 0.5f;
    const float uwpix = uw * float(resu);
    const float dupix = 2.0f * uwpix;
    const int u1 = int(std::ceil(upix - dupix)), u2 = int(std::ceil(upix + dupix));
    ku = u1;
    kw = u2 - u1;
    const float x1 = (float(u1) - upix) / uwpix, step = 1.0f / uwpix;
    for (int i = 0; i < kw; ++i) w[i] = bspline(x1 + float(i) * step, c);
}

struct Filter {
    const QFace* faces;
    int nfaces;
    const uint16_t* texels;
    Coeffs co;
    float result[3];
    float weight;

    void apply(Kernel& k, int faceid) {
        if (k.uw <= 0 || k.vw <= 0) return;
        const QFace& f = faces[faceid];
        const uint16_t* d = texels + size_t(f.offset) * 3;
        if (f.constant) {
            const float w = k.weight();
            for (int c = 0; c < 3; ++c) result[c] += half_bits_to_float(d[c]) * w;
            return;
        }
        const int resu = k.resu();
        for (int j = 0; j < k.vw; ++j) {
            const uint16_t* p = d + (size_t(k.v + j) * resu + k.u) * 3;
            float row[3];
            for (int c = 0; c < 3; ++c) row[c] = half_bits_to_float(p[c]) * k.KU()[0];
            for (int i = 1; i < k.uw; ++i)
                for (int c = 0; c < 3; ++c) row[c] += half_bits_to_float(p[3 * i + c]) * k.KU()[i];
            for (int c = 0; c < 3; ++c) result[c] += row[c] * k.KV()[j];
        }
    }

    void across_edge(Kernel& k, int faceid, int eid) {
        const QFace& f = faces[faceid];
        const int afid = f.adj[eid], aeid = f.adjedge[eid];
        k.rotate(eid - aeid + 2);
        apply(k, afid);
    }

    void corner_face(Kernel& k, int eid, int cfid, int ceid) {
        k.rotate(eid - ceid + 2);
        apply(k, cfid);
    }

    void to_corner(Kernel& k, int faceid, int eid) {
        int afid = faceid, aeid = eid;
        const QFace* af = &faces[faceid];
        const int kMaxValence = 10;
        int cface[kMaxValence], cedge[kMaxValence];
        int num = 0;
        for (int i = 0; i < kMaxValence; ++i) {
            const int a = af->adj[aeid];
            aeid = (af->adjedge[aeid] + 1) % 4;
            afid = a;
            if (afid < 0 || (afid == faceid && aeid == eid)) {
                num = i - 2;
                break;
            }
            af = &faces[afid];
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
            weight += nw * float(num) - initial;
        } else {
            weight -= k.weight();
        }
    }

    void split_and_apply(Kernel& k, int faceid) {
        const QFace& f = faces[faceid];
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

    bool eval(int faceid, float u, float v, float* out) {
        if (faceid < 0 || faceid >= nfaces) return false;
        const QFace& f = faces[faceid];
        if (f.nbconstant) {
            const uint16_t* d = texels + size_t(f.offset) * 3;
            for (int c = 0; c < 3; ++c) out[c] = half_bits_to_float(d[c]);
            return true;
        }
        u = std::min(std::max(u, 0.0f), 1.0f);
        v = std::min(std::max(v, 0.0f), 1.0f);
        Kernel k;
        build_axis(k.ulog2, k.u, k.uw, k.kub, u, 0.0f, f.log2, co.c);
        build_axis(k.vlog2, k.v, k.vw, k.kvb, v, 0.0f, f.log2, co.c);
        k.strip_zeros();
        weight = k.weight();
        result[0] = result[1] = result[2] = 0.0f;
        split_and_apply(k, faceid);
        const float scale = 1.0f / (weight * 1.0f);
        for (int c = 0; c < 3; ++c) out[c] = float(result[c] * scale);
        return true;
    }
};

// The writer's face flags: constant (every texel the same bits) and, for a constant face, a neighbourhood of
// constant faces of the same value around each of its vertices (PtexMainWriter::flagConstantNeighorhoods with
// clamp borders and no subfaces).
void flag_constant(std::vector<QFace>& faces, const uint16_t* texels) {
    for (QFace& f : faces) {
        const size_t n = size_t(1) << (2 * f.log2);
        const uint16_t* d = texels + size_t(f.offset) * 3;
        f.constant = true;
        for (size_t i = 1; i < n && f.constant; ++i) f.constant = std::memcmp(d, d + 3 * i, 6) == 0;
        f.nbconstant = false;
    }
    const int n = int(faces.size());
    for (int faceid = 0; faceid < n; ++faceid) {
        QFace& f = faces[faceid];
        if (!f.constant) continue;
        const uint16_t* cd = texels + size_t(f.offset) * 3;
        auto same = [&](int afid) {
            return faces[afid].constant && std::memcmp(cd, texels + size_t(faces[afid].offset) * 3, 6) == 0;
        };
        bool is_const = true;
        for (int eid = 0; is_const && eid < 4; ++eid) {
            int afid = f.adj[eid], aeid = f.adjedge[eid];
            int count = 0;
            while (afid != faceid && afid >= 0 && ++count < 10) {
                if (!same(afid)) { is_const = false; break; }
                const QFace& af = faces[afid];
                aeid = (aeid + 1) % 4;
                afid = af.adj[aeid];
                aeid = af.adjedge[aeid];
            }
            if (afid < 0 && is_const) {
                aeid = (aeid - 1 + 4) % 4;
                afid = f.adj[aeid];
                aeid = f.adjedge[aeid];
                count = 0;
                while (afid != faceid && afid >= 0 && ++count < 10) {
                    if (!same(afid)) { is_const = false; break; }
                    const QFace& af = faces[afid];
                    aeid = (aeid - 1 + 4) % 4;
                    afid = af.adj[aeid];
                    aeid = af.adjedge[aeid];
                }
            }
        }
        f.nbconstant = is_const;
    }
}

struct QuadState {
    std::vector<QFace> faces;
    std::vector<uint16_t> texels;
};

std::vector<QFace> read_rows(const int32_t* rows, int nfaces) {
    std::vector<QFace> faces(size_t(nfaces > 0 ? nfaces : 0));
    for (int i = 0; i < nfaces; ++i) {
        const int32_t* r = rows + 10 * i;
        faces[i].log2 = r[0];
        faces[i].offset = uint32_t(r[1]);
        for (int e = 0; e < 4; ++e) {
            faces[i].adj[e] = r[2 + e];
            faces[i].adjedge[e] = r[6 + e];
        }
    }
    return faces;
}

}  // namespace

#include "oracle_ptex.h"

namespace orp {

QuadTexture::QuadTexture(const int32_t* rows, int n, const uint16_t* texels, size_t texel_count) {
    QuadState* s = new QuadState;
    s->faces = read_rows(rows, n);
    s->texels.assign(texels, texels + texel_count);
    flag_constant(s->faces, s->texels.data());
    state = s;
}

QuadTexture::~QuadTexture() { delete static_cast<QuadState*>(state); }

bool QuadTexture::eval(int face, float u, float v, float* out) const {
    const QuadState* s = static_cast<const QuadState*>(state);
    Filter flt;
    flt.faces = s->faces.data();
    flt.nfaces = int(s->faces.size());
    flt.texels = s->texels.data();
    return flt.eval(face, u, v, out);
}

}  // namespace orp

extern "C" {

// faces: nfaces x 10 ints (log2, texel offset, adj0..3, adjedge0..3); texels: half RGB; queries: n x (face as
// int bits, u, v); out: n x 3 (untouched for invalid faces).
void oracle_ptex_quad_eval(const int32_t* rows, int nfaces, const uint16_t* texels, const float* queries, int64_t n,
                           float* out) {
    std::vector<QFace> faces = read_rows(rows, nfaces);
    flag_constant(faces, texels);
    Filter flt;
    flt.faces = faces.data();
    flt.nfaces = nfaces;
    flt.texels = texels;
    for (int64_t i = 0; i < n; ++i) {
        int32_t face;
        std::memcpy(&face, &queries[3 * i], 4);
        flt.eval(face, queries[3 * i + 1], queries[3 * i + 2], out + 3 * i);
    }
}

}  // extern "C"
