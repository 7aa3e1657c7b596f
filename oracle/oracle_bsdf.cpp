// ORACLE - test infrastructure only (see oracle_query.cpp).
//
// CPU restatement of the reference BSDF, pinned against tests/golden/bsdf_golden.npz (generated from the
// reference's own Disney.cpp / Ggx.cpp / Fresnel.cpp / DiracTransparent.cpp):
//   EvaluateBsdf        Source/Core/Shading/SurfaceScattering.cpp:41-60 -> Disney.cpp:525-614
//   SampleBsdfFunction  Source/Core/Shading/SurfaceScattering.cpp:18-38 -> Disney.cpp:617-659,
//                       DiracTransparent.cpp:20-68
// Also exported to the oracle path tracer (oracle_pt.cpp) through oracle_bsdf.h.

#include "oracle_bsdf.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

namespace orc {

namespace {

const float kPi = 3.141592653589793f;
const float kInvPi = 1.0f / kPi;

float Sat(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }
float Clampf(float x, float a, float b) { return x < a ? a : (x > b ? b : x); }
float Sq(float x) { return x * x; }
float Lerp(float a, float b, float t) { return (1.0f - t) * a + t * b; }
V3 Lerp(V3 a, V3 b, float t) { return (1.0f - t) * a + t * b; }
float Abs(float x) { return x < 0 ? -x : x; }

// y-up tangent space helpers, MathLib/Trigonometric.h:51-108
float SinT(const V3& w) { return std::sqrt(std::fmax(0.0f, 1.0f - w.y * w.y)); }
float TanT(const V3& w) { return SinT(w) / w.y; }
float CosP(const V3& w) { float s = SinT(w); return s == 0 ? 1.0f : Clampf(w.x / s, -1.0f, 1.0f); }
float SinP(const V3& w) { float s = SinT(w); return s == 0 ? 1.0f : Clampf(w.z / s, -1.0f, 1.0f); }

// Fresnel.cpp:19-84
float SchlickW(float u) { float m = Sat(1.0f - u); float m2 = m * m; return m * m2 * m2; }
float SchlickS(float r0, float c) { return Lerp(1.0f, SchlickW(c), r0); }
V3 SchlickC(V3 r0, float c) { float e = std::pow(1.0f - c, 5.0f); return r0 + (V3(1.0f) - r0) * e; }
float R0(float eta) { return Sq(eta - 1.0f) / Sq(eta + 1.0f); }
float Dielectric(float ci, float ni, float nt) {
    ci = Clampf(ci, -1.0f, 1.0f);
    if (ci < 0.0f) { float t = ni; ni = nt; nt = t; ci = -ci; }
    float si = std::sqrt(std::fmax(0.0f, 1.0f - ci * ci));
    float st = ni / nt * si;
    if (st >= 1) return 1;
    float ct = std::sqrt(std::fmax(0.0f, 1.0f - st * st));
    float a = ((nt * ci) - (ni * ct)) / ((nt * ci) + (ni * ct));
    float b = ((ni * ci) - (nt * ct)) / ((ni * ci) + (nt * ct));
    return (a * a + b * b) / 2;
}

// Ggx.cpp
float G1(const V3& w, float ax, float ay) {
    float at = Abs(TanT(w));
    if (std::isinf(at)) return 0.0f;
    float a = std::sqrt(Sq(CosP(w)) * ax * ax + Sq(SinP(w)) * ay * ay);
    float l = 0.5f * (-1.0f + std::sqrt(1.0f + Sq(a * at)));
    return 1.0f / (1.0f + l);
}
float G1Iso(const V3& w, float a) {
    float a2 = a * a, c = Abs(w.y);
    return 2.0f / (1.0f + std::sqrt(a2 + (1 - a2) * c * c));
}
float D(const V3& m, float ax, float ay) {
    return 1.0f / (kPi * ax * ay * Sq(Sq(m.x) / Sq(ax) + Sq(m.z) / Sq(ay) + m.y * m.y));
}
V3 SampleVndf(const V3& wo, float ax, float ay, float u1, float u2) {
    V3 v = Norm(V3(wo.x * ax, wo.y, wo.z * ay));
    V3 t1 = (v.y < 0.9999f) ? Norm(Cross(v, V3(0, 1, 0))) : V3(1, 0, 0);
    V3 t2 = Cross(t1, v);
    float a = 1.0f / (1.0f + v.y);
    float r = std::sqrt(u1);
    float phi = (u2 < a) ? (u2 / a) * kPi : kPi + (u2 - a) / (1.0f - a) * kPi;
    float p1 = r * std::cos(phi);
    float p2 = r * std::sin(phi) * ((u2 < a) ? 1.0f : v.y);
    V3 n = p1 * t1 + p2 * t2 + std::sqrt(std::fmax(0.0f, 1.0f - p1 * p1 - p2 * p2)) * v;
    return Norm(V3(ax * n.x, n.y, ay * n.z));
}
void VndfPdfs(const V3& wi, const V3& wm, const V3& wo, float ax, float ay, float& f, float& r) {
    float d = D(wm, ax, ay);
    f = G1(wo, ax, ay) * Abs(Dot(wm, wi)) * d / Abs(wi.y);
    r = G1(wi, ax, ay) * Abs(Dot(wm, wo)) * d / Abs(wo.y);
}

// FloatFuncs.h:348-366
V3 Reflect(V3 n, V3 l) { return 2.0f * Dot(n, l) * n - l; }
bool Transmit(V3 wm, V3 wi, float n, V3& wo) {
    float c = Dot(wi, wm);
    if (c < 0.0f) { c = -c; wm = -1.0f * wm; }
    float root = 1.0f - n * n * (1.0f - c * c);
    if (root <= 0) return false;
    wo = (n * c - std::sqrt(root)) * wm - n * wi;
    return true;
}

struct Lobes { float spec, diff, coat, trans; };
Lobes LobePdfs(const Surf& s) {  // Disney.cpp:25-44
    float mb = s.metallic, sb = (1.0f - s.metallic) * s.specTrans, db = (1.0f - s.specTrans) * (1.0f - s.metallic);
    float ws = mb + db, wt = sb, wd = db, wc = 1.0f * Sat(s.clearcoat);
    float nrm = 1.0f / (ws + wt + wd + wc);
    return {ws * nrm, wd * nrm, wc * nrm, wt * nrm};
}
float ThinRough(float ior, float r) { return Sat((0.65f * ior - 0.35f) * r); }
void Aniso(float r, float an, float& ax, float& ay) {
    float asp = std::sqrt(1.0f - 0.9f * an);
    ax = std::fmax(0.001f, Sq(r) / asp);
    ay = std::fmax(0.001f, Sq(r) * asp);
}
V3 Tint(V3 c) { float l = Dot(V3(0.3f, 0.6f, 1.0f), c); return l > 0.0f ? c * (1.0f / l) : V3(1.0f); }
float Gtr1(float h, float a) {
    if (a >= 1) return kInvPi;
    float a2 = a * a;
    return (a2 - 1.0f) / (kPi * std::log2(a2) * (1.0f + (a2 - 1.0f) * h * h));
}
V3 Sheen(const Surf& s, V3 wm, V3 wi) {
    if (s.sheen <= 0.0f) return V3(0.0f);
    return s.sheen * Lerp(V3(1.0f), Tint(s.baseColor), s.sheenTint) * SchlickW(Abs(Dot(wm, wi)));
}
V3 DFresnel(const Surf& s, V3 wo, V3 wm, V3 wi) {
    V3 r0 = R0(s.relativeIOR) * Lerp(V3(1.0f), Tint(s.baseColor), s.specularTint);
    r0 = Lerp(r0, s.baseColor, s.metallic);
    return Lerp(V3(Dielectric(Dot(wm, wo), 1.0f, s.ior)), SchlickC(r0, Dot(wi, wm)), s.metallic);
}
float Diffuse(const Surf& s, V3 wo, V3 wm, V3 wi, bool thin) {
    float nl = Abs(wi.y), nv = Abs(wo.y), fl = SchlickW(nl), fv = SchlickW(nv);
    float hk = 0.0f;
    if (thin && s.flatness > 0.0f) {
        float r = s.roughness * s.roughness, hl = Dot(wm, wi), f90 = hl * hl * r;
        float fss = Lerp(1.0f, f90, fl) * Lerp(1.0f, f90, fv);
        hk = 1.25f * (fss * (1.0f / (nl + nv) - 0.5f) + 0.5f);
    }
    float r = s.roughness * s.roughness, rr = 0.5f + 2.0f * nl * nl * r;
    float retro = rr * (fl + fv + fl * fv * (rr - 1.0f));
    float ssa = Lerp(1.0f, hk, thin ? s.flatness : 0.0f);
    return kInvPi * (retro + ssa * (1.0f - 0.5f * fl) * (1.0f - 0.5f * fv));
}
// Disney.cpp:337-343 with the reference's float / float3 operator (FloatFuncs.h:147-151), which divides
// the vector by the scalar: 1.0f / (s * d) evaluates to s * d.
V3 Extinction(V3 a, float d) {
    V3 s = V3(1.9f) - a + 3.5f * (a - V3(0.8f)) * (a - V3(0.8f));
    return (s * d) / V3(1.0f);
}
V3 Local(const Surf& s, V3 v) { return V3(Dot(v, s.t), Dot(v, s.n), Dot(v, s.b)); }
V3 World(const Surf& s, V3 w) { return w.x * s.t + w.y * s.n + w.z * s.b; }
void Clear(Sample& o) { o.fwd = o.rev = 0.0f; o.refl = V3(0.0f); o.wi = V3(0.0f); }

V3 EvalDisney(const Surf& s, V3 v, V3 l, bool thin, float& fwd, float& rev) {
    V3 wo = Norm(Local(s, v)), wi = Norm(Local(s, l)), wm = Norm(wo + wi);
    float nv = wo.y, nl = wi.y;
    V3 refl(0.0f);
    fwd = rev = 0.0f;
    Lobes p = LobePdfs(s);
    float ax, ay;
    Aniso(s.roughness, s.anisotropic, ax, ay);
    float wd = (1.0f - s.metallic) * (1.0f - s.specTrans), wt = (1.0f - s.metallic) * s.specTrans;
    bool up = nl > 0.0f && nv > 0.0f;
    if (up && s.clearcoat > 0.0f) {  // Disney.cpp:85-106
        float d = Gtr1(Abs(wm.y), Lerp(0.1f, 0.001f, s.clearcoatGloss));
        float f = SchlickS(0.04f, Dot(wm, wi));
        float c = 0.25f * s.clearcoat * d * f * G1Iso(wi, 0.25f) * G1Iso(wo, 0.25f);
        refl = refl + V3(c);
        fwd += p.coat * (d / (4.0f * Abs(Dot(wo, wm))));
        rev += p.coat * (d / (4.0f * Abs(Dot(wi, wm))));
    }
    if (wd > 0.0f) {
        float d = Diffuse(s, wo, wm, wi, thin);
        refl = refl + wd * (d * s.baseColor + Sheen(s, wm, wi));
        fwd += p.diff * Abs(wi.y);
        rev += p.diff * Abs(wo.y);
    }
    if (wt > 0.0f) {  // Disney.cpp:214-245, 585-601
        float rs = thin ? ThinRough(s.ior, s.roughness) : s.roughness;
        float tax, tay;
        Aniso(rs, s.anisotropic, tax, tay);
        float rel = s.relativeIOR, n2 = rel * rel;
        float hl = Dot(wm, wi), hv = Dot(wm, wo);
        float d = D(wm, tax, tay), gl = G1(wi, tax, tay), gv = G1(wo, tax, tay);
        float f = Dielectric(hv, 1.0f, s.ior);
        V3 col = thin ? Sqrt(s.baseColor) : s.baseColor;
        float c = (Abs(hl) * Abs(hv)) / (Abs(wi.y) * Abs(wo.y));
        float t = n2 / Sq(hl + rel * hv);
        refl = refl + wt * (col * (c * t * (1.0f - f) * gl * gv * d));
        float ft, rt;
        VndfPdfs(wi, wm, wo, tax, tay, ft, rt);
        fwd += p.trans * ft / Sq(hl + s.relativeIOR * hv);
        rev += p.trans * rt / Sq(hv + s.relativeIOR * hl);
    }
    if (up) {  // Disney.cpp:140-166
        float fm = 0, rm = 0;
        V3 sp(0.0f);
        if (nl > 0.0f && nv > 0.0f) {
            float d = D(wm, ax, ay), gl = G1(wi, ax, ay), gv = G1(wo, ax, ay);
            V3 F = DFresnel(s, wo, wm, wi);
            VndfPdfs(wi, wm, wo, ax, ay, fm, rm);
            fm *= (1.0f / (4 * Abs(Dot(wo, wm))));
            rm *= (1.0f / (4 * Abs(Dot(wi, wm))));
            sp = d * gl * gv * F * (1.0f / (4.0f * nl * nv));
        }
        refl = refl + sp;
        fwd += p.spec * fm / (4 * Abs(Dot(wo, wm)));
        rev += p.spec * rm / (4 * Abs(Dot(wi, wm)));
    }
    return refl * Abs(nl);
}

struct Uniforms {
    const float* u;
    int used;
    float next() { return u[used++]; }
};

bool SampBrdf(const Surf& s, V3 v, Uniforms& u, Sample& o) {  // Disney.cpp:169-211
    V3 wo = Norm(Local(s, v));
    float ax, ay;
    Aniso(s.roughness, s.anisotropic, ax, ay);
    float r0 = u.next(), r1 = u.next();
    V3 wm = SampleVndf(wo, ax, ay, r0, r1);
    V3 wi = Norm(Reflect(wm, wo));
    if (wi.y <= 0.0f) { Clear(o); return false; }
    o.flags = 1;
    o.refl = G1(wo, ax, ay) * DFresnel(s, wo, wm, wi);
    o.wi = Norm(World(s, wi));
    VndfPdfs(wi, wm, wo, ax, ay, o.fwd, o.rev);
    o.fwd *= (1.0f / (4 * Abs(Dot(wo, wm))));
    o.rev *= (1.0f / (4 * Abs(Dot(wi, wm))));
    return true;
}
bool SampCoat(const Surf& s, V3 v, Uniforms& u, Sample& o) {  // Disney.cpp:293-334
    V3 wo = Norm(Local(s, v));
    float a2 = 0.25f * 0.25f;
    float r0 = u.next(), r1 = u.next();
    float ct = std::sqrt(std::fmax(0.0f, (1.0f - std::pow(a2, 1.0f - r0)) / (1.0f - a2)));
    float st = std::sqrt(std::fmax(0.0f, 1.0f - ct * ct));
    float phi = 2.0f * kPi * r1;
    V3 wm(st * std::cos(phi), ct, st * std::sin(phi));
    if (Dot(wm, wo) < 0.0f) wm = -1.0f * wm;
    V3 wi = Reflect(wm, wo);
    if (Dot(wi, wo) < 0.0f) return false;
    float d = Gtr1(Abs(wm.y), Lerp(0.1f, 0.001f, s.clearcoatGloss));
    float f = SchlickS(0.04f, Dot(wm, wi));
    float g = G1Iso(wi, 0.25f) * G1Iso(wo, 0.25f);
    float fp = d / (4.0f * Dot(wo, wm));
    o.refl = V3(0.25f * s.clearcoat * g * f * d) / V3(fp);
    o.wi = Norm(World(s, wi));
    o.fwd = fp;
    o.rev = d / (4.0f * Dot(wi, wm));
    return true;
}
bool SampTrans(const Surf& s, V3 v, bool thin, Uniforms& u, Sample& o) {  // Disney.cpp:346-448
    V3 wo = Local(s, v);
    if (wo.y == 0.0) { Clear(o); return false; }
    float rs = thin ? ThinRough(s.ior, s.roughness) : s.roughness;
    float tax, tay;
    Aniso(rs, s.anisotropic, tax, tay);
    float r0 = u.next(), r1 = u.next();
    V3 wm = SampleVndf(wo, tax, tay, r0, r1);
    float vh = Dot(wo, wm);
    if (wm.y < 0.0f) vh = -vh;
    float ni = wo.y > 0.0f ? 1.0f : s.ior, nt = wo.y > 0.0f ? s.ior : 1.0f;
    float F = Dielectric(vh, 1.0f, s.ior);
    float g1v = G1(wo, tax, tay);
    float pdf;
    V3 wi;
    if (u.next() <= F) {
        wi = Norm(Reflect(wm, wo));
        o.flags = 1;
        o.refl = g1v * s.baseColor;
        pdf = F / (4 * Abs(Dot(wo, wm)));
    } else {
        if (thin) {
            wi = Reflect(wm, wo);
            wi.y = -wi.y;
            o.refl = g1v * Sqrt(s.baseColor);
            o.flags = 1;
        } else {
            if (Transmit(wm, wo, ni / nt, wi)) {
                o.flags = 2;
                o.phase = vh > 0.0f ? 1 : 0;
                o.ext = Extinction(s.transmittanceColor, s.scatterDistance);
            } else {
                o.flags = 1;
                wi = Reflect(wm, wo);
            }
            o.refl = g1v * s.baseColor;
        }
        wi = Norm(wi);
        float lh = Abs(Dot(wi, wm));
        pdf = (1.0f - F) / (lh / Sq(lh + s.relativeIOR * vh));
    }
    if (wi.y == 0.0f) { Clear(o); return false; }
    if (s.roughness < 0.01f) o.flags |= 4;
    VndfPdfs(wi, wm, wo, tax, tay, o.fwd, o.rev);
    o.fwd *= pdf;
    o.rev *= pdf;
    o.wi = Norm(World(s, wi));
    return true;
}
bool SampDiff(const Surf& s, V3 v, bool thin, Uniforms& u, Sample& o) {  // Disney.cpp:461-518
    V3 wo = Local(s, v);
    float sign = wo.y < 0.0f ? -1.0f : (wo.y > 0.0f ? 1.0f : 0.0f);
    float r0 = u.next(), r1 = u.next();
    float r = std::sqrt(r0), th = 2.0f * kPi * r1;
    V3 wi = sign * V3(r * std::cos(th), std::sqrt(std::fmax(0.0f, 1 - r0)), r * std::sin(th));
    V3 wm = Norm(wi + wo);
    float nl = wi.y;
    if (nl == 0.0f) { Clear(o); return false; }
    float nv = wo.y, pdf;
    unsigned ev = 1;
    V3 col = s.baseColor;
    if (u.next() <= s.diffTrans) {
        wi = -1.0f * wi;
        pdf = s.diffTrans;
        if (thin) {
            col = Sqrt(col);
        } else {
            ev = 2;
            o.phase = 1;
            o.ext = Extinction(s.transmittanceColor, s.scatterDistance);
        }
    } else {
        pdf = 1.0f - s.diffTrans;
    }
    V3 sh = Sheen(s, wm, wi);
    float d = Diffuse(s, wo, wm, wi, thin);
    o.refl = sh + col * (d / pdf);
    o.wi = Norm(World(s, wi));
    o.fwd = Abs(nl) * pdf;
    o.rev = Abs(nv) * pdf;
    o.flags = ev;
    return true;
}
bool SampDisney(const Surf& s, V3 v, bool thin, Uniforms& u, Sample& o) {
    Lobes p = LobePdfs(s);
    float x = u.next();
    bool ok;
    float pl;
    if (x <= p.spec) { ok = SampBrdf(s, v, u, o); pl = p.spec; }
    else if (x <= p.spec + p.coat) { ok = SampCoat(s, v, u, o); pl = p.coat; }
    else if (x <= p.spec + p.coat + p.diff) { ok = SampDiff(s, v, thin, u, o); pl = p.diff; }
    else { ok = SampTrans(s, v, thin, u, o); pl = p.trans; }
    if (pl > 0.0f) {
        o.refl = o.refl * (1.0f / pl);
        o.fwd *= pl;
        o.rev *= pl;
    }
    return ok;
}
bool SampDirac(const Surf& s, V3 v, Uniforms& u, Sample& o) {  // DiracTransparent.cpp:20-68
    V3 n = s.n;
    float vh = Dot(v, n);
    float ni = vh > 0.0f ? 1.0f : s.ior, nt = vh > 0.0f ? s.ior : 1.0f;
    float F = Dielectric(vh, ni, nt), pdf;
    V3 wi;
    if (u.next() < F) {
        wi = Norm(Reflect(n, v));
        o.flags = 1;
        pdf = F;
    } else {
        if (Transmit(n, v, ni / nt, wi)) o.flags = 2;
        else { wi = Reflect(n, v); o.flags = 1; }
        wi = Norm(wi);
        pdf = 1.0f - F;
    }
    o.flags |= 4;
    o.refl = s.baseColor / V3(pdf);
    o.wi = wi;
    o.fwd = o.rev = pdf;
    return true;
}

}  // namespace

Surf surf_from_record(const float* r) {
    Surf s;
    s.t = V3(r[0], r[1], r[2]);
    s.n = V3(r[3], r[4], r[5]);
    s.b = V3(r[6], r[7], r[8]);
    s.baseColor = V3(r[9], r[10], r[11]);
    s.transmittanceColor = V3(r[12], r[13], r[14]);
    s.sheen = r[15]; s.sheenTint = r[16]; s.clearcoat = r[17]; s.clearcoatGloss = r[18];
    s.metallic = r[19]; s.specTrans = r[20]; s.diffTrans = r[21]; s.flatness = r[22];
    s.anisotropic = r[23]; s.relativeIOR = r[24]; s.specularTint = r[25]; s.roughness = r[26];
    s.scatterDistance = r[27]; s.ior = r[28];
    int32_t sh;
    std::memcpy(&sh, &r[29], 4);
    s.shader = sh;
    return s;
}

// Test switch: a BSDF whose sampling weights are exactly f * cos / density (opaque Lambert with albedo
// baseColor, cosine sampling, pdf cos / pi).  The reference Disney model is not of that kind (its diffuse
// sample weight is baseColor * f_d and its diffuse pdf is |cos| rather than |cos| / pi, Disney.cpp:466-519),
// so different estimators of the same path converge to different images on it; the integrators' estimator
// bookkeeping is checked on this one, where every unbiased estimator converges to the same image.
std::atomic<int> g_consistent_lambert{0};

static V3 EvalLambert(const Surf& s, V3 v, V3 l, float& fwd, float& rev) {
    const float cl = Dot(s.n, l), cv = Dot(s.n, v);
    if (cl * cv <= 0.0f) return V3(0.0f);
    fwd = std::fabs(cl) * float(1.0 / M_PI);
    rev = std::fabs(cv) * float(1.0 / M_PI);
    return s.baseColor * fwd;
}

static bool SampLambert(const Surf& s, V3 v, Uniforms& un, Sample& o) {
    const float r0 = un.next(), r1 = un.next();
    const float r = std::sqrt(r0), ph = float(2.0 * M_PI) * r1, ct = std::sqrt(std::max(0.0f, 1.0f - r0));
    const float side = Dot(s.n, v) < 0.0f ? -1.0f : 1.0f;
    o.wi = Norm(r * std::cos(ph) * s.t + (side * ct) * s.n + r * std::sin(ph) * s.b);
    if (!(ct > 0.0f)) return false;
    o.refl = s.baseColor;
    o.fwd = ct * float(1.0 / M_PI);
    o.rev = std::fabs(Dot(s.n, v)) * float(1.0 / M_PI);
    o.flags = 1;
    return true;
}

V3 bsdf_evaluate(const Surf& s, V3 v, V3 l, float& fwd, float& rev) {
    fwd = rev = 0.0f;
    if (g_consistent_lambert.load(std::memory_order_relaxed) && s.shader != 2) return EvalLambert(s, v, l, fwd, rev);
    if (s.shader == 0) return EvalDisney(s, v, l, true, fwd, rev);
    if (s.shader == 1) return EvalDisney(s, v, l, false, fwd, rev);
    return V3(0.0f);
}

bool bsdf_sample(const Surf& s, V3 v, const float* u, int& used, Sample& o) {
    o = Sample();
    Uniforms un{u, used};
    bool ok = false;
    if (g_consistent_lambert.load(std::memory_order_relaxed) && s.shader != 2) ok = SampLambert(s, v, un, o);
    else if (s.shader == 0) ok = SampDisney(s, v, true, un, o);
    else if (s.shader == 1) ok = SampDisney(s, v, false, un, o);
    else if (s.shader == 2) ok = SampDirac(s, v, un, o);
    used = un.used;
    return ok;
}

}  // namespace orc

extern "C" {

void oracle_set_consistent_lambert(int on) { orc::g_consistent_lambert.store(on); }

// surf: 32-word SelSurface records (shader as int32 bits); out as sel_bsdf_evaluate_device.
void oracle_bsdf_evaluate(const float* surf, const float* wo, const float* wi, int64_t n, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        const orc::Surf s = orc::surf_from_record(surf + 32 * i);
        float f, r;
        const orc::V3 e = orc::bsdf_evaluate(s, orc::V3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]),
                                             orc::V3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]), f, r);
        float* o = out + 5 * i;
        o[0] = e.x; o[1] = e.y; o[2] = e.z; o[3] = f; o[4] = r;
    }
}

void oracle_bsdf_sample(const float* surf, const float* wo, const float* u, int64_t n, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        const orc::Surf s = orc::surf_from_record(surf + 32 * i);
        orc::Sample bs;
        int used = 0;
        const bool ok = orc::bsdf_sample(s, orc::V3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), u + 4 * i, used, bs);
        float* o = out + 16 * i;
        o[0] = ok ? 1.0f : 0.0f;
        o[1] = float(bs.flags);
        o[2] = bs.refl.x; o[3] = bs.refl.y; o[4] = bs.refl.z;
        o[5] = bs.wi.x; o[6] = bs.wi.y; o[7] = bs.wi.z;
        o[8] = bs.fwd; o[9] = bs.rev;
        o[10] = float(bs.phase);
        o[11] = bs.ext.x; o[12] = bs.ext.y; o[13] = bs.ext.z;
        o[14] = float(used);
        o[15] = 0.0f;
    }
}

}  // extern "C"
