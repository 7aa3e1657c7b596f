// Disney BSDF (thin and solid), GGX with visible-normal sampling, dielectric Fresnel and the Dirac
// transparent shader, as device functions.
//
// Restates the reference's shading math (Source/Core/Shading/Disney.cpp, Ggx.cpp, Fresnel.cpp,
// DiracTransparent.cpp, SurfaceScattering.cpp) formula for formula, including its particular choices,
// so that f and the pdfs agree with it to FP32 rounding:
//   * the tint luminance uses weights (0.3, 0.6, 1.0) (Disney.cpp:64-70);
//   * the scalar Schlick term is Lerp(1, SchlickWeight(cos), r0) (Fresnel.cpp:26-29);
//   * the lobe after diffuse is always specular transmission (Disney.cpp:639-642);
//   * spec-transmission and diffuse sampling do not renormalise the tangent-space view vector
//     (Disney.cpp:349, 464) while the other paths do;
//   * the medium extinction is s * scatterDistance (see extinction() below).
// Tangent space is y-up: (t, n, b) = (x, y, z) (MathLib/Trigonometric.h:49-108).
#pragma once

#include "vecmath.cuh"

namespace sel {

enum ShaderKind : int { kDisneyThin = 0, kDisneySolid = 1, kDiracTransparent = 2 };
enum EventFlags : unsigned { kScatterEvent = 1u, kTransmissionEvent = 2u, kDiracEvent = 4u };

// A shading point: world-space frame rows and the Disney parameters in the units SurfaceParameters
// holds them (baseColor linear, diffTrans already halved) -- layout of SelSurface.
struct Surface {
    float3 t, n, b;
    float3 base_color;
    float3 transmittance_color;
    float sheen, sheen_tint, clearcoat, clearcoat_gloss;
    float metallic, spec_trans, diff_trans, flatness;
    float anisotropic, relative_ior, specular_tint, roughness;
    float scatter_distance, ior;
    int shader;
};

struct BsdfSampleOut {
    unsigned flags;
    int medium_phase;  // 0 vacuum, 1 isotropic
    float3 extinction;
    float3 reflectance;
    float3 wi;
    float forward_pdf, reverse_pdf;
};

namespace disney {

SEL_HD float3 to_local(const Surface& s, float3 v) { return f3(dot(v, s.t), dot(v, s.n), dot(v, s.b)); }
SEL_HD float3 to_world(const Surface& s, float3 w) { return w.x * s.t + w.y * s.n + w.z * s.b; }

// y-up trigonometry (Trigonometric.h:51-108)
SEL_HD float cos2_theta(float3 w) { return w.y * w.y; }
SEL_HD float sin_theta(float3 w) { return sqrtf(fmaxf(0.0f, 1.0f - cos2_theta(w))); }
SEL_HD float tan_theta(float3 w) { return sin_theta(w) / w.y; }
SEL_HD float cos_phi(float3 w) { float s = sin_theta(w); return s == 0.0f ? 1.0f : clampf(w.x / s, -1.0f, 1.0f); }
SEL_HD float sin_phi(float3 w) { float s = sin_theta(w); return s == 0.0f ? 1.0f : clampf(w.z / s, -1.0f, 1.0f); }

// Fresnel.cpp:19-84
SEL_HD float schlick_weight(float u) {
    const float m = saturate(1.0f - u);
    const float m2 = m * m;
    return m * m2 * m2;
}
SEL_HD float schlick_scalar(float r0, float c) { return lerpf(1.0f, schlick_weight(c), r0); }
SEL_HD float3 schlick_color(float3 r0, float c) {
    const float e = powf(1.0f - c, 5.0f);
    return r0 + (f3(1.0f) - r0) * e;
}
SEL_HD float schlick_r0(float eta) { return sqr(eta - 1.0f) / sqr(eta + 1.0f); }
SEL_HD float dielectric(float cos_i, float ni, float nt) {
    cos_i = clampf(cos_i, -1.0f, 1.0f);
    if (cos_i < 0.0f) {
        const float tmp = ni;
        ni = nt;
        nt = tmp;
        cos_i = -cos_i;
    }
    const float sin_i = sqrtf(fmaxf(0.0f, 1.0f - cos_i * cos_i));
    const float sin_t = ni / nt * sin_i;
    if (sin_t >= 1.0f) return 1.0f;
    const float cos_t = sqrtf(fmaxf(0.0f, 1.0f - sin_t * sin_t));
    const float r_par = ((nt * cos_i) - (ni * cos_t)) / ((nt * cos_i) + (ni * cos_t));
    const float r_perp = ((ni * cos_i) - (nt * cos_t)) / ((ni * cos_i) + (nt * cos_t));
    return (r_par * r_par + r_perp * r_perp) / 2.0f;
}

// Ggx.cpp:19-46, 73-83
SEL_HD float smith_g1(float3 w, float ax, float ay) {
    const float abs_tan = fabsf(tan_theta(w));
    if (isinf(abs_tan)) return 0.0f;
    const float cp = cos_phi(w), sp = sin_phi(w);
    const float a = sqrtf(cp * cp * ax * ax + sp * sp * ay * ay);
    const float a2t2 = sqr(a * abs_tan);
    const float lambda = 0.5f * (-1.0f + sqrtf(1.0f + a2t2));
    return 1.0f / (1.0f + lambda);
}
SEL_HD float smith_g1_iso(float3 w, float a) {
    const float a2 = a * a;
    const float c = fabsf(w.y);
    return 2.0f / (1.0f + sqrtf(a2 + (1.0f - a2) * c * c));
}
SEL_HD float ggx_d(float3 wm, float ax, float ay) {
    const float hx2 = sqr(wm.x), hy2 = sqr(wm.z), c2 = cos2_theta(wm);
    const float ax2 = sqr(ax), ay2 = sqr(ay);
    return 1.0f / (kPi * ax * ay * sqr(hx2 / ax2 + hy2 / ay2 + c2));
}
// Heitz 2018 visible-normal sampling (Ggx.cpp:105-128)
SEL_HD float3 sample_vndf(float3 wo, float ax, float ay, float u1, float u2) {
    const float3 v = normalize(f3(wo.x * ax, wo.y, wo.z * ay));
    const float3 t1 = (v.y < 0.9999f) ? normalize(cross(v, f3(0.0f, 1.0f, 0.0f))) : f3(1.0f, 0.0f, 0.0f);
    const float3 t2 = cross(t1, v);
    const float a = 1.0f / (1.0f + v.y);
    const float r = sqrtf(u1);
    const float phi = (u2 < a) ? (u2 / a) * kPi : kPi + (u2 - a) / (1.0f - a) * kPi;
    const float p1 = r * cosf(phi);
    const float p2 = r * sinf(phi) * ((u2 < a) ? 1.0f : v.y);
    const float3 n = p1 * t1 + p2 * t2 + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * v;
    return normalize(f3(ax * n.x, n.y, ay * n.z));
}
// forward and reverse visible-normal pdfs (Ggx.cpp:143-156)
SEL_HD void vndf_pdfs(float3 wi, float3 wm, float3 wo, float ax, float ay, float& fwd, float& rev) {
    const float d = ggx_d(wm, ax, ay);
    fwd = smith_g1(wo, ax, ay) * fabsf(dot(wm, wi)) * d / fabsf(wi.y);
    rev = smith_g1(wi, ax, ay) * fabsf(dot(wm, wo)) * d / fabsf(wo.y);
}

SEL_HD float3 reflect(float3 n, float3 l) { return 2.0f * dot(n, l) * n - l; }
SEL_HD bool transmit(float3 wm, float3 wi, float n, float3& wo) {
    float c = dot(wi, wm);
    if (c < 0.0f) {
        c = -c;
        wm = -wm;
    }
    const float root = 1.0f - n * n * (1.0f - c * c);
    if (root <= 0.0f) return false;
    wo = (n * c - sqrtf(root)) * wm - n * wi;
    return true;
}

// Disney.cpp:25-44
SEL_HD void lobe_pdfs(const Surface& s, float& p_spec, float& p_diff, float& p_coat, float& p_trans) {
    const float metallic_brdf = s.metallic;
    const float specular_bsdf = (1.0f - s.metallic) * s.spec_trans;
    const float dielectric_brdf = (1.0f - s.spec_trans) * (1.0f - s.metallic);
    const float w_spec = metallic_brdf + dielectric_brdf;
    const float w_trans = specular_bsdf;
    const float w_diff = dielectric_brdf;
    const float w_coat = 1.0f * saturate(s.clearcoat);
    const float norm = 1.0f / (w_spec + w_trans + w_diff + w_coat);
    p_spec = w_spec * norm;
    p_trans = w_trans * norm;
    p_diff = w_diff * norm;
    p_coat = w_coat * norm;
}
SEL_HD float thin_roughness(float ior, float r) { return saturate((0.65f * ior - 0.35f) * r); }
SEL_HD void aniso(float r, float anisotropic, float& ax, float& ay) {
    const float aspect = sqrtf(1.0f - 0.9f * anisotropic);
    ax = fmaxf(0.001f, sqr(r) / aspect);
    ay = fmaxf(0.001f, sqr(r) * aspect);
}
SEL_HD float3 tint(float3 c) {
    const float lum = dot(f3(0.3f, 0.6f, 1.0f), c);
    return lum > 0.0f ? c * (1.0f / lum) : f3(1.0f);
}
SEL_HD float gtr1(float abs_h, float a) {
    if (a >= 1.0f) return kInvPi;
    const float a2 = a * a;
    return (a2 - 1.0f) / (kPi * log2f(a2) * (1.0f + (a2 - 1.0f) * abs_h * abs_h));
}
SEL_HD float clearcoat_eval(float coat, float alpha, float3 wo, float3 wm, float3 wi, float& fpdf, float& rpdf) {
    if (coat <= 0.0f) return 0.0f;
    const float abs_nh = fabsf(wm.y);
    const float hl = dot(wm, wi);
    const float d = gtr1(abs_nh, lerpf(0.1f, 0.001f, alpha));
    const float f = schlick_scalar(0.04f, hl);
    const float gl = smith_g1_iso(wi, 0.25f);
    const float gv = smith_g1_iso(wo, 0.25f);
    fpdf = d / (4.0f * fabsf(dot(wo, wm)));
    rpdf = d / (4.0f * fabsf(dot(wi, wm)));
    return 0.25f * coat * d * f * gl * gv;
}
SEL_HD float3 sheen_eval(const Surface& s, float3 wm, float3 wi) {
    if (s.sheen <= 0.0f) return f3(0.0f);
    const float hl = fabsf(dot(wm, wi));
    return s.sheen * lerp3(f3(1.0f), tint(s.base_color), s.sheen_tint) * schlick_weight(hl);
}
SEL_HD float3 disney_fresnel(const Surface& s, float3 wo, float3 wm, float3 wi) {
    const float hv = dot(wm, wo);
    float3 r0 = schlick_r0(s.relative_ior) * lerp3(f3(1.0f), tint(s.base_color), s.specular_tint);
    r0 = lerp3(r0, s.base_color, s.metallic);
    const float fd = dielectric(hv, 1.0f, s.ior);
    const float3 fm = schlick_color(r0, dot(wi, wm));
    return lerp3(f3(fd), fm, s.metallic);
}
SEL_HD float3 brdf_eval(const Surface& s, float3 wo, float3 wm, float3 wi, float& fpdf, float& rpdf) {
    fpdf = 0.0f;
    rpdf = 0.0f;
    const float nl = wi.y, nv = wo.y;
    if (nl <= 0.0f || nv <= 0.0f) return f3(0.0f);
    float ax, ay;
    aniso(s.roughness, s.anisotropic, ax, ay);
    const float d = ggx_d(wm, ax, ay);
    const float gl = smith_g1(wi, ax, ay);
    const float gv = smith_g1(wo, ax, ay);
    const float3 f = disney_fresnel(s, wo, wm, wi);
    vndf_pdfs(wi, wm, wo, ax, ay, fpdf, rpdf);
    fpdf *= (1.0f / (4.0f * fabsf(dot(wo, wm))));
    rpdf *= (1.0f / (4.0f * fabsf(dot(wi, wm))));
    return d * gl * gv * f * (1.0f / (4.0f * nl * nv));
}
SEL_HD float3 spec_trans_eval(const Surface& s, float3 wo, float3 wm, float3 wi, float ax, float ay, bool thin) {
    const float rel = s.relative_ior;
    const float n2 = rel * rel;
    const float abs_nl = fabsf(wi.y), abs_nv = fabsf(wo.y);
    const float hl = dot(wm, wi), hv = dot(wm, wo);
    const float abs_hl = fabsf(hl), abs_hv = fabsf(hv);
    const float d = ggx_d(wm, ax, ay);
    const float gl = smith_g1(wi, ax, ay);
    const float gv = smith_g1(wo, ax, ay);
    const float f = dielectric(hv, 1.0f, s.ior);
    const float3 color = thin ? sqrt3(s.base_color) : s.base_color;
    const float c = (abs_hl * abs_hv) / (abs_nl * abs_nv);
    const float t = n2 / sqr(hl + rel * hv);
    return color * (c * t * (1.0f - f) * gl * gv * d);
}
SEL_HD float retro_diffuse(const Surface& s, float3 wo, float3 wi) {
    const float nl = fabsf(wi.y), nv = fabsf(wo.y);
    const float r = s.roughness * s.roughness;
    const float rr = 0.5f + 2.0f * nl * nl * r;
    const float fl = schlick_weight(nl), fv = schlick_weight(nv);
    return rr * (fl + fv + fl * fv * (rr - 1.0f));
}
SEL_HD float diffuse_eval(const Surface& s, float3 wo, float3 wm, float3 wi, bool thin) {
    const float nl = fabsf(wi.y), nv = fabsf(wo.y);
    const float fl = schlick_weight(nl), fv = schlick_weight(nv);
    float hk = 0.0f;
    if (thin && s.flatness > 0.0f) {
        const float r = s.roughness * s.roughness;
        const float hl = dot(wm, wi);
        const float fss90 = hl * hl * r;
        const float fss = lerpf(1.0f, fss90, fl) * lerpf(1.0f, fss90, fv);
        hk = 1.25f * (fss * (1.0f / (nl + nv) - 0.5f) + 0.5f);
    }
    const float retro = retro_diffuse(s, wo, wi);
    const float ss = lerpf(1.0f, hk, thin ? s.flatness : 0.0f);
    return kInvPi * (retro + ss * (1.0f - 0.5f * fl) * (1.0f - 0.5f * fv));
}
// CalculateExtinction (Disney.cpp:337-343) writes 1.0f / (s * d), but the reference's operator/(float,
// float3) returns rhs / lhs (MathLib/FloatFuncs.h:147-151), so the value it produces is s * d.
SEL_HD float3 extinction(float3 a, float dist) {
    const float3 s = f3(1.9f) - a + 3.5f * (a - f3(0.8f)) * (a - f3(0.8f));
    return s * dist;
}

// EvaluateDisney (Disney.cpp:525-614); v = toward the viewer, l = toward the light, world space.
SEL_HD float3 evaluate(const Surface& s, float3 v, float3 l, bool thin, float& fwd, float& rev) {
    const float3 wo = normalize(to_local(s, v));
    const float3 wi = normalize(to_local(s, l));
    const float3 wm = normalize(wo + wi);
    const float nv = wo.y, nl = wi.y;
    float3 refl = f3(0.0f);
    fwd = 0.0f;
    rev = 0.0f;
    float p_brdf, p_diff, p_coat, p_trans;
    lobe_pdfs(s, p_brdf, p_diff, p_coat, p_trans);
    float ax, ay;
    aniso(s.roughness, s.anisotropic, ax, ay);
    const float w_diff = (1.0f - s.metallic) * (1.0f - s.spec_trans);
    const float w_trans = (1.0f - s.metallic) * s.spec_trans;
    const bool upper = nl > 0.0f && nv > 0.0f;
    if (upper && s.clearcoat > 0.0f) {
        float fc, rc;
        const float c = clearcoat_eval(s.clearcoat, s.clearcoat_gloss, wo, wm, wi, fc, rc);
        refl += f3(c);
        fwd += p_coat * fc;
        rev += p_coat * rc;
    }
    if (w_diff > 0.0f) {
        const float fd = fabsf(wi.y), rd = fabsf(wo.y);
        const float d = diffuse_eval(s, wo, wm, wi, thin);
        const float3 sh = sheen_eval(s, wm, wi);
        refl += w_diff * (d * s.base_color + sh);
        fwd += p_diff * fd;
        rev += p_diff * rd;
    }
    if (w_trans > 0.0f) {
        const float rs = thin ? thin_roughness(s.ior, s.roughness) : s.roughness;
        float tax, tay;
        aniso(rs, s.anisotropic, tax, tay);
        const float3 tr = spec_trans_eval(s, wo, wm, wi, tax, tay, thin);
        refl += w_trans * tr;
        float ft, rt;
        vndf_pdfs(wi, wm, wo, tax, tay, ft, rt);
        const float lh = dot(wm, wi), vh = dot(wm, wo);
        fwd += p_trans * ft / sqr(lh + s.relative_ior * vh);
        rev += p_trans * rt / sqr(vh + s.relative_ior * lh);
    }
    if (upper) {
        float fm, rm;
        const float3 sp = brdf_eval(s, wo, wm, wi, fm, rm);
        refl += sp;
        fwd += p_brdf * fm / (4.0f * fabsf(dot(wo, wm)));
        rev += p_brdf * rm / (4.0f * fabsf(dot(wi, wm)));
    }
    return refl * fabsf(nl);
}

SEL_HD void clear_sample(BsdfSampleOut& o) {
    o.forward_pdf = 0.0f;
    o.reverse_pdf = 0.0f;
    o.reflectance = f3(0.0f);
    o.wi = f3(0.0f);
}

// Each sampler below draws its uniforms from u[] in the order the reference draws them.
SEL_HD bool sample_brdf(const Surface& s, float3 v, const float* u, int& used, BsdfSampleOut& o) {
    const float3 wo = normalize(to_local(s, v));
    float ax, ay;
    aniso(s.roughness, s.anisotropic, ax, ay);
    const float r0 = u[used++], r1 = u[used++];
    const float3 wm = sample_vndf(wo, ax, ay, r0, r1);
    const float3 wi = normalize(reflect(wm, wo));
    if (wi.y <= 0.0f) {
        clear_sample(o);
        return false;
    }
    const float3 F = disney_fresnel(s, wo, wm, wi);
    const float g1v = smith_g1(wo, ax, ay);
    o.flags = kScatterEvent;
    o.reflectance = g1v * F;
    o.wi = normalize(to_world(s, wi));
    vndf_pdfs(wi, wm, wo, ax, ay, o.forward_pdf, o.reverse_pdf);
    o.forward_pdf *= (1.0f / (4.0f * fabsf(dot(wo, wm))));
    o.reverse_pdf *= (1.0f / (4.0f * fabsf(dot(wi, wm))));
    return true;
}

SEL_HD bool sample_clearcoat(const Surface& s, float3 v, const float* u, int& used, BsdfSampleOut& o) {
    const float3 wo = normalize(to_local(s, v));
    const float a = 0.25f, a2 = a * a;
    const float r0 = u[used++], r1 = u[used++];
    const float ct = sqrtf(fmaxf(0.0f, (1.0f - powf(a2, 1.0f - r0)) / (1.0f - a2)));
    const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    const float phi = kTwoPi * r1;
    float3 wm = f3(st * cosf(phi), ct, st * sinf(phi));
    if (dot(wm, wo) < 0.0f) wm = -wm;
    const float3 wi = reflect(wm, wo);
    if (dot(wi, wo) < 0.0f) return false;
    const float nh = wm.y, lh = dot(wm, wi);
    const float d = gtr1(fabsf(nh), lerpf(0.1f, 0.001f, s.clearcoat_gloss));
    const float f = schlick_scalar(0.04f, lh);
    const float g = smith_g1_iso(wi, 0.25f) * smith_g1_iso(wo, 0.25f);
    const float fpdf = d / (4.0f * dot(wo, wm));
    o.reflectance = f3(0.25f * s.clearcoat * g * f * d) / f3(fpdf);
    o.wi = normalize(to_world(s, wi));
    o.forward_pdf = fpdf;
    o.reverse_pdf = d / (4.0f * dot(wi, wm));
    return true;
}

SEL_HD bool sample_spec_trans(const Surface& s, float3 v, bool thin, const float* u, int& used, BsdfSampleOut& o) {
    const float3 wo = to_local(s, v);
    if (wo.y == 0.0f) {
        clear_sample(o);
        return false;
    }
    const float rs = thin ? thin_roughness(s.ior, s.roughness) : s.roughness;
    float tax, tay;
    aniso(rs, s.anisotropic, tax, tay);
    const float r0 = u[used++], r1 = u[used++];
    const float3 wm = sample_vndf(wo, tax, tay, r0, r1);
    float vh = dot(wo, wm);
    if (wm.y < 0.0f) vh = -vh;
    const float ni = wo.y > 0.0f ? 1.0f : s.ior;
    const float nt = wo.y > 0.0f ? s.ior : 1.0f;
    const float rel = ni / nt;
    const float F = dielectric(vh, 1.0f, s.ior);
    const float g1v = smith_g1(wo, tax, tay);
    float pdf;
    float3 wi;
    if (u[used++] <= F) {
        wi = normalize(reflect(wm, wo));
        o.flags = kScatterEvent;
        o.reflectance = g1v * s.base_color;
        pdf = F / (4.0f * fabsf(dot(wo, wm)));
    } else {
        if (thin) {
            wi = reflect(wm, wo);
            wi.y = -wi.y;
            o.reflectance = g1v * sqrt3(s.base_color);
            o.flags = kScatterEvent;
        } else {
            if (transmit(wm, wo, rel, wi)) {
                o.flags = kTransmissionEvent;
                o.medium_phase = vh > 0.0f ? 1 : 0;
                o.extinction = extinction(s.transmittance_color, s.scatter_distance);
            } else {
                o.flags = kScatterEvent;
                wi = reflect(wm, wo);
            }
            o.reflectance = g1v * s.base_color;
        }
        wi = normalize(wi);
        const float lh = fabsf(dot(wi, wm));
        const float jac = lh / sqr(lh + s.relative_ior * vh);
        pdf = (1.0f - F) / jac;
    }
    if (wi.y == 0.0f) {
        clear_sample(o);
        return false;
    }
    if (s.roughness < 0.01f) o.flags |= kDiracEvent;
    vndf_pdfs(wi, wm, wo, tax, tay, o.forward_pdf, o.reverse_pdf);
    o.forward_pdf *= pdf;
    o.reverse_pdf *= pdf;
    o.wi = normalize(to_world(s, wi));
    return true;
}

SEL_HD bool sample_diffuse(const Surface& s, float3 v, bool thin, const float* u, int& used, BsdfSampleOut& o) {
    const float3 wo = to_local(s, v);
    const float sign = wo.y > 0.0f ? 1.0f : (wo.y < 0.0f ? -1.0f : 0.0f);
    const float r0 = u[used++], r1 = u[used++];
    const float rr = sqrtf(r0);
    const float th = kTwoPi * r1;
    float3 wi = sign * f3(rr * cosf(th), sqrtf(fmaxf(0.0f, 1.0f - r0)), rr * sinf(th));
    const float3 wm = normalize(wi + wo);
    const float nl = wi.y;
    if (nl == 0.0f) {
        clear_sample(o);
        return false;
    }
    const float nv = wo.y;
    float pdf;
    unsigned ev = kScatterEvent;
    float3 color = s.base_color;
    if (u[used++] <= s.diff_trans) {
        wi = -wi;
        pdf = s.diff_trans;
        if (thin) {
            color = sqrt3(color);
        } else {
            ev = kTransmissionEvent;
            o.medium_phase = 1;
            o.extinction = extinction(s.transmittance_color, s.scatter_distance);
        }
    } else {
        pdf = 1.0f - s.diff_trans;
    }
    const float3 sh = sheen_eval(s, wm, wi);
    const float d = diffuse_eval(s, wo, wm, wi, thin);
    o.reflectance = sh + color * (d / pdf);
    o.wi = normalize(to_world(s, wi));
    o.forward_pdf = fabsf(nl) * pdf;
    o.reverse_pdf = fabsf(nv) * pdf;
    o.flags = ev;
    return true;
}

// SampleDisney (Disney.cpp:617-659)
SEL_HD bool sample(const Surface& s, float3 v, bool thin, const float* u, int& used, BsdfSampleOut& o) {
    float p_spec, p_diff, p_coat, p_trans;
    lobe_pdfs(s, p_spec, p_diff, p_coat, p_trans);
    bool ok;
    float p_lobe;
    const float p = u[used++];
    if (p <= p_spec) {
        ok = sample_brdf(s, v, u, used, o);
        p_lobe = p_spec;
    } else if (p <= p_spec + p_coat) {
        ok = sample_clearcoat(s, v, u, used, o);
        p_lobe = p_coat;
    } else if (p <= p_spec + p_coat + p_diff) {
        ok = sample_diffuse(s, v, thin, u, used, o);
        p_lobe = p_diff;
    } else {
        ok = sample_spec_trans(s, v, thin, u, used, o);
        p_lobe = p_trans;
    }
    if (p_lobe > 0.0f) {
        o.reflectance = o.reflectance * (1.0f / p_lobe);
        o.forward_pdf *= p_lobe;
        o.reverse_pdf *= p_lobe;
    }
    return ok;
}

}  // namespace disney

// SampleDiracTransparent (DiracTransparent.cpp:20-68): world space, geometric normal = frame normal.
SEL_HD bool sample_dirac_transparent(const Surface& s, float3 v, const float* u, int& used, BsdfSampleOut& o) {
    const float3 n = s.n;
    const float vh = dot(v, n);
    const float ni = vh > 0.0f ? 1.0f : s.ior;
    const float nt = vh > 0.0f ? s.ior : 1.0f;
    const float eta = ni / nt;
    const float F = disney::dielectric(vh, ni, nt);
    float pdf;
    float3 wi;
    if (u[used++] < F) {
        wi = normalize(disney::reflect(n, v));
        o.flags = kScatterEvent;
        pdf = F;
    } else {
        if (disney::transmit(n, v, eta, wi)) {
            o.flags = kTransmissionEvent;
        } else {
            wi = disney::reflect(n, v);
            o.flags = kScatterEvent;
        }
        wi = normalize(wi);
        pdf = 1.0f - F;
    }
    o.flags |= kDiracEvent;
    o.reflectance = s.base_color * (1.0f / pdf);
    o.wi = wi;
    o.forward_pdf = pdf;
    o.reverse_pdf = pdf;
    return true;
}

// SampleBsdfFunction / EvaluateBsdf dispatch (SurfaceScattering.cpp:18-60)
SEL_HD bool bsdf_sample(const Surface& s, float3 v, const float* u, int& used, BsdfSampleOut& o) {
    o.flags = 0;
    o.medium_phase = 0;
    o.extinction = f3(0.0f);
    o.reflectance = f3(0.0f);
    o.wi = f3(0.0f);
    o.forward_pdf = 0.0f;
    o.reverse_pdf = 0.0f;
    if (s.shader == kDisneyThin) return disney::sample(s, v, true, u, used, o);
    if (s.shader == kDisneySolid) return disney::sample(s, v, false, u, used, o);
    if (s.shader == kDiracTransparent) return sample_dirac_transparent(s, v, u, used, o);
    return false;
}

SEL_HD float3 bsdf_evaluate(const Surface& s, float3 v, float3 l, float& fwd, float& rev) {
    fwd = 0.0f;
    rev = 0.0f;
    if (s.shader == kDisneyThin) return disney::evaluate(s, v, l, true, fwd, rev);
    if (s.shader == kDisneySolid) return disney::evaluate(s, v, l, false, fwd, rev);
    return f3(0.0f);
}

// The same dispatch for surfaces known to have shader kShader (-1: any), so that a kernel that shades one kind
// of surface carries only that shader's code.
template <int kShader>
SEL_HD bool bsdf_sample_as(const Surface& s, float3 v, const float* u, int& used, BsdfSampleOut& o) {
    if constexpr (kShader < 0) {
        return bsdf_sample(s, v, u, used, o);
    } else {
        o.flags = 0;
        o.medium_phase = 0;
        o.extinction = f3(0.0f);
        o.reflectance = f3(0.0f);
        o.wi = f3(0.0f);
        o.forward_pdf = 0.0f;
        o.reverse_pdf = 0.0f;
        if constexpr (kShader == kDisneyThin) return disney::sample(s, v, true, u, used, o);
        else if constexpr (kShader == kDisneySolid) return disney::sample(s, v, false, u, used, o);
        else return sample_dirac_transparent(s, v, u, used, o);
    }
}

template <int kShader>
SEL_HD float3 bsdf_evaluate_as(const Surface& s, float3 v, float3 l, float& fwd, float& rev) {
    if constexpr (kShader < 0) {
        return bsdf_evaluate(s, v, l, fwd, rev);
    } else {
        fwd = 0.0f;
        rev = 0.0f;
        if constexpr (kShader == kDisneyThin) return disney::evaluate(s, v, l, true, fwd, rev);
        else if constexpr (kShader == kDisneySolid) return disney::evaluate(s, v, l, false, fwd, rev);
        else return f3(0.0f);
    }
}

}  // namespace sel
