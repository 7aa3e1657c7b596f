// Round B-spline curves (Embree's RTC_GEOMETRY_TYPE_ROUND_BSPLINE_CURVE as the reference attaches them,
// Source/Core/SceneLib/ModelResource.cpp:300-332): segment k of a curve geometry is the uniform cubic B-spline of
// the four control points index[k] .. index[k] + 3 (x, y, z, radius), swept by a sphere whose radius follows the
// same spline.
//
// Embree is a closed binary in the reference, so the intersection is defined here, deterministically: each
// segment is split at u = j / kCurvePieces into pieces whose ends are the spline's centres and radii there, and
// each piece is the round cone through its two end spheres (the union of the spheres of linearly interpolated
// centre and radius).  A hit reports t, u = (j + s) / kCurvePieces where s is the parameter of the piece's sphere
// that touches the hit point, v = 0, and Ng = hit point - that sphere's centre.  Every operation is a single
// rounded IEEE add, multiply, divide or square root (no fused multiply-add), so the CPU oracle's restatement
// returns the same bits.
//
// Leaf records: a curve segment is a TriRecord of kind kTriCurve whose prim / geom words are Embree's primID and
// geomID, and whose v0.x / v0.y hold, as an int64, the byte offset from the record to the segment's data: four
// float4 control points (x, y, z, radius), stored after the scene's leaf records.
#pragma once

#include <cstdint>

#include "vecmath.cuh"

namespace sel {

constexpr int kCurvePieces = 8;

namespace crv {

__device__ __forceinline__ float m(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float a(float x, float y) { return __fadd_rn(x, y); }
__device__ __forceinline__ float s(float x, float y) { return __fsub_rn(x, y); }
__device__ __forceinline__ float d(float x, float y) { return __fdiv_rn(x, y); }
__device__ __forceinline__ float sq(float x) { return __fsqrt_rn(x); }

struct P4 {
    float x, y, z, r;
};

// Uniform cubic B-spline at u (basis (1-u)^3/6, (3u^3-6u^2+4)/6, (-3u^3+3u^2+3u+1)/6, u^3/6).
__device__ __forceinline__ P4 eval(const float4* cp, float u) {
    const float u2 = m(u, u), u3 = m(u2, u), iu = s(1.0f, u);
    const float b0 = d(m(m(iu, iu), iu), 6.0f);
    const float b1 = d(a(s(m(3.0f, u3), m(6.0f, u2)), 4.0f), 6.0f);
    const float b2 = d(a(a(a(m(-3.0f, u3), m(3.0f, u2)), m(3.0f, u)), 1.0f), 6.0f);
    const float b3 = d(u3, 6.0f);
    P4 p;
    p.x = a(a(a(m(b0, cp[0].x), m(b1, cp[1].x)), m(b2, cp[2].x)), m(b3, cp[3].x));
    p.y = a(a(a(m(b0, cp[0].y), m(b1, cp[1].y)), m(b2, cp[2].y)), m(b3, cp[3].y));
    p.z = a(a(a(m(b0, cp[0].z), m(b1, cp[1].z)), m(b2, cp[2].z)), m(b3, cp[3].z));
    p.r = a(a(a(m(b0, cp[0].w), m(b1, cp[1].w)), m(b2, cp[2].w)), m(b3, cp[3].w));
    return p;
}

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return a(a(m(ax, bx), m(ay, by)), m(az, bz));
}

struct Ray3 {
    float ox, oy, oz, dx, dy, dz;
};

// Round cone of end spheres (p0, r0) and (p1, r1): nearest hit with t in [tnear, tfar]; returns false if none.
// s: parameter (0..1) of the touching sphere.
__device__ __forceinline__ bool round_cone(const Ray3& ray, const P4& p0, const P4& p1, float tnear, float tfar,
                                           float& t_out, float& s_out) {
    const float bx = s(p1.x, p0.x), by = s(p1.y, p0.y), bz = s(p1.z, p0.z);
    const float L2 = dot3(bx, by, bz, bx, by, bz);
    const float dr = s(p1.r, p0.r);
    const float ox = s(ray.ox, p0.x), oy = s(ray.oy, p0.y), oz = s(ray.oz, p0.z);
    const float dd = dot3(ray.dx, ray.dy, ray.dz, ray.dx, ray.dy, ray.dz);
    bool found = false;
    float best = tfar;
    // the sphere (c, r) at parameter sp, keeping roots whose point lies on its cap (cap: sign * (z - zc) >= 0)
    auto sphere = [&](float cx, float cy, float cz, float r, float sp, int cap, float zc) {
        const float qx = s(ray.ox, cx), qy = s(ray.oy, cy), qz = s(ray.oz, cz);
        const float hb = dot3(qx, qy, qz, ray.dx, ray.dy, ray.dz);
        const float c = s(dot3(qx, qy, qz, qx, qy, qz), m(r, r));
        const float disc = s(m(hb, hb), m(dd, c));
        if (!(disc >= 0.0f)) return;
        const float root = sq(disc);
        const float ts[2] = {d(s(-hb, root), dd), d(a(-hb, root), dd)};
        for (int i = 0; i < 2; ++i) {
            const float t = ts[i];
            if (!(t >= tnear && t <= best)) continue;
            if (cap != 0 && L2 > 0.0f) {
                // axial coordinate of the hit point relative to p0, scaled by |b|
                const float px = a(ox, m(t, ray.dx)), py = a(oy, m(t, ray.dy)), pz = a(oz, m(t, ray.dz));
                const float z = dot3(px, py, pz, bx, by, bz);
                if (cap < 0 ? z > zc : z < zc) continue;
            }
            best = t;
            s_out = sp;
            found = true;
        }
    };
    const float Lsq = L2;
    if (!(Lsq > 0.0f) || !(m(dr, dr) < Lsq)) {
        // one sphere holds the other (or the piece is a point): the larger sphere
        if (p1.r > p0.r) sphere(p1.x, p1.y, p1.z, p1.r, 1.0f, 0, 0.0f);
        else sphere(p0.x, p0.y, p0.z, p0.r, 0.0f, 0, 0.0f);
        t_out = best;
        return found;
    }
    // contact circles: z (= (P - p0) . b) at the caps' rims: z0 = -r0 dr, z1 = L2 - r1 dr
    const float z0 = m(-p0.r, dr), z1 = s(Lsq, m(p1.r, dr));
    sphere(p0.x, p0.y, p0.z, p0.r, 0.0f, -1, z0);
    sphere(p1.x, p1.y, p1.z, p1.r, 1.0f, 1, z1);
    // tangent cone, the envelope of the spheres (p0 + s b, r0 + s dr): with q = P - p0 and z = q . b its points
    // satisfy (L2 - dr^2) (L2 |q|^2 - z^2) = (L2 r0 + dr z)^2 with L2 r0 + dr z >= 0; for q = o' + t d that is
    // A t^2 + 2 B t + C = 0
    const float h2 = s(Lsq, m(dr, dr));
    const float zo = dot3(ox, oy, oz, bx, by, bz), zd = dot3(ray.dx, ray.dy, ray.dz, bx, by, bz);
    const float qo = dot3(ox, oy, oz, ox, oy, oz), qd = dot3(ox, oy, oz, ray.dx, ray.dy, ray.dz);
    const float wo = a(m(Lsq, p0.r), m(dr, zo)), wd = m(dr, zd);
    const float A = s(m(h2, s(m(Lsq, dd), m(zd, zd))), m(wd, wd));
    const float B = s(m(h2, s(m(Lsq, qd), m(zo, zd))), m(wo, wd));
    const float C = s(m(h2, s(m(Lsq, qo), m(zo, zo))), m(wo, wo));
    if (A != 0.0f) {
        const float disc = s(m(B, B), m(A, C));
        if (disc >= 0.0f) {
            const float root = sq(disc);
            const float ts[2] = {d(s(-B, root), A), d(a(-B, root), A)};
            for (int i = 0; i < 2; ++i) {
                const float t = ts[i];
                if (!(t >= tnear && t <= best)) continue;
                const float z = a(zo, m(t, zd));
                const float w = a(m(Lsq, p0.r), m(dr, z));  // > 0 on the cone's nappe of positive radii
                if (!(w > 0.0f) || z < z0 || z > z1) continue;
                // touching sphere: z = s L2 - r(s) dr  =>  s = (z + r0 dr) / h2
                const float sp = d(a(z, m(p0.r, dr)), h2);
                best = t;
                s_out = fminf(fmaxf(sp, 0.0f), 1.0f);
                found = true;
            }
        }
    }
    t_out = best;
    return found;
}

}  // namespace crv

// Closest hit of the ray with curve segment `cp` (four control points) in [tnear, tfar]: t and u (among equal t,
// the last piece and candidate tested).
static __device__ __noinline__ bool curve_intersect(const float4* cp, float ox, float oy, float oz, float dx, float dy,
                                             float dz, float tnear, float tfar, float& t_out, float& u_out) {
    crv::Ray3 ray{ox, oy, oz, dx, dy, dz};
    bool hit = false;
    float best = tfar;
    crv::P4 prev = crv::eval(cp, 0.0f);
    for (int j = 0; j < kCurvePieces; ++j) {
        const crv::P4 next = crv::eval(cp, crv::d(float(j + 1), float(kCurvePieces)));
        float t, sp;
        if (crv::round_cone(ray, prev, next, tnear, best, t, sp)) {
            best = t;
            u_out = crv::d(crv::a(float(j), sp), float(kCurvePieces));
            hit = true;
        }
        prev = next;
    }
    t_out = best;
    return hit;
}

// Geometric normal of a curve hit at (t, u): hit point minus the centre of the touching sphere of its piece.
__device__ __forceinline__ float3 curve_ng(const float4* cp, float ox, float oy, float oz, float dx, float dy, float dz,
                                           float t, float u) {
    const float uj = crv::m(u, float(kCurvePieces));
    int j = int(floorf(uj));
    j = j < 0 ? 0 : (j > kCurvePieces - 1 ? kCurvePieces - 1 : j);
    const float sp = crv::s(uj, float(j));
    const crv::P4 p0 = crv::eval(cp, crv::d(float(j), float(kCurvePieces)));
    const crv::P4 p1 = crv::eval(cp, crv::d(float(j + 1), float(kCurvePieces)));
    const float cx = crv::a(p0.x, crv::m(sp, crv::s(p1.x, p0.x)));
    const float cy = crv::a(p0.y, crv::m(sp, crv::s(p1.y, p0.y)));
    const float cz = crv::a(p0.z, crv::m(sp, crv::s(p1.z, p0.z)));
    const float px = crv::a(ox, crv::m(t, dx)), py = crv::a(oy, crv::m(t, dy)), pz = crv::a(oz, crv::m(t, dz));
    return make_float3(crv::s(px, cx), crv::s(py, cy), crv::s(pz, cz));
}

// The control points of a curve leaf record (kind kTriCurve): v0.x / v0.y hold the byte offset to them.
__device__ __forceinline__ const float4* curve_points(const float4* record, float4 p0) {
    const int64_t off = int64_t((uint64_t(__float_as_uint(p0.y)) << 32) | __float_as_uint(p0.x));
    return reinterpret_cast<const float4*>(reinterpret_cast<const char*>(record) + off);
}

}  // namespace sel
