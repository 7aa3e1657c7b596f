// ORACLE - test infrastructure only (see oracle_query.cpp).
//
// CPU restatement of the round B-spline curve hits the product defines (Embree's RTC_GEOMETRY_TYPE_ROUND_
// BSPLINE_CURVE, attached by Source/Core/SceneLib/ModelResource.cpp:300-332, is a closed binary, so there is no
// reference result to pin): a segment is the uniform cubic B-spline of four control points (x, y, z, radius), cut
// at u = j / 8 into round cones between the spline's spheres there; a hit reports t, u = the touching sphere's
// parameter, v = 0 and Ng = hit point - that sphere's centre.  Written from the definition with every operation a
// single IEEE rounding (built with -ffp-contract=off), so the device's results are matched bit for bit.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <vector>

#include "oracle_curve.h"

namespace {

constexpr int kPieces = 8;

struct P4 {
    float x, y, z, r;
};

P4 eval(const float* cp, float u) {
    const float u2 = u * u, u3 = u2 * u, iu = 1.0f - u;
    const float b0 = ((iu * iu) * iu) / 6.0f;
    const float b1 = ((3.0f * u3 - 6.0f * u2) + 4.0f) / 6.0f;
    const float b2 = (((-3.0f * u3 + 3.0f * u2) + 3.0f * u) + 1.0f) / 6.0f;
    const float b3 = u3 / 6.0f;
    P4 p;
    p.x = ((b0 * cp[0] + b1 * cp[4]) + b2 * cp[8]) + b3 * cp[12];
    p.y = ((b0 * cp[1] + b1 * cp[5]) + b2 * cp[9]) + b3 * cp[13];
    p.z = ((b0 * cp[2] + b1 * cp[6]) + b2 * cp[10]) + b3 * cp[14];
    p.r = ((b0 * cp[3] + b1 * cp[7]) + b2 * cp[11]) + b3 * cp[15];
    return p;
}

float dot3(float ax, float ay, float az, float bx, float by, float bz) { return (ax * bx + ay * by) + az * bz; }

struct Ray {
    float ox, oy, oz, dx, dy, dz;
};

// Nearest point of the round cone (p0, p1) with t in [tnear, best]; equal t: the later candidate.
bool round_cone(const Ray& ray, const P4& p0, const P4& p1, float tnear, float tfar, float& t_out, float& s_out) {
    const float bx = p1.x - p0.x, by = p1.y - p0.y, bz = p1.z - p0.z;
    const float L2 = dot3(bx, by, bz, bx, by, bz);
    const float dr = p1.r - p0.r;
    const float ox = ray.ox - p0.x, oy = ray.oy - p0.y, oz = ray.oz - p0.z;
    const float dd = dot3(ray.dx, ray.dy, ray.dz, ray.dx, ray.dy, ray.dz);
    bool found = false;
    float best = tfar;
    auto sphere = [&](float cx, float cy, float cz, float r, float sp, int cap, float zc) {
        const float qx = ray.ox - cx, qy = ray.oy - cy, qz = ray.oz - cz;
        const float hb = dot3(qx, qy, qz, ray.dx, ray.dy, ray.dz);
        const float c = dot3(qx, qy, qz, qx, qy, qz) - r * r;
        const float disc = hb * hb - dd * c;
        if (!(disc >= 0.0f)) return;
        const float root = std::sqrt(disc);
        const float ts[2] = {(-hb - root) / dd, (-hb + root) / dd};
        for (float t : ts) {
            if (!(t >= tnear && t <= best)) continue;
            if (cap != 0 && L2 > 0.0f) {
                const float px = ox + t * ray.dx, py = oy + t * ray.dy, pz = oz + t * ray.dz;
                const float z = dot3(px, py, pz, bx, by, bz);
                if (cap < 0 ? z > zc : z < zc) continue;
            }
            best = t;
            s_out = sp;
            found = true;
        }
    };
    if (!(L2 > 0.0f) || !(dr * dr < L2)) {
        if (p1.r > p0.r) sphere(p1.x, p1.y, p1.z, p1.r, 1.0f, 0, 0.0f);
        else sphere(p0.x, p0.y, p0.z, p0.r, 0.0f, 0, 0.0f);
        t_out = best;
        return found;
    }
    const float z0 = -p0.r * dr, z1 = L2 - p1.r * dr;
    sphere(p0.x, p0.y, p0.z, p0.r, 0.0f, -1, z0);
    sphere(p1.x, p1.y, p1.z, p1.r, 1.0f, 1, z1);
    // the spheres' envelope: (L2 - dr^2) (L2 |q|^2 - z^2) = (L2 r0 + dr z)^2, L2 r0 + dr z >= 0, q = P - p0, z = q.b
    const float h2 = L2 - dr * dr;
    const float zo = dot3(ox, oy, oz, bx, by, bz), zd = dot3(ray.dx, ray.dy, ray.dz, bx, by, bz);
    const float qo = dot3(ox, oy, oz, ox, oy, oz), qd = dot3(ox, oy, oz, ray.dx, ray.dy, ray.dz);
    const float wo = L2 * p0.r + dr * zo, wd = dr * zd;
    const float A = h2 * (L2 * dd - zd * zd) - wd * wd;
    const float B = h2 * (L2 * qd - zo * zd) - wo * wd;
    const float C = h2 * (L2 * qo - zo * zo) - wo * wo;
    if (A != 0.0f) {
        const float disc = B * B - A * C;
        if (disc >= 0.0f) {
            const float root = std::sqrt(disc);
            const float ts[2] = {(-B - root) / A, (-B + root) / A};
            for (float t : ts) {
                if (!(t >= tnear && t <= best)) continue;
                const float z = zo + t * zd;
                const float w = L2 * p0.r + dr * z;
                if (!(w > 0.0f) || z < z0 || z > z1) continue;
                const float sp = (z + p0.r * dr) / h2;
                best = t;
                s_out = std::fmin(std::fmax(sp, 0.0f), 1.0f);
                found = true;
            }
        }
    }
    t_out = best;
    return found;
}

bool curve_hit(const float* cp, const Ray& ray, float tnear, float tfar, float& t_out, float& u_out) {
    bool hit = false;
    float best = tfar;
    P4 prev = eval(cp, 0.0f);
    for (int j = 0; j < kPieces; ++j) {
        const P4 next = eval(cp, float(j + 1) / float(kPieces));
        float t, sp;
        if (round_cone(ray, prev, next, tnear, best, t, sp)) {
            best = t;
            u_out = (float(j) + sp) / float(kPieces);
            hit = true;
        }
        prev = next;
    }
    t_out = best;
    return hit;
}

void curve_ng(const float* cp, const Ray& ray, float t, float u, float ng[3]) {
    const float uj = u * float(kPieces);
    int j = int(std::floor(uj));
    j = j < 0 ? 0 : (j > kPieces - 1 ? kPieces - 1 : j);
    const float sp = uj - float(j);
    const P4 p0 = eval(cp, float(j) / float(kPieces));
    const P4 p1 = eval(cp, float(j + 1) / float(kPieces));
    const float cx = p0.x + sp * (p1.x - p0.x), cy = p0.y + sp * (p1.y - p0.y), cz = p0.z + sp * (p1.z - p0.z);
    ng[0] = (ray.ox + t * ray.dx) - cx;
    ng[1] = (ray.oy + t * ray.dy) - cy;
    ng[2] = (ray.oz + t * ray.dz) - cz;
}

// Curve geometries of the render oracle's scenes (oracle_set_curves), by scene index.
struct Segment {
    double lo[3], hi[3];  // the control points' hull grown by their largest radius (holds every piece)
    uint32_t first, prim;
};
struct CurveGeom {
    uint32_t geom;
    std::vector<float> points;
    std::vector<Segment> segs;
};
std::map<uint32_t, std::vector<CurveGeom>> g_curves;

bool seg_box_hit(const Segment& b, const float* o, const float* d, float tnear, float tfar) {
    double t0 = tnear, t1 = tfar;
    for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0f) {
            if (o[a] < b.lo[a] || o[a] > b.hi[a]) return false;
            continue;
        }
        double n = (b.lo[a] - o[a]) / double(d[a]);
        double f = (b.hi[a] - o[a]) / double(d[a]);
        if (n > f) std::swap(n, f);
        t0 = std::max(t0, n);
        t1 = std::min(t1, f);
    }
    return t0 <= t1;
}

}  // namespace

namespace orcv {

bool any(uint32_t scene) { return g_curves.count(scene) != 0; }

bool bounds(uint32_t scene, float lo[3], float hi[3]) {
    const auto it = g_curves.find(scene);
    if (it == g_curves.end()) return false;
    double l[3] = {INFINITY, INFINITY, INFINITY}, h[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (const CurveGeom& c : it->second)
        for (const Segment& s : c.segs)
            for (int a = 0; a < 3; ++a) {
                l[a] = std::min(l[a], s.lo[a]);
                h[a] = std::max(h[a], s.hi[a]);
            }
    for (int a = 0; a < 3; ++a) {
        lo[a] = std::nextafter(float(l[a]), -INFINITY);
        hi[a] = std::nextafter(float(h[a]), INFINITY);
    }
    return l[0] <= h[0];
}

bool closest(uint32_t scene, const float* o, const float* d, float tnear, float tfar, float& t_out, float& u_out,
             float ng[3], uint32_t& prim, uint32_t& geom) {
    const auto it = g_curves.find(scene);
    if (it == g_curves.end()) return false;
    const Ray ray{o[0], o[1], o[2], d[0], d[1], d[2]};
    bool found = false;
    uint64_t best_key = ~0ull;
    const float* best_cp = nullptr;
    for (const CurveGeom& c : it->second)
        for (const Segment& s : c.segs) {
            if (!seg_box_hit(s, o, d, tnear, tfar)) continue;
            float t, u;
            const float* cp = c.points.data() + 4 * size_t(s.first);
            if (!curve_hit(cp, ray, tnear, tfar, t, u)) continue;
            const uint64_t key = (uint64_t(c.geom) << 32) | s.prim;
            if (found && !(t < tfar || key < best_key)) continue;
            found = true;
            tfar = t;
            best_key = key;
            best_cp = cp;
            t_out = t;
            u_out = u;
        }
    if (!found) return false;
    curve_ng(best_cp, ray, t_out, u_out, ng);
    prim = uint32_t(best_key);
    geom = uint32_t(best_key >> 32);
    return true;
}

bool occluded(uint32_t scene, const float* o, const float* d, float tnear, float tfar) {
    const auto it = g_curves.find(scene);
    if (it == g_curves.end()) return false;
    const Ray ray{o[0], o[1], o[2], d[0], d[1], d[2]};
    for (const CurveGeom& c : it->second)
        for (const Segment& s : c.segs) {
            float t, u;
            if (seg_box_hit(s, o, d, tnear, tfar) && curve_hit(c.points.data() + 4 * size_t(s.first), ray, tnear, tfar, t, u))
                return true;
        }
    return false;
}

}  // namespace orcv

extern "C" {

// Curve geometries of the next oracle renders: n geometries, geometry k in scene keys[2k] with geomID keys[2k+1],
// its points (float4) points[point_offs[k] ..] and segment first points indices[index_offs[k] ..] (relative to
// its own points); n = 0 clears them.
void oracle_set_curves(int n, const uint32_t* keys, const int64_t* point_offs, const float* points,
                       const int64_t* index_offs, const uint32_t* indices) {
    g_curves.clear();
    for (int k = 0; k < n; ++k) {
        CurveGeom c;
        c.geom = keys[2 * k + 1];
        c.points.assign(points + 4 * point_offs[k], points + 4 * point_offs[k + 1]);
        for (int64_t i = index_offs[k]; i < index_offs[k + 1]; ++i) {
            Segment s;
            s.first = indices[i];
            s.prim = uint32_t(i - index_offs[k]);
            const float* cp = c.points.data() + 4 * size_t(s.first);
            float r = 0.0f;
            for (int a = 0; a < 3; ++a) {
                s.lo[a] = INFINITY;
                s.hi[a] = -INFINITY;
            }
            for (int j = 0; j < 4; ++j) {
                r = std::max(r, cp[4 * j + 3]);
                for (int a = 0; a < 3; ++a) {
                    s.lo[a] = std::min(s.lo[a], double(cp[4 * j + a]));
                    s.hi[a] = std::max(s.hi[a], double(cp[4 * j + a]));
                }
            }
            for (int a = 0; a < 3; ++a) {  // radius, and room for the pieces' rounding
                const double pad = double(r) + (std::fabs(s.lo[a]) + std::fabs(s.hi[a]) + double(r)) * 1e-5 + 1e-30;
                s.lo[a] -= pad;
                s.hi[a] += pad;
            }
            c.segs.push_back(s);
        }
        g_curves[keys[2 * k]].push_back(std::move(c));
    }
}

// Brute force over the segments of one curve geometry (points: 4 floats each; indices: first point of each
// segment) for records of `stride` bytes (96: RTCRayHit, closest hit; 48: RTCRay, any hit): a record takes the
// curve's hit when it is nearer than the record's tfar, or as near with a smaller (geomID, primID).
void oracle_curve_hits(const float* points, const uint32_t* indices, int64_t nseg, uint32_t geom, void* records,
                       int64_t n, int stride) {
    for (int64_t i = 0; i < n; ++i) {
        float* r = reinterpret_cast<float*>(static_cast<char*>(records) + i * stride);
        const Ray ray{r[0], r[1], r[2], r[4], r[5], r[6]};
        const float tnear = r[3];
        float tfar = r[8];
        if (stride == 48) {
            if (!(tfar >= tnear)) continue;  // already occluded
            for (int64_t k = 0; k < nseg; ++k) {
                float t, u;
                if (curve_hit(points + 4 * size_t(indices[k]), ray, tnear, tfar, t, u)) {
                    r[8] = -std::numeric_limits<float>::infinity();
                    break;
                }
            }
            continue;
        }
        uint32_t* w = reinterpret_cast<uint32_t*>(r);
        for (int64_t k = 0; k < nseg; ++k) {
            float t, u;
            if (!curve_hit(points + 4 * size_t(indices[k]), ray, tnear, tfar, t, u)) continue;
            const uint64_t key = (uint64_t(geom) << 32) | uint64_t(k);
            const uint64_t cur = (uint64_t(w[18]) << 32) | uint64_t(w[17]);
            if (!(t < tfar || (t == tfar && key < cur))) continue;
            float ng[3];
            curve_ng(points + 4 * size_t(indices[k]), ray, t, u, ng);
            tfar = t;
            r[8] = t;
            r[12] = ng[0];
            r[13] = ng[1];
            r[14] = ng[2];
            r[15] = u;
            r[16] = 0.0f;
            w[17] = uint32_t(k);
            w[18] = geom;
            w[19] = 0xffffffffu;
            w[20] = 0xffffffffu;
        }
    }
}

}  // extern "C"
