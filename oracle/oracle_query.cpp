// ORACLE - test infrastructure only.  Nothing in the product links or calls this file; only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load liboracle.so, as the checker.
//
// CPU restatement of the ray-query contract the reference integrators rely on:
//   * closest hit  - Embree rtcIntersect1 as called by RayPick, Source/Applications/Selas/Source/PathTracer.cpp:95-139
//                    (tnear/tfar in, tfar/Ng/u/v/primID/geomID/instID out; geomID stays -1 on a miss);
//   * any hit      - Embree rtcOccluded1 as called by OcclusionRay, PathTracer.cpp:71-92 (tfar = -inf on a hit).
// Embree 3.2 itself ships only as a Windows/macOS binary (Middleware/embree-latest), so parity against it
// is unpinned here; this file pins the contract instead with an independent CPU implementation of the
// watertight test of Woop, Benthin and Wald (JCGT 2013) and the order-independent tie rule (smallest t,
// then smallest (geomID, primID)).  Two traversals are provided: brute force over every triangle (the
// definition) and an SAH BVH of this file's own (for large scenes and for the CPU baseline).
//
// Instanced scenes (two levels, as the reference's subscene instances of model instances,
// Source/Core/SceneLib/SceneResource.cpp:73-187 and SubsceneResource.cpp:63-79) are restated by brute force:
// the ray is carried into each instance by its world-to-local rows (fma chains), t stays in the world ray's
// parametrisation, and ties on t go to the smaller (instID[0], instID[1], geomID, primID).
//
// Compiled with -ffp-contract=off; every fused multiply-add is an explicit std::fma.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "oracle_curve.h"

namespace {

struct Ray {
    float org[3];
    float tnear;
    float dir[3];
    float time;
    float tfar;
    uint32_t mask, id, flags;
};
struct RayHit {
    Ray ray;
    float ng[3];
    float u, v;
    uint32_t prim, geom, inst[2];
    uint32_t pad[3];
};
static_assert(sizeof(Ray) == 48, "Ray");
static_assert(sizeof(RayHit) == 96, "RayHit");

struct Tri {
    float v[3][3];
    uint32_t prim, geom;
};

struct Setup {
    int kx, ky, kz;
    float sx, sy, sz;
};

Setup setup(const float* d) {
    Setup s;
    const float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    s.kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    s.kx = s.kz == 2 ? 0 : s.kz + 1;
    s.ky = s.kx == 2 ? 0 : s.kx + 1;
    if (d[s.kz] < 0.0f) std::swap(s.kx, s.ky);
    s.sx = d[s.kx] / d[s.kz];
    s.sy = d[s.ky] / d[s.kz];
    s.sz = 1.0f / d[s.kz];
    return s;
}

bool intersect(const Setup& s, const float* o, const Tri& tri, float tnear, float tfar, float& t, float& u, float& v) {
    float A[3], B[3], C[3];
    for (int k = 0; k < 3; ++k) {
        A[k] = tri.v[0][k] - o[k];
        B[k] = tri.v[1][k] - o[k];
        C[k] = tri.v[2][k] - o[k];
    }
    const float Ax = std::fma(-s.sx, A[s.kz], A[s.kx]);
    const float Ay = std::fma(-s.sy, A[s.kz], A[s.ky]);
    const float Bx = std::fma(-s.sx, B[s.kz], B[s.kx]);
    const float By = std::fma(-s.sy, B[s.kz], B[s.ky]);
    const float Cx = std::fma(-s.sx, C[s.kz], C[s.kx]);
    const float Cy = std::fma(-s.sy, C[s.kz], C[s.ky]);
    const float cybx = Cy * Bx, aycx = Ay * Cx, byax = By * Ax;
    float U = std::fma(Cx, By, -cybx);
    float V = std::fma(Ax, Cy, -aycx);
    float W = std::fma(Bx, Ay, -byax);
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = float(double(Cx) * double(By) - double(Cy) * double(Bx));
        V = float(double(Ax) * double(Cy) - double(Ay) * double(Cx));
        W = float(double(Bx) * double(Ay) - double(By) * double(Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = s.sz * A[s.kz], Bz = s.sz * B[s.kz], Cz = s.sz * C[s.kz];
    const float wcz = W * Cz;
    const float T = std::fma(U, Az, std::fma(V, Bz, wcz));
    const float rcp = 1.0f / det;
    const float tt = T * rcp;
    if (!(tt >= tnear && tt <= tfar)) return false;
    t = tt;
    u = V * rcp;
    v = W * rcp;
    return true;
}

void normal(const Tri& tri, float* ng) {
    float e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
        e1[k] = tri.v[1][k] - tri.v[0][k];
        e2[k] = tri.v[2][k] - tri.v[0][k];
    }
    const float a = e1[2] * e2[1], b = e1[0] * e2[2], c = e1[1] * e2[0];
    ng[0] = std::fma(e1[1], e2[2], -a);
    ng[1] = std::fma(e1[2], e2[0], -b);
    ng[2] = std::fma(e1[0], e2[1], -c);
}

uint64_t key_of(const Tri& t) { return (uint64_t(t.geom) << 32) | t.prim; }

struct Best {
    float t, u, v;
    int64_t tri = -1;
    uint64_t key = ~0ull;
};

// candidate accepted when tnear <= t <= current tfar; ties on t go to the smaller key
inline void offer(const Setup& s, const Ray& r, const Tri& tri, int64_t index, float& tfar, Best& best) {
    float t, u, v;
    if (!intersect(s, r.org, tri, r.tnear, tfar, t, u, v)) return;
    const uint64_t k = key_of(tri);
    if (t < tfar || k < best.key) {
        tfar = t;
        best.t = t; best.u = u; best.v = v; best.tri = index; best.key = k;
    }
}

void write_hit(RayHit& rh, const Tri& tri, const Best& b) {
    rh.ray.tfar = b.t;
    normal(tri, rh.ng);
    rh.u = b.u;
    rh.v = b.v;
    rh.prim = tri.prim;
    rh.geom = tri.geom;
    rh.inst[0] = rh.inst[1] = 0xffffffffu;
}

// ---------------------------------------------------------------------------------------------------
// Oracle BVH: binary, binned SAH (16 bins), leaves of <= 4 triangles.
// ---------------------------------------------------------------------------------------------------
struct Box {
    float lo[3], hi[3];
    void reset() { for (int a = 0; a < 3; ++a) { lo[a] = INFINITY; hi[a] = -INFINITY; } }
    void grow(const Box& b) { for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); } }
    float area() const {
        if (lo[0] > hi[0]) return 0.0f;
        const float x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
        return 2.0f * (x * y + y * z + z * x);
    }
};

struct Node {
    Box box;
    int32_t left, right;  // internal: child indices; leaf: left = first, right = -count
};

struct Bvh {
    std::vector<Tri> tris;  // reordered to leaf order
    std::vector<Node> nodes;
};

struct Item {
    Box box;
    float c[3];
    uint32_t tri;
};

int build_node(std::vector<Node>& nodes, std::vector<Item>& items, int first, int count) {
    const int index = int(nodes.size());
    nodes.push_back(Node());
    Box box, cb;
    box.reset();
    cb.reset();
    for (int i = first; i < first + count; ++i) {
        box.grow(items[i].box);
        for (int a = 0; a < 3; ++a) { cb.lo[a] = std::min(cb.lo[a], items[i].c[a]); cb.hi[a] = std::max(cb.hi[a], items[i].c[a]); }
    }
    nodes[index].box = box;
    int axis = 0;
    for (int a = 1; a < 3; ++a) if (cb.hi[a] - cb.lo[a] > cb.hi[axis] - cb.lo[axis]) axis = a;
    if (count <= 4 || !(cb.hi[axis] > cb.lo[axis])) {
        if (count <= 4) {
            nodes[index].left = first;
            nodes[index].right = -count;
            return index;
        }
    }
    int mid = first + count / 2;
    if (cb.hi[axis] > cb.lo[axis]) {
        constexpr int kB = 16;
        Box bins[kB];
        int cnt[kB] = {};
        for (int b = 0; b < kB; ++b) bins[b].reset();
        const float scale = kB * 0.999999f / (cb.hi[axis] - cb.lo[axis]);
        for (int i = first; i < first + count; ++i) {
            int b = std::min(kB - 1, std::max(0, int((items[i].c[axis] - cb.lo[axis]) * scale)));
            bins[b].grow(items[i].box);
            cnt[b]++;
        }
        float best = INFINITY;
        int best_b = -1;
        for (int s = 0; s < kB - 1; ++s) {
            Box l, r;
            l.reset(); r.reset();
            int nl = 0, nr = 0;
            for (int b = 0; b <= s; ++b) { l.grow(bins[b]); nl += cnt[b]; }
            for (int b = s + 1; b < kB; ++b) { r.grow(bins[b]); nr += cnt[b]; }
            if (!nl || !nr) continue;
            const float c = l.area() * nl + r.area() * nr;
            if (c < best) { best = c; best_b = s; }
        }
        if (best_b >= 0) {
            auto it = std::partition(items.begin() + first, items.begin() + first + count, [&](const Item& it2) {
                int b = std::min(kB - 1, std::max(0, int((it2.c[axis] - cb.lo[axis]) * scale)));
                return b <= best_b;
            });
            mid = int(it - items.begin());
        }
        if (mid == first || mid == first + count) {
            mid = first + count / 2;
            std::nth_element(items.begin() + first, items.begin() + mid, items.begin() + first + count,
                             [axis](const Item& a, const Item& b) { return a.c[axis] < b.c[axis]; });
        }
    }
    const int l = build_node(nodes, items, first, mid - first);
    const int r = build_node(nodes, items, mid, first + count - mid);
    nodes[index].left = l;
    nodes[index].right = r;
    return index;
}

// Slab test in double on boxes padded by 2^-20 of their magnitude; a zero direction component constrains
// nothing when the origin lies inside the slab and rejects the box otherwise.
inline bool box_hit(const Box& b, const float* o, const float* dir, float tnear, float tfar, float& tmin) {
    double t0 = tnear, t1 = tfar;
    for (int a = 0; a < 3; ++a) {
        const double pad = std::ldexp(std::max(std::fabs(double(b.lo[a])), std::fabs(double(b.hi[a]))), -20) + 1e-30;
        const double lo = double(b.lo[a]) - pad, hi = double(b.hi[a]) + pad;
        if (dir[a] == 0.0f) {
            if (o[a] < lo || o[a] > hi) return false;
            continue;
        }
        double n = (lo - o[a]) / double(dir[a]);
        double f = (hi - o[a]) / double(dir[a]);
        if (n > f) std::swap(n, f);
        t0 = std::max(t0, n);
        t1 = std::min(t1, f);
    }
    tmin = float(t0);
    return t0 <= t1;
}

template <bool kAny>
bool trace(const Bvh& bvh, const Ray& r, Best& best) {
    const Setup s = setup(r.dir);
    const float* inv = r.dir;
    const float margin = 1.0f / 262144.0f;
    float tfar = r.tfar;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node& n = bvh.nodes[stack[--sp]];
        float tmin;
        if (!box_hit(n.box, r.org, inv, r.tnear - std::fabs(r.tnear) * margin, tfar + std::fabs(tfar) * margin, tmin))
            continue;
        if (n.right <= 0) {
            for (int i = n.left; i < n.left - n.right; ++i) {
                if (kAny) {
                    float t, u, v;
                    if (intersect(s, r.org, bvh.tris[i], r.tnear, r.tfar, t, u, v)) return true;
                } else {
                    offer(s, r, bvh.tris[i], i, tfar, best);
                }
            }
            continue;
        }
        const Node& l = bvh.nodes[n.left];
        const Node& rr = bvh.nodes[n.right];
        float tl, tr;
        const bool hl = box_hit(l.box, r.org, inv, r.tnear - std::fabs(r.tnear) * margin, tfar + std::fabs(tfar) * margin, tl);
        const bool hr = box_hit(rr.box, r.org, inv, r.tnear - std::fabs(r.tnear) * margin, tfar + std::fabs(tfar) * margin, tr);
        if (hl && hr) {
            if (tl <= tr) { stack[sp++] = n.right; stack[sp++] = n.left; }
            else { stack[sp++] = n.left; stack[sp++] = n.right; }
        } else if (hl) {
            stack[sp++] = n.left;
        } else if (hr) {
            stack[sp++] = n.right;
        }
        if (sp > 120) break;  // cannot happen for trees built above (depth < 64)
    }
    return best.tri >= 0;
}

// ---------------------------------------------------------------------------------------------------
// Instanced scenes, brute force
// ---------------------------------------------------------------------------------------------------
struct OInst {
    float w2l[12];
    uint32_t id, proto;
};
struct OScene {
    std::vector<Tri> tris;
    std::vector<OInst> insts;
};
struct IBest {
    float t = 0, u = 0, v = 0;
    const Tri* tri = nullptr;
    uint64_t inst = ~0ull, key = ~0ull;
};

void xpoint(const float* m, const float* p, float* o) {
    for (int r = 0; r < 3; ++r) o[r] = std::fma(m[4 * r], p[0], std::fma(m[4 * r + 1], p[1], std::fma(m[4 * r + 2], p[2], m[4 * r + 3])));
}
void xvector(const float* m, const float* d, float* o) {
    for (int r = 0; r < 3; ++r) o[r] = std::fma(m[4 * r], d[0], std::fma(m[4 * r + 1], d[1], m[4 * r + 2] * d[2]));
}
bool untraceable(const float* o, const float* d) {
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(o[k]) || !std::isfinite(d[k])) return true;
    return d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f;
}

// Returns true when an any-hit query found a hit.
bool brute_instanced(const std::vector<OScene>& S, uint32_t s, const float* o, const float* d, float tnear, float& tfar,
                     uint64_t cur, int level, IBest& best, bool any) {
    const Setup st = setup(d);
    for (const Tri& tri : S[s].tris) {
        float t, u, v;
        if (!intersect(st, o, tri, tnear, tfar, t, u, v)) continue;
        if (any) return true;
        const uint64_t k = key_of(tri);
        if (t < tfar || cur < best.inst || (cur == best.inst && k < best.key)) {
            tfar = t;
            best.t = t; best.u = u; best.v = v; best.tri = &tri; best.inst = cur; best.key = k;
        }
    }
    for (const OInst& in : S[s].insts) {
        if (level >= 2) continue;
        float o2[3], d2[3];
        xpoint(in.w2l, o, o2);
        xvector(in.w2l, d, d2);
        if (untraceable(o2, d2)) continue;
        const uint64_t ci = level == 0 ? ((uint64_t(in.id) << 32) | 0xffffffffull) : ((cur & 0xffffffff00000000ull) | in.id);
        if (brute_instanced(S, in.proto, o2, d2, tnear, tfar, ci, level + 1, best, any)) return true;
    }
    return false;
}

std::vector<Tri> make_tris(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t n) {
    std::vector<Tri> tris(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        std::memcpy(tris[size_t(i)].v, verts + 9 * i, 36);
        tris[size_t(i)].prim = prim[i];
        tris[size_t(i)].geom = geom[i];
    }
    return tris;
}

template <typename F>
void parallel_for(int64_t n, int threads, F f) {
    if (threads <= 1 || n < 256) {
        for (int64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&] {
            for (;;) {
                const int64_t start = next.fetch_add(64);
                if (start >= n) break;
                const int64_t end = std::min(n, start + 64);
                for (int64_t i = start; i < end; ++i) f(i);
            }
        });
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

// verts: n x 9 floats (v0, v1, v2); prim/geom: n ids.  Brute force over every triangle.
void oracle_intersect_bruteforce(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t n,
                                 void* rayhits, int64_t m, int threads) {
    const std::vector<Tri> tris = make_tris(verts, prim, geom, n);
    RayHit* rh = static_cast<RayHit*>(rayhits);
    parallel_for(m, threads, [&](int64_t i) {
        RayHit& q = rh[i];
        const Setup s = setup(q.ray.dir);
        float tfar = q.ray.tfar;
        Best best;
        for (int64_t k = 0; k < n; ++k) offer(s, q.ray, tris[size_t(k)], k, tfar, best);
        if (best.tri >= 0) write_hit(q, tris[size_t(best.tri)], best);
    });
}

void oracle_occluded_bruteforce(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t n, void* rays,
                                int64_t m, int threads) {
    const std::vector<Tri> tris = make_tris(verts, prim, geom, n);
    Ray* rs = static_cast<Ray*>(rays);
    parallel_for(m, threads, [&](int64_t i) {
        Ray& r = rs[i];
        const Setup s = setup(r.dir);
        for (int64_t k = 0; k < n; ++k) {
            float t, u, v;
            if (intersect(s, r.org, tris[size_t(k)], r.tnear, r.tfar, t, u, v)) {
                r.tfar = -INFINITY;
                return;
            }
        }
    });
}

void* oracle_bvh_build(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t n) {
    Bvh* bvh = new Bvh();
    std::vector<Tri> tris = make_tris(verts, prim, geom, n);
    std::vector<Item> items(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        Item& it = items[size_t(i)];
        it.box.reset();
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) {
                it.box.lo[a] = std::min(it.box.lo[a], tris[size_t(i)].v[k][a]);
                it.box.hi[a] = std::max(it.box.hi[a], tris[size_t(i)].v[k][a]);
            }
        for (int a = 0; a < 3; ++a) it.c[a] = 0.5f * (it.box.lo[a] + it.box.hi[a]);
        it.tri = uint32_t(i);
    }
    bvh->nodes.reserve(size_t(2 * n));
    build_node(bvh->nodes, items, 0, int(n));
    bvh->tris.resize(size_t(n));
    for (int64_t i = 0; i < n; ++i) bvh->tris[size_t(i)] = tris[items[size_t(i)].tri];
    return bvh;
}

void oracle_bvh_free(void* h) { delete static_cast<Bvh*>(h); }

void oracle_intersect_bvh(void* h, void* rayhits, int64_t m, int threads) {
    const Bvh& bvh = *static_cast<Bvh*>(h);
    RayHit* rh = static_cast<RayHit*>(rayhits);
    parallel_for(m, threads, [&](int64_t i) {
        Best best;
        if (trace<false>(bvh, rh[i].ray, best)) write_hit(rh[i], bvh.tris[size_t(best.tri)], best);
    });
}

// Instanced scenes.  Triangles: verts (ntri x 9), prim, geom and the scene each belongs to (tri_scene);
// instances: w2l rows (ninst x 12), instID, the scene holding the instance and the instanced scene; `top` is
// the scene queried.  any_hit = 0: rayhits are SelRayHit records (Ng in the hit mesh's object space); else
// SelRay records (tfar = -inf on a hit).
void oracle_instanced_query(int n_scenes, const float* verts, const uint32_t* prim, const uint32_t* geom,
                            const uint32_t* tri_scene, int64_t ntri, const float* w2l, const uint32_t* inst_id,
                            const uint32_t* inst_scene, const uint32_t* inst_proto, int64_t ninst, int top, void* rays,
                            int64_t m, int any_hit, int threads) {
    std::vector<OScene> S(size_t(std::max(n_scenes, 1)));
    const std::vector<Tri> tris = make_tris(verts, prim, geom, ntri);
    for (int64_t i = 0; i < ntri; ++i) S[tri_scene[i]].tris.push_back(tris[size_t(i)]);
    for (int64_t i = 0; i < ninst; ++i) {
        OInst in;
        std::memcpy(in.w2l, w2l + 12 * i, 48);
        in.id = inst_id[i];
        in.proto = inst_proto[i];
        S[inst_scene[i]].insts.push_back(in);
    }
    parallel_for(m, threads, [&](int64_t i) {
        Ray& r = any_hit ? static_cast<Ray*>(rays)[i] : static_cast<RayHit*>(rays)[i].ray;
        if (untraceable(r.org, r.dir)) return;
        float tfar = r.tfar;
        IBest best;
        const bool hit = brute_instanced(S, uint32_t(top), r.org, r.dir, r.tnear, tfar, ~0ull, 0, best, any_hit != 0);
        if (any_hit) {
            if (hit) r.tfar = -INFINITY;
            return;
        }
        if (!best.tri) return;
        RayHit& rh = static_cast<RayHit*>(rays)[i];
        Best b;
        b.t = best.t; b.u = best.u; b.v = best.v;
        write_hit(rh, *best.tri, b);
        rh.inst[0] = uint32_t(best.inst >> 32);
        rh.inst[1] = uint32_t(best.inst);
    });
}

// World-to-local rows of an affine local-to-world (rows): cofactor inverse and -inv . t in double, rounded
// to float (the product's instance transform, restated).  Returns 0 when singular or not finite.
int oracle_affine_inverse(const float* l2w, float* w2l) {
    const double a00 = l2w[0], a01 = l2w[1], a02 = l2w[2], t0 = l2w[3];
    const double a10 = l2w[4], a11 = l2w[5], a12 = l2w[6], t1 = l2w[7];
    const double a20 = l2w[8], a21 = l2w[9], a22 = l2w[10], t2 = l2w[11];
    const double cof[3][3] = {{a11 * a22 - a12 * a21, a12 * a20 - a10 * a22, a10 * a21 - a11 * a20},
                              {a02 * a21 - a01 * a22, a00 * a22 - a02 * a20, a01 * a20 - a00 * a21},
                              {a01 * a12 - a02 * a11, a02 * a10 - a00 * a12, a00 * a11 - a01 * a10}};
    const double det = a00 * cof[0][0] + a01 * cof[0][1] + a02 * cof[0][2];
    if (!(det != 0.0) || !std::isfinite(det)) return 0;
    for (int r = 0; r < 3; ++r) {
        const double i0 = cof[0][r] / det, i1 = cof[1][r] / det, i2 = cof[2][r] / det;
        const double tr = -(i0 * t0 + i1 * t1 + i2 * t2);
        w2l[4 * r] = float(i0);
        w2l[4 * r + 1] = float(i1);
        w2l[4 * r + 2] = float(i2);
        w2l[4 * r + 3] = float(tr);
    }
    for (int k = 0; k < 12; ++k)
        if (!std::isfinite(w2l[k])) return 0;
    return 1;
}

void oracle_occluded_bvh(void* h, void* rays, int64_t m, int threads) {
    const Bvh& bvh = *static_cast<Bvh*>(h);
    Ray* rs = static_cast<Ray*>(rays);
    parallel_for(m, threads, [&](int64_t i) {
        Best best;
        if (trace<true>(bvh, rs[i], best)) rs[i].tfar = -INFINITY;
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------
// Entry points for the oracle integrators (oracle_query.h).
// ---------------------------------------------------------------------------------------------------
#include "oracle_query.h"

namespace orq {

void* build(const float* verts, const uint32_t* prim, const uint32_t* geom, int64_t n) {
    return oracle_bvh_build(verts, prim, geom, n);
}

bool closest(const void* h, const float* org, const float* dir, float tnear, float tfar, Hit& out) {
    const Bvh& bvh = *static_cast<const Bvh*>(h);
    Ray r;
    std::memcpy(r.org, org, 12);
    std::memcpy(r.dir, dir, 12);
    r.tnear = tnear;
    r.tfar = tfar;
    Best best;
    const bool tri = !bvh.nodes.empty() && trace<false>(bvh, r, best);
    float ct, cu;
    uint32_t cp, cg;
    if (orcv::closest(0, org, dir, tnear, tri ? best.t : tfar, ct, cu, out.ng, cp, cg) &&
        (!tri || ct < best.t || ((uint64_t(cg) << 32) | cp) < best.key)) {  // a curve of the scene (oracle_curve.cpp)
        out.t = ct;
        out.u = cu;
        out.v = 0.0f;
        out.prim = cp;
        out.geom = cg;
        return true;
    }
    if (!tri) return false;
    const Tri& t = bvh.tris[size_t(best.tri)];
    out.t = best.t;
    out.u = best.u;
    out.v = best.v;
    normal(t, out.ng);
    out.prim = t.prim;
    out.geom = t.geom;
    return true;
}

void release(void* h) { oracle_bvh_free(h); }

bool occluded(const void* h, const float* org, const float* dir, float tnear, float tfar) {
    const Bvh& bvh = *static_cast<const Bvh*>(h);
    Ray r;
    std::memcpy(r.org, org, 12);
    std::memcpy(r.dir, dir, 12);
    r.tnear = tnear;
    r.tfar = tfar;
    Best best;
    return (!bvh.nodes.empty() && trace<true>(bvh, r, best)) || orcv::occluded(0, org, dir, tnear, tfar);
}

// ---------------------------------------------------------------------------------------------------
// Instanced graphs with per-scene BVHs (the render oracle's form of oracle_instanced_query)
// ---------------------------------------------------------------------------------------------------
namespace {

struct GInst {
    float w2l[12], l2w[12];
    uint32_t id, proto;
    Box box;  // world box in the owning scene's frame, padded generously (culling only)
};
struct GScene {
    Bvh* bvh = nullptr;
    std::vector<GInst> insts;
    Box bounds;
};
struct Graph {
    std::vector<GScene> scenes;
    uint32_t top = 0;
    ~Graph() {
        for (GScene& s : scenes) delete s.bvh;
    }
};
struct GBest {
    float t = 0, u = 0, v = 0;
    const Tri* tri = nullptr;
    bool curve = false;  // the best hit is a curve's (cng, cprim, cgeom)
    float cng[3] = {0, 0, 0};
    uint32_t cprim = 0, cgeom = 0;
    uint64_t inst = ~0ull, key = ~0ull;
    uint32_t scene = 0;
    const float* l2w[2] = {nullptr, nullptr};
    uint64_t updates = 0;
};

void scene_bounds(Graph& G, uint32_t s, std::vector<int>& done) {
    if (done[s]) return;
    GScene& S = G.scenes[s];
    S.bounds.reset();
    if (S.bvh && !S.bvh->nodes.empty()) S.bounds.grow(S.bvh->nodes[0].box);
    Box cb;
    if (orcv::bounds(s, cb.lo, cb.hi)) S.bounds.grow(cb);
    for (GInst& in : S.insts) {
        scene_bounds(G, in.proto, done);
        const Box& pb = G.scenes[in.proto].bounds;
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int k = 0; k < 8; ++k) {
            const double p[3] = {(k & 1) ? pb.hi[0] : pb.lo[0], (k & 2) ? pb.hi[1] : pb.lo[1], (k & 4) ? pb.hi[2] : pb.lo[2]};
            for (int r = 0; r < 3; ++r) {
                const double w = double(in.l2w[4 * r]) * p[0] + double(in.l2w[4 * r + 1]) * p[1] +
                                 double(in.l2w[4 * r + 2]) * p[2] + double(in.l2w[4 * r + 3]);
                lo[r] = std::min(lo[r], w);
                hi[r] = std::max(hi[r], w);
            }
        }
        for (int r = 0; r < 3; ++r) {
            const double pad = (std::max(std::fabs(lo[r]), std::fabs(hi[r])) + (hi[r] - lo[r])) * 1e-3 + 1e-20;
            in.box.lo[r] = float(lo[r] - pad);
            in.box.hi[r] = float(hi[r] + pad);
        }
        S.bounds.grow(in.box);
    }
    done[s] = 1;
}

// Closest hit in scene s at instance level `level`, merged into `best` by (t, instance ids, geomID, primID).
void gclosest(const Graph& G, uint32_t s, const float* o, const float* d, float tnear, float& tfar, uint64_t cur,
              int level, const float* chain0, GBest& best) {
    const GScene& S = G.scenes[s];
    if (S.bvh && !S.bvh->nodes.empty()) {
        Ray r;
        std::memcpy(r.org, o, 12);
        std::memcpy(r.dir, d, 12);
        r.tnear = tnear;
        r.tfar = tfar;
        Best b;
        if (trace<false>(*S.bvh, r, b)) {
            const uint64_t k = b.key;
            if (b.t < tfar || cur < best.inst || (cur == best.inst && k < best.key)) {
                tfar = b.t;
                best.t = b.t; best.u = b.u; best.v = b.v;
                best.tri = &S.bvh->tris[size_t(b.tri)];
                best.curve = false;
                best.inst = cur;
                best.key = k;
                best.scene = s;
                best.l2w[0] = chain0;
                best.l2w[1] = nullptr;
                ++best.updates;
            }
        }
    }
    float ct, cu, cng[3];
    uint32_t cp, cg;
    if (orcv::closest(s, o, d, tnear, tfar, ct, cu, cng, cp, cg)) {  // the scene's curves (oracle_curve.cpp)
        const uint64_t k = (uint64_t(cg) << 32) | cp;
        if (ct < tfar || cur < best.inst || (cur == best.inst && k < best.key)) {
            tfar = ct;
            best.t = ct; best.u = cu; best.v = 0.0f;
            best.tri = nullptr;
            best.curve = true;
            std::memcpy(best.cng, cng, 12);
            best.cprim = cp;
            best.cgeom = cg;
            best.inst = cur;
            best.key = k;
            best.scene = s;
            best.l2w[0] = chain0;
            best.l2w[1] = nullptr;
            ++best.updates;
        }
    }
    if (level >= 2) return;
    for (const GInst& in : S.insts) {
        float tmin;
        if (!box_hit(in.box, o, d, tnear, tfar, tmin)) continue;
        float o2[3], d2[3];
        xpoint(in.w2l, o, o2);
        xvector(in.w2l, d, d2);
        if (untraceable(o2, d2)) continue;
        const uint64_t ci = level == 0 ? ((uint64_t(in.id) << 32) | 0xffffffffull) : ((cur & 0xffffffff00000000ull) | in.id);
        const uint64_t before = best.updates;
        gclosest(G, in.proto, o2, d2, tnear, tfar, ci, level + 1, level == 0 ? in.l2w : chain0, best);
        if (level == 1 && best.updates != before) best.l2w[1] = in.l2w;  // the best hit lies in this inner instance
    }
}

bool goccluded(const Graph& G, uint32_t s, const float* o, const float* d, float tnear, float tfar, int level) {
    const GScene& S = G.scenes[s];
    if (S.bvh && !S.bvh->nodes.empty()) {
        Ray r;
        std::memcpy(r.org, o, 12);
        std::memcpy(r.dir, d, 12);
        r.tnear = tnear;
        r.tfar = tfar;
        Best b;
        if (trace<true>(*S.bvh, r, b)) return true;
    }
    if (orcv::occluded(s, o, d, tnear, tfar)) return true;
    if (level >= 2) return false;
    for (const GInst& in : S.insts) {
        float tmin;
        if (!box_hit(in.box, o, d, tnear, tfar, tmin)) continue;
        float o2[3], d2[3];
        xpoint(in.w2l, o, o2);
        xvector(in.w2l, d, d2);
        if (untraceable(o2, d2)) continue;
        if (goccluded(G, in.proto, o2, d2, tnear, tfar, level + 1)) return true;
    }
    return false;
}

}  // namespace

void* build_graph(int n_scenes, const float* verts, const uint32_t* prim, const uint32_t* geom,
                  const uint32_t* tri_scene, int64_t ntri, const float* l2w, const uint32_t* inst_id,
                  const uint32_t* inst_scene, const uint32_t* inst_proto, int64_t ninst, int top) {
    Graph* G = new Graph();
    G->scenes.resize(size_t(std::max(n_scenes, 1)));
    G->top = uint32_t(top);
    std::vector<std::vector<int64_t>> members(G->scenes.size());
    for (int64_t i = 0; i < ntri; ++i) members[tri_scene[i]].push_back(i);
    for (size_t s = 0; s < G->scenes.size(); ++s) {
        if (members[s].empty()) continue;
        std::vector<float> v;
        std::vector<uint32_t> p, g;
        for (int64_t i : members[s]) {
            v.insert(v.end(), verts + 9 * i, verts + 9 * i + 9);
            p.push_back(prim[i]);
            g.push_back(geom[i]);
        }
        G->scenes[s].bvh = static_cast<Bvh*>(oracle_bvh_build(v.data(), p.data(), g.data(), int64_t(p.size())));
    }
    for (int64_t i = 0; i < ninst; ++i) {
        GInst in;
        std::memcpy(in.l2w, l2w + 12 * i, 48);
        oracle_affine_inverse(in.l2w, in.w2l);
        in.id = inst_id[i];
        in.proto = inst_proto[i];
        G->scenes[inst_scene[i]].insts.push_back(in);
    }
    std::vector<int> done(G->scenes.size(), 0);
    for (uint32_t s = 0; s < G->scenes.size(); ++s) scene_bounds(*G, s, done);
    return G;
}

bool closest_graph(const void* g, const float* org, const float* dir, float tnear, float tfar, Hit& out) {
    const Graph& G = *static_cast<const Graph*>(g);
    if (untraceable(org, dir)) return false;
    GBest best;
    gclosest(G, G.top, org, dir, tnear, tfar, ~0ull, 0, nullptr, best);
    if (!best.tri && !best.curve) return false;
    out.t = best.t;
    out.u = best.u;
    out.v = best.v;
    if (best.curve) {
        std::memcpy(out.ng, best.cng, 12);
        out.prim = best.cprim;
        out.geom = best.cgeom;
    } else {
        normal(*best.tri, out.ng);
        out.prim = best.tri->prim;
        out.geom = best.tri->geom;
    }
    out.scene = best.scene;
    out.l2w[0] = best.l2w[0];
    out.l2w[1] = best.l2w[1];
    return true;
}

bool occluded_graph(const void* g, const float* org, const float* dir, float tnear, float tfar) {
    const Graph& G = *static_cast<const Graph*>(g);
    if (untraceable(org, dir)) return false;
    return goccluded(G, G.top, org, dir, tnear, tfar, 0);
}

void release_graph(void* g) { delete static_cast<Graph*>(g); }

}  // namespace orq

extern "C" {

// The render oracle's instanced traversal (per-scene BVHs) on SelRayHit records, to check it against the
// brute-force instanced query.  Arguments as oracle_instanced_query, with local-to-world rows.
void oracle_graph_intersect(int n_scenes, const float* verts, const uint32_t* prim, const uint32_t* geom,
                            const uint32_t* tri_scene, int64_t ntri, const float* l2w, const uint32_t* inst_id,
                            const uint32_t* inst_scene, const uint32_t* inst_proto, int64_t ninst, int top, void* rayhits,
                            int64_t m, int threads) {
    void* g = orq::build_graph(n_scenes, verts, prim, geom, tri_scene, ntri, l2w, inst_id, inst_scene, inst_proto,
                               ninst, top);
    RayHit* rh = static_cast<RayHit*>(rayhits);
    parallel_for(m, threads, [&](int64_t i) {
        orq::Hit h;
        if (!orq::closest_graph(g, rh[i].ray.org, rh[i].ray.dir, rh[i].ray.tnear, rh[i].ray.tfar, h)) return;
        rh[i].ray.tfar = h.t;
        std::memcpy(rh[i].ng, h.ng, 12);
        rh[i].u = h.u;
        rh[i].v = h.v;
        rh[i].prim = h.prim;
        rh[i].geom = h.geom;
        rh[i].inst[0] = rh[i].inst[1] = 0xffffffffu;
    });
    orq::release_graph(g);
}

}  // extern "C"
