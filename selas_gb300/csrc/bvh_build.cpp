// Host-side SAH-binned BVH builder and the two HBM layouts the traversal kernels read.
//
// Replaces the BVH construction that Embree performs inside rtcCommitScene
// (Source/Core/SceneLib/ModelResource.cpp:461-468, SceneResource.cpp:310-312).  Embree's builder is a
// closed binary; this one is written from the published binned-SAH method (Wald 2007, "On fast
// construction of SAH-based bounding volume hierarchies") followed by a greedy binary-to-8-wide
// collapse and 8-bit outward-rounded child-box quantisation in the spirit of Ylitie, Karras and Laine
// (HPG 2017, "Efficient incoherent ray traversal on GPUs through compressed wide BVHs").
//
// The tree shape never changes which triangle a query reports: the closest-hit rule (smallest t, then
// smallest (geomID, primID)) is order independent, and boxes are only ever rounded outward.

#include "sel_internal.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>

namespace sel {
namespace {

constexpr int kBins = 32;
constexpr uint32_t kMaxLeaf = 3;        // triangles per leaf: eight leaf slots stay within a node's 32 records
static_assert(8 * kMaxLeaf <= kMaxNodeRecords, "a node's leaf children must fit its record mask");
constexpr int kMedianDepth = 40;        // beyond this depth split at the object median (bounds depth)
constexpr uint32_t kParallelGrain = 32768;

struct Box {
    float lo[3], hi[3];
    void reset() {
        for (int a = 0; a < 3; ++a) { lo[a] = std::numeric_limits<float>::infinity(); hi[a] = -lo[a]; }
    }
    void grow(const Box& b) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
    }
    void grow(const float* p) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
    }
    bool empty() const { return lo[0] > hi[0]; }
    float area() const {
        if (empty()) return 0.0f;
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct Prim {
    Box box;
    float c[3];
    uint32_t tri;  // index into the flat triangle list
};

struct Node2 {
    Box box;
    int32_t left = -1, right = -1;  // node indices (internal)
    uint32_t first = 0, count = 0;  // prim range (leaf when count > 0)
};

struct FlatTri {
    float v[3][3];
    uint32_t prim, geom, kind;
};

class BinaryBuilder {
public:
    BinaryBuilder(std::vector<Prim>& prims) : prims_(prims) {
        nodes_.resize(std::max<size_t>(1, 2 * prims.size()));
        unsigned hw = std::thread::hardware_concurrency();
        spare_threads_ = hw > 1 ? int(hw) - 1 : 0;
    }

    // Builds the subtree of prims [first, first+count) into node slot `slot`; the subtree's nodes
    // occupy slots [slot, slot + 2*count - 1), so index assignment is deterministic under threading.
    void build(uint32_t slot, uint32_t first, uint32_t count, int depth) {
        Node2& node = nodes_[slot];
        Box box, cbox;
        box.reset();
        cbox.reset();
        for (uint32_t i = first; i < first + count; ++i) {
            box.grow(prims_[i].box);
            cbox.grow(prims_[i].c);
        }
        node.box = box;
        update_depth(depth);

        if (count <= 1) { make_leaf(node, first, count); return; }

        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (cbox.hi[a] - cbox.lo[a] > cbox.hi[axis] - cbox.lo[axis]) axis = a;
        const bool degenerate = !(cbox.hi[axis] > cbox.lo[axis]);

        uint32_t mid = first;
        if (degenerate || depth >= kMedianDepth) {
            if (count <= kMaxLeaf) { make_leaf(node, first, count); return; }
            mid = first + count / 2;
            if (!degenerate) {
                std::nth_element(prims_.begin() + first, prims_.begin() + mid, prims_.begin() + first + count,
                                 [axis](const Prim& a, const Prim& b) { return a.c[axis] < b.c[axis]; });
            }
        } else {
            // Binned SAH over all three axes.
            float best_cost = std::numeric_limits<float>::infinity();
            int best_axis = -1, best_bin = -1;
            for (int a = 0; a < 3; ++a) {
                float ext = cbox.hi[a] - cbox.lo[a];
                if (!(ext > 0.0f)) continue;
                float k = float(kBins) * (1.0f - 1e-6f) / ext;
                Box bb[kBins];
                uint32_t bc[kBins] = {};
                for (int b = 0; b < kBins; ++b) bb[b].reset();
                for (uint32_t i = first; i < first + count; ++i) {
                    int b = int((prims_[i].c[a] - cbox.lo[a]) * k);
                    b = std::min(std::max(b, 0), kBins - 1);
                    bb[b].grow(prims_[i].box);
                    bc[b]++;
                }
                float right_area[kBins];
                uint32_t right_count[kBins];
                Box acc;
                acc.reset();
                uint32_t n = 0;
                for (int b = kBins - 1; b > 0; --b) {
                    acc.grow(bb[b]);
                    n += bc[b];
                    right_area[b] = acc.area();
                    right_count[b] = n;
                }
                acc.reset();
                n = 0;
                for (int b = 0; b < kBins - 1; ++b) {
                    acc.grow(bb[b]);
                    n += bc[b];
                    if (n == 0 || right_count[b + 1] == 0) continue;
                    float cost = acc.area() * float(n) + right_area[b + 1] * float(right_count[b + 1]);
                    if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = b; }
                }
            }
            const float parent_area = box.area();
            const float leaf_cost = parent_area * float(count);
            const float split_cost = parent_area + best_cost;  // traversal cost ~ one box test
            if (count <= kMaxLeaf && (best_axis < 0 || split_cost >= leaf_cost)) {
                make_leaf(node, first, count);
                return;
            }
            if (best_axis >= 0) {
                float ext = cbox.hi[best_axis] - cbox.lo[best_axis];
                float k = float(kBins) * (1.0f - 1e-6f) / ext;
                float lo = cbox.lo[best_axis];
                int a = best_axis, split = best_bin;
                auto it = std::partition(prims_.begin() + first, prims_.begin() + first + count,
                                         [=](const Prim& p) {
                                             int b = int((p.c[a] - lo) * k);
                                             b = std::min(std::max(b, 0), kBins - 1);
                                             return b <= split;
                                         });
                mid = uint32_t(it - prims_.begin());
            }
            if (mid == first || mid == first + count) {
                mid = first + count / 2;
                std::nth_element(prims_.begin() + first, prims_.begin() + mid, prims_.begin() + first + count,
                                 [axis](const Prim& a, const Prim& b) { return a.c[axis] < b.c[axis]; });
            }
        }

        const uint32_t nl = mid - first, nr = count - nl;
        const uint32_t left_slot = slot + 1, right_slot = slot + 2 * nl;
        node.left = int32_t(left_slot);
        node.right = int32_t(right_slot);
        node.count = 0;

        bool spawned = false;
        std::thread worker;
        if (nl > kParallelGrain && nr > kParallelGrain) {
            int avail = spare_threads_.fetch_sub(1);
            if (avail > 0) {
                worker = std::thread([=] { build(left_slot, first, nl, depth + 1); });
                spawned = true;
            } else {
                spare_threads_.fetch_add(1);
            }
        }
        if (!spawned) build(left_slot, first, nl, depth + 1);
        build(right_slot, mid, nr, depth + 1);
        if (spawned) {
            worker.join();
            spare_threads_.fetch_add(1);
        }
    }

    std::vector<Node2>& nodes() { return nodes_; }
    int max_depth() const { return max_depth_.load(); }

private:
    void make_leaf(Node2& node, uint32_t first, uint32_t count) {
        node.left = node.right = -1;
        node.first = first;
        node.count = count;
    }
    void update_depth(int d) {
        int cur = max_depth_.load();
        while (d + 1 > cur && !max_depth_.compare_exchange_weak(cur, d + 1)) {}
    }

    std::vector<Prim>& prims_;
    std::vector<Node2> nodes_;
    std::atomic<int> spare_threads_{0};
    std::atomic<int> max_depth_{0};
};

// ---------------------------------------------------------------------------------------------------
// 8-wide collapse + quantisation
// ---------------------------------------------------------------------------------------------------
class WideCollapser {
public:
    WideCollapser(const std::vector<Node2>& n2, const std::vector<Prim>& prims, const std::vector<FlatTri>& tris,
                  BuiltBvh& out)
        : n2_(n2), prims_(prims), tris_(tris), out_(out) {}

    std::string run() {
        out_.wide.clear();
        out_.tris.clear();
        out_.wide.resize(1);
        max_depth_ = 0;
        std::string err = fill(0, 0, 1);
        out_.max_depth = uint32_t(max_depth_);
        return err;
    }

private:
    bool is_leaf(int n) const { return n2_[n].count > 0; }

    std::string fill(uint32_t wide_index, int n2_index, int depth) {
        max_depth_ = std::max(max_depth_, depth);
        if (depth > kWideStack) return "8-wide BVH deeper than the traversal stack";
        int children[8];
        int nc = 0;
        if (is_leaf(n2_index)) {
            children[nc++] = n2_index;
        } else {
            children[nc++] = n2_[n2_index].left;
            children[nc++] = n2_[n2_index].right;
            while (nc < 8) {
                int best = -1;
                float best_area = -1.0f;
                for (int i = 0; i < nc; ++i) {
                    if (is_leaf(children[i])) continue;
                    float a = n2_[children[i]].box.area();
                    if (a > best_area) { best_area = a; best = i; }
                }
                if (best < 0) break;
                int opened = children[best];
                children[best] = n2_[opened].left;
                children[nc++] = n2_[opened].right;
            }
        }

        // Slot assignment: the child whose centroid lies furthest along octant direction D(s) takes slot s,
        // D(s) = (s&4 ? +1 : -1, s&2 ? +1 : -1, s&1 ? +1 : -1).  A ray whose direction has sign mask o
        // (bit set for a negative component) meets slot o first, so traversal visits slots in
        // ascending (slot ^ o) order.
        Box nb;
        nb.reset();
        for (int i = 0; i < nc; ++i) nb.grow(n2_[children[i]].box);
        float pc[3];
        for (int a = 0; a < 3; ++a) pc[a] = 0.5f * (nb.lo[a] + nb.hi[a]);
        struct Cand { float cost; int child, slot; };
        Cand cands[64];
        int ncand = 0;
        for (int i = 0; i < nc; ++i) {
            const Box& b = n2_[children[i]].box;
            float off[3];
            for (int a = 0; a < 3; ++a) off[a] = 0.5f * (b.lo[a] + b.hi[a]) - pc[a];
            for (int s = 0; s < 8; ++s) {
                float d = (s & 4 ? off[0] : -off[0]) + (s & 2 ? off[1] : -off[1]) + (s & 1 ? off[2] : -off[2]);
                cands[ncand++] = {-d, i, s};
            }
        }
        std::stable_sort(cands, cands + ncand, [](const Cand& x, const Cand& y) { return x.cost < y.cost; });
        int slot_child[8];
        bool child_done[8] = {};
        for (int s = 0; s < 8; ++s) slot_child[s] = -1;
        for (int k = 0; k < ncand; ++k) {
            const Cand& c = cands[k];
            if (child_done[c.child] || slot_child[c.slot] >= 0) continue;
            slot_child[c.slot] = children[c.child];
            child_done[c.child] = true;
        }

        WideNode node;
        std::memset(&node, 0, sizeof(node));
        std::memset(node.meta, int(kLeafNone), sizeof(node.meta));
        quantise(nb, slot_child, node);

        // internal children: contiguous block in slot order
        int internal_n2[8];
        int ni = 0;
        for (int s = 0; s < 8; ++s) {
            int c = slot_child[s];
            if (c >= 0 && !is_leaf(c)) {
                node.imask |= uint8_t(1u << s);
                internal_n2[ni++] = c;
            }
        }
        node.child_base = uint32_t(out_.wide.size());
        out_.wide.resize(out_.wide.size() + ni);

        // leaf children: triangles appended in slot order
        node.tri_base = uint32_t(out_.tris.size());
        uint32_t offset = 0;
        for (int s = 0; s < 8; ++s) {
            int c = slot_child[s];
            if (c < 0 || !is_leaf(c)) continue;
            const Node2& leaf = n2_[c];
            node.meta[s] = uint8_t(((leaf.count - 1u) << 5) | offset);
            for (uint32_t k = 0; k < leaf.count; ++k) {
                const FlatTri& t = tris_[prims_[leaf.first + k].tri];
                TriRecord r;
                std::memcpy(r.v0, t.v[0], 12);
                std::memcpy(r.v1, t.v[1], 12);
                std::memcpy(r.v2, t.v[2], 12);
                r.prim = t.prim;
                r.geom = t.geom;
                r.kind = t.kind;
                out_.tris.push_back(r);
            }
            offset += leaf.count;
        }
        out_.wide[wide_index] = node;

        for (int i = 0; i < ni; ++i) {
            std::string err = fill(node.child_base + i, internal_n2[i], depth + 1);
            if (!err.empty()) return err;
        }
        return "";
    }

    // Child boxes are stored strictly larger than their true boxes: the node origin p sits one quantum
    // below the node box and every child bound is pushed out by at least half a quantum more than the
    // rounding needs.  The quantum is at least 2^-20 of the node's coordinate magnitude and 2^-60
    // absolute, so a ray whose direction has a zero component and whose origin lies on a true box face
    // still sees an open slab with the clamped reciprocal used by the traversal.
    void quantise(const Box& nb, const int* slot_child, WideNode& node) {
        for (int a = 0; a < 3; ++a) {
            const double ext = double(nb.hi[a]) - double(nb.lo[a]);
            const double mag = std::max(std::fabs(double(nb.lo[a])), std::fabs(double(nb.hi[a])));
            const double min_q = std::max(std::ldexp(mag, -20), std::ldexp(1.0, -60));
            int e;
            std::frexp(std::max(ext / 250.0, min_q), &e);  // 2^e >= max(ext/250, min_q)
            for (;; ++e) {
                const double scale = std::ldexp(1.0, e);
                float p = float(double(nb.lo[a]) - scale);
                if (double(p) > double(nb.lo[a]) - scale) p = std::nextafter(p, -INFINITY);
                bool ok = true;
                for (int s = 0; s < 8; ++s) {
                    const int c = slot_child[s];
                    if (c < 0) {
                        node.qlo[a][s] = 255;
                        node.qhi[a][s] = 0;
                        continue;
                    }
                    const Box& b = n2_[c].box;
                    double lo = std::floor((double(b.lo[a]) - p) / scale) - 1.0;
                    double hi = std::ceil((double(b.hi[a]) - p) / scale) + 1.0;
                    while (lo > 0.0 && double(p) + lo * scale > double(b.lo[a]) - 0.5 * scale) lo -= 1.0;
                    while (double(p) + hi * scale < double(b.hi[a]) + 0.5 * scale) hi += 1.0;
                    if (lo < 0.0 || hi > 255.0 || double(p) + lo * scale > double(b.lo[a]) - 0.5 * scale) {
                        ok = false;
                        break;
                    }
                    node.qlo[a][s] = uint8_t(lo);
                    node.qhi[a][s] = uint8_t(hi);
                }
                if (ok) {
                    node.p[a] = p;
                    node.e[a] = uint8_t(e + 127);
                    break;
                }
            }
        }
    }

    const std::vector<Node2>& n2_;
    const std::vector<Prim>& prims_;
    const std::vector<FlatTri>& tris_;
    BuiltBvh& out_;
    int max_depth_ = 0;
};

// ---------------------------------------------------------------------------------------------------
// Binary FP32 layout
// ---------------------------------------------------------------------------------------------------
std::string emit_binary(const std::vector<Node2>& n2, const std::vector<Prim>& prims, const std::vector<FlatTri>& tris,
                        int depth2, BuiltBvh& out) {
    if (depth2 > kBinaryStack) return "binary BVH deeper than the traversal stack";
    out.binary.clear();
    out.tris.clear();
    out.tris.reserve(prims.size());
    for (const Prim& p : prims) {
        const FlatTri& t = tris[p.tri];
        TriRecord r;
        std::memcpy(r.v0, t.v[0], 12);
        std::memcpy(r.v1, t.v[1], 12);
        std::memcpy(r.v2, t.v[2], 12);
        r.prim = t.prim;
        r.geom = t.geom;
        r.kind = t.kind;
        out.tris.push_back(r);
    }
    // Renumber reachable internal nodes densely (DFS, left first); a root leaf becomes a node whose
    // first child is that leaf and whose second child is empty.
    std::vector<int32_t> remap(n2.size(), -1);
    std::vector<int> order;
    std::vector<int> stack{0};
    while (!stack.empty()) {
        int n = stack.back();
        stack.pop_back();
        remap[n] = int32_t(order.size());
        order.push_back(n);
        if (n2[n].count == 0) {
            if (n2[n2[n].right].count == 0) stack.push_back(n2[n].right);
            if (n2[n2[n].left].count == 0) stack.push_back(n2[n].left);
        }
    }
    out.binary.resize(order.size());
    // Stored child boxes are padded outward by 2^-20 of the coordinate magnitude (at least 2^-60), so a
    // ray with a zero direction component whose origin lies on a true box face still sees an open slab.
    auto pad_lo = [](float lo, float hi) {
        const double m = std::max(std::ldexp(std::max(std::fabs(double(lo)), std::fabs(double(hi))), -20), std::ldexp(1.0, -60));
        float r = float(double(lo) - m);
        if (double(r) > double(lo) - m) r = std::nextafter(r, -INFINITY);
        return r;
    };
    auto pad_hi = [](float lo, float hi) {
        const double m = std::max(std::ldexp(std::max(std::fabs(double(lo)), std::fabs(double(hi))), -20), std::ldexp(1.0, -60));
        float r = float(double(hi) + m);
        if (double(r) < double(hi) + m) r = std::nextafter(r, INFINITY);
        return r;
    };
    auto set_child = [&](BinaryNode& bn, int k, int c) {
        Box b = n2[c].box;
        for (int a = 0; a < 3; ++a) {
            const float lo = b.lo[a], hi = b.hi[a];
            b.lo[a] = pad_lo(lo, hi);
            b.hi[a] = pad_hi(lo, hi);
        }
        float* cx = k == 0 ? bn.c0x : bn.c1x;
        float* cy = k == 0 ? bn.c0y : bn.c1y;
        float* cz = k == 0 ? bn.c0z : bn.c1z;
        cx[0] = b.lo[0]; cx[1] = b.hi[0];
        cy[0] = b.lo[1]; cy[1] = b.hi[1];
        cz[0] = b.lo[2]; cz[1] = b.hi[2];
        if (n2[c].count > 0) {
            bn.ref[k] = int32_t(n2[c].first);
            bn.count[k] = int32_t(n2[c].count);
        } else {
            bn.ref[k] = remap[c];
            bn.count[k] = 0;
        }
    };
    for (size_t i = 0; i < order.size(); ++i) {
        int n = order[i];
        BinaryNode bn;
        std::memset(&bn, 0, sizeof(bn));
        if (n2[n].count > 0) {
            set_child(bn, 0, n);
            // empty second child: inverted box never hit
            bn.c1x[0] = bn.c1y[0] = bn.c1z[0] = std::numeric_limits<float>::infinity();
            bn.c1x[1] = bn.c1y[1] = bn.c1z[1] = -std::numeric_limits<float>::infinity();
            bn.ref[1] = 0;
            bn.count[1] = -1;  // never entered (box is empty as well)
        } else {
            set_child(bn, 0, n2[n].left);
            set_child(bn, 1, n2[n].right);
        }
        out.binary[i] = bn;
    }
    out.max_depth = uint32_t(depth2);
    return "";
}

}  // namespace

std::string build_bvh(const std::vector<MeshInput>& meshes, int kind, BuiltBvh& out) {
    if (kind != SEL_BVH_WIDE8_Q8 && kind != SEL_BVH_BINARY_FP32) return "unknown BVH kind";
    std::vector<FlatTri> tris;
    size_t total = 0;
    for (const MeshInput& m : meshes) total += m.indices.size() / 3;
    if (total == 0) return "scene has no triangles";
    if (total > (size_t(1) << 31)) return "too many triangles";
    tris.reserve(total);
    for (const MeshInput& m : meshes) {
        const size_t nv = m.vertices.size() / 3;
        const size_t nt = m.indices.size() / 3;
        for (size_t t = 0; t < nt; ++t) {
            FlatTri ft;
            for (int k = 0; k < 3; ++k) {
                uint32_t vi = m.indices[3 * t + k];
                if (vi >= nv) return "triangle index out of range";
                std::memcpy(ft.v[k], &m.vertices[3 * size_t(vi)], 12);
                for (int a = 0; a < 3; ++a)
                    if (!std::isfinite(ft.v[k][a])) return "non-finite vertex";
            }
            ft.prim = uint32_t(t);
            ft.geom = m.geomID;
            ft.kind = m.quads ? kTriQuadHalf : (m.curves ? kTriCurve : kTriPlain);
            tris.push_back(ft);
        }
    }
    // Primitive order is deterministic: geometry order of attachment, then primID.
    std::vector<Prim> prims(tris.size());
    Box scene;
    scene.reset();
    for (size_t i = 0; i < tris.size(); ++i) {
        Prim& p = prims[i];
        p.box.reset();
        for (int k = 0; k < 3; ++k) p.box.grow(tris[i].v[k]);
        for (int a = 0; a < 3; ++a) p.c[a] = 0.5f * (p.box.lo[a] + p.box.hi[a]);
        p.tri = uint32_t(i);
        scene.grow(p.box);
    }
    BinaryBuilder bb(prims);
    bb.build(0, 0, uint32_t(prims.size()), 0);
    for (int a = 0; a < 3; ++a) { out.lo[a] = scene.lo[a]; out.hi[a] = scene.hi[a]; }
    out.kind = kind;
    if (kind == SEL_BVH_WIDE8_Q8) {
        out.binary.clear();
        WideCollapser wc(bb.nodes(), prims, tris, out);
        return wc.run();
    }
    out.wide.clear();
    return emit_binary(bb.nodes(), prims, tris, bb.max_depth(), out);
}

}  // namespace sel
