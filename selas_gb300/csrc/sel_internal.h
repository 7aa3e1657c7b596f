// Internal declarations shared by the host-side builder (bvh_build.cpp) and the CUDA translation units.
// Nothing here crosses the C ABI.
#pragma once

#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/selas.h"

namespace sel {

// ---------------------------------------------------------------------------------------------------
// Acceleration-structure layouts in HBM
// ---------------------------------------------------------------------------------------------------

// Triangle record, 48 bytes = 3 x float4, in the leaf order of the BVH that references it.
//   v0.xyz, w = primID (bits)      v1.xyz, w = geomID (bits)      v2.xyz, w = 0
struct TriRecord {
    float v0[3]; uint32_t prim;
    float v1[3]; uint32_t geom;
    float v2[3]; uint32_t kind;  // kTriPlain, or kTriQuadHalf: prim = 2 * quad + half (half 0: v0 v1 v3, 1: v2 v3 v1)
};
constexpr uint32_t kTriPlain = 0u;
constexpr uint32_t kTriQuadHalf = 1u;
// a round B-spline curve segment (curve.cuh): v0.x / v0.y hold the byte offset from the record to its four
// control points; while the BVH is built, v0 / v1 are the corners of the segment's box
constexpr uint32_t kTriCurve = 2u;
static_assert(sizeof(TriRecord) == 48, "TriRecord must be 48 bytes");

// 8-wide node with child boxes quantised to 8 bits per axis (80 bytes = 5 x uint4).
//   origin p (float3), per-axis exponent byte e (scale = 2^(e-127)), internal-child mask imask,
//   child_base (index of the first internal child; internal children are contiguous in slot order),
//   tri_base (index of the first triangle; leaf children are contiguous),
//   meta[8]: leaf slot -> ((count - 1) << 5) | offset, count in 1..8, offset + count <= 32 (a node's leaf
//   children hold 32 records at most); kLeafNone (0xff) for internal and empty slots,
//   qlo/qhi[axis][8]: child box = p + scale * q, rounded outward when built.
struct WideNode {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(WideNode) == 80, "WideNode must be 80 bytes");
constexpr uint32_t kLeafNone = 0xffu;       // WideNode::meta of a slot that is not a leaf
constexpr uint32_t kMaxNodeRecords = 32u;   // leaf records under one node (the traversal's 32-bit record mask)
constexpr uint32_t kMaxLeafRecords = 8u;    // records of one leaf slot

// Binary node with FP32 child boxes (64 bytes = 4 x float4):
//   [c0.lo.x c0.hi.x c0.lo.y c0.hi.y] [c1.lo.x c1.hi.x c1.lo.y c1.hi.y] [c0.lo.z c0.hi.z c1.lo.z c1.hi.z]
//   [ref0 ref1 count0 count1]: ref >= 0 and count == 0 -> internal node index; count > 0 -> leaf of
//   `count` triangles starting at triangle index ref.
struct BinaryNode {
    float c0x[2], c0y[2];
    float c1x[2], c1y[2];
    float c0z[2], c1z[2];
    int32_t ref[2];
    int32_t count[2];
};
static_assert(sizeof(BinaryNode) == 64, "BinaryNode must be 64 bytes");

// ---------------------------------------------------------------------------------------------------
// Host-side build
// ---------------------------------------------------------------------------------------------------
struct MeshInput {
    uint32_t geomID;
    std::vector<float> vertices;   // xyz packed
    std::vector<uint32_t> indices; // 3 per triangle; a quad mesh holds each quad as two triangles (see quads)
    bool quads = false;            // RTC_GEOMETRY_TYPE_QUAD: triangle 2q is (v0, v1, v3), 2q + 1 is (v2, v3, v1)
    bool curves = false;           // box triangles (lo, hi, lo) standing for curve segments (kTriCurve records)
    std::vector<float> attr[4];    // per-vertex attributes (sel_scene_set_vertex_attribute), attr_n[slot] floats each
    uint32_t attr_n[4] = {0, 0, 0, 0};
};

struct BuiltBvh {
    int kind = SEL_BVH_WIDE8_Q8;
    std::vector<WideNode> wide;
    std::vector<BinaryNode> binary;
    std::vector<TriRecord> tris;
    uint32_t max_depth = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};

// Returns an empty string on success or an error message.
std::string build_bvh(const std::vector<MeshInput>& meshes, int kind, BuiltBvh& out);

// The 8-wide quantised BVH built on the current CUDA device (bvh_device.cu): node and triangle arrays in
// device memory, handed to the caller (cudaFree).
struct DeviceBuild {
    void* d_nodes = nullptr;  // WideNode[node_count]
    void* d_tris = nullptr;   // TriRecord[tri_count], leaf order
    uint32_t node_count = 0, tri_count = 0, max_depth = 0, binary_depth = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    double build_ms = 0.0;    // upload of the triangles + all build kernels
};
std::string build_wide_device(const std::vector<MeshInput>& meshes, uint32_t max_leaf, DeviceBuild& out);

// Traversal stack capacities (entries per thread); the builder rejects trees deeper than these.
constexpr int kWideStack = 24;
constexpr int kBinaryStack = 64;

// ---------------------------------------------------------------------------------------------------
// Instances (two levels, as Embree's RTC_MAX_INSTANCE_LEVEL_COUNT = 2)
// ---------------------------------------------------------------------------------------------------
// An instance enters its parent's BVH as a leaf record whose geomID word is kInstanceGeom and whose primID
// word is the instance's index in the parent's instance table; its vertices (lo, hi, lo) span the world box.
constexpr uint32_t kInstanceGeom = 0xFFFFFFFEu;
// Stack entries per thread of the instanced traversal: the sum over the levels a ray can enter of the tree
// depth, plus 2 per instance level (a pending-leaf entry and a level marker); commit rejects deeper nestings.
constexpr int kInstStack = 40;

// Device record of one instance (144 bytes = 9 x float4), in the parent scene's instance table.
//   w2l: world-to-local affine rows (object point = w2l . (x, y, z, 1)); l2w: local-to-world rows;
//   nodes / tris / insts: the instanced scene's 8-wide BVH, leaf records and own instance table (null: none);
//   shading: the instanced scene's shading view for the integrators (null until its shading data is synced).
struct InstanceRecord {
    float w2l[12];
    float l2w[12];
    const void* nodes;
    const void* tris;
    const InstanceRecord* insts;
    const void* shading;
    uint32_t instID;
    uint32_t pad[3];
};
static_assert(sizeof(InstanceRecord) == 144, "InstanceRecord must be 144 bytes");

// World-to-local rows of an affine local-to-world (rows, 12 floats): the 3 x 3 inverse by cofactors and the
// translation -inv . t, in double, rounded to float.  Returns false when the 3 x 3 part is singular or the
// result is not finite.
bool affine_inverse(const float l2w[12], float w2l[12]);

}  // namespace sel
