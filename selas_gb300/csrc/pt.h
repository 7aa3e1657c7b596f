// Host interface of the wavefront path tracer (pt.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "graph.h"

namespace sel {

struct MaterialDev;
struct QuadLight;

constexpr int kPtCounters = 8;  // [0],[1] queue lengths, [2] shadow queue length, [3],[4] fetch cursors;
                                // [8] holds the current batch size

// Device-resident path state (structure of arrays), carved from one allocation.
struct PtState {
    float4* ray_o;    // origin, tnear
    float4* ray_d;    // direction, tfar
    float4* thr;      // throughput, isDeltaOnly
    float4* medium;   // phase (0 vacuum / 1 isotropic), extinction
    float4* hit;      // t, u, v, triangle (bits; all ones = miss)
    uint32_t* pixel;
    uint32_t* path_id;
    uint64_t* rng;
    uint32_t* queue[2];
    float4* sh_o;     // shadow rays: origin, tnear
    float4* sh_d;     // direction, tfar
    float4* sh_c;     // contribution, pixel (bits)
    uint32_t* counters;
    uint64_t* first;  // first path of the current batch (device-resident, inside the counters block)
    uint32_t capacity;
};

struct PtScene {
    const void* nodes;  // 8-wide quantised (bvh_kind 0) or binary FP32 (bvh_kind 1) node array
    int bvh_kind;
    const float4* tris;
    const MaterialDev* materials;
    uint32_t material_count;
    const QuadLight* lights;
    const uint2* light_sets;
    uint32_t light_set_count;
    const void* ptex_faces;   // PtexFace[] of all bound geometries
    const void* ptex_texels;  // half RGB
    uint32_t ptex_face_count;
    float background[3];
};

// RayCastCameraSettings (GeometryLib/Camera.h:24-42) as InitializeRayCastCamera computes it.
struct PtCamera {
    float x[3], y[3], z[3], position[3];
    uint32_t width, height;
};

struct PtSettings {
    uint32_t spp;
    uint32_t max_bounces;
    uint64_t seed;
};

size_t pt_state_block_bytes(uint32_t paths);
PtState pt_state_carve(void* block, uint32_t paths);
// With `graphs`, one batch of paths is captured as a CUDA graph (once per argument set) and replayed per batch.
cudaError_t pt_render(const PtScene& sc, const PtCamera& cam, const PtSettings& set, const PtState& st, double* d_accum,
                      uint32_t* d_err, cudaStream_t stream, GraphCache* graphs);
cudaError_t pt_resolve(const double* d_accum, uint32_t values, double scale, float* d_out, cudaStream_t stream);

}  // namespace sel
