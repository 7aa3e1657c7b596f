// Host interface of the wavefront path tracer (pt.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "graph.h"

namespace sel {

struct MaterialDev;
struct QuadLight;
struct InstanceRecord;
struct IblDev;
struct MeshAttrDev;

constexpr int kPtCounters = 8;  // [0],[1] queue lengths, [2] shadow queue length, [3],[4] fetch cursors;
                                // [8] holds the current batch size, [32..47] material-class counts,
                                // [48..63] their scatter cursors
constexpr int kPtClasses = 16;
constexpr int kMaxPtJobs = 16;  // jobs sharing one wavefront (shadow records pack the job in 4 bits)

// Scene view the integrators read.
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
    uint32_t sort_hint;  // 1: the scene has Ptex materials or several material classes (sort before shading)
    const InstanceRecord* insts;  // instance table (null: no instances); lights and background stay this scene's
    const IblDev* ibl;            // image-based light (null: the uniform background)
    const MeshAttrDev* attrs;     // vertex attributes by geomID (null: none)
    uint32_t attr_count;
    float lo[3], hi[3];           // bounds (the origin cells of the ray sort)
    uint32_t ray_sort;            // 1: sort each bounce's continuing rays (SEL_OPTION_RAY_SORT)
    uint32_t tex2d;               // 1: a material takes its base colour from a 2D image (kMaterialUsesTexture)
    uint32_t shader_kinds;        // bit s: a material of the scene or the scenes it instances has shader s
    uint32_t ptex_quads;          // 1: a quad mesh of the scene or the scenes it instances has a Ptex texture
};

// RayCastCameraSettings (GeometryLib/Camera.h:24-42) as InitializeRayCastCamera computes it.
struct PtCamera {
    float x[3], y[3], z[3], position[3];
    uint32_t width, height;
};

// Integrator of a job: PathTracer::EvaluatePath, or DeferredPathTracer (DeferredPathTracer.cpp:61-148).
enum : uint32_t { kPtModePath = 0, kPtModeDeferred = 1 };

struct PtSettings {
    uint32_t spp;          // kPtModeDeferred: samples_per_axis^2
    uint32_t max_bounces;  // kPtModeDeferred: cap on path segments (the reference has none)
    uint64_t seed;
    uint32_t mode;
    uint32_t samples_per_axis;  // kPtModeDeferred: correlated multi-jittered pattern m x m
};

// One render job of the shared wavefront (an entry of the device-resident job table).
struct PtJob {
    PtScene scene;
    PtCamera cam;
    uint32_t max_bounces;
    uint32_t mode;              // kPtModePath / kPtModeDeferred
    uint32_t samples_per_axis;  // kPtModeDeferred
    uint32_t pad;
    uint64_t seed;
    uint64_t total;  // paths of the job: width * height * spp
    double* accum;   // kPtModePath: [2][height][width][3]; kPtModeDeferred: [height][width][3]
};

// Device-resident batch control: which paths of each job the next batch takes.  The host writes `next`
// and `quota` when a job enters a slot; k_batch_begin derives count and prefix, k_batch_end advances next.
struct PtControl {
    uint64_t next[kMaxPtJobs];   // paths of the job already issued
    uint32_t quota[kMaxPtJobs];  // paths of the job a batch may take (0: slot idle)
    uint32_t count[kMaxPtJobs];  // paths of the job in the current batch
    uint32_t prefix[kMaxPtJobs + 1];
    uint32_t njobs;              // slots in use: 0..njobs-1
    uint32_t pad[2];
};

// Device-resident path state (structure of arrays), carved from one allocation.
struct PtState {
    float4* ray_o;    // origin, tnear
    float4* ray_d;    // direction, tfar
    float4* thr;      // throughput, isDeltaOnly
    float4* medium;   // phase (0 vacuum / 1 isotropic), extinction
    float4* hit;      // t, u, v, triangle (bits; all ones = miss)
    uint2* hinst;     // instances entered to the hit, as 1 + index in the parent's table (0: none)
    uint32_t* pixel;
    uint32_t* job;    // job slot of the path
    uint64_t* path_id;  // index of the path within its job (its PCG32 stream)
    uint64_t* rng;
    uint32_t* queue[2];
    uint32_t* queue_sorted;  // the current queue ordered by material class (counting sort; textured scenes:
                             // class, then Ptex face, by radix sort)
    uint32_t* cls;    // material class of each current queue entry
    float4* base;     // Ptex base colour (authored, before the 2.2 power) of the path's current hit
    float4* sh_o;     // shadow rays (2 per path slot): origin, tnear
    float4* sh_d;     // direction, tfar
    float4* sh_c;     // contribution, (job << 28 | pixel) bits
    uint32_t* counters;
    unsigned long long* rays;  // [0] closest-hit, [1] any-hit rays traced, running totals
    uint32_t* rkeys[2];       // ray sort: keys and the ping-pong partner of the queue
    uint32_t* rvals;
    uint32_t* rhist;          // digit counts per tile and their scan
    uint32_t* rhist_off;
    uint32_t* rscan_tmp;
    PtControl* control;
    PtJob* jobs;      // job table (kMaxPtJobs entries)
    uint32_t capacity;
};

size_t pt_state_block_bytes(uint32_t paths);
PtState pt_state_carve(void* block, uint32_t paths);

// Launches `batches` batches of the shared wavefront over the jobs in st.jobs / st.control (uploaded by the
// caller).  `bounces` is the number of extend/shade/shadow rounds per batch (the largest max_bounces of the
// jobs).  With `graphs`, one batch is captured as a CUDA graph and replayed.
// `sort`: order each bounce's queue by material class before shading (Ptex is filtered by a kernel of its own
// either way, in shading order).
// `trace_block`: threads per block of the traversal kernels (128, or 256 with the 8-wide layout).
// `modes`: integrators of the jobs, bit 0 kPtModePath, bit 1 kPtModeDeferred.
// `instanced`: a job's scene has instances (the instanced traversal, which also walks flat scenes).
cudaError_t pt_run_batches(int bvh_kind, uint32_t bounces, bool sort, const PtState& st, uint32_t* d_err,
                           uint64_t batches, cudaStream_t stream, GraphCache* graphs, int trace_block = 128,
                           uint32_t modes = 1u, bool instanced = false, bool texture = true, bool ray_sort = false,
                           uint64_t batch_paths = 0, uint32_t shader_kinds = 7u, bool quad_ptex = true);
// `ray_sort`: order each bounce's continuing rays by (direction bin, origin cell) before tracing them.
// `texture`: a job's hits may need Ptex (see pt_scene_textured); the Ptex kernel runs only then.
// `quad_ptex`: a job's scene has quad-mesh Ptex (the Ptex kernel compiled with the quad filter runs only then).
// `shader_kinds`: bit s set when a job's scene has a material of shader s.  Shading runs a kernel compiled for
// one shader: over the whole queue when the jobs have one kind of shader, else per shader over its classes of
// the class-ordered queue (without the class order: one kernel for every shader).
// `batch_paths`: paths a batch holds; with `sort` and `texture`, batches of kFaceOrderPaths or more of flat scenes
// order the textured hits by Ptex face as well (the face order's radix passes cost more than it saves on smaller
// batches, and on the instanced terrain, whose 4 x 4-texel faces filter cheaply: 110.6 against 114.8 M paths/s).
bool pt_scene_textured(const PtScene& sc);

// Batch size from which textured hits are ordered by Ptex face (room at 1280 x 720, 16 spp: 1M paths per batch
// 159.8 against 160.1 ms, 2M 143.5 against 149.6, 4M 134.2 against 143.4, 8M 128.9 against 139.5).
constexpr uint64_t kFaceOrderPaths = 1ull << 21;

// Single render (PathTracer::GenerateImage, or DeferredPathTracer::GenerateImage with set.mode =
// kPtModeDeferred): one job, batches until all its paths are done.
cudaError_t pt_render(const PtScene& sc, const PtCamera& cam, const PtSettings& set, const PtState& st, double* d_accum,
                      uint32_t* d_err, cudaStream_t stream, GraphCache* graphs, int trace_block = 128);
cudaError_t pt_resolve(const double* d_accum, uint32_t values, double scale, float* d_out, cudaStream_t stream);

}  // namespace sel
