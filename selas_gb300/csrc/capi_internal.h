// Handle types behind the opaque C ABI pointers and the shared error helpers.
#pragma once

#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "graph.h"
#include "scene_types.h"
#include "sel_internal.h"

struct SelDeviceTy {
    int cuda_device = 0;
    cudaStream_t stream = nullptr;  // internal stream for the host-memory entry points
    cudaStream_t qstream[4] = {nullptr, nullptr, nullptr, nullptr};  // pipelined host-memory queries (chunk k on k % 4)
    uint32_t* d_err = nullptr;      // kernel error word (iteration cap / stack overflow bits)
    cudaMemPool_t order_pool = nullptr;  // stream-ordered scratch of ordered queries (keeps freed memory)
    bool graph_replay = true;       // SEL_OPTION_GRAPH_REPLAY
    bool material_sort = true;      // SEL_OPTION_MATERIAL_SORT
    bool ray_sort = false;          // SEL_OPTION_RAY_SORT
    bool zero_copy = true;          // SEL_OPTION_ZERO_COPY
    void* noalloc_staging = nullptr;  // device address of sel_intersect1M_noalloc's fixed array on this GPU
    std::mutex mu;
};

struct SelSceneTy {
    SelDeviceTy* dev = nullptr;
    int kind = SEL_BVH_WIDE8_Q8;
    int build_mode = SEL_BUILD_DEVICE;  // 8-wide layout built by GPU kernels (binary: always host)
    uint32_t leaf_size = 3;             // triangles per leaf of the device-built 8-wide layout
    uint32_t tuned_paths_in_flight = 0; // sel_scene_autotune's choices (0: built-in defaults)
    uint32_t tuned_trace_block = 0;
    std::vector<sel::MeshInput> meshes;
    // round B-spline curve geometries (sel_scene_attach_curve_mesh): control points (x, y, z, radius) and the
    // first control point of each segment
    struct CurveInput {
        uint32_t geomID;
        std::vector<float> points;
        std::vector<uint32_t> indices;
    };
    std::vector<CurveInput> curves;
    // instances of other committed scenes (sel_scene_attach_instance): id, instanced scene, transforms
    struct InstanceInput {
        uint32_t instID;
        SelSceneTy* scene;
        float l2w[12], w2l[12];  // rows
    };
    std::vector<InstanceInput> instances;
    void* d_insts = nullptr;                  // InstanceRecord[instances] of the last commit
    void* d_view = nullptr;                   // ShadeView of this scene (allocated by the first commit)
    uint32_t class_mask = 0;                  // material classes of the meshes (bit shader * 4 + Ptex * 2 + transp.)
    bool sort_hint_ptex = false;              // a material of this scene uses Ptex
    uint32_t inst_levels = 0;                 // instance levels below this scene at the last commit (0..2)
    uint32_t stack_need = 0;                  // worst-case instanced-traversal stack entries from here down
    uint64_t generation = 0;                  // incremented by every commit
    std::vector<std::pair<SelSceneTy*, uint64_t>> referenced;  // instanced scenes and their generations
    int instanced_by = 0;                     // committed scenes whose instances reference this one
    bool committed = false;
    void* d_nodes = nullptr;
    void* d_tris = nullptr;
    SelSceneInfo info{};
    void* scratch = nullptr;  // staging buffer of the host-memory query forms
    const unsigned long long* last_rays = nullptr;  // [closest, any] ray counters of the most recent render
    size_t scratch_bytes = 0;

    // shading data (materials indexed by geomID, quad-light sets, background) and its HBM copies
    std::vector<sel::MaterialDev> materials;
    std::vector<std::vector<sel::QuadLight>> light_sets;
    float background[3] = {1.0f, 1.0f, 1.0f};  // backgroundIntensity default (CSceneBuildProcessor.cpp:59)
    // image-based light (sel_scene_set_ibl): RGB images, densities built on upload
    std::vector<float> ibl_light, ibl_miss;
    uint32_t ibl_w = 0, ibl_h = 0, ibl_mw = 0, ibl_mh = 0;
    float ibl_rotation = 0.0f, ibl_exposure = 1.0f;
    void* d_ibl = nullptr;  // IblDev followed by its arrays (null: no image)
    void* d_attrs = nullptr;  // MeshAttrDev table by geomID, then the index, normal and tangent arrays
    uint32_t attr_count = 0;
    bool shading_dirty = true;
    struct PtexBinding {
        uint32_t geomID;
        bool quads = false;               // sel_scene_set_ptex_quads: faces hold PtexQuadFace records
        std::vector<SelPtexFace> faces;   // 32-byte face records (triangle faces or quad faces)
        std::vector<uint16_t> texels;
    };
    std::vector<PtexBinding> ptex;
    struct TextureBinding {  // sel_scene_set_texture: a 2D base-colour image, RGBA floats
        uint32_t geomID, width, height;
        std::vector<float> rgba;
    };
    std::vector<TextureBinding> textures;
    void* d_textures = nullptr;  // their texels, one block
    bool tex2d = false;          // a material samples one (set by the shading upload)
    void* d_ptex_faces = nullptr;
    void* d_ptex_texels = nullptr;
    uint32_t ptex_face_count = 0;
    uint32_t sort_hint = 0;  // Ptex materials or more than one material class among the meshes
    void* d_materials = nullptr;
    void* d_lights = nullptr;
    void* d_light_sets = nullptr;
    // path-tracer scratch: path state for `pt_capacity` paths and the FP64 accumulator
    void* pt_block = nullptr;
    uint32_t pt_capacity = 0;
    void* d_accum = nullptr;
    size_t accum_bytes = 0;
    // VCM scratch: light vertices, hash grid and constants table for `vcm_paths` paths per pass
    void* vcm_block = nullptr;
    uint32_t vcm_paths = 0, vcm_len = 0, vcm_passes = 0;
    // captured per-batch / per-pass launch graphs of the integrators
    sel::GraphCache pt_graph, vcm_graph;
    // scenes released with this one, after it (sel_scene_load_cooked: the subscene and model scenes)
    std::vector<SelSceneTy*> owned;
    std::mutex mu;
};

namespace sel {
struct DeviceBvh;
struct PtCamera;
struct PtScene;
struct VcmConsts;
struct VcmSettings;
// render_capi.cu
int sync_shading(SelSceneTy* sc);              // uploads materials, lights, Ptex and the IBL when they changed
// sel_scene_set_material with the eTransparent flag given instead of derived (cooked materials keep theirs)
int set_material_flags(SelSceneTy* sc, unsigned int geomID, const SelMaterial& material, bool transparent);
// The Ptex writer's constant and constant-neighbourhood flags of `count` PtexQuadFace records (ptex_quad.cuh)
void flag_constant_quads(void* records, size_t count, const uint16_t* texels);
// curve.cu: replaces *d_tris (`records` leaf records) by a copy followed by the segments' control points (nseg x
// 16 floats) and points each kTriCurve record at its segment (geoms[k] / bases[k]: geomID and first segment)
cudaError_t attach_curve_data(void** d_tris, uint64_t records, const float* data, size_t nseg, const uint32_t* geoms,
                              const uint32_t* bases, uint32_t ngeoms);
// capi.cpp: `top` releases `scenes` (created after the scenes they instance) when it is released
void adopt_scenes(SelSceneTy* top, const std::vector<SelSceneTy*>& scenes);
// CalculateIntensityMap + CalculateStrataDistributionFunctions (BuildImageBasedLight.cpp:18-107): marginal CDF
// (height) and conditional CDFs (width x height) of sin(theta) x luma of an RGB latitude-longitude image.
void ibl_densities(const float* rgb, uint32_t width, uint32_t height, std::vector<float>& mdf, std::vector<float>& cdf);
PtScene scene_view(const SelSceneTy* sc);       // device pointers of a committed, synced scene
float vcm_default_radius(const SelSceneTy* sc);
void vcm_constants(float radius0, float alpha, uint32_t paths, bool merging, uint32_t pass, VcmConsts& c);
void vcm_lights(const SelSceneTy* sc, VcmSettings& set);
int check_render_args(SelScene scene, const SelCamera* camera, const SelPtSettings* settings);
// capi.cpp: every scene instanced (directly or below) is still the one committed when `sc` was committed
bool instances_fresh(const SelSceneTy* sc);
// Deferred path tracer: check_render_args plus samplesPerPixel = m * m (m <= 256) and maxBounces 1..1024.
int check_deferred_args(SelScene scene, const SelCamera* camera, const SelPtSettings* settings);
uint32_t deferred_axis(const SelPtSettings& settings);
int check_vcm_args(SelScene scene, const SelCamera* camera, const SelVcmSettings* settings);
int check_vcm_materials(const SelSceneTy* scene);  // after sync_shading: material tables below 2^56
void init_camera(const SelCamera& c, PtCamera& out);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
int set_device(SelDeviceTy* dev);
int read_error_word(SelDeviceTy* dev, cudaStream_t s);
DeviceBvh device_bvh(const SelSceneTy* sc);
// noalloc.cu: looks up the device address of the fixed staging array on dev's GPU (dev's device current)
int resolve_noalloc_staging(SelDeviceTy* dev);
}  // namespace sel
