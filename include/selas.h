/*
 * selas.h - C ABI of the GB300-native Selas render hot path.
 *
 * One shared library, libselas_gb300.so, exports every function declared here.  All functions return
 * an int status (SEL_OK == 0) and never abort; sel_get_last_error() describes the most recent failure
 * on the calling host thread.  No function takes or returns a PyTorch, CUDA-runtime or C++ type:
 * device memory is passed as plain pointers and CUDA streams as void*.
 *
 * Ray/hit records are byte-identical to Embree 3.2's RTCRay / RTCHit / RTCRayHit
 * (Middleware/embree-latest/include/embree3/rtcore_ray.h:26-61), so arrays built for rtcIntersect1M /
 * rtcOccluded1M can be handed to the functions below unchanged.
 */
#ifndef SELAS_GB300_H
#define SELAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------------------------ */
/* Status codes                                                                                      */
/* ------------------------------------------------------------------------------------------------ */
enum {
    SEL_OK = 0,
    SEL_ERR_INVALID_ARGUMENT = 1,  /* null handle, bad size or stride, unknown enum value          */
    SEL_ERR_OUT_OF_MEMORY = 2,     /* device or host allocation failed                             */
    SEL_ERR_CUDA = 3,              /* a CUDA runtime call failed (text in sel_get_last_error)      */
    SEL_ERR_INVALID_OPERATION = 4, /* e.g. query on a scene that was never committed               */
    SEL_ERR_DEVICE_LIMIT = 5,      /* a kernel hit its iteration cap or stack limit and stopped    */
    SEL_ERR_IO = 6                 /* an asset file is missing, unreadable or malformed            */
};

/* Mirrors RTC_INVALID_GEOMETRY_ID and RTC_MAX_INSTANCE_LEVEL_COUNT (rtcore_common.h:66,72). */
#define SEL_INVALID_GEOMETRY_ID ((unsigned int)-1)
#define SEL_MAX_INSTANCE_LEVEL_COUNT 2

/* Layout of RTCRay (rtcore_ray.h:26-43): 48 bytes, 16-byte aligned. */
typedef struct __attribute__((aligned(16))) SelRay {
    float org_x, org_y, org_z;
    float tnear;
    float dir_x, dir_y, dir_z;
    float time;
    float tfar;
    unsigned int mask;
    unsigned int id;
    unsigned int flags;
} SelRay;

/* Layout of RTCHit (rtcore_ray.h:46-57): 36 bytes. */
typedef struct SelHit {
    float Ng_x, Ng_y, Ng_z;
    float u, v;
    unsigned int primID;
    unsigned int geomID;
    unsigned int instID[SEL_MAX_INSTANCE_LEVEL_COUNT];
} SelHit;

/* Layout of RTCRayHit (rtcore_ray.h:59-63): 96 bytes (hit at offset 48). */
typedef struct SelRayHit {
    SelRay ray;
    SelHit hit;
} SelRayHit;

typedef struct SelDeviceTy* SelDevice; /* replaces RTCDevice (rtcore_device.h) */
typedef struct SelSceneTy* SelScene;   /* replaces RTCScene  (rtcore_scene.h)  */

/* Acceleration structure built by sel_scene_commit. */
enum {
    SEL_BVH_WIDE8_Q8 = 0,    /* 8-wide BVH, child bounds quantised to 8 bits per axis, rounded outward */
    SEL_BVH_BINARY_FP32 = 1  /* binary BVH with FP32 child bounds: the plain GPU path                   */
};

typedef struct SelSceneInfo {
    uint64_t triangle_count;
    uint64_t node_count;
    uint64_t device_bytes;     /* nodes + triangles resident in HBM                */
    uint32_t bvh_kind;
    uint32_t max_depth;        /* deepest node level (root = 1)                    */
    double build_ms;           /* host-side SAH build + layout                     */
    double upload_ms;          /* host -> HBM copy                                 */
    float bounds_lo[3];
    float bounds_hi[3];
} SelSceneInfo;

/* ------------------------------------------------------------------------------------------------ */
/* Errors                                                                                            */
/* ------------------------------------------------------------------------------------------------ */
const char* sel_get_last_error(void);

/* ------------------------------------------------------------------------------------------------ */
/* Device lifetime.  Replaces rtcNewDevice / rtcReleaseDevice (rtcore_device.h; called at           */
/* Source/Applications/Selas/Source/main.cpp:99).  cuda_device selects the GPU.                      */
/* ------------------------------------------------------------------------------------------------ */
int sel_device_new(int cuda_device, SelDevice* out_device);
int sel_device_release(SelDevice device);
/* Waits for `stream` and returns SEL_ERR_DEVICE_LIMIT if any kernel of this device raised its error
 * word since the last call (the word is cleared by the call). */
int sel_device_sync(SelDevice device, void* stream);

/* Device options (no reference counterpart: tuning switches of this implementation). */
enum {
    SEL_OPTION_GRAPH_REPLAY = 1,  /* 1 (default): the integrators capture one path batch / VCM pass as a CUDA
                                     graph per argument set and replay it; 0: launch kernel by kernel */
    SEL_OPTION_MATERIAL_SORT = 2, /* 1 (default): before shading, the integrators order each bounce's hits by
                                     material class and filter Ptex in a kernel of their own when the scene has
                                     Ptex or several material classes; 0: shade in queue order */
    SEL_OPTION_RAY_SORT = 3,      /* 1: the path tracers order each bounce's continuing rays by direction bin
                                     (dominant axis and sign) and a Morton code of the origin before tracing
                                     them (PathTracingBatcher.cpp:162-258), and the queries trace batches of
                                     at least 1,048,576 records in HBM (8-wide layout, no instances) in the
                                     order of the direction's octant and a Morton code of the origin, unless
                                     the batch's neighbouring rays run nearly parallel; 0 (default): queue
                                     and record order */
    SEL_OPTION_ZERO_COPY = 4      /* 1 (default): the host-memory queries (sel_intersect1M etc.) trace records
                                     that lie in page-locked host memory the GPU can address (cudaHostAlloc /
                                     cudaHostRegister) in place, the kernel reading rays and writing hits over
                                     the host link, except batches of more than 524,288 records whose rays
                                     run nearly parallel record to record (camera rays: their traversal is
                                     too short to hide the link, so full-duplex staged copies are faster);
                                     0: always stage them through HBM with pipelined copies */
};
int sel_device_set_option(SelDevice device, int option, int value);

/* ------------------------------------------------------------------------------------------------ */
/* Scene lifetime.  Replaces rtcNewScene, rtcNewGeometry(RTC_GEOMETRY_TYPE_TRIANGLE) +               */
/* rtcSetSharedGeometryBuffer + rtcAttachGeometryByID, rtcCommitScene and rtcReleaseScene as used in */
/* Source/Core/SceneLib/ModelResource.cpp:236-297,461-468 and SceneResource.cpp:310-312.            */
/* ------------------------------------------------------------------------------------------------ */
int sel_scene_new(SelDevice device, SelScene* out_scene);
int sel_scene_set_bvh_kind(SelScene scene, int bvh_kind);

/* Where sel_scene_commit builds the BVH (no reference counterpart: Embree builds on the host with TBB).
 * SEL_BUILD_DEVICE (the default) builds the 8-wide layout with GPU kernels (binned SAH, collapse,
 * quantisation); the binary layout is always built on the host.  Results of queries do not depend on the
 * builder. */
enum { SEL_BUILD_HOST = 0, SEL_BUILD_DEVICE = 1 };
int sel_scene_set_build_mode(SelScene scene, int build_mode);
/* Triangles per leaf of the device-built 8-wide layout, 1..8 (default 3; the host builder uses 3).  A node's leaf
 * children hold 32 triangles at most: with leaves above 4, the largest leaves of a node that would hold more
 * move one level down, each into a node of its own. */
int sel_scene_set_leaf_size(SelScene scene, unsigned int leaf_size);
/* vertices: vertex_count records of 3 floats (x,y,z) every vertex_stride_bytes bytes (>= 12);
 * indices: triangle_count x 3 unsigned ints.  The data is copied; the caller may free it after the
 * call.  geomID is reported in SelHit.geomID; primID is the triangle's index within this mesh. */
int sel_scene_attach_triangle_mesh(SelScene scene, unsigned int geomID, const float* vertices,
                                   size_t vertex_count, size_t vertex_stride_bytes,
                                   const unsigned int* indices, size_t triangle_count);
/* Replaces rtcNewGeometry(RTC_GEOMETRY_TYPE_QUAD) + index/vertex buffers, the geometry the reference makes for
 * meshes cooked with four indices per face (Source/Core/SceneLib/ModelResource.cpp:272-281).  indices: 4 per quad.
 * As in Embree (RTC_GEOMETRY_TYPE_QUAD.3embree3) a quad is the triangles (v0, v1, v3) and (v2, v3, v1); a hit
 * reports primID = the quad's index, Ng of the triangle hit, and (u, v) of the quad's parametrisation (the second
 * triangle's (u', v') become (1 - u', 1 - v')), so that p = v0 + u (v1 - v0) + v (v3 - v0) on a planar quad.  Ties
 * on t between the two triangles of one quad go to the first.  Vertex attributes interpolate bilinearly,
 * t_uv = (1 - v)((1 - u) t0 + u t1) + v((1 - u) t3 + u t2).  Fewer than 2^31 quads per mesh; quad meshes take no
 * Ptex texture (the reference filters quad Ptex with the separable bicubic filter, not provided). */
int sel_scene_attach_quad_mesh(SelScene scene, unsigned int geomID, const float* vertices, size_t vertex_count,
                               size_t vertex_stride_bytes, const unsigned int* indices, size_t quad_count);
/* Instances, two levels at most (RTC_MAX_INSTANCE_LEVEL_COUNT = 2): rtcNewGeometry(RTC_GEOMETRY_TYPE_INSTANCE)
 * + rtcSetGeometryInstancedScene + rtcSetGeometryTransform(RTC_FORMAT_FLOAT4X4_COLUMN_MAJOR) +
 * rtcAttachGeometryByID (SubsceneResource.cpp:63-79), and the subscene-instance user geometry whose callbacks
 * transform the ray into the subscene (SceneResource.cpp:73-187).  Attaches `instanced`, a committed scene of
 * the 8-wide layout, to `scene` under instID (unique among the scene's geomIDs and instIDs) with the affine
 * localToWorld (16 floats, column-major, last row 0 0 0 1).  Queries report, for a hit inside instances,
 * instID[0] = the outermost instance's id and instID[1] = the next one's (SEL_INVALID_GEOMETRY_ID where there
 * is none), geomID / primID of the hit mesh within its scene, Ng in that mesh's object space (untransformed,
 * as Embree reports it) and t in the world ray's parametrisation.  `instanced` must stay committed and alive
 * while `scene` uses it (releasing it fails while a committed scene instances it); committing it again
 * requires committing `scene` again.  Scenes with instances use the SEL_BVH_WIDE8_Q8 layout. */
int sel_scene_attach_instance(SelScene scene, unsigned int instID, SelScene instanced, const float* localToWorld);
/* Round B-spline curves: rtcNewGeometry(RTC_GEOMETRY_TYPE_ROUND_BSPLINE_CURVE) + the index buffer (RTC_FORMAT_UINT,
 * one entry per segment) + the vertex buffer (RTC_FORMAT_FLOAT4: x, y, z, radius) (ModelResource.cpp:300-332).
 * Segment k is the uniform cubic B-spline of points indices[k] .. indices[k] + 3, swept by a sphere whose radius
 * follows the same spline.  Embree's curve intersector is closed, so hits are defined here: the segment is cut
 * at u = j / 8 into round cones (the union of spheres of linearly interpolated centre and radius between its
 * pieces' end spheres); a hit reports t, u = the touching sphere's parameter along the segment, v = 0, Ng = hit
 * point - that sphere's centre (object space), primID = k.  Scenes with curves use the 8-wide layout and are
 * traversed by the instanced traversal.  points: point_count x 4 floats; data copied. */
int sel_scene_attach_curve_mesh(SelScene scene, unsigned int geomID, const float* points, size_t point_count,
                                const unsigned int* indices, size_t segment_count);
int sel_scene_commit(SelScene scene);
/* Per-vertex attributes: rtcSetGeometryVertexAttributeCount + rtcSetSharedGeometryBuffer(
 * RTC_BUFFER_TYPE_VERTEX_ATTRIBUTE, slot, RTC_FORMAT_FLOAT<components>) (ModelResource.cpp:183-197).  Slot 0..3
 * of mesh geomID gets vertex_count records of `components` (1..4) floats (copied; vertex_count must equal the
 * mesh's).  As CalculateSurfaceParams reads them (SurfaceParameters.cpp:157-184), the integrators take slot 0
 * (3 floats) as shading normals and slot 1 (4 floats: xyz and the bitangent sign) as tangents; slot 2 holds uvs. */
int sel_scene_set_vertex_attribute(SelScene scene, unsigned int geomID, unsigned int slot, const float* data,
                                   size_t vertex_count, unsigned int components);
/* rtcInterpolate0 (rtcore_geometry.h; called at SurfaceParameters.cpp:162,176,188): attribute `slot` of mesh
 * geomID at barycentrics (u, v) of triangle primID, (1 - u - v) a0 + u a1 + v a2 per component, `count` floats
 * (at most the attribute's components) to out.  Host-side, from the scene's copies. */
int sel_interpolate0(SelScene scene, unsigned int geomID, unsigned int primID, float u, float v, unsigned int slot,
                     float* out, unsigned int count);
int sel_scene_get_info(SelScene scene, SelSceneInfo* out_info);
int sel_scene_release(SelScene scene);

/* ------------------------------------------------------------------------------------------------ */
/* Ray queries.                                                                                      */
/* Closest hit: a triangle is hit when the watertight test of Woop, Benthin and Wald (JCGT 2013)     */
/* accepts it with tnear <= t <= tfar.  Of all hit triangles the one with the smallest t wins; equal */
/* t is decided by the smaller (geomID, primID).  On a hit tfar, Ng = (v1-v0)x(v2-v0), u, v (so that */
/* p = (1-u-v)v0 + u v1 + v v2), primID, geomID are written and instID[0..1] are set to             */
/* SEL_INVALID_GEOMETRY_ID; on a miss the record is left untouched.                                  */
/* Any hit: tfar is set to -inf when some triangle is hit in [tnear, tfar].                          */
/* ------------------------------------------------------------------------------------------------ */

/* Host-memory forms.  Replace rtcIntersect1 / rtcOccluded1 (rtcore_scene.h:94,118; called at        */
/* Source/Applications/Selas/Source/PathTracer.cpp:88,116) and the stream forms rtcIntersect1M /     */
/* rtcOccluded1M (rtcore_scene.h:106,130).  They copy the records to HBM, trace, copy back and       */
/* return when the results are in host memory.                                                       */
int sel_intersect1(SelScene scene, SelRayHit* rayhit);
int sel_occluded1(SelScene scene, SelRay* ray);
int sel_intersect1M(SelScene scene, SelRayHit* rayhits, unsigned int M, size_t byte_stride);
int sel_occluded1M(SelScene scene, SelRay* rays, unsigned int M, size_t byte_stride);

/* Same closest-hit query as sel_intersect1M for callers that must not allocate GPU memory: a host
 * application that owns the GPU's memory through its own pool (a plugin inside a renderer or engine),
 * a real-time loop that cannot risk the device synchronisation cudaMalloc/cudaFree may cause, or code
 * with every byte of HBM budgeted up front.  It has no counterpart in the reference.  The call allocates
 * nothing: it stages records in one fixed array of 65536 SelRayHit records (6 MiB) that every GPU
 * loading the library holds until exit, and rejects M > 65536 with SEL_ERR_INVALID_ARGUMENT.
 * sel_device_new looks up that array's device address (loading the module that holds it), so the query
 * itself loads nothing.  Like every query it refuses, with SEL_ERR_INVALID_OPERATION and before any
 * launch, a scene whose instanced scenes were re-committed after it.  All calls share the array (its contents are whatever the last call left; every call overwrites the
 * records it uses first).  Calls through one SelDevice are serialised; calls through different SelDevice
 * handles on the same GPU that overlap on the GPU race on the array. */
int sel_intersect1M_noalloc(SelScene scene, SelRayHit* rayhits, unsigned int M, size_t byte_stride);

/* Device-memory forms: d_rayhits / d_rays point to HBM, work is queued on `stream` (void* holding a
 * cudaStream_t, NULL = default stream) and the call returns without waiting.  Replace the packet
 * queries rtcIntersect8 / rtcOccluded8 of Source/Applications/Selas/Source/DeferredPathTracer.cpp:191,267
 * for whole ray batches.  Use sel_device_sync to wait and collect kernel errors.  With SEL_OPTION_RAY_SORT,
 * batches of 1,048,576 records or more take stream-ordered scratch for their key sort (16 bytes a record, from a
 * memory pool the SelDevice owns and keeps filled); otherwise the calls allocate nothing. */
int sel_intersect_device(SelScene scene, SelRayHit* d_rayhits, unsigned int n, void* stream);
int sel_occluded_device(SelScene scene, SelRay* d_rays, unsigned int n, void* stream);

/* ------------------------------------------------------------------------------------------------ */
/* BSDF evaluation and sampling (device memory, asynchronous on `stream`).                           */
/* ------------------------------------------------------------------------------------------------ */

/* Shader kinds: ShaderType (Source/Core/SceneLib/ModelResource.h:27-34). */
enum { SEL_SHADER_DISNEY_THIN = 0, SEL_SHADER_DISNEY_SOLID = 1, SEL_SHADER_DIRAC_TRANSPARENT = 2 };
/* Event flags: SurfaceEventFlags (Source/Core/Shading/Scattering.h:12-17). */
enum { SEL_EVENT_SCATTER = 1, SEL_EVENT_TRANSMISSION = 2, SEL_EVENT_DIRAC = 4 };

/* A shading point: the fields of SurfaceParameters (Source/Core/Shading/SurfaceParameters.h:15-48) that
 * the BSDF reads.  tangent/normal/bitangent are the world-space rows of tangentToWorld (worldToTangent is
 * their transpose); baseColor is linear; diffTrans is the halved value CalculateSurfaceParams stores.
 * 128 bytes. */
typedef struct SelSurface {
    float tangent[3], normal[3], bitangent[3];
    float baseColor[3];
    float transmittanceColor[3];
    float sheen, sheenTint, clearcoat, clearcoatGloss;
    float metallic, specTrans, diffTrans, flatness;
    float anisotropic, relativeIOR, specularTint, roughness;
    float scatterDistance, ior;
    int32_t shader;
    float pad[2];
} SelSurface;

/* EvaluateBsdf (Source/Core/Shading/SurfaceScattering.h:16): for each i, wo[i] (toward the viewer) and
 * wi[i] (toward the light) are 3 floats; out[5*i..] = f.x f.y f.z forwardPdfW reversePdfW, where f already
 * includes |cos(theta_i)| as in the reference. */
int sel_bsdf_evaluate_device(const SelSurface* d_surfaces, const float* d_wo, const float* d_wi, unsigned int n,
                             float* d_out, void* stream);
/* SampleBsdfFunction (Source/Core/Shading/SurfaceScattering.h:15) with the sampler's uniforms given
 * explicitly: u[4*i..4*i+3] are consumed in the order the reference draws them.  out[16*i..] = success
 * flags reflectance[3] wi[3] forwardPdfW reversePdfW mediumPhase extinction[3] uniformsUsed 0. */
int sel_bsdf_sample_device(const SelSurface* d_surfaces, const float* d_wo, const float* d_u, unsigned int n,
                           float* d_out, void* stream);

/* Shading probes (no counterpart in the reference: diagnostic entry points that run the integrators' own device
 * functions on given inputs, so that each step can be compared with the reference's function of the same name on
 * identical inputs).  All take a committed scene without instances; buffers are device memory, work is queued on
 * `stream`.
 *
 * CalculateSurfaceParams + OffsetRayOrigin (Source/Core/Shading/SurfaceParameters.cpp:144-247,403-408) on hits as
 * RayPick forms them (Source/Applications/Selas/Source/PathTracer.cpp:122-136): d_hits n x 12 floats (position,
 * Ng, ray direction, u, v, t), d_ids n x 2 (geomID, primID).  d_out n x 40 floats: worldToTangent rows (9),
 * baseColor (3, after Ptex / 2D image and the power 2.2), transmittanceColor (3), sheen, sheenTint, clearcoat,
 * clearcoatGloss, metallic, specTrans, diffTrans, flatness, anisotropic, specularTint, roughness, scatterDistance,
 * ior, relativeIOR, error, shader, materialFlags (eTransparent 1 | eUsesPtex 16), lightSetIndex, the bounce
 * origin OffsetRayOrigin(-d, 1) (3), the shadow origin OffsetRayOrigin(-d, 0.1) (3), 0. */
int sel_surface_probe_device(SelScene scene, const float* d_hits, const unsigned int* d_ids, unsigned int n,
                             float* d_out, void* stream);
/* NextEventEstimation (Source/Core/Shading/AreaLighting.cpp:113-153,353-373) with its three uniforms given:
 * d_points n x 6 (position, normal), d_light_sets n, d_u n x 3 (light pick, spherical-rectangle u, v).
 * d_out n x 9: direction, radiance, distance, pdfW, light index in the set; zeros without a light. */
int sel_light_probe_device(SelScene scene, const float* d_points, const unsigned int* d_light_sets, const float* d_u,
                           unsigned int n, float* d_out, void* stream);
/* The scene's image-based light: Ibl + SphericalToCartesian + SampleIbl(x, y)
 * (Source/Core/SceneLib/ImageBasedLightResource.cpp:118-151,264-267) for n uniform pairs d_r -> d_samples n x 7
 * (direction, radiance, pdf); SampleIBlPdf, SampleIbl(wi), SampleIblMiss(wi) (:154-261) for m directions
 * d_dirs -> d_eval m x 7 (pdf, radiance, miss radiance). */
int sel_ibl_probe_device(SelScene scene, const float* d_r, unsigned int n, float* d_samples, const float* d_dirs,
                         unsigned int m, float* d_eval, void* stream);

/* ------------------------------------------------------------------------------------------------ */
/* Shading data of a scene.                                                                          */
/* ------------------------------------------------------------------------------------------------ */

/* The MaterialResourceData fields the renderer reads (Source/Core/SceneLib/ModelResource.h:68-88), with
 * the scalar attributes in eMaterialProperty order (Source/Core/BuildCommon/ImportMaterial.cpp:36-52).
 * baseColor is as authored: shading raises it to the power 2.2 (Shading/SurfaceParameters.cpp:210-212).
 * The transparent flag is derived as the reference's build step does (BuildCommon/BuildModel.cpp:60-65). */
typedef struct SelMaterial {
    int32_t shader;
    uint32_t lightSetIndex;
    float baseColor[3];
    float transmittanceColor[3];
    float metallic, specularTint, roughness, anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss;
    float specTrans, diffuseTrans, flatness, ior, scatterDistance;
    uint32_t usesPtex;   /* 1: base colour from the geometry's per-face Ptex texels */
} SelMaterial;

/* Fills the reference's default material (CreateDefaultMaterial, SceneLib/ModelResource.cpp:203-211). */
int sel_material_defaults(SelMaterial* out);
/* Material of geometry geomID (geomID < 65536); geometries without one use the default material. */
int sel_scene_set_material(SelScene scene, unsigned int geomID, const SelMaterial* material);

/* A material from the text of one material JSON file (ImportMaterial, BuildCommon/ImportMaterial.cpp:56-88, then
 * BuildMaterial, BuildCommon/BuildModel.cpp:22-64): "shaderName" (DisneyThin, DisneySolid or DeltaTransparent,
 * any case; DisneySolid otherwise), "baseColor" ([r, g, b], default 0.6 grey; a string names a texture, written
 * NUL-terminated to base_color_texture (truncated to texture_capacity - 1 bytes, may be null) with the colour left
 * 0.6 grey), "transmittanceColor" (default 0), the scalar attributes with the importer's defaults (metallic 0.3,
 * roughness 0.5, ior 1.5, the others 0; a string there names a texture, which is not sampled: the default is
 * kept), "usesPtex" (default false).  alphaTesting, invertDisplacement and displacement have no use here.
 * Malformed JSON or a document that is not an object: SEL_ERR_INVALID_ARGUMENT, with the offset in the message.
 * Needs no device. */
int sel_material_from_json(const char* json, SelMaterial* out, char* base_color_texture, unsigned int texture_capacity);

/* One entry of a Disney-island materials file. */
typedef struct SelNamedMaterial {
    char name[64];        /* material or assignment name, NUL-terminated (truncated to 63 bytes) */
    SelMaterial material;
    char colorMap[256];   /* Ptex path with '/' separators ("" when the material has none) */
} SelNamedMaterial;

/* The materials of a Disney-island materials file (ImportDisneyMaterials, ImportMaterial.cpp:91-146, then
 * BuildMaterial): an object of named materials, each with "baseColor" (default 1), the scalar attributes (the
 * importer's defaults), "type" ("solid": DisneySolid, else DisneyThin), an optional "colorMap" (usesPtex when
 * non-empty) and an optional "assignment" array of further names that take the same material; transmittance
 * colour 1.  Entries are written in document order, each material followed by its assignment names; *count
 * receives the number of entries, of which the first `capacity` are written (call with capacity 0 to size
 * `out`).  Needs no device. */
int sel_disney_materials_from_json(const char* json, SelNamedMaterial* out, unsigned int capacity, unsigned int* count);

/* One model or subscene instance of a scene file. */
typedef struct SelSceneInstance {
    char asset[256];        /* the "model" or "scene" name, NUL-terminated ("" when absent) */
    float localToWorld[16]; /* "transform": the file's 16 numbers as they stand, rows r0..r3 of the reference's
                               row-vector matrix (translation in r3), which is the column-major localToWorld that
                               sel_scene_attach_instance takes; the identity unless an array of 16 numbers */
} SelSceneInstance;

typedef struct SelSceneDescription {
    float backgroundIntensity[3];   /* default 1 (sel_scene_set_background) */
    char ibl[256];                  /* image-based light name, "" when none */
    unsigned int modelCount;        /* entries of "instances" in the document */
    unsigned int sceneCount;        /* entries of "scenes" */
} SelSceneDescription;

/* A scene file (ParseSceneFile, BuildCommon/CSceneBuildProcessor.cpp:32-63): model instances ("instances":
 * {"model", "transform"}), subscene instances ("scenes": {"scene", "transform"}), "backgroundIntensity" and
 * "ibl".  The first model_capacity / scene_capacity instances are written (capacities 0 to size the arrays);
 * the caller builds a scene per model or subscene name and attaches them with sel_scene_attach_instance.
 * Malformed JSON, or "instances" / "scenes" that are not arrays of objects: SEL_ERR_INVALID_ARGUMENT.  Needs
 * no device. */
int sel_scene_description_from_json(const char* json, SelSceneDescription* out, SelSceneInstance* models,
                                    unsigned int model_capacity, SelSceneInstance* scenes, unsigned int scene_capacity);

/* SceneLight (SceneLib/SceneResource.h) as the lighting code reads it: quad centre, facing direction,
 * full edge vectors x and z, emitted radiance (AreaLighting.cpp:113-153). */
typedef struct SelQuadLight {
    float position[3];
    float direction[3];
    float x[3];
    float z[3];
    float radiance[3];
} SelQuadLight;
int sel_scene_add_quad_light(SelScene scene, unsigned int lightSetIndex, const SelQuadLight* light);
/* backgroundIntensity (default 1, BuildCommon/CSceneBuildProcessor.cpp:59). */
int sel_scene_set_background(SelScene scene, float r, float g, float b);
/* Image-based light (SceneResource::iblResource; ImageBasedLightResource.h:24-35): a latitude-longitude RGB
 * image of width x height (row y at polar angle (y + 0.5) pi / height from +y, column x at azimuth
 * (x + 0.5) 2 pi / width + rotationRadians - pi from +x towards +z), scaled by exposureScale, which lights
 * the scene and is importance-sampled through marginal / conditional densities of sin(theta) x luma
 * (BuildCommon/BuildImageBasedLight.cpp:18-107, built here); `miss` (may be null: the light image times the
 * exposure) is what camera rays and pure-specular chains see (EvaluateBackgroundMiss).  Replaces the uniform
 * background in the path tracer (misses) and the deferred path tracer (misses, background next-event
 * estimation and its MIS).  In VCM it is an environment emitter beside the quad lights of light set 0 (light
 * sub-paths from a disc of the scene's bounding-sphere radius, next-event estimation, camera paths that leave
 * the scene; GenerateLightSample, VCMCommon.cpp:37-62), sampled with the density of the directions whose lookup
 * returns each texel; without it VCM's misses carry no radiance.  width == 0 removes the image. */
int sel_scene_set_ibl(SelScene scene, const float* rgb, unsigned int width, unsigned int height, const float* miss_rgb,
                      unsigned int miss_width, unsigned int miss_height, float rotationRadians, float exposureScale);

/* A 2D base-colour image for geometry geomID, the reference's non-Ptex texture path (CalculateSurfaceParams,
 * SurfaceParameters.cpp:186-213): a material without Ptex takes its base colour from the image at the hit's uvs
 * (vertex attribute slot 2 as (u, v) pairs, sel_scene_set_vertex_attribute; (0, 0) without them), filtered by
 * TextureFiltering::Triangle at mip level 0 (bilinear, texel centres at (i + 0.5) / size, Repeat wrapping by the
 * signed remainder, TextureFiltering.h:30-100), converted from sRGB to linear (SrgbToLinearPrecise) and then,
 * as every base colour, raised to 2.2.  width x height texels of `channels` floats (1: grey, 3: RGB, 4: RGBA,
 * alpha unused), row 0 at v = 0.  width or height 0 removes the image.  Applies from the next render. */
int sel_scene_set_texture(SelScene scene, unsigned int geomID, const float* data, unsigned int width,
                          unsigned int height, unsigned int channels);

/* ------------------------------------------------------------------------------------------------ */
/* Ptex per-face textures.                                                                           */
/* ------------------------------------------------------------------------------------------------ */

/* One triangle face of a Ptex texture (Ptex FaceInfo, Middleware/ptex/Include/Ptexture.h:228-300):
 * square resolution 2^log2 (all faces of a mesh share it), offset of its texels in the texel array (in
 * texels), neighbouring face across edge i (edge i runs from vertex i to vertex i+1; -1 = boundary) and
 * the neighbour's edge id for that edge.  32 bytes. */
typedef struct SelPtexFace {
    int32_t log2;
    uint32_t offset;
    int32_t adjfaces[3];
    int32_t adjedges[3];
} SelPtexFace;

/* PtexFilter::getFilter(f_bspline) + eval on a triangle texture as CalculateSurfaceParams calls it
 * (Source/Core/Shading/SurfaceParameters.cpp:196-206: faceid = primId, u/v = barycentrics, widths 0):
 * d_texels holds half-float RGB texels, d_queries n x (face id as int32 bits, u, v), d_out n x 3 floats
 * (rows of invalid face ids are left untouched).  Device memory, asynchronous on `stream`. */
int sel_ptex_filter_device(SelDevice device, const SelPtexFace* d_faces, unsigned int nfaces, const uint16_t* d_texels,
                           const float* d_queries, unsigned int n, float* d_out, void* stream);

/* Binds a Ptex texture to triangle mesh geomID (replaces TextureCache::FetchPtex of the per-mesh .ptx,
 * Source/Core/TextureLib/TextureCache.cpp:168-185): face_count must equal the geometry's triangle count;
 * materials with usesPtex take their base colour from it.  Host arrays, copied.  A quad mesh: use
 * sel_scene_set_ptex_quads. */
int sel_scene_set_ptex(SelScene scene, unsigned int geomID, const SelPtexFace* faces, size_t face_count,
                       const uint16_t* texels, size_t texel_count);

/* One quad face of a Ptex texture (Ptex FaceInfo of an mt_quad texture): square resolution 2^log2 (all faces of
 * a mesh share it), texel offset (in texels), neighbouring face across edge i (bottom, right, top, left: edge i
 * runs from vertex i to vertex i + 1, u along edge 0, v along edge 3 reversed; -1 = boundary) and the
 * neighbour's edge id for that edge.  40 bytes. */
typedef struct SelPtexQuadFace {
    int32_t log2;
    uint32_t offset;
    int32_t adjfaces[4];
    int32_t adjedges[4];
} SelPtexQuadFace;

/* Binds a Ptex texture to quad mesh geomID: face_count must equal the geometry's quad count (face q is quad q,
 * sampled at the quad's (u, v) as Embree reports them).  Materials with usesPtex take their base colour from the
 * separable bicubic filter with B-spline weights that PtexFilter::getFilter(f_bspline) gives a quad texture
 * (Middleware/ptex/Include/PtexFilters.cpp:116-285,419-441, PtexSeparableFilter.cpp:47-359), with filter
 * widths 0 as SurfaceParameters.cpp:196-206 evaluates it.  Faces whose texels are all equal, and such faces
 * amid equal neighbours, take the reader's constant-face forms (flagged here as the Ptex writer flags them).
 * Host arrays, copied. */
int sel_scene_set_ptex_quads(SelScene scene, unsigned int geomID, const SelPtexQuadFace* faces, size_t face_count,
                             const uint16_t* texels, size_t texel_count);

/* The quad filter on device arrays (as sel_ptex_filter_device): d_faces holds nfaces SelPtexQuadFace records,
 * d_texels half RGB, d_queries n x (face id as int32 bits, u, v); d_out n x 3 (rows of invalid face ids left
 * untouched).  Needs no scene; asynchronous on `stream`. */
int sel_ptex_quad_filter_device(SelDevice device, const SelPtexQuadFace* d_faces, unsigned int nfaces,
                                const uint16_t* d_texels, const float* d_queries, unsigned int n, float* d_out,
                                void* stream);

/* ------------------------------------------------------------------------------------------------ */
/* Integrator entry points.                                                                          */
/* ------------------------------------------------------------------------------------------------ */

/* CameraSettings (GeometryLib/Camera.h:13-21: position, lookAt, up, horizontal fovDegrees) and the
 * viewport InitializeRayCastCamera receives (GeometryLib/Camera.cpp:89-115). */
typedef struct SelCamera {
    float position[3];
    float lookAt[3];
    float up[3];
    float fovDegrees;
    uint32_t width, height;
} SelCamera;

typedef struct SelPtSettings {
    uint32_t samplesPerPixel;  /* PathsPerPixel_ (PathTracer.cpp:45) */
    uint32_t maxBounces;       /* MaxBounceCount_ (PathTracer.cpp:42) */
    uint64_t seed;             /* PCG32 seed; path k uses stream k */
    uint32_t pathsInFlight;    /* wavefront batch (0 = the scene's tuned value, else 4,194,304) */
    uint32_t traceBlockSize;   /* threads per traversal block: 128 or 256 (0 = the scene's tuned value, else 128) */
} SelPtSettings;

/* PathTracer::GenerateImage (Source/Applications/Selas/Source/PathTracer.h:20-21): renders the scene
 * with the wavefront path tracer and writes the two framebuffer layers, already scaled by 1/spp
 * (FrameBuffer_Scale, PathTracer.cpp:346), to out_layers: [2][height][width][3] floats in host memory.
 * Layer 0 is the first-bounce BSDF sample weight, layer 1 the radiance estimate.  Accumulation is FP64. */
int sel_pt_generate_image(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, float* out_layers);
/* Device form: adds the un-normalised FP64 sums into d_accum ([2][height][width][3] doubles in HBM) on
 * `stream` and returns without waiting. */
int sel_pt_render_device(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, double* d_accum,
                         void* stream);

/* DeferredPathTracer::GenerateImage (Source/Applications/Selas/Source/DeferredPathTracer.h:20-21, the
 * integrator main.cpp:121 runs): samplesPerPixel = m * m correlated multi-jittered samples per pixel (m = 4,
 * SamplesPerPixelX_ x SamplesPerPixelY_, in the reference; samplesPerPixel must be a square, m <= 256), quad-light
 * and background next-event estimation, balance-heuristic MIS against the background and Russian roulette
 * from 7 tracked bounces.  The reference has no bounce limit: maxBounces caps the segments of a path (1..1024;
 * sel_deferred_settings_defaults gives 64).  Writes the one framebuffer layer scaled by 1/spp (FrameBuffer_Scale,
 * DeferredPathTracer.cpp:465) to out_rgb: [height][width][3] floats in host memory.  Accumulation is FP64. */
int sel_deferred_settings_defaults(SelPtSettings* out);
int sel_deferred_generate_image(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, float* out_rgb);
/* Device form: adds the un-normalised FP64 sums into d_accum ([height][width][3] doubles in HBM) on `stream` and
 * returns without waiting. */
int sel_deferred_render_device(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, double* d_accum,
                               void* stream);

/* Several views of one scene in one shared wavefront (no reference counterpart: main.cpp renders one camera per
 * run).  1..16 cameras; integrator SEL_INTEGRATOR_PT or SEL_INTEGRATOR_DEFERRED with the settings those entry
 * points take.  View k uses seed settings->seed + k, so its image equals the single-view entry point's with that
 * seed; every wavefront batch takes an equal share of paths from each view, and one batch is captured as a CUDA
 * graph and replayed until all views are done.  out: the views' images one after another, each laid out as the
 * single-view entry point writes it (already scaled by 1/spp); the device form adds FP64 sums into d_accum laid
 * out the same way. */
int sel_render_views(SelScene scene, const SelCamera* cameras, unsigned int count, unsigned int integrator,
                     const SelPtSettings* settings, float* out);
int sel_render_views_device(SelScene scene, const SelCamera* cameras, unsigned int count, unsigned int integrator,
                            const SelPtSettings* settings, double* d_accum, void* stream);

/* Autotuner (no reference counterpart).  Renders the given path-tracer workload (timed with CUDA events,
 * after one untimed render per configuration) over BVH layout and leaf size {8-wide quantised with 2, 3, 4, 8
 * triangles per leaf; binary FP32 (scenes without instances)}, wavefront capacity {1,048,576; 4,194,304;
 * 8,388,608 paths} and traversal block size {128, 256 (8-wide only)}; rebuilds the scene with the fastest layout and keeps the fastest
 * capacity and block size as its defaults (used when SelPtSettings leaves them 0).  Images do not depend on
 * any of these choices. */
typedef struct SelTuneTrial {
    uint32_t bvh_kind, leaf_size, paths_in_flight, trace_block;
    double ms;  /* one render */
} SelTuneTrial;
typedef struct SelTuneResult {
    SelTuneTrial best;
    uint32_t trials;
    uint32_t reserved;
    SelTuneTrial trial[32];
} SelTuneResult;
int sel_scene_autotune(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, SelTuneResult* out);

/* Vertex connection and merging: VCM::GenerateImage (Source/Applications/Selas/Source/VCM.h:18,
 * VCM.cpp:751-808, commented out in the reference and restated from the VCM technical report it cites).
 * A pass traces width * height light paths (from light set 0) and as many camera paths; the pass index
 * i = firstPass + k sets the merge radius r0 / (i + 1)^((1 - alpha) / 2) (VCMCommon.cpp:91-112) and the
 * random streams, so a render split over several calls equals one call over all its passes. */
typedef struct SelVcmSettings {
    uint32_t passes;          /* iterations (the reference integrates for IntegrationSeconds_ = 30 s) */
    uint32_t firstPass;       /* global index of the first pass */
    uint32_t maxPathLength;   /* path segments, 2..32 (MaxBounceCount_ = 10, VCMCommon.cpp:24) */
    uint32_t disableMerging;  /* nonzero: bidirectional path tracing (no merge term or merge weights) */
    uint64_t seed;            /* PCG32 seed */
    float radius;             /* r0; 0 = VcmRadiusFactor_ (0.0025) x the bounding-sphere radius of the
                                 scene bounds (half their diagonal), as VCM.cpp:778 */
    float radiusAlpha;        /* VcmRadiusAlpha_ = 0.75 (VCMCommon.cpp:30) */
} SelVcmSettings;

int sel_vcm_settings_defaults(SelVcmSettings* out);
/* Rays traced by the scene's most recent render (any integrator, any form): out[0] closest-hit (extension)
 * rays, out[1] any-hit (shadow) rays.  Call once that render's stream has been synchronised.  No reference
 * counterpart: the measurement counts of the integrators. */
int sel_scene_last_render_rays(SelScene scene, uint64_t* out);
/* The per-pass constants of a VCM pass: VCMCommon::CalculateIterationConstants
 * (Source/Applications/Selas/Source/VCMCommon.cpp:85-112) with vcCount = 1 and iterationIndex = pass + 1, for
 * base radius radius0, radius alpha and `paths` light paths a pass.  out[5] = vmSearchRadius, vmSearchRadiusSqr,
 * vmNormalization, vmWeight, vcWeight.  Host computation: needs no GPU. */
int sel_vcm_pass_constants(float radius0, float alpha, unsigned int paths, unsigned int pass, float* out);
/* Renders and writes the mean over the passes, [height][width][3] floats in host memory (FP64 sums). */
int sel_vcm_generate_image(SelScene scene, const SelCamera* camera, const SelVcmSettings* settings, float* out_rgb);
/* Device form: adds the per-pass sums into d_accum ([height][width][3] doubles in HBM) on `stream` and
 * returns without waiting. */
int sel_vcm_render_device(SelScene scene, const SelCamera* camera, const SelVcmSettings* settings, double* d_accum,
                          void* stream);

/* ------------------------------------------------------------------------------------------------ */
/* Render server (no reference counterpart: the reference renders one image per process,            */
/* main.cpp:120-123).  Jobs of differing scene, resolution, spp and integrator are admitted while   */
/* device memory (a byte budget) and job slots allow, and their work overlaps on the GPU: path-tracer */
/* jobs share the wavefront launches (a batch takes a fair share of paths from every admitted job),  */
/* VCM jobs advance one pass per round on their own streams.  Scenes stay resident; each job holds   */
/* its accumulator (and VCM state) from admission to completion.  A job's image does not depend on    */
/* the other jobs: its paths use the same random streams alone and in a mix.                         */
/* ------------------------------------------------------------------------------------------------ */
typedef struct SelServerTy* SelServer;

enum { SEL_INTEGRATOR_PT = 0, SEL_INTEGRATOR_VCM = 1, SEL_INTEGRATOR_DEFERRED = 2 };

typedef struct SelServerConfig {
    uint64_t hbm_budget_bytes;  /* device bytes admitted jobs may hold (0: free HBM minus the reserve)  */
    uint64_t hbm_reserve_bytes; /* left free when hbm_budget_bytes is 0 (default 2 GiB)                */
    uint32_t max_jobs;          /* jobs admitted at once, 1..16 (default 16)                           */
    uint32_t paths_in_flight;   /* shared path-tracer wavefront capacity (default 4,194,304)           */
    uint32_t max_bounces;       /* 1..64: path-tracer and deferred jobs may ask for at most this many
                                   bounces (default 8); a batch runs the most its jobs ask for         */
    uint32_t reserved;
} SelServerConfig;

typedef struct SelJob {
    SelScene scene;             /* committed with SEL_BVH_WIDE8_Q8; must outlive the job               */
    SelCamera camera;
    uint32_t integrator;        /* SEL_INTEGRATOR_PT, SEL_INTEGRATOR_VCM or SEL_INTEGRATOR_DEFERRED      */
    uint32_t reserved;
    SelPtSettings pt;           /* used by SEL_INTEGRATOR_PT and _DEFERRED (pathsInFlight is ignored)   */
    SelVcmSettings vcm;         /* used by SEL_INTEGRATOR_VCM                                           */
} SelJob;

typedef struct SelJobStats {
    double queue_ms;            /* submit -> admission                                                  */
    double run_ms;              /* admission -> result in host memory                                   */
    double latency_ms;          /* submit -> result in host memory                                      */
    uint64_t device_bytes;      /* device memory the job held                                           */
    int32_t status;             /* SEL_OK or the error the job ended with                                */
    uint32_t reserved;
} SelJobStats;

typedef struct SelServerStats {
    uint64_t submitted, completed;
    uint64_t rays;              /* closest-hit + any-hit rays traced by finished work                    */
    uint64_t peak_jobs;         /* most jobs admitted at once                                           */
    uint64_t peak_bytes;        /* most device bytes held by admitted jobs at once                      */
    uint64_t graph_captures;    /* shared path-tracer batches captured as CUDA graphs                   */
} SelServerStats;

int sel_server_config_defaults(SelServerConfig* out);
int sel_server_new(SelDevice device, const SelServerConfig* config, SelServer* out_server);
/* Queues a job and returns at once with its id.  The result size is sel_server_result_floats. */
int sel_server_submit(SelServer server, const SelJob* job, uint64_t* out_job_id);
int sel_server_result_floats(const SelJob* job, size_t* out_floats);
/* done = 1 when the job's result is in host memory. */
int sel_server_poll(SelServer server, uint64_t job_id, int* out_done);
/* Blocks until the job is done, copies its image (path tracer: the two layers [2][H][W][3] scaled by
 * 1/spp; deferred path tracer: [H][W][3] scaled by 1/spp; VCM: [H][W][3], the mean over the passes) to out (out_floats >= the result size) and its
 * statistics to stats (may be null), and forgets the job.  Returns the job's status. */
int sel_server_wait(SelServer server, uint64_t job_id, float* out, size_t out_floats, SelJobStats* stats);
int sel_server_stats(SelServer server, SelServerStats* out);
/* Finishes every queued job, then stops the server. */
int sel_server_release(SelServer server);

/* ------------------------------------------------------------------------------------------------ */
/* Cooked assets.                                                                                    */
/* ------------------------------------------------------------------------------------------------ */

/* The reference's cooked asset blobs under <asset_root>/_Assets/<type>/<version>/<name>.bin
 * (AssetFileUtils::AssetFilePath, Assets/AssetFileUtils.cpp:109-116): SceneResource (version 1539147471),
 * SubsceneResource (1539551841), ModelResource and ModelGeometryResource (1539636447), Textures (1534887410) and
 * IBL (1538087123), as SerializeToBinary writes them (IoLib/BinaryStreamSerializer.h:15-32).  Replaces
 * ReadSceneResource + InitializeSceneResource (SceneLib/SceneResource.cpp:271-315) with its subscenes
 * (SubsceneResource.cpp:101-160) and models (ModelResource.cpp:432-471). */

/* sel_scene_load_cooked flag: materials that sample Ptex (eUsesPtex) render with their base colour instead of
 * refusing the scene (the loader reads no .ptx files; bind Ptex with sel_scene_set_ptex on scenes built by hand). */
#define SEL_COOKED_PTEX_AS_BASE_COLOR 1u

typedef struct SelCookedSceneInfo {
    uint32_t subscenes;             /* subsceneNames */
    uint32_t subsceneInstances;
    uint32_t models;                /* models loaded: each subscene loads its own copy of each model it names */
    uint32_t modelInstances;        /* over all subscenes */
    uint32_t meshes;                /* over all loaded models */
    uint32_t quadMeshes;            /* meshes of 4 indices per face (RTC_GEOMETRY_TYPE_QUAD) */
    uint64_t faces;                 /* triangles plus quads */
    uint32_t lights;
    uint32_t lightSets;             /* lightSetRanges */
    uint32_t cameras;
    uint32_t textures;              /* distinct Textures assets the meshes' materials load */
    uint32_t ptexMeshes;            /* meshes whose material samples Ptex */
    uint32_t curves;                /* curve geometries of the loaded models */
    float backgroundIntensity[4];
    char ibl[512];                  /* iblName ("" when none) */
    SelCamera camera;               /* SetupSceneCamera(scene, 0): cameras[0] when valid (fovDegrees > 0, zfar >
                                       znear), else DefaultCameraSettings; width and height 0 */
} SelCookedSceneInfo;

/* One mesh of a cooked scene as the reference's loader sets it up (InitializeGeometryUserDatas,
 * ModelResource.cpp:300-344). */
typedef struct SelCookedMesh {
    uint32_t subscene;        /* index into the scene's subsceneNames */
    uint32_t model;           /* index into that subscene's modelNames */
    uint32_t mesh;            /* index into the model's meshes: its geomID in the model scene */
    uint32_t indicesPerFace;  /* 3 or 4 */
    uint32_t faces;
    uint32_t materialFlags;   /* MaterialFlags of the resolved material (eTransparent 1, eUsesPtex 16, ...) */
    SelMaterial material;     /* FindMeshMaterial (ModelResource.cpp:213-229): the model's materials by binary search
                                 of their sorted name hashes, then the subscene's scene materials, else the default;
                                 lightSetIndex = the subscene's lightSetIndex */
    char texture[512];        /* the material's baseColorTexture: a Textures asset name, or a Ptex content path */
    char name[64];            /* MeshMetaData::name */
} SelCookedMesh;

/* Parses the scene blob, its subscene blobs and their model and geometry blobs (no device): fills *out_info and
 * the first `capacity` meshes in load order (subscene, model, mesh).  A missing file or a blob whose offsets or
 * counts leave the file: SEL_ERR_IO, with the path in the message. */
int sel_cooked_scene_describe(const char* asset_root, const char* scene_name, SelCookedSceneInfo* out_info,
                              SelCookedMesh* meshes, unsigned int capacity);

/* Loads a cooked scene into *out_scene, a committed scene of the 8-wide layout:
 *   top scene:       instance i = subsceneInstances[i], of the scene built for subsceneNames[index];
 *   subscene scene:  instance j = modelInstances[j], of that subscene's copy of modelNames[index];
 *   model scene:     geomID k = meshes[k], a triangle or quad mesh with the model's normals (slot 0), tangents
 *                    (slot 1) and uvs (slot 2), the material FindMeshMaterial resolves (the stored eTransparent
 *                    flag kept) and, for a non-Ptex material naming a texture, mip 0 of that Textures asset as
 *                    its base-colour image (read as RGB float triples, as TextureFiltering::Triangle<float3>
 *                    reads it);
 * the scene's quad lights in light sets by lightSetRanges, its backgroundIntensity and, when iblName is set, the
 * IBL asset's light and miss images with its rotation and exposure (the densities are derived again from the
 * light image).  Queries on *out_scene report instID[0] = i, instID[1] = j and geomID = k, the ids the reference's
 * Embree scenes report.  A model's curves (InitializeCurves, ModelResource.cpp:300-332) follow its meshes as
 * geomIDs meshes + c, round B-spline curves (sel_scene_attach_curve_mesh) with the material of the model's
 * curveModelName.  Releasing *out_scene releases the subscene and model scenes with it.  Refused with
 * SEL_ERR_INVALID_OPERATION: Ptex materials unless SEL_COOKED_PTEX_AS_BASE_COLOR.
 * out_info may be null. */
int sel_scene_load_cooked(SelDevice device, const char* asset_root, const char* scene_name, unsigned int flags,
                          SelScene* out_scene, SelCookedSceneInfo* out_info);

#ifdef __cplusplus
}
#endif

#endif /* SELAS_GB300_H */
