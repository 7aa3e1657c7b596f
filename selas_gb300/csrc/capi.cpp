// C ABI: device and scene lifetime plus the ray-query entry points declared in include/selas.h.
// Status codes instead of exceptions; the message of the last failure is kept per host thread.
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "capi_internal.h"
#include "pt.h"
#include "query.h"

using sel::BuiltBvh;
using sel::DeviceBvh;
using sel::MeshInput;

namespace sel {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(SEL_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int set_device(SelDeviceTy* dev) {
    cudaError_t e = cudaSetDevice(dev->cuda_device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return SEL_OK;
}

int ensure_scratch(SelSceneTy* sc, size_t bytes) {
    if (sc->scratch_bytes >= bytes) return SEL_OK;
    if (sc->scratch) cudaFree(sc->scratch);
    sc->scratch = nullptr;
    sc->scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&sc->scratch, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(query staging)");
    sc->scratch_bytes = bytes;
    return SEL_OK;
}

int read_error_word(SelDeviceTy* dev, cudaStream_t s) {
    uint32_t word = 0;
    cudaError_t e = cudaMemcpyAsync(&word, dev->d_err, sizeof(word), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "reading device error word");
    if (word) {
        cudaMemsetAsync(dev->d_err, 0, sizeof(uint32_t), s);
        cudaStreamSynchronize(s);
        const char* what = (word & 2u)    ? "traversal stack overflow"
                           : (word & 4u)  ? "Ptex filter frame stack overflow"
                           : (word & 8u)  ? "render queue overflow"
                           : (word & 16u) ? "instances nested deeper than two levels"
                                          : "kernel iteration cap reached";
        return fail(SEL_ERR_DEVICE_LIMIT, what);
    }
    return SEL_OK;
}

DeviceBvh device_bvh(const SelSceneTy* sc) {
    DeviceBvh b;
    b.kind = sc->info.bvh_kind;
    b.nodes = sc->d_nodes;
    b.tris = static_cast<const float4*>(sc->d_tris);
    b.tri_count = uint32_t(sc->info.triangle_count);
    b.insts = static_cast<const InstanceRecord*>(sc->d_insts);
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = sc->info.bounds_lo[a];
        b.hi[a] = sc->info.bounds_hi[a];
    }
    b.order_rays = sc->dev->ray_sort;
    b.pool = sc->dev->order_pool;
    return b;
}

bool instances_fresh(const SelSceneTy* sc) {
    for (const auto& r : sc->referenced) {
        if (!r.first->committed || r.first->generation != r.second) return false;
        if (!instances_fresh(r.first)) return false;
    }
    return true;
}

void adopt_scenes(SelSceneTy* top, const std::vector<SelSceneTy*>& scenes) {
    top->owned.insert(top->owned.end(), scenes.begin(), scenes.end());
}

}  // namespace sel

using namespace sel;

extern "C" {

const char* sel_get_last_error(void) { return g_last_error.c_str(); }

int sel_device_new(int cuda_device, SelDevice* out_device) {
    if (!out_device) return fail(SEL_ERR_INVALID_ARGUMENT, "out_device is null");
    *out_device = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (cuda_device < 0 || cuda_device >= count) return fail(SEL_ERR_INVALID_ARGUMENT, "no such CUDA device");
    SelDeviceTy* dev = new (std::nothrow) SelDeviceTy();
    if (!dev) return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
    dev->cuda_device = cuda_device;
    if (int rc = set_device(dev)) { delete dev; return rc; }
    e = cudaStreamCreateWithFlags(&dev->stream, cudaStreamNonBlocking);
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaStreamCreateWithFlags(&dev->qstream[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&dev->d_err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(dev->d_err, 0, sizeof(uint32_t));
    // The allocation-free query's staging array: resolving its address here loads its module (and so
    // creates the array) while the device is being set up, not inside the first allocation-free call.
    if (e == cudaSuccess && resolve_noalloc_staging(dev) != SEL_OK) e = cudaErrorInvalidSymbol;
    // The ray-order scratch of large queries is stream-ordered, from a pool of the device's own that keeps freed
    // memory for the next query instead of returning it at every synchronisation.
    if (e == cudaSuccess) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = cuda_device;
        e = cudaMemPoolCreate(&dev->order_pool, &props);
        uint64_t keep = ~uint64_t(0);
        if (e == cudaSuccess) e = cudaMemPoolSetAttribute(dev->order_pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e != cudaSuccess) {
        if (dev->order_pool) cudaMemPoolDestroy(dev->order_pool);
        if (dev->stream) cudaStreamDestroy(dev->stream);
        for (cudaStream_t q : dev->qstream)
            if (q) cudaStreamDestroy(q);
        if (dev->d_err) cudaFree(dev->d_err);
        delete dev;
        return cuda_fail(e, "device setup");
    }
    *out_device = dev;
    return SEL_OK;
}

int sel_device_release(SelDevice device) {
    if (!device) return fail(SEL_ERR_INVALID_ARGUMENT, "device is null");
    set_device(device);
    cudaStreamSynchronize(device->stream);
    cudaStreamDestroy(device->stream);
    for (cudaStream_t q : device->qstream) {
        cudaStreamSynchronize(q);
        cudaStreamDestroy(q);
    }
    cudaFree(device->d_err);
    if (device->order_pool) cudaMemPoolDestroy(device->order_pool);  // released once its last block is freed
    delete device;
    return SEL_OK;
}

int sel_device_sync(SelDevice device, void* stream) {
    if (!device) return fail(SEL_ERR_INVALID_ARGUMENT, "device is null");
    if (int rc = set_device(device)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    std::lock_guard<std::mutex> lock(device->mu);
    return read_error_word(device, device->stream);
}

int sel_scene_new(SelDevice device, SelScene* out_scene) {
    if (!device || !out_scene) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    SelSceneTy* sc = new (std::nothrow) SelSceneTy();
    if (!sc) return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
    sc->dev = device;
    *out_scene = sc;
    return SEL_OK;
}

int sel_scene_set_bvh_kind(SelScene scene, int bvh_kind) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if (bvh_kind != SEL_BVH_WIDE8_Q8 && bvh_kind != SEL_BVH_BINARY_FP32)
        return fail(SEL_ERR_INVALID_ARGUMENT, "unknown BVH kind");
    std::lock_guard<std::mutex> lock(scene->mu);
    scene->kind = bvh_kind;
    return SEL_OK;
}

int sel_scene_attach_triangle_mesh(SelScene scene, unsigned int geomID, const float* vertices, size_t vertex_count,
                                   size_t vertex_stride_bytes, const unsigned int* indices, size_t triangle_count) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if ((vertex_count && !vertices) || (triangle_count && !indices))
        return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    if (vertex_stride_bytes < 12 || vertex_stride_bytes % 4)
        return fail(SEL_ERR_INVALID_ARGUMENT, "vertex stride must be >= 12 and a multiple of 4");
    if (geomID >= kInstanceGeom) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID must be below 0xFFFFFFFE");
    std::lock_guard<std::mutex> lock(scene->mu);
    for (const MeshInput& m : scene->meshes)
        if (m.geomID == geomID) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID already attached");
    for (const SelSceneTy::CurveInput& c : scene->curves)
        if (c.geomID == geomID) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID already attached");
    for (const SelSceneTy::InstanceInput& ii : scene->instances)
        if (ii.instID == geomID) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID already used by an instance");
    MeshInput m;
    m.geomID = geomID;
    try {
        m.vertices.resize(vertex_count * 3);
        const char* vb = reinterpret_cast<const char*>(vertices);
        for (size_t i = 0; i < vertex_count; ++i) std::memcpy(&m.vertices[3 * i], vb + i * vertex_stride_bytes, 12);
        m.indices.assign(indices, indices + triangle_count * 3);
    } catch (const std::bad_alloc&) {
        return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    for (uint32_t idx : m.indices)
        if (idx >= vertex_count) return fail(SEL_ERR_INVALID_ARGUMENT, "triangle index out of range");
    scene->meshes.push_back(std::move(m));
    scene->committed = false;
    return SEL_OK;
}

int sel_scene_attach_quad_mesh(SelScene scene, unsigned int geomID, const float* vertices, size_t vertex_count,
                               size_t vertex_stride_bytes, const unsigned int* indices, size_t quad_count) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if (quad_count && !indices) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    if (quad_count >= (size_t(1) << 31)) return fail(SEL_ERR_INVALID_ARGUMENT, "a quad mesh holds fewer than 2^31 quads");
    // Embree handles a quad as the triangles (v0, v1, v3) and (v2, v3, v1) (RTC_GEOMETRY_TYPE_QUAD.3embree3):
    // stored that way, as triangles 2q and 2q + 1 of the mesh
    std::vector<unsigned int> pairs;
    try {
        pairs.resize(quad_count * 6);
    } catch (const std::bad_alloc&) {
        return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    for (size_t q = 0; q < quad_count; ++q) {
        const unsigned int* v = indices + 4 * q;
        unsigned int* t = pairs.data() + 6 * q;
        t[0] = v[0]; t[1] = v[1]; t[2] = v[3];
        t[3] = v[2]; t[4] = v[3]; t[5] = v[1];
    }
    if (int rc = sel_scene_attach_triangle_mesh(scene, geomID, vertices, vertex_count, vertex_stride_bytes,
                                                pairs.data(), 2 * quad_count))
        return rc;
    std::lock_guard<std::mutex> lock(scene->mu);
    scene->meshes.back().quads = true;
    return SEL_OK;
}

int sel_scene_attach_curve_mesh(SelScene scene, unsigned int geomID, const float* points, size_t point_count,
                                const unsigned int* indices, size_t segment_count) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if ((point_count && !points) || (segment_count && !indices)) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    if (geomID >= kInstanceGeom) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID must be below 0xFFFFFFFE");
    if (segment_count >= (size_t(1) << 31)) return fail(SEL_ERR_INVALID_ARGUMENT, "fewer than 2^31 segments");
    for (size_t k = 0; k < segment_count; ++k)
        if (size_t(indices[k]) + 3 >= point_count)
            return fail(SEL_ERR_INVALID_ARGUMENT, "a segment's four control points run past the point array");
    for (size_t i = 0; i < 4 * point_count; ++i)
        if (!std::isfinite(points[i])) return fail(SEL_ERR_INVALID_ARGUMENT, "non-finite control point");
    for (size_t i = 0; i < point_count; ++i)
        if (points[4 * i + 3] < 0.0f) return fail(SEL_ERR_INVALID_ARGUMENT, "negative curve radius");
    std::lock_guard<std::mutex> lock(scene->mu);
    for (const MeshInput& m : scene->meshes)
        if (m.geomID == geomID) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID already attached");
    for (const SelSceneTy::CurveInput& c : scene->curves)
        if (c.geomID == geomID) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID already attached");
    for (const SelSceneTy::InstanceInput& ii : scene->instances)
        if (ii.instID == geomID) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID already used by an instance");
    for (const SelSceneTy::TextureBinding& t : scene->textures)
        if (t.geomID == geomID) return fail(SEL_ERR_INVALID_OPERATION, "a texture is bound to this geomID; curves take none");
    SelSceneTy::CurveInput c;
    c.geomID = geomID;
    try {
        c.points.assign(points, points + 4 * point_count);
        c.indices.assign(indices, indices + segment_count);
    } catch (const std::bad_alloc&) {
        return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    scene->curves.push_back(std::move(c));
    scene->committed = false;
    return SEL_OK;
}

int sel_scene_attach_instance(SelScene scene, unsigned int instID, SelScene instanced, const float* localToWorld) {
    if (!scene || !instanced || !localToWorld) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (instanced == scene) return fail(SEL_ERR_INVALID_ARGUMENT, "a scene cannot instance itself");
    if (instanced->dev != scene->dev) return fail(SEL_ERR_INVALID_ARGUMENT, "scenes of different devices");
    if (instID >= kInstanceGeom) return fail(SEL_ERR_INVALID_ARGUMENT, "instID must be below 0xFFFFFFFE");
    const float* m = localToWorld;  // column-major 4 x 4: element (row r, column c) at m[4 c + r]
    for (int k = 0; k < 16; ++k)
        if (!std::isfinite(m[k])) return fail(SEL_ERR_INVALID_ARGUMENT, "non-finite transform");
    if (m[3] != 0.0f || m[7] != 0.0f || m[11] != 0.0f || m[15] != 1.0f)
        return fail(SEL_ERR_INVALID_ARGUMENT, "localToWorld must be affine (last row 0 0 0 1)");
    SelSceneTy::InstanceInput ii;
    ii.instID = instID;
    ii.scene = instanced;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) ii.l2w[4 * r + c] = m[4 * c + r];
    if (!affine_inverse(ii.l2w, ii.w2l)) return fail(SEL_ERR_INVALID_ARGUMENT, "localToWorld is singular");
    std::lock_guard<std::mutex> lock(scene->mu);
    for (const MeshInput& mi : scene->meshes)
        if (mi.geomID == instID) return fail(SEL_ERR_INVALID_ARGUMENT, "instID already used by a mesh");
    for (const SelSceneTy::CurveInput& c : scene->curves)
        if (c.geomID == instID) return fail(SEL_ERR_INVALID_ARGUMENT, "instID already used by a curve geometry");
    for (const SelSceneTy::InstanceInput& o : scene->instances)
        if (o.instID == instID) return fail(SEL_ERR_INVALID_ARGUMENT, "instID already attached");
    scene->instances.push_back(ii);
    scene->committed = false;
    return SEL_OK;
}

int sel_scene_set_vertex_attribute(SelScene scene, unsigned int geomID, unsigned int slot, const float* data,
                                   size_t vertex_count, unsigned int components) {
    if (!scene || (!data && vertex_count)) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (slot > 3 || components < 1 || components > 4)
        return fail(SEL_ERR_INVALID_ARGUMENT, "slot must lie in 0..3 and components in 1..4");
    if ((slot == 0 && components != 3) || (slot == 1 && components != 4))
        return fail(SEL_ERR_INVALID_ARGUMENT, "slot 0 (normals) takes 3 floats and slot 1 (tangents) 4");
    std::lock_guard<std::mutex> lock(scene->mu);
    for (MeshInput& m : scene->meshes) {
        if (m.geomID != geomID) continue;
        if (vertex_count != m.vertices.size() / 3)
            return fail(SEL_ERR_INVALID_ARGUMENT, "vertex_count differs from the mesh's vertex count");
        for (size_t i = 0; i < vertex_count * components; ++i)
            if (!std::isfinite(data[i])) return fail(SEL_ERR_INVALID_ARGUMENT, "non-finite attribute");
        try {
            m.attr[slot].assign(data, data + vertex_count * components);
        } catch (const std::bad_alloc&) {
            return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
        }
        m.attr_n[slot] = components;
        scene->shading_dirty = true;
        return SEL_OK;
    }
    return fail(SEL_ERR_INVALID_ARGUMENT, "no mesh with this geomID");
}

int sel_interpolate0(SelScene scene, unsigned int geomID, unsigned int primID, float u, float v, unsigned int slot,
                     float* out, unsigned int count) {
    if (!scene || !out) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (slot > 3) return fail(SEL_ERR_INVALID_ARGUMENT, "slot must lie in 0..3");
    std::lock_guard<std::mutex> lock(scene->mu);
    for (const MeshInput& m : scene->meshes) {
        if (m.geomID != geomID) continue;
        const uint32_t n = m.attr_n[slot];
        if (!n) return fail(SEL_ERR_INVALID_OPERATION, "the mesh has no attribute in this slot");
        if (count > n) return fail(SEL_ERR_INVALID_ARGUMENT, "count exceeds the attribute's components");
        if (m.quads) {
            // bilinear over the quad (RTC_GEOMETRY_TYPE_QUAD.3embree3): t_uv = (1-v)((1-u) t0 + u t1) + v((1-u) t3 + u t2)
            if (size_t(primID) * 6 + 5 >= m.indices.size()) return fail(SEL_ERR_INVALID_ARGUMENT, "primID out of range");
            const uint32_t* t = &m.indices[6 * size_t(primID)];  // (v0, v1, v3), (v2, v3, v1)
            const float* a0 = &m.attr[slot][size_t(t[0]) * n];
            const float* a1 = &m.attr[slot][size_t(t[1]) * n];
            const float* a2 = &m.attr[slot][size_t(t[3]) * n];
            const float* a3 = &m.attr[slot][size_t(t[2]) * n];
            const float iu = 1.0f - u, iv = 1.0f - v;
            for (unsigned int k = 0; k < count; ++k) out[k] = iv * (iu * a0[k] + u * a1[k]) + v * (iu * a3[k] + u * a2[k]);
            return SEL_OK;
        }
        if (size_t(primID) * 3 + 2 >= m.indices.size()) return fail(SEL_ERR_INVALID_ARGUMENT, "primID out of range");
        const float* a0 = &m.attr[slot][size_t(m.indices[3 * size_t(primID)]) * n];
        const float* a1 = &m.attr[slot][size_t(m.indices[3 * size_t(primID) + 1]) * n];
        const float* a2 = &m.attr[slot][size_t(m.indices[3 * size_t(primID) + 2]) * n];
        const float w = 1.0f - u - v;
        for (unsigned int k = 0; k < count; ++k) out[k] = w * a0[k] + u * a1[k] + v * a2[k];
        return SEL_OK;
    }
    return fail(SEL_ERR_INVALID_ARGUMENT, "no mesh with this geomID");
}

int sel_scene_set_build_mode(SelScene scene, int build_mode) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if (build_mode != SEL_BUILD_HOST && build_mode != SEL_BUILD_DEVICE)
        return fail(SEL_ERR_INVALID_ARGUMENT, "unknown build mode");
    std::lock_guard<std::mutex> lock(scene->mu);
    scene->build_mode = build_mode;
    return SEL_OK;
}

int sel_scene_set_leaf_size(SelScene scene, unsigned int leaf_size) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if (leaf_size < 1 || leaf_size > kMaxLeafRecords)
        return fail(SEL_ERR_INVALID_ARGUMENT, "leaf_size must lie in 1..8");
    std::lock_guard<std::mutex> lock(scene->mu);
    scene->leaf_size = leaf_size;
    return SEL_OK;
}

}  // extern "C"

namespace {

// World box of an instance: the instanced scene's bounds transformed corner by corner in double, rounded
// outward and padded by 2^-16 of its magnitude and extent, so that the box holds every point the object-space
// test can hit despite the rounding of the two transforms.
void instance_box(const SelSceneTy::InstanceInput& ii, float lo[3], float hi[3]) {
    const SelSceneInfo& pi = ii.scene->info;
    double blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < 8; ++k) {
        const double p[3] = {(k & 1) ? pi.bounds_hi[0] : pi.bounds_lo[0], (k & 2) ? pi.bounds_hi[1] : pi.bounds_lo[1],
                             (k & 4) ? pi.bounds_hi[2] : pi.bounds_lo[2]};
        for (int r = 0; r < 3; ++r) {
            const double w = double(ii.l2w[4 * r]) * p[0] + double(ii.l2w[4 * r + 1]) * p[1] +
                             double(ii.l2w[4 * r + 2]) * p[2] + double(ii.l2w[4 * r + 3]);
            blo[r] = std::min(blo[r], w);
            bhi[r] = std::max(bhi[r], w);
        }
    }
    for (int r = 0; r < 3; ++r) {
        const double pad = (std::max(std::fabs(blo[r]), std::fabs(bhi[r])) + (bhi[r] - blo[r])) * std::ldexp(1.0, -16) +
                           std::ldexp(1.0, -100);
        lo[r] = std::nextafter(float(blo[r] - pad), -INFINITY);
        hi[r] = std::nextafter(float(bhi[r] + pad), INFINITY);
    }
}

// Checks the instances of a scene about to be committed and appends the leaf records that stand for them (a
// mesh of geomID kInstanceGeom whose triangle i spans instance i's world box).
int prepare_instances(SelSceneTy* scene, MeshInput& mesh, uint32_t& levels, uint32_t& below) {
    levels = 0;
    below = 0;
    mesh.geomID = kInstanceGeom;
    mesh.vertices.clear();
    mesh.indices.clear();
    if (scene->kind != SEL_BVH_WIDE8_Q8)
        return fail(SEL_ERR_INVALID_OPERATION, "scenes with instances need the SEL_BVH_WIDE8_Q8 layout");
    for (size_t i = 0; i < scene->instances.size(); ++i) {
        const SelSceneTy::InstanceInput& ii = scene->instances[i];
        SelSceneTy* p = ii.scene;
        if (!p->committed) return fail(SEL_ERR_INVALID_OPERATION, "an instanced scene is not committed");
        if (p->info.bvh_kind != SEL_BVH_WIDE8_Q8)
            return fail(SEL_ERR_INVALID_OPERATION, "instanced scenes need the SEL_BVH_WIDE8_Q8 layout");
        if (p->inst_levels >= 2) return fail(SEL_ERR_INVALID_OPERATION, "instances nest at most two levels");
        if (!instances_fresh(p)) return fail(SEL_ERR_INVALID_OPERATION, "an instanced scene is out of date");
        levels = std::max(levels, 1u + p->inst_levels);
        below = std::max(below, p->stack_need);
        float lo[3], hi[3];
        instance_box(ii, lo, hi);
        const uint32_t v = uint32_t(mesh.vertices.size() / 3);
        mesh.vertices.insert(mesh.vertices.end(), {lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]});
        mesh.indices.insert(mesh.indices.end(), {v, v + 1, v});
    }
    return SEL_OK;
}

// After a successful build: the instance table, the nesting bounds and the references of a scene.
int finish_instances(SelSceneTy* scene, uint32_t levels, uint32_t below) {
    if (scene->d_insts) cudaFree(scene->d_insts);
    scene->d_insts = nullptr;
    const size_t n = scene->instances.size();
    scene->stack_need = scene->info.max_depth + (n ? 2u + below : 0u);
    if (n && scene->stack_need > uint32_t(kInstStack))
        return fail(SEL_ERR_INVALID_OPERATION, "instance nesting too deep for the traversal stack");
    std::vector<InstanceRecord> recs(n);
    for (size_t i = 0; i < n; ++i) {
        const SelSceneTy::InstanceInput& ii = scene->instances[i];
        InstanceRecord& r = recs[i];
        std::memset(&r, 0, sizeof(r));
        std::memcpy(r.w2l, ii.w2l, sizeof(r.w2l));
        std::memcpy(r.l2w, ii.l2w, sizeof(r.l2w));
        r.nodes = ii.scene->d_nodes;
        r.tris = ii.scene->d_tris;
        r.insts = static_cast<const InstanceRecord*>(ii.scene->d_insts);
        r.shading = ii.scene->d_view;
        r.instID = ii.instID;
    }
    if (n) {
        cudaError_t e = cudaMalloc(&scene->d_insts, n * sizeof(InstanceRecord));
        if (e == cudaSuccess) e = cudaMemcpy(scene->d_insts, recs.data(), n * sizeof(InstanceRecord), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, "instance table");
        scene->info.triangle_count -= n;
        scene->info.device_bytes += n * sizeof(InstanceRecord);
    } else if (!scene->curves.empty()) {
        // curve segments are intersected by the instanced traversal only: a scene with curves and no instances
        // takes it through an instance table of one unused record
        cudaError_t e = cudaMalloc(&scene->d_insts, sizeof(InstanceRecord));
        if (e == cudaSuccess) e = cudaMemset(scene->d_insts, 0, sizeof(InstanceRecord));
        if (e != cudaSuccess) return cuda_fail(e, "instance table");
    }
    scene->inst_levels = levels;
    for (auto& r : scene->referenced) --r.first->instanced_by;
    scene->referenced.clear();
    for (const SelSceneTy::InstanceInput& ii : scene->instances) {
        bool seen = false;
        for (const auto& r : scene->referenced) seen |= r.first == ii.scene;
        if (seen) continue;
        scene->referenced.push_back({ii.scene, ii.scene->generation});
        ++ii.scene->instanced_by;
    }
    return SEL_OK;
}

int commit_geometry(SelSceneTy* scene);

// The build's stand-in for a curve geometry: per segment a box "triangle" (lo, hi, lo), the box of its four
// control points grown by their largest radius (the B-spline and its radius stay inside their hull).
MeshInput curve_boxes(const SelSceneTy::CurveInput& c) {
    MeshInput m;
    m.geomID = c.geomID;
    m.curves = true;
    m.vertices.reserve(c.indices.size() * 6);
    m.indices.reserve(c.indices.size() * 3);
    for (size_t k = 0; k < c.indices.size(); ++k) {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}, r = 0.0f;
        for (int j = 0; j < 4; ++j) {
            const float* p = &c.points[4 * (size_t(c.indices[k]) + j)];
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], p[a]);
                hi[a] = std::max(hi[a], p[a]);
            }
            r = std::max(r, p[3]);
        }
        for (int a = 0; a < 3; ++a) {
            const float pad = r + (std::fabs(lo[a]) + std::fabs(hi[a]) + r) * std::ldexp(1.0f, -20);
            lo[a] = std::nextafter(lo[a] - pad, -INFINITY);
            hi[a] = std::nextafter(hi[a] + pad, INFINITY);
        }
        const uint32_t v = uint32_t(m.vertices.size() / 3);
        m.vertices.insert(m.vertices.end(), {lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]});
        m.indices.insert(m.indices.end(), {v, v + 1, v});
    }
    return m;
}

// After the build: the segments' control points appended to the leaf records and each curve record pointed at
// its own (curve.cu).
int finish_curves(SelSceneTy* scene) {
    std::vector<float> data;
    std::vector<uint32_t> geoms, bases;
    size_t nseg = 0;
    for (const SelSceneTy::CurveInput& c : scene->curves) nseg += c.indices.size();
    try {
        data.reserve(nseg * 16);
        for (const SelSceneTy::CurveInput& c : scene->curves) {
            geoms.push_back(c.geomID);
            bases.push_back(uint32_t(data.size() / 16));
            for (uint32_t first : c.indices)
                data.insert(data.end(), c.points.begin() + 4 * size_t(first), c.points.begin() + 4 * (size_t(first) + 4));
        }
    } catch (const std::bad_alloc&) {
        return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    void* tris = scene->d_tris;
    const uint64_t records = scene->info.triangle_count;
    cudaError_t e = attach_curve_data(&tris, records, data.data(), nseg, geoms.data(), bases.data(),
                                      uint32_t(geoms.size()));
    if (e != cudaSuccess) return cuda_fail(e, "curve segment data");
    scene->d_tris = tris;
    scene->info.device_bytes += nseg * 64;
    return SEL_OK;
}

}  // namespace

extern "C" int sel_scene_commit(SelScene scene) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    uint32_t levels = 0, below = 0;
    const bool has_instances = !scene->instances.empty();
    if (has_instances) {
        MeshInput mesh;
        try {
            if (int rc = prepare_instances(scene, mesh, levels, below)) return rc;
        } catch (const std::bad_alloc&) {
            return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
        }
        scene->meshes.push_back(std::move(mesh));  // the instance records, for the duration of the build
    }
    // curve geometries enter the build as boxes, one per segment (their records are finished afterwards)
    const size_t mesh_count = scene->meshes.size();
    if (!scene->curves.empty()) {
        if (scene->kind != SEL_BVH_WIDE8_Q8) {
            if (has_instances) scene->meshes.pop_back();
            return fail(SEL_ERR_INVALID_OPERATION, "scenes with curves need the SEL_BVH_WIDE8_Q8 layout");
        }
        try {
            for (const SelSceneTy::CurveInput& c : scene->curves) scene->meshes.push_back(curve_boxes(c));
        } catch (const std::bad_alloc&) {
            scene->meshes.resize(mesh_count);
            if (has_instances) scene->meshes.pop_back();
            return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
        }
    }
    scene->committed = false;
    int rc = commit_geometry(scene);
    scene->meshes.resize(mesh_count);
    if (has_instances) scene->meshes.pop_back();
    if (rc == SEL_OK && !scene->curves.empty()) rc = finish_curves(scene);
    if (rc == SEL_OK) rc = finish_instances(scene, levels, below);
    if (rc != SEL_OK) {
        scene->committed = false;
        return rc;
    }
    if (!scene->d_view) {
        cudaError_t e = cudaMalloc(&scene->d_view, sizeof(ShadeView));
        if (e == cudaSuccess) e = cudaMemset(scene->d_view, 0, sizeof(ShadeView));
        if (e != cudaSuccess) {
            scene->d_view = nullptr;
            return cuda_fail(e, "cudaMalloc(shading view)");
        }
        scene->shading_dirty = true;  // the view is written by the next shading upload
    }
    ++scene->generation;
    scene->committed = true;
    return SEL_OK;
}

namespace {

int commit_geometry(SelSceneTy* scene) {
    if (scene->kind == SEL_BVH_WIDE8_Q8 && scene->build_mode == SEL_BUILD_DEVICE) {
        DeviceBuild db;
        std::string derr;
        try {
            derr = build_wide_device(scene->meshes, scene->leaf_size, db);
        } catch (const std::bad_alloc&) {
            return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed during BVH build");
        }
        if (!derr.empty()) return fail(SEL_ERR_INVALID_OPERATION, derr);
        if (scene->d_nodes) cudaFree(scene->d_nodes);
        if (scene->d_tris) cudaFree(scene->d_tris);
        scene->d_nodes = db.d_nodes;
        scene->d_tris = db.d_tris;
        SelSceneInfo& info = scene->info;
        std::memset(&info, 0, sizeof(info));
        info.triangle_count = db.tri_count;
        info.node_count = db.node_count;
        info.device_bytes = uint64_t(db.node_count) * sizeof(WideNode) + uint64_t(db.tri_count) * sizeof(TriRecord);
        info.bvh_kind = SEL_BVH_WIDE8_Q8;
        info.max_depth = db.max_depth;
        info.build_ms = db.build_ms;
        info.upload_ms = 0.0;
        for (int a = 0; a < 3; ++a) { info.bounds_lo[a] = db.lo[a]; info.bounds_hi[a] = db.hi[a]; }
        return SEL_OK;
    }
    BuiltBvh built;
    auto t0 = std::chrono::steady_clock::now();
    std::string err;
    try {
        err = build_bvh(scene->meshes, scene->kind, built);
    } catch (const std::bad_alloc&) {
        return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed during BVH build");
    }
    if (!err.empty()) return fail(SEL_ERR_INVALID_OPERATION, err);
    auto t1 = std::chrono::steady_clock::now();
    const void* nodes_src = scene->kind == SEL_BVH_WIDE8_Q8 ? static_cast<const void*>(built.wide.data())
                                                            : static_cast<const void*>(built.binary.data());
    const size_t node_count = scene->kind == SEL_BVH_WIDE8_Q8 ? built.wide.size() : built.binary.size();
    const size_t node_bytes = node_count * (scene->kind == SEL_BVH_WIDE8_Q8 ? sizeof(WideNode) : sizeof(BinaryNode));
    const size_t tri_bytes = built.tris.size() * sizeof(TriRecord);
    if (scene->d_nodes) cudaFree(scene->d_nodes);
    if (scene->d_tris) cudaFree(scene->d_tris);
    scene->d_nodes = scene->d_tris = nullptr;
    cudaError_t e = cudaMalloc(&scene->d_nodes, node_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&scene->d_tris, tri_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(scene)");
    e = cudaMemcpy(scene->d_nodes, nodes_src, node_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(scene->d_tris, built.tris.data(), tri_bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(scene)");
    auto t2 = std::chrono::steady_clock::now();
    SelSceneInfo& info = scene->info;
    std::memset(&info, 0, sizeof(info));
    info.triangle_count = built.tris.size();
    info.node_count = node_count;
    info.device_bytes = node_bytes + tri_bytes;
    info.bvh_kind = uint32_t(scene->kind);
    info.max_depth = built.max_depth;
    info.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    info.upload_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    for (int a = 0; a < 3; ++a) { info.bounds_lo[a] = built.lo[a]; info.bounds_hi[a] = built.hi[a]; }
    return SEL_OK;
}

}  // namespace

extern "C" {

int sel_scene_get_info(SelScene scene, SelSceneInfo* out_info) {
    if (!scene || !out_info) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (!scene->committed) return fail(SEL_ERR_INVALID_OPERATION, "scene not committed");
    *out_info = scene->info;
    return SEL_OK;
}

int sel_device_set_option(SelDevice device, int option, int value) {
    if (!device) return fail(SEL_ERR_INVALID_ARGUMENT, "device is null");
    std::lock_guard<std::mutex> lock(device->mu);
    switch (option) {
        case SEL_OPTION_GRAPH_REPLAY:
            device->graph_replay = value != 0;
            return SEL_OK;
        case SEL_OPTION_MATERIAL_SORT:
            device->material_sort = value != 0;
            return SEL_OK;
        case SEL_OPTION_RAY_SORT:
            device->ray_sort = value != 0;
            return SEL_OK;
        case SEL_OPTION_ZERO_COPY:
            device->zero_copy = value != 0;
            return SEL_OK;
        default:
            return fail(SEL_ERR_INVALID_ARGUMENT, "unknown option");
    }
}

int sel_scene_release(SelScene scene) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if (scene->instanced_by > 0)
        return fail(SEL_ERR_INVALID_OPERATION, "scene is instanced by a committed scene: release that one first");
    set_device(scene->dev);
    cudaStreamSynchronize(scene->dev->stream);
    for (auto& r : scene->referenced) --r.first->instanced_by;
    for (void* p : {scene->d_nodes, scene->d_tris, scene->scratch, scene->d_materials, scene->d_lights,
                    scene->d_light_sets, scene->pt_block, scene->d_accum, scene->d_ptex_faces, scene->d_ptex_texels,
                    scene->vcm_block, scene->d_insts, scene->d_view, scene->d_ibl, scene->d_attrs, scene->d_textures})
        if (p) cudaFree(p);
    std::vector<SelSceneTy*> owned = std::move(scene->owned);
    delete scene;
    for (auto it = owned.rbegin(); it != owned.rend(); ++it) sel_scene_release(*it);
    return SEL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------
// Queries
// ---------------------------------------------------------------------------------------------------
static int check_query(SelScene scene) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if (!scene->committed) return fail(SEL_ERR_INVALID_OPERATION, "scene not committed");
    if (!instances_fresh(scene))
        return fail(SEL_ERR_INVALID_OPERATION, "an instanced scene changed since this scene was committed");
    return SEL_OK;
}

// The device address of `bytes` of host memory at p when the whole range is page-locked memory that the current
// device can address (cudaHostAlloc / cudaMallocHost / cudaHostRegister under unified addressing): both ends
// must belong to pinned memory mapped contiguously into the device's address space.
static bool mapped_host_range(const void* p, size_t bytes, int device, void** dptr) {
    cudaPointerAttributes a{}, b{};
    const char* first = static_cast<const char*>(p);
    const char* last = first + bytes - 1;
    if (cudaPointerGetAttributes(&a, first) != cudaSuccess || cudaPointerGetAttributes(&b, last) != cudaSuccess) {
        cudaGetLastError();  // unregistered memory on older runtimes reports an error: not mapped
        return false;
    }
    if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer || !b.devicePointer)
        return false;
    if (a.device != device || b.device != device) return false;
    if (static_cast<const char*>(b.devicePointer) - static_cast<const char*>(a.devicePointer) != last - first)
        return false;
    *dptr = a.devicePointer;
    return true;
}

// Whether a batch's rays run nearly parallel from one record to the next (camera rays in pixel order): sampled
// pairs of neighbouring records, directions within about 2.5 degrees.  Such rays traverse so fast that moving
// the records over the host link is the whole cost, and the copy engines' full-duplex staging moves them
// fastest; incoherent rays traverse long enough to hide the link's latency, and the query kernel reads and
// writes them in place.
static bool coherent_batch(const void* recs, size_t byte_stride, unsigned int M) {
    constexpr unsigned kPairs = 256;
    if (M < 2) return false;
    const unsigned pairs = std::min(M - 1, kPairs);
    const size_t step = size_t(M - 1) / pairs;
    const char* base = static_cast<const char*>(recs);
    unsigned close = 0;
    for (unsigned k = 0; k < pairs; ++k) {
        const float* a = reinterpret_cast<const float*>(base + size_t(k) * step * byte_stride) + 4;
        const float* b = reinterpret_cast<const float*>(base + (size_t(k) * step + 1) * byte_stride) + 4;
        const double d = double(a[0]) * b[0] + double(a[1]) * b[1] + double(a[2]) * b[2];
        const double n = std::sqrt((double(a[0]) * a[0] + double(a[1]) * a[1] + double(a[2]) * a[2]) *
                                   (double(b[0]) * b[0] + double(b[1]) * b[1] + double(b[2]) * b[2]));
        if (n > 0.0 && d > 0.999 * n) ++close;
    }
    return 2 * close > pairs;
}

template <typename Rec, bool kHit>
static int host_query(SelScene scene, Rec* recs, unsigned int M, size_t byte_stride) {
    if (int rc = check_query(scene)) return rc;
    if (M == 0) return SEL_OK;
    if (!recs) return fail(SEL_ERR_INVALID_ARGUMENT, "ray buffer is null");
    if (byte_stride < sizeof(Rec)) return fail(SEL_ERR_INVALID_ARGUMENT, "byte_stride smaller than the record");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    SelDeviceTy* dev = scene->dev;
    std::lock_guard<std::mutex> dlock(dev->mu);
    const size_t bytes = size_t(M) * sizeof(Rec);
    const bool dense = byte_stride == sizeof(Rec);
    cudaError_t e = cudaSuccess;
    // Records in page-locked host memory the GPU can address (over NVLink-C2C on Grace): the query kernel reads
    // each ray and writes each hit in place, so only the fields it touches cross the link and no staging buffer
    // or copy is needed.  Any 16-byte aligned stride that is a multiple of 16 works.  Large dense batches of
    // coherent rays take the staged pipeline below instead (coherent_batch).
    constexpr unsigned kChunk = 1u << 18;
    const bool staged_pipeline = dense && M > 2 * kChunk;
    void* mapped = nullptr;
    if (dev->zero_copy && byte_stride % 16 == 0 && (reinterpret_cast<uintptr_t>(recs) & 15u) == 0 &&
        !(staged_pipeline && coherent_batch(recs, byte_stride, M)) &&
        mapped_host_range(recs, size_t(M - 1) * byte_stride + sizeof(Rec), dev->cuda_device, &mapped)) {
        e = launch_query_strided(!kHit, device_bvh(scene), mapped, byte_stride, M, dev->d_err, dev->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(dev->stream);
        if (e != cudaSuccess) return cuda_fail(e, "zero-copy query");
        return read_error_word(dev, dev->stream);
    }
    // Large dense batches: chunks pipelined over four streams, so that uploads, traversals and downloads of
    // different chunks overlap (the copy engines move both directions at once while the SMs traverse).
    if (staged_pipeline) {
        if (int rc = ensure_scratch(scene, 4 * size_t(kChunk) * sizeof(Rec))) return rc;
        Rec* slots = static_cast<Rec*>(scene->scratch);
        const DeviceBvh bvh = device_bvh(scene);
        for (unsigned c0 = 0, c = 0; c0 < M && e == cudaSuccess; c0 += kChunk, ++c) {
            const unsigned n = std::min(kChunk, M - c0);
            cudaStream_t q = dev->qstream[c % 4];
            Rec* d = slots + size_t(c % 4) * kChunk;
            e = cudaMemcpyAsync(d, recs + c0, size_t(n) * sizeof(Rec), cudaMemcpyHostToDevice, q);
            if (e != cudaSuccess) break;
            e = kHit ? launch_intersect(bvh, reinterpret_cast<SelRayHit*>(d), n, dev->d_err, q)
                     : launch_occluded(bvh, reinterpret_cast<SelRay*>(d), n, dev->d_err, q);
            if (e != cudaSuccess) break;
            e = cudaMemcpyAsync(recs + c0, d, size_t(n) * sizeof(Rec), cudaMemcpyDeviceToHost, q);
        }
        for (cudaStream_t q : dev->qstream) {
            const cudaError_t es = cudaStreamSynchronize(q);
            if (e == cudaSuccess) e = es;
        }
        if (e != cudaSuccess) return cuda_fail(e, "pipelined query");
        return read_error_word(dev, dev->stream);
    }
    if (int rc = ensure_scratch(scene, bytes)) return rc;
    cudaStream_t s = dev->stream;
    std::vector<Rec> packed;
    if (dense) {
        e = cudaMemcpyAsync(scene->scratch, recs, bytes, cudaMemcpyHostToDevice, s);
    } else {
        packed.resize(M);
        const char* src = reinterpret_cast<const char*>(recs);
        for (unsigned i = 0; i < M; ++i) std::memcpy(&packed[i], src + size_t(i) * byte_stride, sizeof(Rec));
        e = cudaMemcpyAsync(scene->scratch, packed.data(), bytes, cudaMemcpyHostToDevice, s);
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(rays to device)");
    if (kHit)
        e = launch_intersect(device_bvh(scene), static_cast<SelRayHit*>(scene->scratch), M, dev->d_err, s);
    else
        e = launch_occluded(device_bvh(scene), static_cast<SelRay*>(scene->scratch), M, dev->d_err, s);
    if (e != cudaSuccess) return cuda_fail(e, "query launch");
    if (dense) {
        e = cudaMemcpyAsync(recs, scene->scratch, bytes, cudaMemcpyDeviceToHost, s);
    } else {
        e = cudaMemcpyAsync(packed.data(), scene->scratch, bytes, cudaMemcpyDeviceToHost, s);
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(rays to host)");
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "query");
    if (!dense) {
        char* dst = reinterpret_cast<char*>(recs);
        for (unsigned i = 0; i < M; ++i) std::memcpy(dst + size_t(i) * byte_stride, &packed[i], sizeof(Rec));
    }
    return read_error_word(dev, s);
}

extern "C" {

int sel_intersect1(SelScene scene, SelRayHit* rayhit) {
    return host_query<SelRayHit, true>(scene, rayhit, 1, sizeof(SelRayHit));
}

int sel_occluded1(SelScene scene, SelRay* ray) { return host_query<SelRay, false>(scene, ray, 1, sizeof(SelRay)); }

int sel_intersect1M(SelScene scene, SelRayHit* rayhits, unsigned int M, size_t byte_stride) {
    return host_query<SelRayHit, true>(scene, rayhits, M, byte_stride);
}

int sel_occluded1M(SelScene scene, SelRay* rays, unsigned int M, size_t byte_stride) {
    return host_query<SelRay, false>(scene, rays, M, byte_stride);
}

int sel_intersect_device(SelScene scene, SelRayHit* d_rayhits, unsigned int n, void* stream) {
    if (int rc = check_query(scene)) return rc;
    if (n == 0) return SEL_OK;
    if (!d_rayhits || (reinterpret_cast<uintptr_t>(d_rayhits) & 15u))
        return fail(SEL_ERR_INVALID_ARGUMENT, "d_rayhits must be a 16-byte aligned device pointer");
    if (int rc = set_device(scene->dev)) return rc;
    cudaError_t e = launch_intersect(device_bvh(scene), d_rayhits, n, scene->dev->d_err, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "intersect launch");
    return SEL_OK;
}

int sel_occluded_device(SelScene scene, SelRay* d_rays, unsigned int n, void* stream) {
    if (int rc = check_query(scene)) return rc;
    if (n == 0) return SEL_OK;
    if (!d_rays || (reinterpret_cast<uintptr_t>(d_rays) & 15u))
        return fail(SEL_ERR_INVALID_ARGUMENT, "d_rays must be a 16-byte aligned device pointer");
    if (int rc = set_device(scene->dev)) return rc;
    cudaError_t e = launch_occluded(device_bvh(scene), d_rays, n, scene->dev->d_err, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "occluded launch");
    return SEL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------
// Camera set-up on the host (compiled without contraction so the CPU oracle, which restates the same
// steps, derives a bit-identical basis): InitializeRayCastCamera (GeometryLib/Camera.cpp:89-115).
// ---------------------------------------------------------------------------------------------------
namespace sel {

void init_camera(const SelCamera& c, PtCamera& out) {
    auto sub = [](const float* a, const float* b, float* o) { for (int i = 0; i < 3; ++i) o[i] = a[i] - b[i]; };
    auto norm = [](float* v) {
        const float il = 1.0f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int i = 0; i < 3; ++i) v[i] = v[i] * il;
    };
    auto cross = [](const float* a, const float* b, float* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    const float widthf = float(c.width), heightf = float(c.height);
    const float aspect = widthf / heightf;
    const float hfov = c.fovDegrees * (3.141592653589793f / 180.0f);
    const float hlen = std::tan(hfov * 0.5f);
    const float vfov = 2.0f * std::atan(hlen / aspect);
    const float vlen = std::tan(vfov * 0.5f);
    float fwd[3], right[3], upv[3];
    sub(c.lookAt, c.position, fwd);
    norm(fwd);
    cross(c.up, fwd, right);
    norm(right);
    cross(fwd, right, upv);
    for (int i = 0; i < 3; ++i) {
        out.x[i] = hlen * right[i];
        out.y[i] = vlen * upv[i];
        out.z[i] = fwd[i];
        out.position[i] = c.position[i];
    }
    out.width = c.width;
    out.height = c.height;
}

}  // namespace sel
