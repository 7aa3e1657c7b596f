// Cooked asset loading: the reference's binary SceneResource / SubsceneResource / ModelResource /
// ModelGeometryResource / Textures / IBL blobs read into device scenes.
//
// The reference reads each blob whole and attaches it in place (ReadSceneResource, SceneResource.cpp:271-283;
// ReadSubsceneResource, SubsceneResource.cpp:101-113; ReadModelResource / LoadModelGeometry,
// ModelResource.cpp:432-467; ReadTextureResource, TextureResource.cpp:46-58; ReadImageBasedLightResource,
// ImageBasedLightResource.cpp:52-65): AttachToBinary (IoLib/BinaryStreamSerializer.h:34-44) rewrites every
// pointer field, which SerializeToBinary stored as a byte offset from the start of the file, into an address.
// Here the blob is read into host memory and every field is read at its offset with bounds checks instead; no
// pointer is patched, and a blob whose offsets or counts leave the file is refused.
//
// The scene graph becomes the two-level instancing of sel_scene_attach_instance, with the ids the reference's
// Embree scenes give (SceneResource.cpp:229-256, SubsceneResource.cpp:63-79, ModelResource.cpp:231-298):
//   top scene           instance i  = subsceneInstances[i]  of the subscene scene subsceneNames[index]
//   subscene scene      instance j  = modelInstances[j]     of the model scene modelNames[index]
//   model scene         geomID k    = meshes[k]             (a triangle or quad mesh)
// so hits report instID[0] = i, instID[1] = j, geomID = k, as ModelDataFromRayIds expects
// (SceneResource.cpp:362-378).  Each subscene loads its own copy of each model it names, as
// InitializeSubsceneResource does (SubsceneResource.cpp:116-137): materials and light sets are per subscene.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "selas.h"

using sel::fail;

namespace {

// ------------------------------------------------------------------------------------------------
// Blob layouts (x86-64 and aarch64 alike: natural alignment, no padding between the fields listed).
// ------------------------------------------------------------------------------------------------

// CArray<T> (ContainersLib/CArray.h:57-63): flags u32, padding u32, count u64, capacity u64, data (file offset).
constexpr size_t kArrCount = 8, kArrData = 24;
constexpr size_t kPath = 512;  // FilePathString = FixedString<MaxPath_>

// SceneResourceData (SceneLib/SceneResource.h:49-59)
constexpr size_t kSceneIbl = 512, kSceneBackground = 1024, kSceneSubsceneNames = 1040,
                 kSceneSubsceneInstances = 1072, kSceneLights = 1104, kSceneLightSetRanges = 1136, kSceneCameras = 1168,
                 kSceneSize = 1200;
// Instance (SubsceneResource.h:26-36): index u64, localToWorld float4x4.
constexpr size_t kInstance = 72;
// SceneLight (SceneResource.h:32-40): type u32, position, direction, x, z, radiance (float3 each).
constexpr size_t kLight = 64;
// CameraSettings (GeometryLib/Camera.h:17-26): name FixedString128, position, fovDegrees, lookAt, znear, up, zfar.
constexpr size_t kCamera = 176, kCamPosition = 128, kCamFov = 140, kCamLookAt = 144, kCamNear = 156, kCamUp = 160,
                 kCamFar = 172;
// SubsceneResourceData (SubsceneResource.h:39-47)
constexpr size_t kSubLightSet = 512, kSubModelNames = 520, kSubModelInstances = 552, kSubMaterialNames = 584,
                 kSubMaterials = 616, kSubSize = 648;
// MaterialResourceData (ModelResource.h:68-88): baseColorTexture, shader, flags, baseColor, transmittanceColor,
// scalarAttributeValues[eMaterialPropertyCount = 14].
constexpr size_t kMaterial = 600, kMatShader = 512, kMatFlags = 516, kMatBase = 520, kMatTrans = 532, kMatScalars = 544;
constexpr uint32_t kFlagTransparent = 1u, kFlagUsesPtex = 16u;  // MaterialFlags (ModelResource.h:36-43)
// MeshMetaData (ModelResource.h:113-123): indexCount, indexOffset, vertexCount, vertexOffset, materialHash,
// indicesPerFace, nameHash (u32 each), name FixedString64.
constexpr size_t kMesh = 92, kMeshName = 28;
// ModelResourceData (ModelResource.h:125-149)
constexpr size_t kModelVertexCount = 24, kModelCurveVertexCount = 28, kModelCurveName = 32, kModelMaterials = 168,
                 kModelMaterialHashes = 200, kModelMeshes = 232, kModelCurves = 264, kModelSize = 296;
// ModelGeometryData (ModelResource.h:151-170): eight u64 sizes (index, faceIndex, position, normals, tangents, uvs,
// curveIndex, curveVertex), then the eight arrays (file offsets) in the same order.
constexpr size_t kGeomSizes = 0, kGeomPtrs = 64, kGeomSize = 128;
// TextureResourceData (TextureLib/TextureResource.h:12-34): mipCount, dataSize, mipWidths[16], mipHeights[16],
// mipOffsets[16] (u64), format, pad, texture.
constexpr size_t kTexMipCount = 0, kTexDataSize = 4, kTexWidths = 8, kTexHeights = 72, kTexOffsets = 136,
                 kTexFormat = 264, kTexData = 272, kTexSize = 280;
// ImageBasedLightResourceData (SceneLib/ImageBasedLightResource.h:16-35): densityfunctions {width u64, height u64,
// marginal, conditional}, missWidth u64, missHeight u64, rotationRadians, exposureScale, lightData, missData.
constexpr size_t kIblWidth = 0, kIblHeight = 8, kIblMissWidth = 32, kIblMissHeight = 40, kIblRotation = 48,
                 kIblExposure = 52, kIblLight = 56, kIblMiss = 64, kIblSize = 72;

// Asset type names and versions (kDataType / kDataVersion of each resource).
constexpr const char* kSceneType = "SceneResource";
constexpr unsigned long long kSceneVersion = 1539147471ull;
constexpr const char* kSubsceneType = "SubsceneResource";
constexpr unsigned long long kSubsceneVersion = 1539551841ull;
constexpr const char* kModelType = "ModelResource";
constexpr const char* kModelGeometryType = "ModelGeometryResource";
constexpr unsigned long long kModelVersion = 1539636447ull;
constexpr const char* kTextureType = "Textures";
constexpr unsigned long long kTextureVersion = 1534887410ull;
constexpr const char* kIblType = "IBL";
constexpr unsigned long long kIblVersion = 1538087123ull;

struct BlobError {
    std::string msg;
};

// A whole blob in host memory with checked field reads.
struct Blob {
    std::string path;
    std::vector<unsigned char> bytes;

    void need(size_t off, size_t n) const {
        if (off > bytes.size() || n > bytes.size() - off)
            throw BlobError{path + ": field at byte " + std::to_string(off) + " (+" + std::to_string(n) +
                            ") lies past the end of the file (" + std::to_string(bytes.size()) + " bytes)"};
    }
    template <typename T>
    T get(size_t off) const {
        need(off, sizeof(T));
        T v;
        std::memcpy(&v, bytes.data() + off, sizeof(T));
        return v;
    }
    std::string str(size_t off, size_t cap) const {
        need(off, cap);
        const char* p = reinterpret_cast<const char*>(bytes.data() + off);
        return std::string(p, strnlen(p, cap));
    }
    // An array of `count` elements of `elem` bytes at the file offset stored at `ptr_off`.
    size_t array(size_t ptr_off, uint64_t count, size_t elem, const char* what) const {
        const uint64_t data = get<uint64_t>(ptr_off);
        if (count == 0) return 0;
        if (count > (uint64_t(1) << 40) / std::max<size_t>(elem, 1))
            throw BlobError{path + ": " + what + " count " + std::to_string(count) + " is not plausible"};
        need(size_t(data), size_t(count) * elem);
        return size_t(data);
    }
    // A CArray field at `off`: (count, offset of element 0).
    std::pair<uint64_t, size_t> carray(size_t off, size_t elem, const char* what) const {
        const uint64_t count = get<uint64_t>(off + kArrCount);
        return {count, array(off + kArrData, count, elem, what)};
    }
};

Blob read_blob(const std::string& root, const char* type, unsigned long long version, const std::string& name) {
    Blob b;
    b.path = root + "/_Assets/" + type + "/" + std::to_string(version) + "/" + name + ".bin";
    FILE* f = std::fopen(b.path.c_str(), "rb");
    if (!f) throw BlobError{"cannot open " + b.path};
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (size < 0) {
        std::fclose(f);
        throw BlobError{"cannot size " + b.path};
    }
    b.bytes.resize(size_t(size));
    const bool ok = size == 0 || std::fread(b.bytes.data(), 1, size_t(size), f) == size_t(size);
    std::fclose(f);
    if (!ok) throw BlobError{"cannot read " + b.path};
    return b;
}

void read_floats(const Blob& b, size_t off, float* out, int n) {
    for (int i = 0; i < n; ++i) out[i] = b.get<float>(off + 4 * size_t(i));
}

// ------------------------------------------------------------------------------------------------
// Parsed asset graph.
// ------------------------------------------------------------------------------------------------

struct Material {
    std::string texture;
    uint32_t shader = 1, flags = 0;
    float base[3] = {0.6f, 0.6f, 0.6f}, trans[3] = {0.0f, 0.0f, 0.0f};
    float scalars[14] = {};
};

Material default_material() {  // CreateDefaultMaterial (ModelResource.cpp:203-211)
    Material m;
    m.scalars[11] = 1.5f;      // eIor
    return m;
}

Material parse_material(const Blob& b, size_t off) {
    Material m;
    m.texture = b.str(off, kPath);
    m.shader = b.get<uint32_t>(off + kMatShader);
    m.flags = b.get<uint32_t>(off + kMatFlags);
    read_floats(b, off + kMatBase, m.base, 3);
    read_floats(b, off + kMatTrans, m.trans, 3);
    read_floats(b, off + kMatScalars, m.scalars, 14);
    if (m.shader > 2u) throw BlobError{b.path + ": material shader " + std::to_string(m.shader) + " is not a ShaderType"};
    return m;
}

struct Instance {
    uint64_t index;
    float l2w[16];  // the float4x4 as stored: the column-major localToWorld
};

std::vector<Instance> parse_instances(const Blob& b, size_t field, size_t targets, const char* what) {
    const auto arr = b.carray(field, kInstance, what);
    std::vector<Instance> out(arr.first);
    for (size_t i = 0; i < out.size(); ++i) {
        const size_t o = arr.second + i * kInstance;
        out[i].index = b.get<uint64_t>(o);
        read_floats(b, o + 8, out[i].l2w, 16);
        if (out[i].index >= targets)
            throw BlobError{b.path + ": " + what + " " + std::to_string(i) + " names entry " +
                            std::to_string(out[i].index) + " of " + std::to_string(targets)};
    }
    return out;
}

std::vector<std::string> parse_names(const Blob& b, size_t field, const char* what) {
    const auto arr = b.carray(field, kPath, what);
    std::vector<std::string> out(arr.first);
    for (size_t i = 0; i < out.size(); ++i) out[i] = b.str(arr.second + i * kPath, kPath);
    return out;
}

struct Mesh {
    uint32_t index_count, index_offset, material_hash, per_face;
    std::string name;
};

struct Model {
    std::string name;
    uint32_t vertex_count = 0;
    std::vector<uint32_t> hashes;  // sorted by the build step (BinarySearch needs it)
    std::vector<Material> materials;
    std::vector<Mesh> meshes;
    uint64_t curves = 0;
    std::vector<std::pair<uint32_t, uint32_t>> curve_ranges;  // CurveMetaData: (indexOffset, indexCount)
    uint32_t curve_material = 0;                              // curveModelName (a material name hash)
    uint32_t curve_vertex_count = 0;
    size_t curve_indices = 0, curve_vertices = 0;             // offsets in the geometry blob
    Blob geometry;
    size_t indices = 0, positions = 0, normals = 0, tangents = 0, uvs = 0;  // offsets (0: absent)
    uint64_t index_count = 0;
    bool has_normals = false, has_tangents = false, has_uvs = false;
};

struct Subscene {
    std::string name;
    uint64_t light_set = 0;
    std::vector<std::string> model_names;
    std::vector<Instance> instances;
    std::vector<uint32_t> material_names;
    std::vector<Material> materials;
    std::vector<Model> models;  // one per model name: this subscene's own copy
};

struct Camera {
    float position[3], look_at[3], up[3], fov, znear, zfar;
};

struct SceneAssets {
    std::string root, name, ibl;
    float background[4];
    std::vector<std::string> subscene_names;
    std::vector<Instance> instances;
    struct Light {
        uint32_t type;
        float v[15];
    };
    std::vector<Light> lights;
    std::vector<std::pair<uint32_t, uint32_t>> ranges;
    std::vector<Camera> cameras;
    std::vector<Subscene> subscenes;
};

Model load_model(const std::string& root, const std::string& name) {
    Model m;
    m.name = name;
    const Blob b = read_blob(root, kModelType, kModelVersion, name);
    b.need(0, kModelSize);
    m.vertex_count = b.get<uint32_t>(kModelVertexCount);
    const auto mats = b.carray(kModelMaterials, kMaterial, "materials");
    const auto hashes = b.carray(kModelMaterialHashes, 4, "materialHashes");
    if (mats.first != hashes.first) throw BlobError{b.path + ": materials and materialHashes differ in count"};
    for (uint64_t i = 0; i < mats.first; ++i) {
        m.materials.push_back(parse_material(b, mats.second + i * kMaterial));
        m.hashes.push_back(b.get<uint32_t>(hashes.second + i * 4));
    }
    const auto meshes = b.carray(kModelMeshes, kMesh, "meshes");
    for (uint64_t i = 0; i < meshes.first; ++i) {
        const size_t o = meshes.second + i * kMesh;
        Mesh x;
        x.index_count = b.get<uint32_t>(o);
        x.index_offset = b.get<uint32_t>(o + 4);
        x.material_hash = b.get<uint32_t>(o + 16);
        x.per_face = b.get<uint32_t>(o + 20);
        x.name = b.str(o + kMeshName, 64);
        if (x.per_face != 3u && x.per_face != 4u)
            throw BlobError{b.path + ": mesh " + x.name + " has " + std::to_string(x.per_face) +
                            " indices per face (3: triangles, 4: quads)"};
        if (x.index_count % x.per_face)
            throw BlobError{b.path + ": mesh " + x.name + " index count is not a multiple of its face size"};
        m.meshes.push_back(x);
    }
    const auto curves = b.carray(kModelCurves, 8, "curves");
    m.curves = curves.first;
    for (uint64_t i = 0; i < curves.first; ++i)  // CurveMetaData (ModelResource.h:107-111): indexOffset, indexCount
        m.curve_ranges.emplace_back(b.get<uint32_t>(curves.second + 8 * i), b.get<uint32_t>(curves.second + 8 * i + 4));
    m.curve_vertex_count = b.get<uint32_t>(kModelCurveVertexCount);
    m.curve_material = b.get<uint32_t>(kModelCurveName);

    m.geometry = read_blob(root, kModelGeometryType, kModelVersion, name);
    const Blob& g = m.geometry;
    g.need(0, kGeomSize);
    uint64_t sizes[8];
    for (int i = 0; i < 8; ++i) sizes[i] = g.get<uint64_t>(kGeomSizes + 8 * size_t(i));
    if (sizes[0] % 4) throw BlobError{g.path + ": index bytes not a multiple of 4"};
    const uint64_t nv = m.vertex_count;
    if (sizes[2] != nv * 12) throw BlobError{g.path + ": position bytes do not match totalVertexCount"};
    m.has_normals = sizes[3] > 0;
    m.has_tangents = sizes[4] > 0;
    m.has_uvs = sizes[5] > 0;
    if ((m.has_normals && sizes[3] != nv * 12) || (m.has_tangents && sizes[4] != nv * 16) ||
        (m.has_uvs && sizes[5] != nv * 8))
        throw BlobError{g.path + ": attribute bytes do not match totalVertexCount"};
    m.index_count = sizes[0] / 4;
    m.indices = g.array(kGeomPtrs + 0, m.index_count, 4, "indices");
    m.positions = g.array(kGeomPtrs + 16, nv, 12, "positions");
    if (m.has_normals) m.normals = g.array(kGeomPtrs + 24, nv, 12, "normals");
    if (m.has_tangents) m.tangents = g.array(kGeomPtrs + 32, nv, 16, "tangents");
    if (m.has_uvs) m.uvs = g.array(kGeomPtrs + 40, nv, 8, "uvs");
    for (const Mesh& x : m.meshes) {
        if (uint64_t(x.index_offset) + x.index_count > m.index_count)
            throw BlobError{g.path + ": mesh " + x.name + " indexes past the index array"};
        for (uint32_t k = 0; k < x.index_count; ++k)
            if (g.get<uint32_t>(m.indices + 4 * (size_t(x.index_offset) + k)) >= nv)
                throw BlobError{g.path + ": mesh " + x.name + " indexes past the vertex array"};
    }
    // curves (InitializeCurves, ModelResource.cpp:300-332): one index per segment into the float4 control points
    if (m.curves) {
        const uint64_t ncv = m.curve_vertex_count;
        if (sizes[6] % 4 || sizes[7] != ncv * 16) throw BlobError{g.path + ": curve array sizes"};
        m.curve_indices = g.array(kGeomPtrs + 48, sizes[6] / 4, 4, "curveIndices");
        m.curve_vertices = g.array(kGeomPtrs + 56, ncv, 16, "curveVertices");
        for (const auto& c : m.curve_ranges) {
            if (uint64_t(c.first) + c.second > sizes[6] / 4) throw BlobError{g.path + ": a curve indexes past curveIndices"};
            for (uint32_t k = 0; k < c.second; ++k)
                if (uint64_t(g.get<uint32_t>(m.curve_indices + 4 * (size_t(c.first) + k))) + 3 >= ncv)
                    throw BlobError{g.path + ": a curve segment runs past curveVertices"};
        }
    }
    return m;
}

SceneAssets load_assets(const std::string& root, const std::string& name) {
    SceneAssets s;
    s.root = root;
    s.name = name;
    const Blob b = read_blob(root, kSceneType, kSceneVersion, name);
    b.need(0, kSceneSize);
    s.ibl = b.str(kSceneIbl, kPath);
    read_floats(b, kSceneBackground, s.background, 4);
    s.subscene_names = parse_names(b, kSceneSubsceneNames, "subsceneNames");
    s.instances = parse_instances(b, kSceneSubsceneInstances, s.subscene_names.size(), "subsceneInstances");
    const auto lights = b.carray(kSceneLights, kLight, "lights");
    for (uint64_t i = 0; i < lights.first; ++i) {
        SceneAssets::Light l;
        l.type = b.get<uint32_t>(lights.second + i * kLight);
        read_floats(b, lights.second + i * kLight + 4, l.v, 15);
        if (l.type != 0u) throw BlobError{b.path + ": light type " + std::to_string(l.type) + " is not QuadLight"};
        s.lights.push_back(l);
    }
    const auto ranges = b.carray(kSceneLightSetRanges, 8, "lightSetRanges");
    for (uint64_t i = 0; i < ranges.first; ++i) {
        const uint32_t start = b.get<uint32_t>(ranges.second + i * 8), count = b.get<uint32_t>(ranges.second + i * 8 + 4);
        if (uint64_t(start) + count > s.lights.size())
            throw BlobError{b.path + ": light set range " + std::to_string(i) + " leaves the light array"};
        s.ranges.emplace_back(start, count);
    }
    const auto cams = b.carray(kSceneCameras, kCamera, "cameras");
    for (uint64_t i = 0; i < cams.first; ++i) {
        const size_t o = cams.second + i * kCamera;
        Camera c;
        read_floats(b, o + kCamPosition, c.position, 3);
        c.fov = b.get<float>(o + kCamFov);
        read_floats(b, o + kCamLookAt, c.look_at, 3);
        c.znear = b.get<float>(o + kCamNear);
        read_floats(b, o + kCamUp, c.up, 3);
        c.zfar = b.get<float>(o + kCamFar);
        s.cameras.push_back(c);
    }
    for (const std::string& sn : s.subscene_names) {
        const Blob sb = read_blob(root, kSubsceneType, kSubsceneVersion, sn);
        sb.need(0, kSubSize);
        Subscene sub;
        sub.name = sn;
        sub.light_set = sb.get<uint64_t>(kSubLightSet);
        sub.model_names = parse_names(sb, kSubModelNames, "modelNames");
        sub.instances = parse_instances(sb, kSubModelInstances, sub.model_names.size(), "modelInstances");
        const auto names = sb.carray(kSubMaterialNames, 4, "sceneMaterialNames");
        const auto mats = sb.carray(kSubMaterials, kMaterial, "sceneMaterials");
        if (names.first > mats.first) throw BlobError{sb.path + ": more sceneMaterialNames than sceneMaterials"};
        for (uint64_t i = 0; i < names.first; ++i) {
            sub.material_names.push_back(sb.get<uint32_t>(names.second + i * 4));
            sub.materials.push_back(parse_material(sb, mats.second + i * kMaterial));
        }
        for (const std::string& mn : sub.model_names) sub.models.push_back(load_model(root, mn));
        s.subscenes.push_back(std::move(sub));
    }
    return s;
}

// FindMeshMaterial (ModelResource.cpp:213-229): the model's own materials by BinarySearch over their sorted
// hashes (UtilityLib/BinarySearch.h: the first element >= the key, a match if equal; where every hash is below
// the key the reference reads data[-1], which is taken here as no match), then the subscene's scene materials in
// order, else the default material.
const Material& find_mesh_material(const Model& m, const Subscene& s, uint32_t hash, const Material& fallback) {
    if (!m.materials.empty()) {
        const auto it = std::lower_bound(m.hashes.begin(), m.hashes.end(), hash);
        if (it != m.hashes.end() && *it == hash) return m.materials[size_t(it - m.hashes.begin())];
    }
    for (size_t i = 0; i < s.material_names.size(); ++i)
        if (s.material_names[i] == hash) return s.materials[i];
    return fallback;
}

SelMaterial to_sel(const Material& m, uint32_t light_set) {
    SelMaterial o;
    std::memset(&o, 0, sizeof(o));
    o.shader = int32_t(m.shader);
    o.lightSetIndex = light_set;
    for (int i = 0; i < 3; ++i) {
        o.baseColor[i] = m.base[i];
        o.transmittanceColor[i] = m.trans[i];
    }
    // scalarAttributeValues in ScalarMaterialProperties order (ModelResource.h:45-66)
    o.metallic = m.scalars[0];
    o.specularTint = m.scalars[1];
    o.roughness = m.scalars[2];
    o.anisotropic = m.scalars[3];
    o.sheen = m.scalars[4];
    o.sheenTint = m.scalars[5];
    o.clearcoat = m.scalars[6];
    o.clearcoatGloss = m.scalars[7];
    o.specTrans = m.scalars[8];
    o.diffuseTrans = m.scalars[9];
    o.flatness = m.scalars[10];
    o.ior = m.scalars[11];
    o.scatterDistance = m.scalars[12];
    o.usesPtex = (m.flags & kFlagUsesPtex) ? 1u : 0u;
    return o;
}

void copy_str(char* dst, size_t cap, const std::string& s) {
    const size_t n = std::min(cap - 1, s.size());
    std::memcpy(dst, s.data(), n);
    dst[n] = '\0';
}

// SetupSceneCamera (SceneResource.cpp:330-355): cameras[0] when ValidCamera (fovDegrees > 0 and zfar > znear,
// Camera.cpp:49-52), else DefaultCameraSettings (Camera.cpp:38-46).  The reference indexes cameras[0] even when
// the scene has none; that case takes the default here.
void fill_info(const SceneAssets& s, SelCookedSceneInfo* info) {
    std::memset(info, 0, sizeof(*info));
    info->subscenes = uint32_t(s.subscene_names.size());
    info->subsceneInstances = uint32_t(s.instances.size());
    for (const Subscene& sub : s.subscenes) {
        info->models += uint32_t(sub.models.size());
        info->modelInstances += uint32_t(sub.instances.size());
        for (const Model& m : sub.models) {
            info->meshes += uint32_t(m.meshes.size());
            info->curves += uint32_t(m.curves);
            for (const Mesh& x : m.meshes) {
                info->quadMeshes += x.per_face == 4u ? 1u : 0u;
                info->faces += x.index_count / x.per_face;
            }
        }
    }
    info->lights = uint32_t(s.lights.size());
    info->lightSets = uint32_t(s.ranges.size());
    info->cameras = uint32_t(s.cameras.size());
    std::memcpy(info->backgroundIntensity, s.background, sizeof(s.background));
    copy_str(info->ibl, sizeof(info->ibl), s.ibl);
    Camera c{{0.0f, 0.0f, 5.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, 35.0f, 0.01f, 10000.0f};
    if (!s.cameras.empty() && s.cameras[0].fov > 0.0f && s.cameras[0].zfar > s.cameras[0].znear) c = s.cameras[0];
    std::memcpy(info->camera.position, c.position, 12);
    std::memcpy(info->camera.lookAt, c.look_at, 12);
    std::memcpy(info->camera.up, c.up, 12);
    info->camera.fovDegrees = c.fov;
    info->camera.width = info->camera.height = 0;
}

// Every mesh in load order, with the material FindMeshMaterial resolves; counts Ptex meshes and textures.
struct MeshRow {
    uint32_t subscene, model, mesh;
    const Material* material;
};

std::vector<MeshRow> mesh_rows(const SceneAssets& s, const Material& fallback) {
    std::vector<MeshRow> rows;
    for (size_t si = 0; si < s.subscenes.size(); ++si) {
        const Subscene& sub = s.subscenes[si];
        for (size_t mi = 0; mi < sub.models.size(); ++mi) {
            const Model& m = sub.models[mi];
            for (size_t k = 0; k < m.meshes.size(); ++k)
                rows.push_back({uint32_t(si), uint32_t(mi), uint32_t(k),
                                &find_mesh_material(m, sub, m.meshes[k].material_hash, fallback)});
        }
    }
    return rows;
}

// Texels of mip 0 as the renderer samples them: TextureFiltering::Triangle reads mip 0 as packed float3 texels
// whatever the stored format (SurfaceParameters.cpp:59-73 instantiates it with float3, TextureFiltering.h:53-100),
// so RGB triples are taken from mip 0's offset on; texels past the end of the data read as 0.
std::vector<float> texture_rgb(const Blob& t, uint32_t& width, uint32_t& height) {
    t.need(0, kTexSize);
    const uint32_t mips = t.get<uint32_t>(kTexMipCount), data_size = t.get<uint32_t>(kTexDataSize);
    if (mips == 0 || mips > 16) throw BlobError{t.path + ": mip count " + std::to_string(mips)};
    width = t.get<uint32_t>(kTexWidths);
    height = t.get<uint32_t>(kTexHeights);
    const uint64_t mip0 = t.get<uint64_t>(kTexOffsets);
    if (t.get<uint32_t>(kTexFormat) > 3u) throw BlobError{t.path + ": unknown texture format"};
    if (width == 0 || height == 0 || uint64_t(width) * height > (uint64_t(1) << 28))
        throw BlobError{t.path + ": mip 0 size " + std::to_string(width) + " x " + std::to_string(height)};
    const size_t data = t.array(kTexData, data_size, 1, "texture data");
    std::vector<float> rgb(size_t(width) * height * 3, 0.0f);
    const uint64_t avail = mip0 < data_size ? (data_size - mip0) / 4 : 0;
    const size_t n = size_t(std::min<uint64_t>(avail, rgb.size()));
    if (n) std::memcpy(rgb.data(), t.bytes.data() + data + mip0, n * 4);
    return rgb;
}

struct Texture {
    std::vector<float> rgb;
    uint32_t width = 0, height = 0;
};

// TextureCache::LoadTextureResource (TextureCache.cpp:68-97) loads each name once: the textures of every mesh
// whose resolved material names one and does not sample Ptex.
std::map<std::string, Texture> load_textures(const SceneAssets& s, const std::vector<MeshRow>& rows) {
    std::map<std::string, Texture> out;
    for (const MeshRow& r : rows) {
        const Material& m = *r.material;
        if ((m.flags & kFlagUsesPtex) || m.texture.empty() || out.count(m.texture)) continue;
        Texture t;
        t.rgb = texture_rgb(read_blob(s.root, kTextureType, kTextureVersion, m.texture), t.width, t.height);
        out.emplace(m.texture, std::move(t));
    }
    return out;
}

// The model scene of one subscene's copy of model m: mesh k as geomID k with its vertex attributes, material and
// base-colour image.
int build_model(SelDevice dev, const Subscene& sub, const Model& m, const Material& fallback,
                const std::map<std::string, Texture>& textures, std::vector<SelScene>& built) {
    SelScene sc = nullptr;
    if (int rc = sel_scene_new(dev, &sc)) return rc;
    built.push_back(sc);
    const Blob& g = m.geometry;
    const unsigned char* base = g.bytes.data();
    for (size_t k = 0; k < m.meshes.size(); ++k) {
        const Mesh& x = m.meshes[k];
        // the mesh's vertex range: each geometry holds only the vertices it indexes
        std::vector<uint32_t> idx(x.index_count);
        if (!idx.empty()) std::memcpy(idx.data(), base + m.indices + 4 * size_t(x.index_offset), 4 * idx.size());
        const uint32_t lo = idx.empty() ? 0u : *std::min_element(idx.begin(), idx.end());
        const uint32_t hi = idx.empty() ? 0u : *std::max_element(idx.begin(), idx.end()) + 1u;
        for (uint32_t& i : idx) i -= lo;
        const size_t nv = hi - lo;
        std::vector<float> pos(nv * 3);
        if (nv) std::memcpy(pos.data(), base + m.positions + 12 * size_t(lo), 12 * nv);
        int rc = x.per_face == 4u
                     ? sel_scene_attach_quad_mesh(sc, unsigned(k), pos.data(), nv, 12, idx.data(), idx.size() / 4)
                     : sel_scene_attach_triangle_mesh(sc, unsigned(k), pos.data(), nv, 12, idx.data(), idx.size() / 3);
        if (rc) return rc;
        // SetMeshVertexAttributes (ModelResource.cpp:167-198): slot 0 normals, 1 tangents (float4), 2 uvs
        const size_t offs[3] = {m.has_normals ? m.normals : 0, m.has_tangents ? m.tangents : 0, m.has_uvs ? m.uvs : 0};
        const unsigned comps[3] = {3u, 4u, 2u};
        for (unsigned slot = 0; slot < 3; ++slot) {
            if (!offs[slot] || !nv) continue;
            std::vector<float> a(nv * comps[slot]);
            std::memcpy(a.data(), base + offs[slot] + 4 * size_t(comps[slot]) * lo, 4 * a.size());
            if ((rc = sel_scene_set_vertex_attribute(sc, unsigned(k), slot, a.data(), nv, comps[slot]))) return rc;
        }
        const Material& mat = find_mesh_material(m, sub, x.material_hash, fallback);
        SelMaterial sm = to_sel(mat, uint32_t(sub.light_set));
        const bool ptex = sm.usesPtex != 0u;
        sm.usesPtex = 0u;  // Ptex materials load only under SEL_COOKED_PTEX_AS_BASE_COLOR: their base colour
        if ((rc = sel::set_material_flags(sc, unsigned(k), sm, (mat.flags & kFlagTransparent) != 0u))) return rc;
        if (!ptex && !mat.texture.empty()) {
            const Texture& t = textures.at(mat.texture);
            if ((rc = sel_scene_set_texture(sc, unsigned(k), t.rgb.data(), t.width, t.height, 3))) return rc;
        }
    }
    // curve c as geomID meshes + c, with the material of the model's curveModelName and no texture
    // (InitializeGeometryUserDatas, ModelResource.cpp:346-363)
    for (size_t c = 0; c < m.curve_ranges.size(); ++c) {
        const auto& range = m.curve_ranges[c];
        std::vector<uint32_t> idx(range.second);
        if (!idx.empty()) std::memcpy(idx.data(), base + m.curve_indices + 4 * size_t(range.first), 4 * idx.size());
        const uint32_t lo = idx.empty() ? 0u : *std::min_element(idx.begin(), idx.end());
        const uint32_t hi = idx.empty() ? 0u : *std::max_element(idx.begin(), idx.end()) + 4u;
        for (uint32_t& i : idx) i -= lo;
        std::vector<float> pts(size_t(hi - lo) * 4);
        if (!pts.empty()) std::memcpy(pts.data(), base + m.curve_vertices + 16 * size_t(lo), 4 * pts.size());
        const unsigned geom = unsigned(m.meshes.size() + c);
        int rc = sel_scene_attach_curve_mesh(sc, geom, pts.data(), hi - lo, idx.data(), idx.size());
        if (rc) return rc;
        const Material& mat = find_mesh_material(m, sub, m.curve_material, fallback);
        SelMaterial sm = to_sel(mat, uint32_t(sub.light_set));
        sm.usesPtex = 0u;
        if ((rc = sel::set_material_flags(sc, geom, sm, (mat.flags & kFlagTransparent) != 0u))) return rc;
    }
    return sel_scene_commit(sc);
}

int build_scene(SelDevice dev, const SceneAssets& s, const std::vector<MeshRow>& rows, SelScene* out) {
    const Material fallback = default_material();
    const std::map<std::string, Texture> textures = load_textures(s, rows);
    std::vector<SelScene> built;  // models and subscenes, in creation order
    auto cleanup = [&built]() {
        for (auto it = built.rbegin(); it != built.rend(); ++it) sel_scene_release(*it);
    };
    std::vector<SelScene> subscene_scenes;
    for (const Subscene& sub : s.subscenes) {
        std::vector<SelScene> models;
        for (const Model& m : sub.models) {
            if (int rc = build_model(dev, sub, m, fallback, textures, built)) {
                cleanup();
                return rc;
            }
            models.push_back(built.back());
        }
        SelScene sc = nullptr;
        int rc = sel_scene_new(dev, &sc);
        if (!rc) built.push_back(sc);
        for (size_t j = 0; !rc && j < sub.instances.size(); ++j)
            rc = sel_scene_attach_instance(sc, unsigned(j), models[sub.instances[j].index], sub.instances[j].l2w);
        if (!rc) rc = sel_scene_commit(sc);
        if (rc) {
            cleanup();
            return rc;
        }
        subscene_scenes.push_back(sc);
    }
    SelScene top = nullptr;
    int rc = sel_scene_new(dev, &top);
    if (rc) {
        cleanup();
        return rc;
    }
    for (size_t i = 0; !rc && i < s.instances.size(); ++i)
        rc = sel_scene_attach_instance(top, unsigned(i), subscene_scenes[s.instances[i].index], s.instances[i].l2w);
    // CreateSceneLightSets (SceneResource.cpp:206-215): light set k = lights[start, start + count)
    for (size_t k = 0; !rc && k < s.ranges.size(); ++k)
        for (uint32_t i = s.ranges[k].first; !rc && i < s.ranges[k].first + s.ranges[k].second; ++i) {
            const float* v = s.lights[i].v;
            SelQuadLight q;
            std::memcpy(q.position, v, 12);
            std::memcpy(q.direction, v + 3, 12);
            std::memcpy(q.x, v + 6, 12);
            std::memcpy(q.z, v + 9, 12);
            std::memcpy(q.radiance, v + 12, 12);
            rc = sel_scene_add_quad_light(top, unsigned(k), &q);
        }
    if (!rc) rc = sel_scene_set_background(top, s.background[0], s.background[1], s.background[2]);
    if (!rc && !s.ibl.empty()) {
        // ReadImageBasedLightResource (ImageBasedLightResource.cpp:52-65): the light and miss images; the stored
        // densities are those the IBL build step derives from the light image, which sel_scene_set_ibl derives
        // again (BuildImageBasedLight.cpp:18-107)
        try {
            const Blob b = read_blob(s.root, kIblType, kIblVersion, s.ibl);
            b.need(0, kIblSize);
            const uint64_t w = b.get<uint64_t>(kIblWidth), h = b.get<uint64_t>(kIblHeight);
            const uint64_t mw = b.get<uint64_t>(kIblMissWidth), mh = b.get<uint64_t>(kIblMissHeight);
            if (!w || !h || w * h > (uint64_t(1) << 28) || mw * mh > (uint64_t(1) << 28))
                throw BlobError{b.path + ": image size"};
            const size_t light = b.array(kIblLight, w * h, 12, "lightData");
            const size_t miss = mw && mh ? b.array(kIblMiss, mw * mh, 12, "missData") : 0;
            std::vector<float> L(size_t(w * h) * 3), M(size_t(mw * mh) * 3);
            std::memcpy(L.data(), b.bytes.data() + light, L.size() * 4);
            if (miss) std::memcpy(M.data(), b.bytes.data() + miss, M.size() * 4);
            rc = sel_scene_set_ibl(top, L.data(), unsigned(w), unsigned(h), miss ? M.data() : nullptr, unsigned(mw),
                                   unsigned(mh), b.get<float>(kIblRotation), b.get<float>(kIblExposure));
        } catch (const BlobError& e) {
            rc = fail(SEL_ERR_IO, e.msg);
        }
    }
    if (!rc) rc = sel_scene_commit(top);
    if (rc) {
        sel_scene_release(top);
        cleanup();
        return rc;
    }
    sel::adopt_scenes(top, built);
    *out = top;
    return SEL_OK;
}

}  // namespace

extern "C" {

int sel_cooked_scene_describe(const char* asset_root, const char* scene_name, SelCookedSceneInfo* out_info,
                              SelCookedMesh* meshes, unsigned int capacity) {
    if (!asset_root || !scene_name || !out_info) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (capacity && !meshes) return fail(SEL_ERR_INVALID_ARGUMENT, "meshes is null with a non-zero capacity");
    try {
        const SceneAssets s = load_assets(asset_root, scene_name);
        fill_info(s, out_info);
        const Material fallback = default_material();
        const std::vector<MeshRow> rows = mesh_rows(s, fallback);
        std::map<std::string, int> tex;
        for (const MeshRow& r : rows) {
            if (r.material->flags & kFlagUsesPtex) ++out_info->ptexMeshes;
            else if (!r.material->texture.empty()) tex[r.material->texture] = 1;
        }
        out_info->textures = uint32_t(tex.size());
        for (size_t i = 0; i < rows.size() && i < capacity; ++i) {
            const MeshRow& r = rows[i];
            const Subscene& sub = s.subscenes[r.subscene];
            const Mesh& x = sub.models[r.model].meshes[r.mesh];
            SelCookedMesh& o = meshes[i];
            std::memset(&o, 0, sizeof(o));
            o.subscene = r.subscene;
            o.model = r.model;
            o.mesh = r.mesh;
            o.indicesPerFace = x.per_face;
            o.faces = x.index_count / x.per_face;
            o.materialFlags = r.material->flags;
            o.material = to_sel(*r.material, uint32_t(sub.light_set));
            copy_str(o.texture, sizeof(o.texture), r.material->texture);
            copy_str(o.name, sizeof(o.name), x.name);
        }
        return SEL_OK;
    } catch (const BlobError& e) {
        return fail(SEL_ERR_IO, e.msg);
    } catch (const std::bad_alloc&) {
        return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed while reading cooked assets");
    }
}

int sel_scene_load_cooked(SelDevice device, const char* asset_root, const char* scene_name, unsigned int flags,
                          SelScene* out_scene, SelCookedSceneInfo* out_info) {
    if (!device || !asset_root || !scene_name || !out_scene) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (flags & ~SEL_COOKED_PTEX_AS_BASE_COLOR) return fail(SEL_ERR_INVALID_ARGUMENT, "unknown flag");
    *out_scene = nullptr;
    try {
        const SceneAssets s = load_assets(asset_root, scene_name);
        SelCookedSceneInfo info;
        fill_info(s, &info);
        const Material fallback = default_material();
        const std::vector<MeshRow> rows = mesh_rows(s, fallback);
        std::map<std::string, int> tex;
        for (const MeshRow& r : rows) {
            if (r.material->flags & kFlagUsesPtex) ++info.ptexMeshes;
            else if (!r.material->texture.empty()) tex[r.material->texture] = 1;
        }
        info.textures = uint32_t(tex.size());
        if (info.ptexMeshes && !(flags & SEL_COOKED_PTEX_AS_BASE_COLOR))
            return fail(SEL_ERR_INVALID_OPERATION,
                        std::to_string(info.ptexMeshes) + " meshes sample Ptex textures (.ptx files), which this loader "
                        "does not read: bind them with sel_scene_set_ptex, or pass SEL_COOKED_PTEX_AS_BASE_COLOR");
        if (int rc = build_scene(device, s, rows, out_scene)) return rc;
        if (out_info) *out_info = info;
        return SEL_OK;
    } catch (const BlobError& e) {
        return fail(SEL_ERR_IO, e.msg);
    } catch (const std::bad_alloc&) {
        return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed while reading cooked assets");
    }
}

}  // extern "C"
