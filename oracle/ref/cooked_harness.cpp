// ORACLE harness (test infrastructure only): writes cooked asset blobs with the reference's own serializer, so that
// the fixtures under tests/golden/cooked/ are byte for byte what the reference's build steps write and what its
// loaders attach.  Compiled into oracle/_ref/libref_pt.so (oracle/ref/build_ref.py); the product never loads it.
//
// Reference code run here, unmodified:
//   * SerializeToBinary / AttachToBinary      Source/Core/IoLib/BinaryStreamSerializer.h:15-44 with the size,
//     write and attach serializers of IoLib/SizeSerializer.cpp and IoLib/BinarySerializers.cpp;
//   * the Serialize functions of SceneResourceData (SceneLib/SceneResource.cpp:39-68), SubsceneResourceData
//     (SubsceneResource.cpp:29-37), ModelResourceData and ModelGeometryData (ModelResource.cpp:32-96),
//     TextureResourceData (TextureLib/TextureResource.cpp:21-41), ImageBasedLightResourceData
//     (ImageBasedLightResource.cpp:18-37), CameraSettings (GeometryLib/Camera.cpp:16-25), CArray
//     (ContainersLib/CArray.h:239-250) and FixedString (StringLib/FixedString.h:46-50);
//   * the asset type names and versions (SceneResource::kDataType / kDataVersion and the others) and the path rule
//     <root>/_Assets/<type>/<version>/<name>.bin of AssetFileUtils::AssetFilePath (Assets/AssetFileUtils.cpp:109-116;
//     written out here because the compiled AssetFileUtils needs the environment's root);
//   * the IBL densities of BuildImageBasedLight.cpp:24-101 (through HarnessIblDensities in pt_harness.cpp).
//
// Each ref_cooked_write_* call fills the reference's data structure from flat arrays and writes its blob; each
// ref_cooked_read_* call attaches a blob with AttachToBinary and reads the fields back, the check that a written
// file is what the reference's loader (ReadSceneResource, ReadModelResource, ...) would see.
#include "SceneLib/SceneResource.h"
#include "SceneLib/SubsceneResource.h"
#include "SceneLib/ModelResource.h"
#include "SceneLib/ImageBasedLightResource.h"
#include "TextureLib/TextureResource.h"
#include "IoLib/BinaryStreamSerializer.h"
#include "GeometryLib/Camera.h"

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

namespace Selas {
void HarnessIblDensities(Selas::uint width, Selas::uint height, float3* light, IblDensityFunctions* out);
}

using namespace Selas;

namespace {

int make_dirs(const std::string& path) {
    for (size_t i = 1; i < path.size(); ++i)
        if (path[i] == '/') {
            std::string d = path.substr(0, i);
            if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) return -1;
        }
    return 0;
}

std::string asset_path(const char* root, cpointer type, uint64 version, const char* name) {
    char v[32];
    std::snprintf(v, sizeof(v), "%llu", (unsigned long long)version);
    return std::string(root) + "/_Assets/" + type + "/" + v + "/" + name + ".bin";
}

template <typename T>
int write_blob(const char* root, cpointer type, uint64 version, const char* name, T& object) {
    uint8* data = nullptr;
    Selas::uint size = 0;
    SerializeToBinary(object, data, size);
    const std::string path = asset_path(root, type, version, name);
    int rc = make_dirs(path);
    if (rc == 0) {
        FILE* f = std::fopen(path.c_str(), "wb");
        rc = (f && std::fwrite(data, 1, size, f) == size) ? 0 : -1;
        if (f) std::fclose(f);
    }
    FreeAligned_(data);
    return rc;
}

// Reads a blob into 4096-aligned memory (as File::ReadWholeFile + SerializeToBinary's alignment would give).
template <typename T>
T* attach_blob(const char* root, cpointer type, uint64 version, const char* name, std::vector<uint64>& storage) {
    const std::string path = asset_path(root, type, version, name);
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return nullptr;
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    storage.assign(size_t(size + 7) / 8, 0);
    const bool ok = std::fread(storage.data(), 1, size_t(size), f) == size_t(size);
    std::fclose(f);
    if (!ok) return nullptr;
    T* object = nullptr;
    AttachToBinary(object, reinterpret_cast<uint8*>(storage.data()), Selas::uint(size));
    return object;
}

float3 f3(const float* p) { return float3(p[0], p[1], p[2]); }

// Fixed strings with zeroed tails, so that the blobs are the same bytes on every run.
template <int N>
void set_str(FixedString<N>& s, const char* value) {
    std::memset(s.str, 0, sizeof(s.str));
    s.Copy(value ? value : "");
}

void fill_instances(CArray<Instance>& out, const uint64* index, const float* l2w, uint32 n) {
    for (uint32 i = 0; i < n; ++i) {
        Instance& inst = out.Add();
        inst.index = index[i];
        std::memcpy(&inst.localToWorld, l2w + 16 * i, 64);
    }
}

// Material words: ints = {shader, flags}; floats = {baseColor[3], transmittanceColor[3], scalars[14]}.
void fill_material(MaterialResourceData& m, const uint32* ints, const float* floats, const char* texture) {
    set_str(m.baseColorTexture, texture);
    m.shader = ShaderType(ints[0]);
    m.flags = ints[1];
    m.baseColor = f3(floats);
    m.transmittanceColor = f3(floats + 3);
    for (int k = 0; k < eMaterialPropertyCount; ++k) m.scalarAttributeValues[k] = floats[6 + k];
}

}  // namespace

extern "C" {

// Camera words: position[3], lookAt[3], up[3], fovDegrees, znear, zfar.
int ref_cooked_write_scene(const char* root, const char* name, const char* ibl, const float* background,
                           const char* const* subscene_names, uint32 subscene_count, const uint64* instance_index,
                           const float* instance_l2w, uint32 instance_count, const float* lights, uint32 light_count,
                           const uint32* ranges, uint32 range_count, const float* cameras, uint32 camera_count) {
    SceneResourceData d;
    set_str(d.name, name);
    set_str(d.iblName, ibl);
    d.backgroundIntensity = float4(background[0], background[1], background[2], background[3]);
    for (uint32 i = 0; i < subscene_count; ++i) set_str(d.subsceneNames.Add(), subscene_names[i]);
    fill_instances(d.subsceneInstances, instance_index, instance_l2w, instance_count);
    for (uint32 i = 0; i < light_count; ++i) {  // type, position, direction, x, z, radiance
        const float* l = lights + 16 * i;
        SceneLight& L = d.lights.Add();
        L.type = uint32(l[0]);
        L.position = f3(l + 1);
        L.direction = f3(l + 4);
        L.x = f3(l + 7);
        L.z = f3(l + 10);
        L.radiance = f3(l + 13);
    }
    for (uint32 i = 0; i < range_count; ++i) {
        SceneLightSetRange& r = d.lightSetRanges.Add();
        r.start = ranges[2 * i];
        r.count = ranges[2 * i + 1];
    }
    for (uint32 i = 0; i < camera_count; ++i) {
        const float* c = cameras + 12 * i;
        CameraSettings& s = d.cameras.Add();
        char label[32];
        std::snprintf(label, sizeof(label), "camera%u", i);
        set_str(s.name, label);
        s.position = f3(c);
        s.lookAt = f3(c + 3);
        s.up = f3(c + 6);
        s.fovDegrees = c[9];
        s.znear = c[10];
        s.zfar = c[11];
    }
    return write_blob(root, SceneResource::kDataType, SceneResource::kDataVersion, name, d);
}

int ref_cooked_write_subscene(const char* root, const char* name, uint64 light_set, const char* const* model_names,
                              uint32 model_count, const uint64* instance_index, const float* instance_l2w,
                              uint32 instance_count, const uint32* material_hashes, const uint32* material_ints,
                              const float* material_floats, const char* const* material_textures,
                              uint32 material_count) {
    SubsceneResourceData d;
    set_str(d.name, name);
    d.lightSetIndex = light_set;
    for (uint32 i = 0; i < model_count; ++i) set_str(d.modelNames.Add(), model_names[i]);
    fill_instances(d.modelInstances, instance_index, instance_l2w, instance_count);
    for (uint32 i = 0; i < material_count; ++i) {
        d.sceneMaterialNames.Add(Hash32(material_hashes[i]));
        fill_material(d.sceneMaterials.Add(), material_ints + 2 * i, material_floats + 20 * i,
                      material_textures ? material_textures[i] : nullptr);
    }
    return write_blob(root, SubsceneResource::kDataType, SubsceneResource::kDataVersion, name, d);
}

// Mesh words: indexCount, indexOffset, vertexCount, vertexOffset, materialHash, indicesPerFace, nameHash.
// Curve words: indexOffset, indexCount.  Normals, tangents and uvs may be null.
int ref_cooked_write_model(const char* root, const char* name, uint32 vertex_count, const float* positions,
                           const float* normals, const float* tangents, const float* uvs, uint32 index_count,
                           const uint32* indices, const uint32* mesh_words, const char* const* mesh_names,
                           uint32 mesh_count, const uint32* material_hashes, const uint32* material_ints,
                           const float* material_floats, const char* const* material_textures, uint32 material_count,
                           uint32 curve_model_name, const uint32* curve_words, uint32 curve_count,
                           const uint32* curve_indices, uint32 curve_index_count, const float* curve_vertices,
                           uint32 curve_vertex_count) {
    ModelResourceData d;  // the CArrays start empty; every other field is set below
    d.pad = 0;
    MakeInvalid(&d.aaBox);
    for (uint32 i = 0; i < vertex_count; ++i) IncludePosition(&d.aaBox, f3(positions + 3 * i));
    d.totalVertexCount = vertex_count;
    d.totalCurveVertexCount = curve_vertex_count;
    d.curveModelName = curve_model_name;
    d.indexSize = uint64(index_count) * 4;
    d.faceIndexSize = 0;
    d.positionSize = uint64(vertex_count) * 12;
    d.normalsSize = normals ? uint64(vertex_count) * 12 : 0;
    d.tangentsSize = tangents ? uint64(vertex_count) * 16 : 0;
    d.uvsSize = uvs ? uint64(vertex_count) * 8 : 0;
    d.curveIndexSize = uint64(curve_index_count) * 4;
    d.curveVertexSize = uint64(curve_vertex_count) * 16;
    for (uint32 i = 0; i < material_count; ++i) {
        d.materialHashes.Add(Hash32(material_hashes[i]));
        fill_material(d.materials.Add(), material_ints + 2 * i, material_floats + 20 * i,
                      material_textures ? material_textures[i] : nullptr);
    }
    for (uint32 i = 0; i < mesh_count; ++i) {
        const uint32* w = mesh_words + 7 * i;
        MeshMetaData& m = d.meshes.Add();
        m.indexCount = w[0];
        m.indexOffset = w[1];
        m.vertexCount = w[2];
        m.vertexOffset = w[3];
        m.materialHash = Hash32(w[4]);
        m.indicesPerFace = w[5];
        m.nameHash = Hash32(w[6]);
        set_str(m.name, mesh_names[i]);
    }
    for (uint32 i = 0; i < curve_count; ++i) {
        CurveMetaData& c = d.curves.Add();
        c.indexOffset = curve_words[2 * i];
        c.indexCount = curve_words[2 * i + 1];
    }
    int rc = write_blob(root, ModelResource::kDataType, ModelResource::kDataVersion, name, d);
    if (rc != 0) return rc;

    ModelGeometryData g;
    std::memset(&g, 0, sizeof(g));
    g.indexSize = d.indexSize;
    g.faceIndexSize = 0;
    g.positionSize = d.positionSize;
    g.normalsSize = d.normalsSize;
    g.tangentsSize = d.tangentsSize;
    g.uvsSize = d.uvsSize;
    g.curveIndexSize = d.curveIndexSize;
    g.curveVertexSize = d.curveVertexSize;
    g.indices = const_cast<uint32*>(indices);
    g.positions = reinterpret_cast<float3*>(const_cast<float*>(positions));
    g.normals = reinterpret_cast<float3*>(const_cast<float*>(normals));
    g.tangents = reinterpret_cast<float4*>(const_cast<float*>(tangents));
    g.uvs = reinterpret_cast<float2*>(const_cast<float*>(uvs));
    g.curveIndices = const_cast<uint32*>(curve_indices);
    g.curveVertices = reinterpret_cast<float4*>(const_cast<float*>(curve_vertices));
    return write_blob(root, ModelResource::kGeometryDataType, ModelResource::kDataVersion, name, g);
}

// Mips of `format` (0 Float .. 3 Float4) packed one after the other in `texels`.
int ref_cooked_write_texture(const char* root, const char* name, uint32 format, uint32 mip_count,
                             const uint32* widths, const uint32* heights, const float* texels) {
    TextureResourceData d;
    std::memset(&d, 0, sizeof(d));
    d.mipCount = mip_count;
    d.format = TextureResourceData::TextureDataType(format);
    uint64 offset = 0;
    for (uint32 i = 0; i < mip_count; ++i) {
        d.mipWidths[i] = widths[i];
        d.mipHeights[i] = heights[i];
        d.mipOffsets[i] = offset;
        offset += uint64(widths[i]) * heights[i] * (format + 1) * sizeof(float);
    }
    d.dataSize = uint32(offset);
    d.texture = reinterpret_cast<uint8*>(const_cast<float*>(texels));
    return write_blob(root, TextureResource::kDataType, TextureResource::kDataVersion, name, d);
}

// The light image's densities are built as the reference's IBL build step builds them.
int ref_cooked_write_ibl(const char* root, const char* name, uint32 width, uint32 height, const float* light,
                         uint32 miss_width, uint32 miss_height, const float* miss, float rotation, float exposure) {
    ImageBasedLightResourceData d;
    std::memset(&d, 0, sizeof(d));
    std::vector<float3> L(size_t(width) * height), M(size_t(miss_width) * miss_height);
    for (size_t i = 0; i < L.size(); ++i) L[i] = f3(light + 3 * i);
    for (size_t i = 0; i < M.size(); ++i) M[i] = f3(miss + 3 * i);
    HarnessIblDensities(width, height, L.data(), &d.densityfunctions);
    d.missWidth = miss_width;
    d.missHeight = miss_height;
    d.rotationRadians = rotation;
    d.exposureScale = exposure;
    d.lightData = L.data();
    d.missData = M.data();
    int rc = write_blob(root, ImageBasedLightResource::kDataType, ImageBasedLightResource::kDataVersion, name, d);
    ShutdownDensityFunctions(&d.densityfunctions);
    return rc;
}

// Read-back of a scene blob through AttachToBinary: counts[5] = subscenes, instances, lights, ranges, cameras;
// background[4]; the first instance's index and matrix (17 floats, index first); the first light (16 floats as
// written); the first camera (12 floats).  Returns 0, or -1 when the file is missing.
int ref_cooked_read_scene(const char* root, const char* name, uint64* counts, float* background, float* instance,
                          float* light, float* camera, char* ibl, uint32 ibl_capacity) {
    std::vector<uint64> storage;
    SceneResourceData* d = attach_blob<SceneResourceData>(root, SceneResource::kDataType,
                                                          SceneResource::kDataVersion, name, storage);
    if (!d) return -1;
    counts[0] = d->subsceneNames.Count();
    counts[1] = d->subsceneInstances.Count();
    counts[2] = d->lights.Count();
    counts[3] = d->lightSetRanges.Count();
    counts[4] = d->cameras.Count();
    std::memcpy(background, &d->backgroundIntensity, 16);
    if (d->subsceneInstances.Count()) {
        instance[0] = float(d->subsceneInstances[0].index);
        std::memcpy(instance + 1, &d->subsceneInstances[0].localToWorld, 64);
    }
    if (d->lights.Count()) {
        const SceneLight& L = d->lights[0];
        light[0] = float(L.type);
        std::memcpy(light + 1, &L.position, 12);
        std::memcpy(light + 4, &L.direction, 12);
        std::memcpy(light + 7, &L.x, 12);
        std::memcpy(light + 10, &L.z, 12);
        std::memcpy(light + 13, &L.radiance, 12);
    }
    if (d->cameras.Count()) {
        const CameraSettings& c = d->cameras[0];
        std::memcpy(camera, &c.position, 12);
        std::memcpy(camera + 3, &c.lookAt, 12);
        std::memcpy(camera + 6, &c.up, 12);
        camera[9] = c.fovDegrees;
        camera[10] = c.znear;
        camera[11] = c.zfar;
    }
    std::snprintf(ibl, ibl_capacity, "%s", d->iblName.Ascii());
    return 0;
}

// Read-back of a model and its geometry blob: counts[6] = meshes, materials, curves, vertices, indices, uvsSize;
// mesh_words (7 per mesh, as written; capacity meshes); the index array (capacity_indices).
int ref_cooked_read_model(const char* root, const char* name, uint64* counts, uint32* mesh_words, uint32 capacity,
                          uint32* indices, uint32 capacity_indices) {
    std::vector<uint64> s0, s1;
    ModelResourceData* d = attach_blob<ModelResourceData>(root, ModelResource::kDataType, ModelResource::kDataVersion,
                                                          name, s0);
    ModelGeometryData* g = attach_blob<ModelGeometryData>(root, ModelResource::kGeometryDataType,
                                                          ModelResource::kDataVersion, name, s1);
    if (!d || !g) return -1;
    counts[0] = d->meshes.Count();
    counts[1] = d->materials.Count();
    counts[2] = d->curves.Count();
    counts[3] = d->totalVertexCount;
    counts[4] = g->indexSize / 4;
    counts[5] = g->uvsSize;
    for (uint32 i = 0; i < d->meshes.Count() && i < capacity; ++i) {
        const MeshMetaData& m = d->meshes[i];
        const uint32 w[7] = {m.indexCount, m.indexOffset, m.vertexCount, m.vertexOffset, uint32(m.materialHash),
                             m.indicesPerFace, uint32(m.nameHash)};
        std::memcpy(mesh_words + 7 * i, w, sizeof(w));
    }
    for (uint64 i = 0; i < g->indexSize / 4 && i < capacity_indices; ++i) indices[i] = g->indices[i];
    return 0;
}

}  // extern "C"
