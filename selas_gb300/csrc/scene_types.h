// Scene records shared by host set-up code and the render kernels (plain data, no device code).
#pragma once

#include <cstdint>

#include <vector_types.h>

namespace sel {

// SceneLight as NextEventEstimation reads it (SceneLib/SceneResource.h; AreaLighting.cpp:113-153):
// centre, facing direction, full edge vectors x and z, emitted radiance.
struct QuadLight {
    float3 position, direction, x, z, radiance;
};

// Per-geometry material record in HBM (128 bytes): the MaterialResourceData fields the shading reads
// (SceneLib/ModelResource.h:68-88) plus the geometry's light set and Ptex face range.
struct MaterialDev {
    int shader;
    uint32_t flags;      // kMaterialTransparent | kMaterialUsesPtex | kMaterialUsesTexture
    uint32_t light_set;
    uint32_t ptex_base;  // first face of this geometry in the packed Ptex face table
    float base_color[3];
    float transmittance_color[3];
    float sheen, sheen_tint, clearcoat, clearcoat_gloss, metallic, spec_trans, diffuse_trans, flatness;
    float anisotropic, specular_tint, roughness, scatter_distance, ior;
    uint32_t tex_lo, tex_hi;        // kMaterialUsesTexture: the base-colour image (float4 texels, row-major)
    uint32_t tex_width, tex_height;
    float pad[5];
};
static_assert(sizeof(MaterialDev) == 128, "MaterialDev must be 128 bytes");

// Shading data of one scene as the integrators read it for hits inside instances of that scene (the model data
// ModelDataFromRayIds finds, SceneResource.cpp:362-378): one fixed device record per scene, rewritten whenever
// the scene's shading data is uploaded, so instance records can point at it.
// Vertex attributes of one mesh the shading reads (by geomID): its triangles' vertex indices, shading normals
// (slot 0, 3 floats per vertex) and tangents (slot 1, xyz + bitangent sign); null where absent.
struct MeshAttrDev {
    const uint32_t* indices;  // 3 per stored triangle (a quad mesh: triangles 2q = (v0, v1, v3), 2q + 1 = (v2, v3, v1))
    const float* normals;
    const float4* tangents;
    const float2* uvs;  // slot 2
    uint32_t quads;     // 1: a quad mesh, interpolated bilinearly over each quad
    uint32_t pad;
};

struct ShadeView {
    const MaterialDev* materials;
    const void* ptex_faces;   // PtexFace[]
    const void* ptex_texels;  // half RGB
    uint32_t material_count;
    uint32_t ptex_face_count;
    const MeshAttrDev* attrs;  // by geomID (null: no mesh has attributes)
    uint32_t attr_count;
    uint32_t pad;
};

constexpr uint32_t kMaterialTransparent = 1u;  // DisneySolid with diffTrans or specTrans (BuildModel.cpp:60-65)
constexpr uint32_t kMaterialUsesPtex = 2u;
constexpr uint32_t kMaterialUsesTexture = 4u;  // base colour from a 2D image at the hit's uvs (not Ptex)
constexpr uint32_t kMaterialTextured = kMaterialUsesPtex | kMaterialUsesTexture;
constexpr uint32_t kMaterialPtexQuad = 8u;  // with kMaterialUsesPtex: the geometry's texture is a quad-mesh texture

}  // namespace sel
