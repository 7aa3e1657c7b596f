// C ABI of the scene shading data and of the path-tracer entry points (include/selas.h).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>

#include <cmath>

#include "capi_internal.h"
#include "ibl.cuh"
#include "pt.h"
#include "ptex_quad.cuh"
#include "vcm.h"

using namespace sel;

namespace {

constexpr uint32_t kMaxGeom = 65536;
constexpr uint32_t kDefaultPathsInFlight = 1u << 22;

MaterialDev to_device(const SelMaterial& m) {
    MaterialDev d;
    std::memset(&d, 0, sizeof(d));
    d.shader = m.shader;
    d.light_set = m.lightSetIndex;
    for (int i = 0; i < 3; ++i) {
        d.base_color[i] = m.baseColor[i];
        d.transmittance_color[i] = m.transmittanceColor[i];
    }
    d.metallic = m.metallic;
    d.specular_tint = m.specularTint;
    d.roughness = m.roughness;
    d.anisotropic = m.anisotropic;
    d.sheen = m.sheen;
    d.sheen_tint = m.sheenTint;
    d.clearcoat = m.clearcoat;
    d.clearcoat_gloss = m.clearcoatGloss;
    d.spec_trans = m.specTrans;
    d.diffuse_trans = m.diffuseTrans;
    d.flatness = m.flatness;
    d.ior = m.ior;
    d.scatter_distance = m.scatterDistance;
    if (m.shader == SEL_SHADER_DISNEY_SOLID && (m.diffuseTrans > 0.0f || m.specTrans > 0.0f))
        d.flags |= kMaterialTransparent;
    if (m.usesPtex) d.flags |= kMaterialUsesPtex;
    return d;
}

SelMaterial default_material() {
    SelMaterial m;
    std::memset(&m, 0, sizeof(m));
    m.shader = SEL_SHADER_DISNEY_SOLID;
    m.baseColor[0] = m.baseColor[1] = m.baseColor[2] = 0.6f;
    m.ior = 1.5f;
    return m;
}

template <typename T>
int upload(void*& dst, const T* src, size_t count) {
    if (dst) cudaFree(dst);
    dst = nullptr;
    const size_t bytes = count ? count * sizeof(T) : sizeof(T);
    cudaError_t e = cudaMalloc(&dst, bytes);
    if (e == cudaSuccess && count) e = cudaMemcpy(dst, src, count * sizeof(T), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "uploading shading data");
}

}  // namespace

namespace sel {

// One past the largest geomID of the scene's meshes and curves: the size of its per-geomID material table.
static uint32_t geom_limit(const SelSceneTy* sc) {
    uint32_t n = 0;
    for (const MeshInput& m : sc->meshes) n = m.geomID + 1 > n ? m.geomID + 1 : n;
    for (const SelSceneTy::CurveInput& c : sc->curves) n = c.geomID + 1 > n ? c.geomID + 1 : n;
    return n;
}

void ibl_densities(const float* rgb, uint32_t width, uint32_t height, std::vector<float>& mdf, std::vector<float>& cdf) {
    mdf.assign(height, 0.0f);
    cdf.assign(size_t(width) * height, 0.0f);
    const float heightf = float(height);
    std::vector<float> intensity(size_t(width) * height);
    for (uint32_t y = 0; y < height; ++y) {
        const float theta = (float(y) + 0.5f) * kPi / heightf;
        const float sin_theta = std::sin(theta);
        for (uint32_t x = 0; x < width; ++x) {
            const float* c = rgb + (size_t(y) * width + x) * 3;
            intensity[size_t(y) * width + x] = sin_theta * (c[0] * 0.299f + c[1] * 0.587f + c[2] * 0.114f);
        }
    }
    float marginal_sum = 0.0f;
    for (uint32_t y = 0; y < height; ++y) {
        float row_sum = 0.0f;
        for (uint32_t x = 0; x < width; ++x) row_sum += intensity[size_t(y) * width + x];
        mdf[y] = row_sum;
        marginal_sum += row_sum;
        if (row_sum > 0.0f) {
            const float oo = 1.0f / row_sum;
            float integral = 0.0f;
            for (uint32_t x = 0; x < width; ++x) {
                integral += oo * intensity[size_t(y) * width + x];
                cdf[size_t(y) * width + x] = integral;
            }
        }
        cdf[size_t(y) * width + width - 1] = 1.0f;  // floating-point imprecision, as the reference
    }
    if (marginal_sum > 0.0f) {
        const float oo = 1.0f / marginal_sum;
        float integral = 0.0f;
        for (uint32_t y = 0; y < height; ++y) {
            integral += mdf[y] * oo;
            mdf[y] = integral;
        }
    }
    mdf[height - 1] = 1.0f;
}

// One device block: the IblDev record, then its marginal and conditional CDFs and the two images (float4 texels).
static int upload_ibl(SelSceneTy* sc) {
    if (sc->d_ibl) cudaFree(sc->d_ibl);
    sc->d_ibl = nullptr;
    if (!sc->ibl_w) return SEL_OK;
    std::vector<float> mdf, cdf;
    ibl_densities(sc->ibl_light.data(), sc->ibl_w, sc->ibl_h, mdf, cdf);
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t n_light = size_t(sc->ibl_w) * sc->ibl_h, n_miss = size_t(sc->ibl_mw) * sc->ibl_mh;
    const size_t o_mdf = up(sizeof(IblDev)), o_cdf = o_mdf + up(mdf.size() * 4), o_light = o_cdf + up(cdf.size() * 4);
    const size_t o_miss = o_light + up(n_light * 16), total = o_miss + up(n_miss * 16);
    std::vector<unsigned char> host(total, 0);
    void* d = nullptr;
    cudaError_t e = cudaMalloc(&d, total);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(image-based light)");
    char* base = static_cast<char*>(d);
    IblDev v;
    v.mdf = reinterpret_cast<const float*>(base + o_mdf);
    v.cdf = reinterpret_cast<const float*>(base + o_cdf);
    v.light = reinterpret_cast<const float4*>(base + o_light);
    v.miss = reinterpret_cast<const float4*>(base + o_miss);
    v.width = sc->ibl_w;
    v.height = sc->ibl_h;
    v.miss_width = sc->ibl_mw;
    v.miss_height = sc->ibl_mh;
    v.rotation = sc->ibl_rotation;
    v.exposure = sc->ibl_exposure;
    std::memcpy(host.data(), &v, sizeof(v));
    std::memcpy(host.data() + o_mdf, mdf.data(), mdf.size() * 4);
    std::memcpy(host.data() + o_cdf, cdf.data(), cdf.size() * 4);
    float* lt = reinterpret_cast<float*>(host.data() + o_light);
    for (size_t i = 0; i < n_light; ++i)
        for (int c = 0; c < 3; ++c) lt[4 * i + c] = sc->ibl_light[3 * i + c];
    float* ms = reinterpret_cast<float*>(host.data() + o_miss);
    for (size_t i = 0; i < n_miss; ++i)
        for (int c = 0; c < 3; ++c) ms[4 * i + c] = sc->ibl_miss[3 * i + c];
    e = cudaMemcpy(d, host.data(), total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "uploading the image-based light");
    }
    sc->d_ibl = d;
    return SEL_OK;
}

// One device block: the MeshAttrDev table (by geomID), then the vertex indices, normals (float3) and tangents
// (float4) of the meshes that have shading normals or tangents.
static int upload_attrs(SelSceneTy* sc) {
    if (sc->d_attrs) cudaFree(sc->d_attrs);
    sc->d_attrs = nullptr;
    sc->attr_count = 0;
    uint32_t max_geom = 0;
    size_t n_idx = 0, n_nrm = 0, n_tan = 0, n_uv = 0;
    auto has_uvs = [](const MeshInput& m) { return m.attr_n[2] == 2; };  // slot 2 as (u, v) pairs
    for (const MeshInput& m : sc->meshes) {
        if (!m.attr_n[0] && !m.attr_n[1] && !has_uvs(m)) continue;
        max_geom = std::max(max_geom, m.geomID + 1);
        n_idx += m.indices.size();
        if (m.attr_n[0]) n_nrm += m.attr[0].size();
        if (m.attr_n[1]) n_tan += m.attr[1].size();
        if (has_uvs(m)) n_uv += m.attr[2].size();
    }
    if (!max_geom) return SEL_OK;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t o_idx = up(sizeof(MeshAttrDev) * max_geom), o_nrm = o_idx + up(n_idx * 4), o_tan = o_nrm + up(n_nrm * 4);
    const size_t o_uv = o_tan + up(n_tan * 4);
    const size_t total = o_uv + up(n_uv * 4);
    void* d = nullptr;
    cudaError_t e = cudaMalloc(&d, total);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(vertex attributes)");
    char* base = static_cast<char*>(d);
    std::vector<unsigned char> host(total, 0);
    MeshAttrDev* table = reinterpret_cast<MeshAttrDev*>(host.data());
    size_t ai = 0, an = 0, at = 0, au = 0;
    for (const MeshInput& m : sc->meshes) {
        if (!m.attr_n[0] && !m.attr_n[1] && !has_uvs(m)) continue;
        MeshAttrDev& t = table[m.geomID];
        t.quads = m.quads ? 1u : 0u;
        t.indices = reinterpret_cast<const uint32_t*>(base + o_idx + ai * 4);
        std::memcpy(host.data() + o_idx + ai * 4, m.indices.data(), m.indices.size() * 4);
        ai += m.indices.size();
        if (m.attr_n[0]) {
            t.normals = reinterpret_cast<const float*>(base + o_nrm + an * 4);
            std::memcpy(host.data() + o_nrm + an * 4, m.attr[0].data(), m.attr[0].size() * 4);
            an += m.attr[0].size();
        }
        if (m.attr_n[1]) {
            t.tangents = reinterpret_cast<const float4*>(base + o_tan + at * 4);
            std::memcpy(host.data() + o_tan + at * 4, m.attr[1].data(), m.attr[1].size() * 4);
            at += m.attr[1].size();
        }
        if (has_uvs(m)) {
            t.uvs = reinterpret_cast<const float2*>(base + o_uv + au * 4);
            std::memcpy(host.data() + o_uv + au * 4, m.attr[2].data(), m.attr[2].size() * 4);
            au += m.attr[2].size();
        }
    }
    e = cudaMemcpy(d, host.data(), total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "uploading vertex attributes");
    }
    sc->d_attrs = d;
    sc->attr_count = max_geom;
    return SEL_OK;
}

// A quad-mesh Ptex texture bound in the scene or the scenes its instances reference.
bool tree_has_quad_ptex(const SelSceneTy* sc) {
    for (const auto& pb : sc->ptex)
        if (pb.quads) return true;
    for (const auto& r : sc->referenced)
        if (tree_has_quad_ptex(r.first)) return true;
    return false;
}

// Material classes (bit shader * 4 + Ptex * 2 + transparent) and Ptex use of a scene and the scenes its
// instances reference.
void tree_classes(const SelSceneTy* sc, uint32_t& mask, bool& ptex) {
    mask |= sc->class_mask;
    ptex |= sc->sort_hint_ptex;
    for (const auto& r : sc->referenced) tree_classes(r.first, mask, ptex);
}

int sync_shading(SelSceneTy* sc) {
    for (const auto& r : sc->referenced)  // instanced scenes first: their views must be current
        if (int rc = sync_shading(r.first)) return rc;
    if (!sc->shading_dirty) {
        uint32_t mask = 0;
        bool ptex = false;
        tree_classes(sc, mask, ptex);
        sc->sort_hint = (ptex || __builtin_popcount(mask) > 1) ? 1u : 0u;
        return SEL_OK;
    }
    const uint32_t max_geom = geom_limit(sc);
    if (max_geom > kMaxGeom) return fail(SEL_ERR_INVALID_OPERATION, "rendering needs geomIDs below 65536");
    std::vector<MaterialDev> mats(max_geom ? max_geom : 1, to_device(default_material()));
    for (size_t i = 0; i < sc->materials.size() && i < mats.size(); ++i)
        if (sc->materials[i].shader >= 0) mats[i] = sc->materials[i];
    std::vector<QuadLight> lights;
    std::vector<uint2> sets;
    for (const auto& set : sc->light_sets) {
        sets.push_back(make_uint2(uint32_t(lights.size()), uint32_t(set.size())));
        lights.insert(lights.end(), set.begin(), set.end());
    }
    // Ptex: one face table for all bound geometries, adjacency and texel offsets rebased
    std::vector<SelPtexFace> faces;
    std::vector<uint16_t> texels;
    for (const auto& pb : sc->ptex) {
        const uint32_t face_base = uint32_t(faces.size());
        const uint32_t texel_base = uint32_t(texels.size() / 3);
        for (SelPtexFace f : pb.faces) {
            if (pb.quads) {
                PtexQuadFace q;
                std::memcpy(&q, &f, sizeof(q));
                q.offset += texel_base;
                for (int e = 0; e < 4; ++e)
                    if (q.adj[e] >= 0) q.adj[e] += int32_t(face_base);
                std::memcpy(&f, &q, sizeof(q));
            } else {
                f.offset += texel_base;
                for (int e = 0; e < 3; ++e)
                    if (f.adjfaces[e] >= 0) f.adjfaces[e] += int32_t(face_base);
            }
            faces.push_back(f);
        }
        texels.insert(texels.end(), pb.texels.begin(), pb.texels.end());
        if (pb.geomID < mats.size()) {
            mats[pb.geomID].ptex_base = face_base;
            mats[pb.geomID].flags = (mats[pb.geomID].flags & ~kMaterialPtexQuad) | (pb.quads ? kMaterialPtexQuad : 0u);
        }
    }
    for (auto& m : mats) {
        bool bound = false;
        for (const auto& pb : sc->ptex) bound |= (&m - mats.data()) == ptrdiff_t(pb.geomID);
        if (!bound) m.flags &= ~kMaterialUsesPtex;  // no texture bound: keep the material's base colour
    }
    // 2D base-colour images: materials without Ptex sample theirs at the hit's uvs
    if (sc->d_textures) cudaFree(sc->d_textures);
    sc->d_textures = nullptr;
    {
        size_t n = 0;
        for (const auto& tb : sc->textures) n += tb.rgba.size();
        if (n) {
            cudaError_t e = cudaMalloc(&sc->d_textures, n * sizeof(float));
            if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(textures)");
            std::vector<float> all;
            all.reserve(n);
            for (const auto& tb : sc->textures) {
                if (tb.geomID < mats.size() && !(mats[tb.geomID].flags & kMaterialUsesPtex)) {
                    MaterialDev& m = mats[tb.geomID];
                    const uint64_t p = reinterpret_cast<uint64_t>(static_cast<float*>(sc->d_textures) + all.size());
                    m.flags |= kMaterialUsesTexture;
                    m.tex_lo = uint32_t(p);
                    m.tex_hi = uint32_t(p >> 32);
                    m.tex_width = tb.width;
                    m.tex_height = tb.height;
                }
                all.insert(all.end(), tb.rgba.begin(), tb.rgba.end());
            }
            e = cudaMemcpy(sc->d_textures, all.data(), n * sizeof(float), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cuda_fail(e, "uploading textures");
        }
    }
    // material classes of the attached meshes (shader x Ptex x transparency, as the path tracer sorts them)
    {
        uint32_t seen = 0;
        auto see = [&](uint32_t geomID) {
            const MaterialDev& m = mats[geomID < mats.size() ? geomID : 0];
            const uint32_t shader = uint32_t(m.shader) < 3u ? uint32_t(m.shader) : 0u;
            seen |= 1u << (shader * 4u + ((m.flags & kMaterialTextured) ? 2u : 0u) + ((m.flags & kMaterialTransparent) ? 1u : 0u));
        };
        for (const MeshInput& mi : sc->meshes) see(mi.geomID);
        for (const SelSceneTy::CurveInput& c : sc->curves) see(c.geomID);
        bool ptex = false;
        for (const auto& m : mats) ptex |= (m.flags & kMaterialTextured) != 0;
        sc->class_mask = seen;
        sc->sort_hint_ptex = ptex;
        sc->tex2d = false;
        for (const auto& m : mats) sc->tex2d |= (m.flags & kMaterialUsesTexture) != 0;
        uint32_t mask = 0;
        tree_classes(sc, mask, ptex);
        sc->sort_hint = (ptex || __builtin_popcount(mask) > 1) ? 1u : 0u;
    }
    if (int rc = upload(sc->d_ptex_faces, faces.data(), faces.size())) return rc;
    if (int rc = upload(sc->d_ptex_texels, texels.data(), texels.size())) return rc;
    sc->ptex_face_count = uint32_t(faces.size());
    if (int rc = upload(sc->d_materials, mats.data(), mats.size())) return rc;
    if (int rc = upload(sc->d_lights, lights.data(), lights.size())) return rc;
    if (int rc = upload(sc->d_light_sets, sets.data(), sets.size())) return rc;
    if (int rc = upload_ibl(sc)) return rc;
    if (int rc = upload_attrs(sc)) return rc;
    if (sc->d_view) {
        ShadeView v;
        v.materials = static_cast<const MaterialDev*>(sc->d_materials);
        v.ptex_faces = sc->d_ptex_faces;
        v.ptex_texels = sc->d_ptex_texels;
        v.material_count = uint32_t(mats.size());
        v.ptex_face_count = sc->ptex_face_count;
        v.attrs = static_cast<const MeshAttrDev*>(sc->d_attrs);
        v.attr_count = sc->attr_count;
        v.pad = 0;
        cudaError_t e = cudaMemcpy(sc->d_view, &v, sizeof(v), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, "shading view");
    }
    sc->shading_dirty = false;
    return SEL_OK;
}

// The Ptex writer's face flags for a quad-mesh texture (PtexWriter.cpp:814-816,996-1075, clamp borders, no
// subfaces): a face whose texels all have the same bits is constant; a constant face is neighbourhood-constant
// when, around each of its vertices (clockwise, and counter-clockwise from a boundary), every face is constant
// with the same value.  The filter applies a constant face through its kernel weight and returns a
// neighbourhood-constant face's value directly, as the reader does.
void flag_constant_quads(void* records, size_t count, const uint16_t* texels) {
    PtexQuadFace* faces = static_cast<PtexQuadFace*>(records);
    for (size_t i = 0; i < count; ++i) {
        PtexQuadFace& f = faces[i];
        const size_t n = size_t(1) << (2 * (f.log2_flags & 0xffu));
        const uint16_t* d = texels + size_t(f.offset) * 3;
        bool c = true;
        for (size_t i = 1; i < n && c; ++i) c = std::memcmp(d, d + 3 * i, 6) == 0;
        if (c) f.log2_flags |= kQuadConstant;
    }
    const int n = int(count);
    auto edge = [&](int f, int e) { return int((faces[f].adjedge >> (8 * e)) & 3u); };
    for (int faceid = 0; faceid < n; ++faceid) {
        PtexQuadFace& f = faces[faceid];
        if (!(f.log2_flags & kQuadConstant)) continue;
        const uint16_t* cd = texels + size_t(f.offset) * 3;
        auto same = [&](int a) {
            return (faces[a].log2_flags & kQuadConstant) && std::memcmp(cd, texels + size_t(faces[a].offset) * 3, 6) == 0;
        };
        bool is_const = true;
        for (int eid = 0; is_const && eid < 4; ++eid) {
            int afid = f.adj[eid], aeid = edge(faceid, eid);
            int count = 0;
            while (afid != faceid && afid >= 0 && ++count < 10) {
                if (!same(afid)) { is_const = false; break; }
                const int next = (aeid + 1) % 4;
                const int nf = faces[afid].adj[next];
                aeid = edge(afid, next);
                afid = nf;
            }
            if (afid < 0 && is_const) {
                aeid = (aeid + 3) % 4;
                afid = f.adj[aeid];
                aeid = edge(faceid, aeid);
                count = 0;
                while (afid != faceid && afid >= 0 && ++count < 10) {
                    if (!same(afid)) { is_const = false; break; }
                    const int prev = (aeid + 3) % 4;
                    const int nf = faces[afid].adj[prev];
                    aeid = edge(afid, prev);
                    afid = nf;
                }
            }
        }
        if (is_const) f.log2_flags |= kQuadNbConstant;
    }
}

int set_material_flags(SelSceneTy* scene, unsigned int geomID, const SelMaterial& material, bool transparent) {
    if (geomID >= kMaxGeom) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID must be below 65536");
    if (material.shader < SEL_SHADER_DISNEY_THIN || material.shader > SEL_SHADER_DIRAC_TRANSPARENT)
        return fail(SEL_ERR_INVALID_ARGUMENT, "unknown shader");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (scene->materials.size() <= geomID) {
        MaterialDev unset;
        std::memset(&unset, 0, sizeof(unset));
        unset.shader = -1;
        scene->materials.resize(geomID + 1, unset);
    }
    MaterialDev d = to_device(material);
    d.flags = (d.flags & ~kMaterialTransparent) | (transparent ? kMaterialTransparent : 0u);
    scene->materials[geomID] = d;
    scene->shading_dirty = true;
    return SEL_OK;
}

}  // namespace sel

namespace {

int ensure_pt_state(SelSceneTy* sc, uint32_t paths) {
    if (sc->pt_block && sc->pt_capacity == paths) return SEL_OK;
    sc->last_rays = nullptr;  // it may point into the block about to be freed
    if (sc->pt_block) cudaFree(sc->pt_block);
    sc->pt_block = nullptr;
    sc->pt_capacity = 0;
    cudaError_t e = cudaMalloc(&sc->pt_block, pt_state_block_bytes(paths));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(path state)");
    sc->pt_capacity = paths;
    return SEL_OK;
}

}  // namespace

namespace sel {

int check_render_args(SelScene scene, const SelCamera* camera, const SelPtSettings* settings) {
    if (!scene || !camera || !settings) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (!scene->committed) return fail(SEL_ERR_INVALID_OPERATION, "scene not committed");
    if (!instances_fresh(scene))
        return fail(SEL_ERR_INVALID_OPERATION, "an instanced scene changed since this scene was committed");
    if (camera->width == 0 || camera->height == 0 || camera->width > 16384 || camera->height > 16384)
        return fail(SEL_ERR_INVALID_ARGUMENT, "viewport must be 1..16384 in each dimension");
    if (!(camera->fovDegrees > 0.0f && camera->fovDegrees < 180.0f))
        return fail(SEL_ERR_INVALID_ARGUMENT, "fovDegrees must lie in (0, 180)");
    if (settings->samplesPerPixel == 0) return fail(SEL_ERR_INVALID_ARGUMENT, "samplesPerPixel must be > 0");
    if (settings->traceBlockSize != 0 && settings->traceBlockSize != 128 && settings->traceBlockSize != 256)
        return fail(SEL_ERR_INVALID_ARGUMENT, "traceBlockSize must be 0, 128 or 256");
    const uint64_t total = uint64_t(camera->width) * camera->height * settings->samplesPerPixel;
    if (total >= (uint64_t(1) << 32)) return fail(SEL_ERR_INVALID_ARGUMENT, "width * height * spp must be < 2^32");
    return SEL_OK;
}

// Samples per axis of a deferred render (samplesPerPixel = m * m), or 0 when the settings are invalid.
uint32_t deferred_axis(const SelPtSettings& settings) {
    uint32_t m = 1;
    while (m * m < settings.samplesPerPixel && m < 256) ++m;
    return m * m == settings.samplesPerPixel ? m : 0u;
}

int check_deferred_args(SelScene scene, const SelCamera* camera, const SelPtSettings* settings) {
    if (int rc = check_render_args(scene, camera, settings)) return rc;
    if (deferred_axis(*settings) == 0)
        return fail(SEL_ERR_INVALID_ARGUMENT, "samplesPerPixel must be m * m with 1 <= m <= 256");
    if (settings->maxBounces == 0 || settings->maxBounces > 1024)
        return fail(SEL_ERR_INVALID_ARGUMENT, "maxBounces must lie in 1..1024");
    return SEL_OK;
}

}  // namespace sel

namespace {

}  // namespace

namespace sel {

PtScene scene_view(const SelSceneTy* sc) {
    PtScene ps;
    ps.nodes = sc->d_nodes;
    ps.bvh_kind = sc->info.bvh_kind == SEL_BVH_WIDE8_Q8 ? 0 : 1;
    ps.tris = static_cast<const float4*>(sc->d_tris);
    ps.materials = static_cast<const MaterialDev*>(sc->d_materials);
    const uint32_t max_geom = geom_limit(sc);
    ps.material_count = max_geom ? max_geom : 1;
    ps.lights = static_cast<const QuadLight*>(sc->d_lights);
    ps.light_sets = static_cast<const uint2*>(sc->d_light_sets);
    ps.light_set_count = uint32_t(sc->light_sets.size());
    ps.ptex_faces = sc->d_ptex_faces;
    ps.ptex_texels = sc->d_ptex_texels;
    ps.ptex_face_count = sc->ptex_face_count;
    for (int i = 0; i < 3; ++i) ps.background[i] = sc->background[i];
    ps.sort_hint = (sc->sort_hint && sc->dev->material_sort) ? 1u : 0u;
    {
        uint32_t mask = 0;
        bool ptex = false;
        tree_classes(sc, mask, ptex);
        ps.shader_kinds = 0u;
        for (uint32_t k = 0; k < 3u; ++k)
            if ((mask >> (4u * k)) & 15u) ps.shader_kinds |= 1u << k;
        ps.ptex_quads = tree_has_quad_ptex(sc) ? 1u : 0u;
    }
    ps.insts = static_cast<const InstanceRecord*>(sc->d_insts);
    ps.ibl = static_cast<const IblDev*>(sc->d_ibl);
    ps.attrs = static_cast<const MeshAttrDev*>(sc->d_attrs);
    ps.attr_count = sc->attr_count;
    for (int a = 0; a < 3; ++a) {
        ps.lo[a] = sc->info.bounds_lo[a];
        ps.hi[a] = sc->info.bounds_hi[a];
    }
    ps.ray_sort = sc->dev->ray_sort ? 1u : 0u;
    ps.tex2d = sc->tex2d ? 1u : 0u;
    return ps;
}

// Default initial merge radius: VcmRadiusFactor_ (0.0025) x the bounding-sphere radius of the scene bounds
// (VCM.cpp:778), the sphere taken about the bounding box.
float vcm_default_radius(const SelSceneTy* sc) {
    float d2 = 0.0f;
    for (int a = 0; a < 3; ++a) {
        const float e = sc->info.bounds_hi[a] - sc->info.bounds_lo[a];
        d2 += e * e;
    }
    const float r = 0.0025f * (0.5f * std::sqrt(d2));
    return r > 0.0f ? r : 1e-3f;
}

// Per-pass constants (CalculateIterationConstants, VCMCommon.cpp:91-112, with vcCount = 1): the float
// expressions of the CPU restatement, so that both compute the same radius and weights.
void vcm_constants(float radius0, float alpha, uint32_t paths, bool merging, uint32_t pass, VcmConsts& c) {
    const float pi = 3.141592653589793f;
    c.radius = radius0 / std::pow(float(pass + 1), 0.5f * (1.0f - alpha));
    c.radius2 = c.radius * c.radius;
    c.n_paths = float(paths);
    const float eta = pi * c.radius2 * c.n_paths;
    c.vm_weight = merging ? eta : 0.0f;
    c.vc_weight = 1.0f / eta;
    c.vm_norm = 1.0f / eta;
    c.pass = pass;
    c.pad = 0;
}

// Light set 0 of the scene as the VCM light source.
void vcm_lights(const SelSceneTy* sc, VcmSettings& set) {
    set.light_first = 0;
    set.light_count = sc->light_sets.empty() ? 0u : uint32_t(sc->light_sets[0].size());
}

}  // namespace sel

namespace {

int render_device(SelSceneTy* sc, const SelCamera& camera, const SelPtSettings& settings, double* d_accum,
                  cudaStream_t stream, uint32_t mode = kPtModePath) {
    if (int rc = sync_shading(sc)) return rc;
    const uint64_t total = uint64_t(camera.width) * camera.height * settings.samplesPerPixel;
    uint32_t cap = settings.pathsInFlight ? settings.pathsInFlight
                   : (sc->tuned_paths_in_flight ? sc->tuned_paths_in_flight : kDefaultPathsInFlight);
    if (uint64_t(cap) > total) cap = uint32_t(total);
    if (int rc = ensure_pt_state(sc, cap)) return rc;
    const PtScene ps = scene_view(sc);
    PtCamera cam;
    init_camera(camera, cam);
    PtSettings set;
    set.spp = settings.samplesPerPixel;
    set.max_bounces = settings.maxBounces;
    set.seed = settings.seed;
    set.mode = mode;
    set.samples_per_axis = mode == kPtModeDeferred ? deferred_axis(settings) : 0u;
    const PtState st = pt_state_carve(sc->pt_block, cap);
    const int block = int(settings.traceBlockSize ? settings.traceBlockSize
                                                  : (sc->tuned_trace_block ? sc->tuned_trace_block : 128u));
    sc->last_rays = st.rays;  // this render's ray counts (sel_scene_last_render_rays)
    if (cudaMemsetAsync(st.rays, 0, 2 * sizeof(unsigned long long), stream) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "ray counters");
    cudaError_t e = pt_render(ps, cam, set, st, d_accum, sc->dev->d_err, stream,
                              sc->dev->graph_replay ? &sc->pt_graph : nullptr, block);
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "path tracer launch");
}

// Several views of one scene in one shared wavefront: view k is job k of the job table (seed + k), each batch
// takes an equal share of the wavefront's paths from every view, and the batch is captured once and replayed.
// d_accum: the views' accumulators one after another (PT: 2 layers, deferred: 1 layer of W x H x 3 doubles).
int render_views_device(SelSceneTy* sc, const SelCamera* cams, uint32_t count, const SelPtSettings& settings,
                        double* d_accum, cudaStream_t stream, uint32_t mode) {
    if (int rc = sync_shading(sc)) return rc;
    uint64_t all = 0;
    for (uint32_t k = 0; k < count; ++k) all += uint64_t(cams[k].width) * cams[k].height * settings.samplesPerPixel;
    uint32_t cap = settings.pathsInFlight ? settings.pathsInFlight
                   : (sc->tuned_paths_in_flight ? sc->tuned_paths_in_flight : kDefaultPathsInFlight);
    if (uint64_t(cap) > all) cap = uint32_t(all);
    if (cap < count) cap = count;
    if (int rc = ensure_pt_state(sc, cap)) return rc;
    const PtScene ps = scene_view(sc);
    const PtState st = pt_state_carve(sc->pt_block, cap);
    sc->last_rays = st.rays;
    if (cudaMemsetAsync(st.rays, 0, 2 * sizeof(unsigned long long), stream) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "ray counters");
    PtJob jobs[kMaxPtJobs];
    PtControl ctl;
    std::memset(jobs, 0, sizeof(jobs));
    std::memset(&ctl, 0, sizeof(ctl));
    const uint32_t layers = mode == kPtModeDeferred ? 1u : 2u;
    uint64_t batches = 0, batch_paths = 0;
    size_t offset = 0;
    for (uint32_t k = 0; k < count; ++k) {
        PtJob& j = jobs[k];
        j.scene = ps;
        init_camera(cams[k], j.cam);
        j.max_bounces = settings.maxBounces;
        j.mode = mode;
        j.samples_per_axis = mode == kPtModeDeferred ? deferred_axis(settings) : 0u;
        j.seed = settings.seed + k;
        j.total = uint64_t(cams[k].width) * cams[k].height * settings.samplesPerPixel;
        j.accum = d_accum + offset;
        offset += size_t(layers) * cams[k].width * cams[k].height * 3;
        ctl.quota[k] = cap / count;
        batches = std::max(batches, (j.total + ctl.quota[k] - 1) / ctl.quota[k]);
        batch_paths += std::min<uint64_t>(j.total, ctl.quota[k]);
    }
    ctl.njobs = count;
    cudaError_t e = cudaMemcpyAsync(st.jobs, jobs, sizeof(PtJob) * kMaxPtJobs, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st.control, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return cuda_fail(e, "view table upload");
    const int block = int(settings.traceBlockSize ? settings.traceBlockSize
                                                  : (sc->tuned_trace_block ? sc->tuned_trace_block : 128u));
    e = pt_run_batches(ps.bvh_kind, settings.maxBounces, ps.sort_hint != 0, st, sc->dev->d_err, batches, stream,
                       sc->dev->graph_replay ? &sc->pt_graph : nullptr, block, mode == kPtModeDeferred ? 2u : 1u,
                       ps.insts != nullptr, pt_scene_textured(ps), ps.ray_sort != 0, batch_paths, ps.shader_kinds,
                       ps.ptex_quads != 0);
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "multi-view render launch");
}

int check_views(SelScene scene, const SelCamera* cams, unsigned int count, unsigned int integrator,
                const SelPtSettings* settings) {
    if (!cams || count == 0 || count > uint32_t(kMaxPtJobs))
        return fail(SEL_ERR_INVALID_ARGUMENT, "1..16 cameras are needed");
    if (integrator != SEL_INTEGRATOR_PT && integrator != SEL_INTEGRATOR_DEFERRED)
        return fail(SEL_ERR_INVALID_ARGUMENT, "integrator must be SEL_INTEGRATOR_PT or SEL_INTEGRATOR_DEFERRED");
    for (unsigned int k = 0; k < count; ++k) {
        const int rc = integrator == SEL_INTEGRATOR_PT ? check_render_args(scene, &cams[k], settings)
                                                       : check_deferred_args(scene, &cams[k], settings);
        if (rc) return rc;
    }
    return SEL_OK;
}

constexpr uint32_t kVcmChunk = 1024;  // passes per constants table

SelVcmSettings default_vcm_settings() {
    SelVcmSettings s;
    std::memset(&s, 0, sizeof(s));
    s.passes = 1;
    s.maxPathLength = 10;      // MaxBounceCount_ (VCMCommon.cpp:24)
    s.seed = 1;
    s.radius = 0.0f;           // VcmRadiusFactor_ x bounding-sphere radius
    s.radiusAlpha = 0.75f;     // VcmRadiusAlpha_ (VCMCommon.cpp:30)
    return s;
}

}  // namespace

namespace sel {

// The scene and every scene it instances (directly or below).
static std::vector<const SelSceneTy*> material_scenes(const SelSceneTy* sc) {
    std::vector<const SelSceneTy*> out{sc};
    for (size_t i = 0; i < out.size(); ++i)
        for (const auto& r : out[i]->referenced)
            if (std::find(out.begin(), out.end(), r.first) == out.end()) out.push_back(r.first);
    return out;
}

// Stored VCM vertices keep their material record's address in 56 bits: checked once the scene's (and its
// instanced scenes') material tables are in HBM.
int check_vcm_materials(const SelSceneTy* scene) {
    for (const SelSceneTy* sc : material_scenes(scene))
        if (reinterpret_cast<uint64_t>(sc->d_materials) >> 56)
            return fail(SEL_ERR_INVALID_OPERATION, "material table above the 2^56 address range VCM vertices hold");
    return SEL_OK;
}

int check_vcm_args(SelScene scene, const SelCamera* camera, const SelVcmSettings* settings) {
    if (!scene || !camera || !settings) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (!scene->committed) return fail(SEL_ERR_INVALID_OPERATION, "scene not committed");
    if (!instances_fresh(scene))
        return fail(SEL_ERR_INVALID_OPERATION, "an instanced scene changed since this scene was committed");
    if (camera->width == 0 || camera->height == 0 || camera->width > 16384 || camera->height > 16384)
        return fail(SEL_ERR_INVALID_ARGUMENT, "viewport must be 1..16384 in each dimension");
    if (!(camera->fovDegrees > 0.0f && camera->fovDegrees < 180.0f))
        return fail(SEL_ERR_INVALID_ARGUMENT, "fovDegrees must lie in (0, 180)");
    if (settings->passes == 0) return fail(SEL_ERR_INVALID_ARGUMENT, "passes must be > 0");
    if (settings->maxPathLength < 2 || settings->maxPathLength > 32)
        return fail(SEL_ERR_INVALID_ARGUMENT, "maxPathLength must lie in 2..32");
    if (!(settings->radius >= 0.0f) || !std::isfinite(settings->radius))
        return fail(SEL_ERR_INVALID_ARGUMENT, "radius must be finite and >= 0");
    if (!(settings->radiusAlpha > 0.0f && settings->radiusAlpha <= 1.0f))
        return fail(SEL_ERR_INVALID_ARGUMENT, "radiusAlpha must lie in (0, 1]");
    const uint64_t paths = uint64_t(camera->width) * camera->height;
    // random streams (2 * pass + 1) * N + p and slot indices p * (maxPathLength - 1) + k stay 32/64-bit exact
    if (paths * (settings->maxPathLength - 1) >= (uint64_t(1) << 31))
        return fail(SEL_ERR_INVALID_ARGUMENT, "width * height * (maxPathLength - 1) must be below 2^31");
    if (uint64_t(settings->firstPass) + settings->passes > (uint64_t(1) << 31))
        return fail(SEL_ERR_INVALID_ARGUMENT, "firstPass + passes must be below 2^31");
    return SEL_OK;
}

}  // namespace sel

namespace {

int ensure_vcm_state(SelSceneTy* sc, uint32_t paths, uint32_t max_len) {
    if (sc->vcm_block && sc->vcm_paths == paths && sc->vcm_len == max_len) return SEL_OK;
    sc->last_rays = nullptr;
    if (sc->vcm_block) cudaFree(sc->vcm_block);
    sc->vcm_block = nullptr;
    sc->vcm_paths = sc->vcm_len = sc->vcm_passes = 0;
    cudaError_t e = cudaMalloc(&sc->vcm_block, vcm_state_block_bytes(paths, max_len, kVcmChunk));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(VCM state)");
    sc->vcm_paths = paths;
    sc->vcm_len = max_len;
    sc->vcm_passes = kVcmChunk;
    return SEL_OK;
}

int vcm_render_device(SelSceneTy* sc, const SelCamera& camera, const SelVcmSettings& settings, double* d_accum,
                      cudaStream_t stream) {
    if (int rc = sync_shading(sc)) return rc;
    if (int rc = check_vcm_materials(sc)) return rc;
    const uint32_t paths = camera.width * camera.height;
    if (int rc = ensure_vcm_state(sc, paths, settings.maxPathLength)) return rc;
    const float radius0 = settings.radius != 0.0f ? settings.radius : vcm_default_radius(sc);
    VcmCamera cam;
    init_camera(camera, cam.cam);
    const float hlen = std::tan(camera.fovDegrees * (3.141592653589793f / 180.0f) * 0.5f);
    cam.image_plane = float(camera.width) / (2.0f * hlen);
    VcmSettings set;
    set.max_len = settings.maxPathLength;
    set.seed = settings.seed;
    set.merging = settings.disableMerging ? 0 : 1;
    set.trace_block = sc->tuned_trace_block;
    vcm_lights(sc, set);
    const PtScene ps = scene_view(sc);
    const VcmState st = vcm_state_carve(sc->vcm_block, paths, settings.maxPathLength, kVcmChunk);
    sc->last_rays = st.rays;
    if (cudaMemsetAsync(st.rays, 0, 2 * sizeof(unsigned long long), stream) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "ray counters");
    std::vector<VcmConsts> consts;
    for (uint32_t done = 0; done < settings.passes;) {
        const uint32_t n = std::min(kVcmChunk, settings.passes - done);
        consts.resize(n);
        for (uint32_t k = 0; k < n; ++k)
            vcm_constants(radius0, settings.radiusAlpha, paths, set.merging != 0, settings.firstPass + done + k, consts[k]);
        cudaError_t e = vcm_render(ps, cam, set, consts.data(), n, st, d_accum, sc->dev->d_err, stream,
                                   sc->dev->graph_replay ? &sc->vcm_graph : nullptr);
        if (e != cudaSuccess) return cuda_fail(e, "VCM launch");
        // the constants table is read by the passes just queued: wait before it is refilled
        if (done + n < settings.passes) {
            e = cudaStreamSynchronize(stream);
            if (e != cudaSuccess) return cuda_fail(e, "VCM");
        }
        done += n;
    }
    return SEL_OK;
}

}  // namespace

extern "C" {

int sel_material_defaults(SelMaterial* out) {
    if (!out) return fail(SEL_ERR_INVALID_ARGUMENT, "out is null");
    *out = default_material();
    return SEL_OK;
}

int sel_scene_set_material(SelScene scene, unsigned int geomID, const SelMaterial* material) {
    if (!scene || !material) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    const bool transparent = material->shader == SEL_SHADER_DISNEY_SOLID &&
                             (material->diffuseTrans > 0.0f || material->specTrans > 0.0f);
    return sel::set_material_flags(scene, geomID, *material, transparent);
}

int sel_scene_add_quad_light(SelScene scene, unsigned int lightSetIndex, const SelQuadLight* light) {
    if (!scene || !light) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (lightSetIndex >= 4096) return fail(SEL_ERR_INVALID_ARGUMENT, "lightSetIndex must be below 4096");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (scene->light_sets.size() <= lightSetIndex) scene->light_sets.resize(lightSetIndex + 1);
    QuadLight q;
    q.position = make_float3(light->position[0], light->position[1], light->position[2]);
    q.direction = make_float3(light->direction[0], light->direction[1], light->direction[2]);
    q.x = make_float3(light->x[0], light->x[1], light->x[2]);
    q.z = make_float3(light->z[0], light->z[1], light->z[2]);
    q.radiance = make_float3(light->radiance[0], light->radiance[1], light->radiance[2]);
    scene->light_sets[lightSetIndex].push_back(q);
    scene->shading_dirty = true;
    return SEL_OK;
}

int sel_scene_set_texture(SelScene scene, unsigned int geomID, const float* data, unsigned int width,
                          unsigned int height, unsigned int channels) {
    if (!scene || (width && height && !data)) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (geomID >= kMaxGeom) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID must be below 65536");
    if (channels != 1 && channels != 3 && channels != 4)
        return fail(SEL_ERR_INVALID_ARGUMENT, "channels must be 1, 3 or 4");
    if (width > 16384 || height > 16384) return fail(SEL_ERR_INVALID_ARGUMENT, "width and height must be at most 16384");
    std::lock_guard<std::mutex> lock(scene->mu);
    for (const SelSceneTy::CurveInput& c : scene->curves)
        if (c.geomID == geomID && width && height)
            return fail(SEL_ERR_INVALID_OPERATION, "curves take no texture (they have no uvs)");
    auto& list = scene->textures;
    for (size_t i = 0; i < list.size(); ++i)
        if (list[i].geomID == geomID) {
            list.erase(list.begin() + ptrdiff_t(i));
            break;
        }
    if (width && height) {
        SelSceneTy::TextureBinding tb;
        tb.geomID = geomID;
        tb.width = width;
        tb.height = height;
        tb.rgba.resize(size_t(width) * height * 4);
        for (size_t i = 0; i < size_t(width) * height; ++i)
            for (int c = 0; c < 4; ++c)  // one channel: grey (SampleTextureFloat3 of a Float image)
                tb.rgba[i * 4 + c] = c < 3 ? data[i * channels + (channels == 1 ? 0 : c)]
                                           : (channels == 4 ? data[i * 4 + 3] : 1.0f);
        list.push_back(std::move(tb));
    }
    scene->shading_dirty = true;
    return SEL_OK;
}

int sel_scene_set_ptex(SelScene scene, unsigned int geomID, const SelPtexFace* faces, size_t face_count,
                       const uint16_t* texels, size_t texel_count) {
    if (!scene || (face_count && !faces) || (texel_count && !texels)) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (geomID >= kMaxGeom) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID must be below 65536");
    std::lock_guard<std::mutex> lock(scene->mu);
    const MeshInput* mesh = nullptr;
    for (const MeshInput& m : scene->meshes)
        if (m.geomID == geomID) mesh = &m;
    if (!mesh) return fail(SEL_ERR_INVALID_ARGUMENT, "no geometry with this geomID");
    if (mesh->quads)
        return fail(SEL_ERR_INVALID_OPERATION, "a quad mesh takes its Ptex texture through sel_scene_set_ptex_quads");
    if (face_count != mesh->indices.size() / 3)
        return fail(SEL_ERR_INVALID_ARGUMENT, "face_count must equal the geometry's triangle count");
    for (size_t i = 0; i < face_count; ++i) {
        const SelPtexFace& f = faces[i];
        if (f.log2 < 0 || f.log2 > 12) return fail(SEL_ERR_INVALID_ARGUMENT, "face log2 resolution out of range");
        const uint64_t need = uint64_t(f.offset) + (uint64_t(1) << (2 * f.log2));
        if (need * 3 > texel_count) return fail(SEL_ERR_INVALID_ARGUMENT, "face texels exceed the texel array");
        if (f.log2 != faces[0].log2) return fail(SEL_ERR_INVALID_ARGUMENT, "all faces must share one resolution");
        for (int e = 0; e < 3; ++e) {
            if (f.adjfaces[e] >= int64_t(face_count) || f.adjfaces[e] < -1 || f.adjedges[e] < 0 || f.adjedges[e] > 2)
                return fail(SEL_ERR_INVALID_ARGUMENT, "adjacency out of range");
        }
    }
    SelSceneTy::PtexBinding pb;
    pb.geomID = geomID;
    pb.faces.assign(faces, faces + face_count);
    pb.texels.assign(texels, texels + texel_count);
    for (auto& existing : scene->ptex)
        if (existing.geomID == geomID) {
            existing = std::move(pb);
            scene->shading_dirty = true;
            return SEL_OK;
        }
    scene->ptex.push_back(std::move(pb));
    scene->shading_dirty = true;
    return SEL_OK;
}

int sel_scene_set_ptex_quads(SelScene scene, unsigned int geomID, const SelPtexQuadFace* faces, size_t face_count,
                             const uint16_t* texels, size_t texel_count) {
    if (!scene || (face_count && !faces) || (texel_count && !texels)) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (geomID >= kMaxGeom) return fail(SEL_ERR_INVALID_ARGUMENT, "geomID must be below 65536");
    std::lock_guard<std::mutex> lock(scene->mu);
    const MeshInput* mesh = nullptr;
    for (const MeshInput& m : scene->meshes)
        if (m.geomID == geomID) mesh = &m;
    if (!mesh) return fail(SEL_ERR_INVALID_ARGUMENT, "no geometry with this geomID");
    if (!mesh->quads) return fail(SEL_ERR_INVALID_OPERATION, "the geometry is not a quad mesh: use sel_scene_set_ptex");
    if (face_count != mesh->indices.size() / 6)
        return fail(SEL_ERR_INVALID_ARGUMENT, "face_count must equal the geometry's quad count");
    std::vector<PtexQuadFace> q(face_count);
    for (size_t i = 0; i < face_count; ++i) {
        const SelPtexQuadFace& f = faces[i];
        if (f.log2 < 0 || f.log2 > 12) return fail(SEL_ERR_INVALID_ARGUMENT, "face log2 resolution out of range");
        if (f.log2 != faces[0].log2) return fail(SEL_ERR_INVALID_ARGUMENT, "all faces must share one resolution");
        const uint64_t need = uint64_t(f.offset) + (uint64_t(1) << (2 * f.log2));
        if (need * 3 > texel_count) return fail(SEL_ERR_INVALID_ARGUMENT, "face texels exceed the texel array");
        q[i].log2_flags = uint32_t(f.log2);
        q[i].offset = f.offset;
        q[i].adjedge = 0;
        q[i].pad = 0;
        for (int e = 0; e < 4; ++e) {
            if (f.adjfaces[e] >= int64_t(face_count) || f.adjfaces[e] < -1 || f.adjedges[e] < 0 || f.adjedges[e] > 3)
                return fail(SEL_ERR_INVALID_ARGUMENT, "adjacency out of range");
            q[i].adj[e] = f.adjfaces[e];
            q[i].adjedge |= uint32_t(f.adjedges[e]) << (8 * e);
        }
    }
    sel::flag_constant_quads(q.data(), q.size(), texels);
    SelSceneTy::PtexBinding pb;
    pb.geomID = geomID;
    pb.quads = true;
    pb.faces.resize(face_count);
    if (face_count) std::memcpy(pb.faces.data(), q.data(), face_count * sizeof(PtexQuadFace));
    pb.texels.assign(texels, texels + texel_count);
    for (auto& existing : scene->ptex)
        if (existing.geomID == geomID) {
            existing = std::move(pb);
            scene->shading_dirty = true;
            return SEL_OK;
        }
    scene->ptex.push_back(std::move(pb));
    scene->shading_dirty = true;
    return SEL_OK;
}

int sel_scene_set_ibl(SelScene scene, const float* rgb, unsigned int width, unsigned int height, const float* miss_rgb,
                      unsigned int miss_width, unsigned int miss_height, float rotationRadians, float exposureScale) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if (width && (!rgb || height == 0)) return fail(SEL_ERR_INVALID_ARGUMENT, "image is null or empty");
    if (width > 32768 || height > 32768) return fail(SEL_ERR_INVALID_ARGUMENT, "image sides must be at most 32768");
    if (miss_rgb && (miss_width == 0 || miss_height == 0 || miss_width > 32768 || miss_height > 32768))
        return fail(SEL_ERR_INVALID_ARGUMENT, "miss image sides must lie in 1..32768");
    if (!std::isfinite(rotationRadians) || !std::isfinite(exposureScale))
        return fail(SEL_ERR_INVALID_ARGUMENT, "rotation and exposure must be finite");
    std::lock_guard<std::mutex> lock(scene->mu);
    try {
        scene->ibl_light.assign(rgb, rgb + size_t(width) * height * 3 * (width ? 1 : 0));
        if (miss_rgb && width) {
            scene->ibl_miss.assign(miss_rgb, miss_rgb + size_t(miss_width) * miss_height * 3);
            scene->ibl_mw = miss_width;
            scene->ibl_mh = miss_height;
        } else {  // the miss image defaults to the light image times the exposure
            scene->ibl_miss.resize(scene->ibl_light.size());
            for (size_t i = 0; i < scene->ibl_light.size(); ++i) scene->ibl_miss[i] = exposureScale * scene->ibl_light[i];
            scene->ibl_mw = width;
            scene->ibl_mh = height;
        }
    } catch (const std::bad_alloc&) {
        return fail(SEL_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    for (float v : scene->ibl_light)
        if (!std::isfinite(v) || v < 0.0f) return fail(SEL_ERR_INVALID_ARGUMENT, "image values must be finite and >= 0");
    scene->ibl_w = width;
    scene->ibl_h = width ? height : 0;
    scene->ibl_rotation = rotationRadians;
    scene->ibl_exposure = exposureScale;
    scene->shading_dirty = true;
    return SEL_OK;
}

int sel_scene_set_background(SelScene scene, float r, float g, float b) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    scene->background[0] = r;
    scene->background[1] = g;
    scene->background[2] = b;
    return SEL_OK;
}

int sel_scene_last_render_rays(SelScene scene, uint64_t* out) {
    if (!scene || !out) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(scene->mu);
    out[0] = out[1] = 0;
    if (!scene->last_rays) return SEL_OK;
    if (int rc = set_device(scene->dev)) return rc;
    std::lock_guard<std::mutex> dlock(scene->dev->mu);
    unsigned long long v[2] = {0, 0};
    cudaError_t e = cudaMemcpyAsync(v, scene->last_rays, sizeof(v), cudaMemcpyDeviceToHost, scene->dev->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(scene->dev->stream);
    if (e != cudaSuccess) return cuda_fail(e, "reading the ray counters");
    out[0] = v[0];
    out[1] = v[1];
    return SEL_OK;
}

int sel_vcm_pass_constants(float radius0, float alpha, unsigned int paths, unsigned int pass, float* out) {
    if (!out) return fail(SEL_ERR_INVALID_ARGUMENT, "out is null");
    VcmConsts c;
    vcm_constants(radius0, alpha, paths, true, pass, c);
    out[0] = c.radius;
    out[1] = c.radius2;
    out[2] = c.vm_norm;
    out[3] = c.vm_weight;
    out[4] = c.vc_weight;
    return SEL_OK;
}

int sel_pt_render_device(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, double* d_accum,
                         void* stream) {
    if (int rc = check_render_args(scene, camera, settings)) return rc;
    if (!d_accum || (reinterpret_cast<uintptr_t>(d_accum) & 7u))
        return fail(SEL_ERR_INVALID_ARGUMENT, "d_accum must be an 8-byte aligned device pointer");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    return render_device(scene, *camera, *settings, d_accum, static_cast<cudaStream_t>(stream));
}

int sel_pt_generate_image(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, float* out_layers) {
    if (int rc = check_render_args(scene, camera, settings)) return rc;
    if (!out_layers) return fail(SEL_ERR_INVALID_ARGUMENT, "out_layers is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    SelDeviceTy* dev = scene->dev;
    std::lock_guard<std::mutex> dlock(dev->mu);
    cudaStream_t s = dev->stream;
    const uint32_t values = 2u * camera->width * camera->height * 3u;
    const size_t accum_bytes = size_t(values) * sizeof(double);
    const size_t need = accum_bytes + size_t(values) * sizeof(float);
    if (scene->accum_bytes < need) {
        if (scene->d_accum) cudaFree(scene->d_accum);
        scene->d_accum = nullptr;
        scene->accum_bytes = 0;
        cudaError_t e = cudaMalloc(&scene->d_accum, need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(accumulator)");
        scene->accum_bytes = need;
    }
    double* acc = static_cast<double*>(scene->d_accum);
    float* res = reinterpret_cast<float*>(static_cast<char*>(scene->d_accum) + accum_bytes);
    cudaError_t e = cudaMemsetAsync(acc, 0, accum_bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(accumulator)");
    if (int rc = render_device(scene, *camera, *settings, acc, s)) return rc;
    e = pt_resolve(acc, values, 1.0 / double(settings->samplesPerPixel), res, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_layers, res, size_t(values) * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "path tracer");
    return read_error_word(dev, s);
}

int sel_render_views_device(SelScene scene, const SelCamera* cameras, unsigned int count, unsigned int integrator,
                            const SelPtSettings* settings, double* d_accum, void* stream) {
    if (int rc = check_views(scene, cameras, count, integrator, settings)) return rc;
    if (!d_accum || (reinterpret_cast<uintptr_t>(d_accum) & 7u))
        return fail(SEL_ERR_INVALID_ARGUMENT, "d_accum must be an 8-byte aligned device pointer");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    return render_views_device(scene, cameras, count, *settings, d_accum, static_cast<cudaStream_t>(stream),
                               integrator == SEL_INTEGRATOR_DEFERRED ? kPtModeDeferred : kPtModePath);
}

int sel_render_views(SelScene scene, const SelCamera* cameras, unsigned int count, unsigned int integrator,
                     const SelPtSettings* settings, float* out) {
    if (int rc = check_views(scene, cameras, count, integrator, settings)) return rc;
    if (!out) return fail(SEL_ERR_INVALID_ARGUMENT, "out is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    SelDeviceTy* dev = scene->dev;
    std::lock_guard<std::mutex> dlock(dev->mu);
    cudaStream_t s = dev->stream;
    const uint32_t layers = integrator == SEL_INTEGRATOR_DEFERRED ? 1u : 2u;
    size_t values = 0;
    for (unsigned int k = 0; k < count; ++k) values += size_t(layers) * cameras[k].width * cameras[k].height * 3;
    const size_t accum_bytes = values * sizeof(double);
    const size_t need = accum_bytes + values * sizeof(float);
    if (scene->accum_bytes < need) {
        if (scene->d_accum) cudaFree(scene->d_accum);
        scene->d_accum = nullptr;
        scene->accum_bytes = 0;
        cudaError_t e = cudaMalloc(&scene->d_accum, need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(accumulator)");
        scene->accum_bytes = need;
    }
    double* acc = static_cast<double*>(scene->d_accum);
    float* res = reinterpret_cast<float*>(static_cast<char*>(scene->d_accum) + accum_bytes);
    cudaError_t e = cudaMemsetAsync(acc, 0, accum_bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(accumulator)");
    if (int rc = render_views_device(scene, cameras, count, *settings, acc, s,
                                     integrator == SEL_INTEGRATOR_DEFERRED ? kPtModeDeferred : kPtModePath))
        return rc;
    e = pt_resolve(acc, uint32_t(values), 1.0 / double(settings->samplesPerPixel), res, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, res, values * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "multi-view render");
    return read_error_word(dev, s);
}

int sel_deferred_settings_defaults(SelPtSettings* out) {
    if (!out) return fail(SEL_ERR_INVALID_ARGUMENT, "out is null");
    std::memset(out, 0, sizeof(*out));
    out->samplesPerPixel = 16;  // SamplesPerPixelX_ x SamplesPerPixelY_ (DeferredPathTracer.cpp:40-41)
    out->maxBounces = 64;
    out->seed = 1;
    return SEL_OK;
}

int sel_deferred_render_device(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, double* d_accum,
                               void* stream) {
    if (int rc = check_deferred_args(scene, camera, settings)) return rc;
    if (!d_accum || (reinterpret_cast<uintptr_t>(d_accum) & 7u))
        return fail(SEL_ERR_INVALID_ARGUMENT, "d_accum must be an 8-byte aligned device pointer");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    return render_device(scene, *camera, *settings, d_accum, static_cast<cudaStream_t>(stream), kPtModeDeferred);
}

int sel_deferred_generate_image(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, float* out_rgb) {
    if (int rc = check_deferred_args(scene, camera, settings)) return rc;
    if (!out_rgb) return fail(SEL_ERR_INVALID_ARGUMENT, "out_rgb is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    SelDeviceTy* dev = scene->dev;
    std::lock_guard<std::mutex> dlock(dev->mu);
    cudaStream_t s = dev->stream;
    const uint32_t values = camera->width * camera->height * 3u;
    const size_t accum_bytes = size_t(values) * sizeof(double);
    const size_t need = accum_bytes + size_t(values) * sizeof(float);
    if (scene->accum_bytes < need) {
        if (scene->d_accum) cudaFree(scene->d_accum);
        scene->d_accum = nullptr;
        scene->accum_bytes = 0;
        cudaError_t e = cudaMalloc(&scene->d_accum, need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(accumulator)");
        scene->accum_bytes = need;
    }
    double* acc = static_cast<double*>(scene->d_accum);
    float* res = reinterpret_cast<float*>(static_cast<char*>(scene->d_accum) + accum_bytes);
    cudaError_t e = cudaMemsetAsync(acc, 0, accum_bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(accumulator)");
    if (int rc = render_device(scene, *camera, *settings, acc, s, kPtModeDeferred)) return rc;
    e = pt_resolve(acc, values, 1.0 / double(settings->samplesPerPixel), res, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_rgb, res, size_t(values) * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "deferred path tracer");
    return read_error_word(dev, s);
}

int sel_vcm_settings_defaults(SelVcmSettings* out) {
    if (!out) return fail(SEL_ERR_INVALID_ARGUMENT, "out is null");
    *out = default_vcm_settings();
    return SEL_OK;
}

int sel_vcm_render_device(SelScene scene, const SelCamera* camera, const SelVcmSettings* settings, double* d_accum,
                          void* stream) {
    if (int rc = check_vcm_args(scene, camera, settings)) return rc;
    if (!d_accum || (reinterpret_cast<uintptr_t>(d_accum) & 7u))
        return fail(SEL_ERR_INVALID_ARGUMENT, "d_accum must be an 8-byte aligned device pointer");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    return vcm_render_device(scene, *camera, *settings, d_accum, static_cast<cudaStream_t>(stream));
}

int sel_vcm_generate_image(SelScene scene, const SelCamera* camera, const SelVcmSettings* settings, float* out_rgb) {
    if (int rc = check_vcm_args(scene, camera, settings)) return rc;
    if (!out_rgb) return fail(SEL_ERR_INVALID_ARGUMENT, "out_rgb is null");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    SelDeviceTy* dev = scene->dev;
    std::lock_guard<std::mutex> dlock(dev->mu);
    cudaStream_t s = dev->stream;
    const uint32_t values = camera->width * camera->height * 3u;
    const size_t accum_bytes = size_t(values) * sizeof(double);
    const size_t need = accum_bytes + size_t(values) * sizeof(float);
    if (scene->accum_bytes < need) {
        if (scene->d_accum) cudaFree(scene->d_accum);
        scene->d_accum = nullptr;
        scene->accum_bytes = 0;
        cudaError_t e = cudaMalloc(&scene->d_accum, need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(accumulator)");
        scene->accum_bytes = need;
    }
    double* acc = static_cast<double*>(scene->d_accum);
    float* res = reinterpret_cast<float*>(static_cast<char*>(scene->d_accum) + accum_bytes);
    cudaError_t e = cudaMemsetAsync(acc, 0, accum_bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(accumulator)");
    if (int rc = vcm_render_device(scene, *camera, *settings, acc, s)) return rc;
    e = pt_resolve(acc, values, 1.0 / double(settings->passes), res, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_rgb, res, size_t(values) * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "VCM");
    return read_error_word(dev, s);
}

int sel_scene_autotune(SelScene scene, const SelCamera* camera, const SelPtSettings* settings, SelTuneResult* out) {
    if (int rc = check_render_args(scene, camera, settings)) return rc;
    if (!out) return fail(SEL_ERR_INVALID_ARGUMENT, "out is null");
    std::memset(out, 0, sizeof(*out));
    if (int rc = set_device(scene->dev)) return rc;
    struct Layout {
        int kind;
        uint32_t leaf;
    };
    const Layout layouts[] = {{SEL_BVH_WIDE8_Q8, 2}, {SEL_BVH_WIDE8_Q8, 3}, {SEL_BVH_WIDE8_Q8, 4}, {SEL_BVH_WIDE8_Q8, 8},
                              {SEL_BVH_BINARY_FP32, 3}};
    const uint32_t capacities[] = {1u << 20, 1u << 22, 1u << 23};
    const int blocks[] = {128, 256};
    const size_t values = 2ull * camera->width * camera->height * 3;
    double* acc = nullptr;
    cudaStream_t s = scene->dev->stream;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaError_t e = cudaMalloc(&acc, values * sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ev1);
    if (e != cudaSuccess) {
        if (acc) cudaFree(acc);
        return cuda_fail(e, "autotune set-up");
    }
    const int kind0 = scene->kind;
    const uint32_t leaf0 = scene->leaf_size;
    SelTuneTrial best;
    std::memset(&best, 0, sizeof(best));
    best.ms = 1e300;
    int rc = SEL_OK;
    for (const Layout& L : layouts) {
        {
            std::lock_guard<std::mutex> lock(scene->mu);
            scene->kind = L.kind;
            scene->leaf_size = L.leaf;
        }
        if (sel_scene_commit(scene) != SEL_OK) continue;  // e.g. a tree deeper than a traversal stack
        for (uint32_t cap : capacities)
            for (int block : blocks) {
                // 256-thread traversal blocks exist for the 8-wide layout only
                if (block == 256 && L.kind != SEL_BVH_WIDE8_Q8) continue;
                SelPtSettings st = *settings;
                st.pathsInFlight = cap;
                st.traceBlockSize = uint32_t(block);
                rc = sel_pt_render_device(scene, camera, &st, acc, s);  // untimed: builds state and graph
                if (rc == SEL_OK) rc = sel_device_sync(scene->dev, s);
                if (rc != SEL_OK) break;
                cudaEventRecord(ev0, s);
                rc = sel_pt_render_device(scene, camera, &st, acc, s);
                cudaEventRecord(ev1, s);
                if (rc == SEL_OK) rc = sel_device_sync(scene->dev, s);
                if (rc != SEL_OK) break;
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, ev0, ev1);
                SelTuneTrial t;
                t.bvh_kind = uint32_t(L.kind);
                t.leaf_size = L.leaf;
                t.paths_in_flight = cap;
                t.trace_block = uint32_t(block);
                t.ms = ms;
                if (out->trials < 32) out->trial[out->trials++] = t;
                if (t.ms < best.ms) best = t;
            }
        if (rc != SEL_OK) break;
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaFree(acc);
    {
        std::lock_guard<std::mutex> lock(scene->mu);
        scene->kind = best.ms < 1e300 ? int(best.bvh_kind) : kind0;
        scene->leaf_size = best.ms < 1e300 ? best.leaf_size : leaf0;
        scene->tuned_paths_in_flight = best.ms < 1e300 ? best.paths_in_flight : 0;
        scene->tuned_trace_block = best.ms < 1e300 ? best.trace_block : 0;
    }
    const int rc_commit = sel_scene_commit(scene);
    if (rc != SEL_OK) return rc;
    if (rc_commit != SEL_OK) return rc_commit;
    out->best = best;
    return SEL_OK;
}

}  // extern "C"
