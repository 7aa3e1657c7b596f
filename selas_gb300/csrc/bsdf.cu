// BSDF kernels behind sel_bsdf_evaluate_device / sel_bsdf_sample_device: one thread per tuple.
#include "capi_internal.h"
#include "disney.cuh"

namespace sel {

__device__ __forceinline__ Surface load_surface(const SelSurface& r) {
    Surface s;
    s.t = ld3(r.tangent);
    s.n = ld3(r.normal);
    s.b = ld3(r.bitangent);
    s.base_color = ld3(r.baseColor);
    s.transmittance_color = ld3(r.transmittanceColor);
    s.sheen = r.sheen;
    s.sheen_tint = r.sheenTint;
    s.clearcoat = r.clearcoat;
    s.clearcoat_gloss = r.clearcoatGloss;
    s.metallic = r.metallic;
    s.spec_trans = r.specTrans;
    s.diff_trans = r.diffTrans;
    s.flatness = r.flatness;
    s.anisotropic = r.anisotropic;
    s.relative_ior = r.relativeIOR;
    s.specular_tint = r.specularTint;
    s.roughness = r.roughness;
    s.scatter_distance = r.scatterDistance;
    s.ior = r.ior;
    s.shader = r.shader;
    return s;
}

namespace {

__global__ void k_bsdf_evaluate(const SelSurface* __restrict__ surf, const float* __restrict__ wo,
                                const float* __restrict__ wi, uint32_t n, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Surface s = load_surface(surf[i]);
    float fwd, rev;
    const float3 f = bsdf_evaluate(s, ld3(wo + 3 * size_t(i)), ld3(wi + 3 * size_t(i)), fwd, rev);
    float* o = out + 5 * size_t(i);
    o[0] = f.x; o[1] = f.y; o[2] = f.z; o[3] = fwd; o[4] = rev;
}

__global__ void k_bsdf_sample(const SelSurface* __restrict__ surf, const float* __restrict__ wo,
                              const float* __restrict__ u, uint32_t n, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Surface s = load_surface(surf[i]);
    float uu[4] = {u[4 * size_t(i)], u[4 * size_t(i) + 1], u[4 * size_t(i) + 2], u[4 * size_t(i) + 3]};
    int used = 0;
    BsdfSampleOut bs;
    const bool ok = bsdf_sample(s, ld3(wo + 3 * size_t(i)), uu, used, bs);
    float* o = out + 16 * size_t(i);
    o[0] = ok ? 1.0f : 0.0f;
    o[1] = float(bs.flags);
    o[2] = bs.reflectance.x; o[3] = bs.reflectance.y; o[4] = bs.reflectance.z;
    o[5] = bs.wi.x; o[6] = bs.wi.y; o[7] = bs.wi.z;
    o[8] = bs.forward_pdf; o[9] = bs.reverse_pdf;
    o[10] = float(bs.medium_phase);
    o[11] = bs.extinction.x; o[12] = bs.extinction.y; o[13] = bs.extinction.z;
    o[14] = float(used);
    o[15] = 0.0f;
}

}  // namespace
}  // namespace sel

using namespace sel;

extern "C" int sel_bsdf_evaluate_device(const SelSurface* d_surfaces, const float* d_wo, const float* d_wi,
                                        unsigned int n, float* d_out, void* stream) {
    if (n == 0) return SEL_OK;
    if (!d_surfaces || !d_wo || !d_wi || !d_out) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    k_bsdf_evaluate<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(d_surfaces, d_wo, d_wi, n, d_out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "bsdf evaluate launch");
}

extern "C" int sel_bsdf_sample_device(const SelSurface* d_surfaces, const float* d_wo, const float* d_u, unsigned int n,
                                      float* d_out, void* stream) {
    if (n == 0) return SEL_OK;
    if (!d_surfaces || !d_wo || !d_u || !d_out) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    k_bsdf_sample<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(d_surfaces, d_wo, d_u, n, d_out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "bsdf sample launch");
}
