// Standalone Ptex filter entry point (sel_ptex_filter_device): one thread per (face, u, v) query.
#include "capi_internal.h"
#include "ptex.cuh"
#include "ptex_quad.cuh"

#include <vector>

namespace sel {
namespace {

__global__ void k_ptex_filter(const PtexFace* __restrict__ faces, int nfaces, const __half* __restrict__ texels,
                              const float* __restrict__ queries, uint32_t n, float* __restrict__ out, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* q = queries + 3 * size_t(i);
    float3 r;
    uint32_t status = 0;
    if (ptex_eval(faces, nfaces, texels, __float_as_int(q[0]), q[1], q[2], r, status)) {
        out[3 * size_t(i)] = r.x;
        out[3 * size_t(i) + 1] = r.y;
        out[3 * size_t(i) + 2] = r.z;
    }
    if (status) atomicOr(err, status);
}

__global__ void k_ptex_quad_filter(const PtexQuadFace* __restrict__ faces, int nfaces, const __half* __restrict__ texels,
                                   const float* __restrict__ queries, uint32_t n, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* q = queries + 3 * size_t(i);
    float3 r;
    if (ptex_quad_eval(faces, nfaces, texels, __float_as_int(q[0]), q[1], q[2], r)) {
        out[3 * size_t(i)] = r.x;
        out[3 * size_t(i) + 1] = r.y;
        out[3 * size_t(i) + 2] = r.z;
    }
}

}  // namespace
}  // namespace sel

using namespace sel;

extern "C" int sel_ptex_filter_device(SelDevice device, const SelPtexFace* d_faces, unsigned int nfaces,
                                      const uint16_t* d_texels, const float* d_queries, unsigned int n, float* d_out,
                                      void* stream) {
    static_assert(sizeof(SelPtexFace) == sizeof(PtexFace), "SelPtexFace and PtexFace must match");
    if (!device) return fail(SEL_ERR_INVALID_ARGUMENT, "device is null");
    if (n == 0) return SEL_OK;
    if (!d_faces || !d_texels || !d_queries || !d_out) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    if (int rc = set_device(device)) return rc;
    if (nfaces > 0x7fffffffu) return fail(SEL_ERR_INVALID_ARGUMENT, "too many faces");
    k_ptex_filter<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const PtexFace*>(d_faces), int(nfaces), reinterpret_cast<const __half*>(d_texels), d_queries,
        n, d_out, device->d_err);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "ptex filter launch");
}

// The face records carry the writer's constant-face flags, which depend on the texels: both arrays are read back
// and the flagged records are staged in a temporary device buffer (a test and benchmark entry point).
extern "C" int sel_ptex_quad_filter_device(SelDevice device, const SelPtexQuadFace* d_faces, unsigned int nfaces,
                                           const uint16_t* d_texels, const float* d_queries, unsigned int n,
                                           float* d_out, void* stream) {
    if (!device) return fail(SEL_ERR_INVALID_ARGUMENT, "device is null");
    if (n == 0) return SEL_OK;
    if (!d_faces || !d_texels || !d_queries || !d_out) return fail(SEL_ERR_INVALID_ARGUMENT, "null buffer");
    if (nfaces == 0 || nfaces > (1u << 26)) return fail(SEL_ERR_INVALID_ARGUMENT, "face count out of range");
    if (int rc = set_device(device)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<SelPtexQuadFace> rows(nfaces);
    cudaError_t e = cudaMemcpyAsync(rows.data(), d_faces, nfaces * sizeof(SelPtexQuadFace), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "reading the face table");
    std::vector<PtexQuadFace> q(nfaces);
    uint64_t texel_end = 0;
    for (unsigned int i = 0; i < nfaces; ++i) {
        const SelPtexQuadFace& f = rows[i];
        if (f.log2 < 0 || f.log2 > 12 || f.log2 != rows[0].log2)
            return fail(SEL_ERR_INVALID_ARGUMENT, "faces must share one log2 resolution in 0..12");
        texel_end = std::max<uint64_t>(texel_end, uint64_t(f.offset) + (uint64_t(1) << (2 * f.log2)));
        q[i].log2_flags = uint32_t(f.log2);
        q[i].offset = f.offset;
        q[i].adjedge = 0;
        q[i].pad = 0;
        for (int k = 0; k < 4; ++k) {
            if (f.adjfaces[k] >= int64_t(nfaces) || f.adjfaces[k] < -1 || f.adjedges[k] < 0 || f.adjedges[k] > 3)
                return fail(SEL_ERR_INVALID_ARGUMENT, "adjacency out of range");
            q[i].adj[k] = f.adjfaces[k];
            q[i].adjedge |= uint32_t(f.adjedges[k]) << (8 * k);
        }
    }
    std::vector<uint16_t> texels(size_t(texel_end) * 3);
    e = cudaMemcpyAsync(texels.data(), d_texels, texels.size() * 2, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "reading the texels");
    flag_constant_quads(q.data(), q.size(), texels.data());
    PtexQuadFace* d_q = nullptr;
    e = cudaMalloc(&d_q, q.size() * sizeof(PtexQuadFace));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(quad faces)");
    e = cudaMemcpyAsync(d_q, q.data(), q.size() * sizeof(PtexQuadFace), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_ptex_quad_filter<<<(n + 127) / 128, 128, 0, s>>>(d_q, int(nfaces), reinterpret_cast<const __half*>(d_texels),
                                                           d_queries, n, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_q);
    return e == cudaSuccess ? SEL_OK : cuda_fail(e, "quad ptex filter");
}
