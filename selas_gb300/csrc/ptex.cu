// Standalone Ptex filter entry point (sel_ptex_filter_device): one thread per (face, u, v) query.
#include "capi_internal.h"
#include "ptex.cuh"

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
