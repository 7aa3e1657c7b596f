// Curve segment data behind the leaf records of a scene with round B-spline curves (curve.cuh).
#include <vector>

#include "capi_internal.h"
#include "curve.cuh"

namespace sel {
namespace {

// Points each curve record (kind kTriCurve) at its segment's control points: the byte offset from the record to
// data_offset + 64 x (first segment of its geometry + primID), as an int64 in v0.x / v0.y.
__global__ void k_patch_curves(float4* recs, uint64_t records, uint64_t data_offset, const uint32_t* geoms,
                               const uint32_t* bases, uint32_t ngeoms) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= records) return;
    float4* r = recs + 3 * i;
    if (__float_as_uint(r[2].w) != kTriCurve) return;
    const uint32_t geom = __float_as_uint(r[1].w), prim = __float_as_uint(r[0].w);
    uint32_t base = 0;
    for (uint32_t k = 0; k < ngeoms; ++k)
        if (geoms[k] == geom) base = bases[k];
    const int64_t off = int64_t(data_offset + 64ull * (uint64_t(base) + prim)) - int64_t(48ull * i);
    r[0].x = __uint_as_float(uint32_t(uint64_t(off)));
    r[0].y = __uint_as_float(uint32_t(uint64_t(off) >> 32));
}

}  // namespace

cudaError_t attach_curve_data(void** d_tris, uint64_t records, const float* data, size_t nseg, const uint32_t* geoms,
                              const uint32_t* bases, uint32_t ngeoms) {
    const uint64_t rec_bytes = records * 48ull, data_bytes = uint64_t(nseg) * 64ull;
    char* out = nullptr;
    uint32_t* table = nullptr;
    cudaError_t e = cudaMalloc(&out, rec_bytes + data_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&table, 2ull * ngeoms * sizeof(uint32_t) + 4);
    if (e == cudaSuccess && rec_bytes) e = cudaMemcpy(out, *d_tris, rec_bytes, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess && data_bytes) e = cudaMemcpy(out + rec_bytes, data, data_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && ngeoms) e = cudaMemcpy(table, geoms, ngeoms * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && ngeoms)
        e = cudaMemcpy(table + ngeoms, bases, ngeoms * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && records) {
        k_patch_curves<<<unsigned((records + 255) / 256), 256>>>(reinterpret_cast<float4*>(out), records, rec_bytes,
                                                                  table, table + ngeoms, ngeoms);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (table) cudaFree(table);
    if (e != cudaSuccess) {
        if (out) cudaFree(out);
        return e;
    }
    cudaFree(*d_tris);
    *d_tris = out;
    return cudaSuccess;
}

}  // namespace sel
