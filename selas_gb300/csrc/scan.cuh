// Device exclusive scan of u32 arrays (three kernels: tile sums, scan of the tile sums in one block, tiles
// with their offsets), shared by the VCM hash grid and the device BVH builder.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace sel {
namespace {

constexpr int kScanTile = 2048;  // 256 threads x 8

__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t x, uint32_t* warp_sums, uint32_t& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = x;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_sums[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < 8 ? warp_sums[lane] : 0u;
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < 8) warp_sums[lane] = s;  // inclusive
    }
    __syncthreads();
    total = warp_sums[7];
    const uint32_t before = w > 0 ? warp_sums[w - 1] : 0u;
    __syncthreads();
    return before + inc - x;
}

__global__ void __launch_bounds__(256) k_scan_tiles(const uint32_t* in, uint32_t n, uint32_t* tile_sums) {
    const size_t base = size_t(blockIdx.x) * kScanTile;
    uint32_t s = 0;
    for (int k = 0; k < kScanTile / 256; ++k) {
        const size_t i = base + size_t(k) * 256 + threadIdx.x;
        if (i < n) s += in[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ uint32_t ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int k = 0; k < 8; ++k) t += ws[k];
        tile_sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(256) k_scan_top(uint32_t* tile_sums, uint32_t ntiles) {
    __shared__ uint32_t ws[8];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < ntiles; base += 256) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t x = i < ntiles ? tile_sums[i] : 0u;
        uint32_t total;
        const uint32_t ex = block_exclusive_scan_256(x, ws, total);
        if (i < ntiles) tile_sums[i] = carry + ex;
        carry += total;
    }
}

// out[0..n) = exclusive scan of in, out[n] = total.  in and out may alias.
__global__ void __launch_bounds__(256) k_scan_apply(const uint32_t* in, uint32_t n, const uint32_t* tile_sums,
                                                    uint32_t* out, uint32_t ntiles) {
    __shared__ uint32_t tile[kScanTile];
    __shared__ uint32_t ws[8];
    const size_t base = size_t(blockIdx.x) * kScanTile;
    for (int k = 0; k < kScanTile / 256; ++k) {
        const size_t i = base + size_t(k) * 256 + threadIdx.x;
        tile[k * 256 + threadIdx.x] = i < n ? in[i] : 0u;
    }
    __syncthreads();
    constexpr int kPer = kScanTile / 256;
    uint32_t loc[kPer];
    uint32_t s = 0;
    for (int k = 0; k < kPer; ++k) {
        loc[k] = tile[threadIdx.x * kPer + k];
        s += loc[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan_256(s, ws, total) + tile_sums[blockIdx.x];
    for (int k = 0; k < kPer; ++k) {
        tile[threadIdx.x * kPer + k] = run;
        run += loc[k];
    }
    __syncthreads();
    for (int k = 0; k < kScanTile / 256; ++k) {
        const size_t i = base + size_t(k) * 256 + threadIdx.x;
        if (i < n) out[i] = tile[k * 256 + threadIdx.x];
    }
    if (blockIdx.x == ntiles - 1 && threadIdx.x == 0) out[n] = tile_sums[blockIdx.x] + total;
}

void scan_exclusive(const uint32_t* in, uint32_t n, uint32_t* out, uint32_t* tmp, cudaStream_t s) {
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<ntiles, 256, 0, s>>>(in, n, tmp);
    k_scan_top<<<1, 256, 0, s>>>(tmp, ntiles);
    k_scan_apply<<<ntiles, 256, 0, s>>>(in, n, tmp, out, ntiles);
}


// Scratch words scan_exclusive needs for n values.
inline size_t scan_scratch_words(size_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

}  // namespace
}  // namespace sel
