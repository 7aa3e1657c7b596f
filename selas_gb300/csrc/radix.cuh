// Stable LSD radix sort of (key, value) pairs by 8-bit digits over tiles of kSortTile keys, with the element count
// read from device memory (so a captured graph sorts whatever a previous kernel produced): per pass, k_radix_hist
// counts digits per tile, an exclusive scan (scan.cuh) turns the digit-major counts into offsets, and
// k_radix_scatter moves the pairs, ranking equal digits within a warp by __match_any_sync.
#pragma once

#include <cstdint>

namespace sel {
namespace {

constexpr int kSortTile = 4096;  // 256 threads x 16

// One pass of a stable LSD radix sort, 8-bit digits, tiles of kSortTile keys.
__global__ void __launch_bounds__(256) k_radix_hist(const uint32_t* keys, const uint32_t* total_ptr, int shift,
                                                    uint32_t* hist, uint32_t ntiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t total = *total_ptr;
    const size_t base = size_t(blockIdx.x) * kSortTile;
    for (int k = 0; k < kSortTile / 256; ++k) {
        const size_t i = base + size_t(k) * 256 + threadIdx.x;
        if (i < total) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[size_t(threadIdx.x) * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(256) k_radix_scatter(const uint32_t* keys_in, const uint32_t* vals_in,
                                                       uint32_t* keys_out, uint32_t* vals_out,
                                                       const uint32_t* total_ptr, int shift, const uint32_t* offsets,
                                                       uint32_t ntiles) {
    __shared__ uint32_t tile_base[256];
    __shared__ uint32_t chunk_count[256];
    __shared__ uint32_t warp_hist[8][256];
    const uint32_t total = *total_ptr;
    const size_t base = size_t(blockIdx.x) * kSortTile;
    if (base >= total) return;  // tiles past the live count (block-uniform)
    tile_base[threadIdx.x] = offsets[size_t(threadIdx.x) * ntiles + blockIdx.x];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (int chunk = 0; chunk < kSortTile / 256; ++chunk) {
        if (base + size_t(chunk) * 256 >= total) break;  // block-uniform
        for (int k = 0; k < 8; ++k) warp_hist[k][threadIdx.x] = 0;
        __syncthreads();
        const size_t i = base + size_t(chunk) * 256 + threadIdx.x;
        const bool valid = i < total;
        const uint32_t key = valid ? keys_in[i] : 0u;
        const uint32_t digit = (key >> shift) & 255u;
        // lanes with the same digit, in lane order; invalid lanes match nobody
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? digit : 256u + uint32_t(lane));
        const uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) warp_hist[w][digit] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = 0;
            for (int k = 0; k < 8; ++k) {
                const uint32_t cnt = warp_hist[k][threadIdx.x];
                warp_hist[k][threadIdx.x] = run;
                run += cnt;
            }
            chunk_count[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t dst = tile_base[digit] + warp_hist[w][digit] + rank;
            keys_out[dst] = key;
            vals_out[dst] = vals_in[i];
        }
        __syncthreads();
        tile_base[threadIdx.x] += chunk_count[threadIdx.x];
        __syncthreads();
    }
}

}  // namespace
}  // namespace sel
