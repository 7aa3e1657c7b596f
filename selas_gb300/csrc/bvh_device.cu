// Device SAH-binned BVH builder: the 8-wide quantised layout of bvh_build.cpp built on the GPU.
//
// Same method as the host builder (binned SAH after Wald 2007, 32 bins per axis, leaves of at most 3
// triangles by default (1..8 selectable), object-median splits beyond depth 40, greedy collapse to 8 children by largest surface area,
// octant slot assignment and outward 8-bit child-box quantisation after Ylitie, Karras and Laine 2017),
// organised for the GPU:
//   1. one thread per triangle: bounds, centroid (box centre, as the host builder);
//   2. binary tree, top levels breadth first: every task of more than kSmall triangles is binned by many
//      blocks (block-local bins flushed with atomics), one warp per task picks the split, and the
//      triangles are partitioned with warp-aggregated cursors;
//   3. subtrees of at most kSmall triangles: one warp each, depth first with a shared-memory task stack;
//   4. collapse and quantisation breadth first: one thread per 8-wide node, scans place the next level's
//      nodes and the leaf triangles.
// Node slots follow the host builder's layout (a subtree of n triangles occupies slots [s, s + 2n - 1),
// left child at s + 1, right child at s + 2 * n_left), so the tree needs no slot allocation.  Traversal
// results do not depend on the tree (order-independent closest-hit rule, outward-rounded boxes).
#include <chrono>
#include <cmath>
#include <cstring>

#include <cuda_runtime.h>

#include "scan.cuh"
#include "sel_internal.h"

namespace sel {

namespace {

constexpr int kBinsD = 32;
constexpr uint32_t kMaxLeafLimit = kMaxLeafRecords;  // leaves beyond a node's 32 records move one level down
constexpr int kMedianDepthD = 40;
constexpr uint32_t kSmall = 1024;   // subtrees at or below this many triangles are built by one warp
constexpr int kWarpStack = 32;
constexpr int kChunk = 2048;        // triangles per block in the large-task kernels (256 threads x 8)
constexpr uint32_t kErrBuildStack = 1u;

__device__ __forceinline__ int f2o(float f) {  // float -> int with the same order
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ float box_area(float3 lo, float3 hi) {
    if (lo.x > hi.x) return 0.0f;
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

struct Build {
    const float4* soup;   // input triangles, 3 x float4 (TriRecord layout), input order
    float4* plo;          // per triangle: box lo, w = input index bits
    float4* phi;          // per triangle: box hi
    uint32_t* idx;        // triangle order (subtree ranges)
    uint32_t* idx_tmp;    // partition scratch
    float4* nlo;          // binary nodes: box lo, w = left slot bits (leaf: all ones)
    float4* nhi;          // box hi, w = right slot bits
    uint2* nrange;        // first, count (count > 0: leaf)
    uint4* tasks[2];      // large tasks: first, count, slot, depth
    uint4* small;         // small subtrees
    int* tbox;            // per large task: box lo/hi, centroid box lo/hi (ordered ints), 12 each
    int* tbins;           // per large task: 3 axes x 32 bins x (6 box ints + count)
    uint4* tsplit;        // per large task: mode (0 bins, 1 position), axis, bin, n_left
    uint32_t* tcursor;    // per large task: left / right partition cursors
    uint32_t* counters;   // [0] next large tasks, [1] small tasks, [2] max large count, [3] depth, [4] error
    int* scene_box;       // 6 ordered ints
    uint32_t n;
    uint32_t max_leaf;    // triangles per leaf, 1..kMaxLeafLimit
};

__global__ void k_init_counters(Build B) {
    if (threadIdx.x < 8) B.counters[threadIdx.x] = 0;
    if (threadIdx.x < 6) B.scene_box[threadIdx.x] = threadIdx.x < 3 ? f2o(INFINITY) : f2o(-INFINITY);
}

__global__ void __launch_bounds__(256) k_prims(Build B) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x) {
        const float4 a = B.soup[size_t(i) * 3], b = B.soup[size_t(i) * 3 + 1], c = B.soup[size_t(i) * 3 + 2];
        const float3 l = make_float3(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z));
        const float3 h = make_float3(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z));
        B.plo[i] = make_float4(l.x, l.y, l.z, __uint_as_float(i));
        B.phi[i] = make_float4(h.x, h.y, h.z, 0.0f);
        B.idx[i] = i;
        lo[0] = fminf(lo[0], l.x); lo[1] = fminf(lo[1], l.y); lo[2] = fminf(lo[2], l.z);
        hi[0] = fmaxf(hi[0], h.x); hi[1] = fmaxf(hi[1], h.y); hi[2] = fmaxf(hi[2], h.z);
    }
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMin(&B.scene_box[a], f2o(lo[a]));
            atomicMax(&B.scene_box[3 + a], f2o(hi[a]));
        }
}

__device__ __forceinline__ float centroid(const Build& B, uint32_t prim, int axis) {
    const float4 l = B.plo[prim], h = B.phi[prim];
    const float lo = axis == 0 ? l.x : (axis == 1 ? l.y : l.z);
    const float hi = axis == 0 ? h.x : (axis == 1 ? h.y : h.z);
    return 0.5f * (lo + hi);
}

// ---------------------------------------------------------------------------------------------------
// Large tasks (more than kSmall triangles), one level at a time.
// ---------------------------------------------------------------------------------------------------
__global__ void k_task_init(Build B, int cur, uint32_t ntasks) {
    const uint32_t words_box = 12, words_bins = 3 * kBinsD * 7;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ntasks * words_bins; i += gridDim.x * blockDim.x) {
        const uint32_t w = i % 7;
        B.tbins[i] = w < 3 ? f2o(INFINITY) : (w < 6 ? f2o(-INFINITY) : 0);
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ntasks * words_box; i += gridDim.x * blockDim.x) {
        const uint32_t w = i % 12;
        B.tbox[i] = (w % 6) < 3 ? f2o(INFINITY) : f2o(-INFINITY);
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * ntasks; i += gridDim.x * blockDim.x) B.tcursor[i] = 0;
    (void)cur;
}

// Block-wide min/max of 12 floats (box lo/hi, centroid lo/hi), then one atomic per value.
__global__ void __launch_bounds__(256) k_task_bounds(Build B, int cur) {
    const uint4 t = B.tasks[cur][blockIdx.y];
    const uint32_t first = t.x, count = t.y;
    const uint32_t begin = blockIdx.x * kChunk;
    if (begin >= count) return;
    const uint32_t end = min(count, begin + kChunk);
    float v[12];
    for (int k = 0; k < 12; ++k) v[k] = (k % 6) < 3 ? INFINITY : -INFINITY;
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
        const uint32_t p = B.idx[first + i];
        const float4 l = B.plo[p], h = B.phi[p];
        const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
        v[0] = fminf(v[0], l.x); v[1] = fminf(v[1], l.y); v[2] = fminf(v[2], l.z);
        v[3] = fmaxf(v[3], h.x); v[4] = fmaxf(v[4], h.y); v[5] = fmaxf(v[5], h.z);
        v[6] = fminf(v[6], c[0]); v[7] = fminf(v[7], c[1]); v[8] = fminf(v[8], c[2]);
        v[9] = fmaxf(v[9], c[0]); v[10] = fmaxf(v[10], c[1]); v[11] = fmaxf(v[11], c[2]);
    }
    __shared__ float red[12][8];
    for (int k = 0; k < 12; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            const float y = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k] = (k % 6) < 3 ? fminf(v[k], y) : fmaxf(v[k], y);
        }
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        const int k = threadIdx.x;
        float r = red[k][0];
        for (int w = 1; w < 8; ++w) r = (k % 6) < 3 ? fminf(r, red[k][w]) : fmaxf(r, red[k][w]);
        int* dst = B.tbox + size_t(blockIdx.y) * 12 + k;
        if ((k % 6) < 3) atomicMin(dst, f2o(r));
        else atomicMax(dst, f2o(r));
    }
}

__device__ __forceinline__ int bin_of(float c, float lo, float k) {
    int b = int((c - lo) * k);
    return b < 0 ? 0 : (b > kBinsD - 1 ? kBinsD - 1 : b);
}

__global__ void __launch_bounds__(256) k_task_bin(Build B, int cur) {
    __shared__ int bins[3 * kBinsD * 7];
    for (int i = threadIdx.x; i < 3 * kBinsD * 7; i += blockDim.x) {
        const int w = i % 7;
        bins[i] = w < 3 ? f2o(INFINITY) : (w < 6 ? f2o(-INFINITY) : 0);
    }
    __syncthreads();
    const uint4 t = B.tasks[cur][blockIdx.y];
    const uint32_t first = t.x, count = t.y;
    const uint32_t begin = blockIdx.x * kChunk;
    const int* tb = B.tbox + size_t(blockIdx.y) * 12;
    float clo[3], kk[3];
    for (int a = 0; a < 3; ++a) {
        clo[a] = o2f(tb[6 + a]);
        const float ext = o2f(tb[9 + a]) - clo[a];
        kk[a] = ext > 0.0f ? float(kBinsD) * (1.0f - 1e-6f) / ext : 0.0f;
    }
    if (begin < count) {
        const uint32_t end = min(count, begin + kChunk);
        for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
            const uint32_t p = B.idx[first + i];
            const float4 l = B.plo[p], h = B.phi[p];
            const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
            const int lo[3] = {f2o(l.x), f2o(l.y), f2o(l.z)}, hi[3] = {f2o(h.x), f2o(h.y), f2o(h.z)};
            for (int a = 0; a < 3; ++a) {
                int* b = bins + (a * kBinsD + bin_of(c[a], clo[a], kk[a])) * 7;
                for (int q = 0; q < 3; ++q) {
                    atomicMin(b + q, lo[q]);
                    atomicMax(b + 3 + q, hi[q]);
                }
                atomicAdd(b + 6, 1);
            }
        }
    }
    __syncthreads();
    int* g = B.tbins + size_t(blockIdx.y) * 3 * kBinsD * 7;
    for (int i = threadIdx.x; i < 3 * kBinsD * 7; i += blockDim.x) {
        const int w = i % 7;
        if (w < 3) atomicMin(g + i, bins[i]);
        else if (w < 6) atomicMax(g + i, bins[i]);
        else if (bins[i]) atomicAdd(g + i, bins[i]);
    }
}

// SAH over 32 bins of one axis, lane b = bin b: returns the lane-0 view of (cost, n_left) of the best split
// after bin b for each lane (cost +inf where a side is empty).
__device__ __forceinline__ void sah_sweep(const int* bins, int lane, float& cost, uint32_t& nleft) {
    const int* b = bins + lane * 7;
    float lo[3] = {o2f(b[0]), o2f(b[1]), o2f(b[2])}, hi[3] = {o2f(b[3]), o2f(b[4]), o2f(b[5])};
    const uint32_t c = uint32_t(b[6]);
    // inclusive prefix (left side of the split after this bin)
    float plo[3] = {lo[0], lo[1], lo[2]}, phi[3] = {hi[0], hi[1], hi[2]};
    uint32_t pc = c;
    // inclusive suffix
    float slo[3] = {lo[0], lo[1], lo[2]}, shi[3] = {hi[0], hi[1], hi[2]};
    uint32_t sc = c;
    for (int o = 1; o < 32; o <<= 1) {
        float t;
        for (int a = 0; a < 3; ++a) {
            t = __shfl_up_sync(0xffffffffu, plo[a], o); if (lane >= o) plo[a] = fminf(plo[a], t);
            t = __shfl_up_sync(0xffffffffu, phi[a], o); if (lane >= o) phi[a] = fmaxf(phi[a], t);
            t = __shfl_down_sync(0xffffffffu, slo[a], o); if (lane + o < 32) slo[a] = fminf(slo[a], t);
            t = __shfl_down_sync(0xffffffffu, shi[a], o); if (lane + o < 32) shi[a] = fmaxf(shi[a], t);
        }
        uint32_t u = __shfl_up_sync(0xffffffffu, pc, o); if (lane >= o) pc += u;
        u = __shfl_down_sync(0xffffffffu, sc, o); if (lane + o < 32) sc += u;
    }
    // split after bin `lane`: left = prefix(lane), right = suffix(lane + 1)
    float rlo[3], rhi[3];
    for (int a = 0; a < 3; ++a) {
        rlo[a] = __shfl_down_sync(0xffffffffu, slo[a], 1);
        rhi[a] = __shfl_down_sync(0xffffffffu, shi[a], 1);
    }
    const uint32_t rc = __shfl_down_sync(0xffffffffu, sc, 1);
    cost = INFINITY;
    nleft = pc;
    if (lane < 31 && pc > 0 && rc > 0) {
        const float la = box_area(make_float3(plo[0], plo[1], plo[2]), make_float3(phi[0], phi[1], phi[2]));
        const float ra = box_area(make_float3(rlo[0], rlo[1], rlo[2]), make_float3(rhi[0], rhi[1], rhi[2]));
        cost = la * float(pc) + ra * float(rc);
    }
}

__global__ void k_task_split(Build B, int cur, uint32_t ntasks) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= ntasks) return;
    const uint4 t = B.tasks[cur][warp];
    const uint32_t first = t.x, count = t.y, slot = t.z, depth = t.w;
    const int* tb = B.tbox + size_t(warp) * 12;
    float lo[3], hi[3], clo[3], chi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = o2f(tb[a]); hi[a] = o2f(tb[3 + a]); clo[a] = o2f(tb[6 + a]); chi[a] = o2f(tb[9 + a]);
    }
    int axis = 0;
    for (int a = 1; a < 3; ++a)
        if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
    const bool degenerate = !(chi[axis] > clo[axis]);
    const int* bins = B.tbins + size_t(warp) * 3 * kBinsD * 7;
    uint32_t mode = 1, split_axis = uint32_t(axis), split_bin = 0, nl = count / 2;
    if (!degenerate && int(depth) < kMedianDepthD) {
        float best = INFINITY;
        for (int a = 0; a < 3; ++a) {
            if (!(chi[a] > clo[a])) continue;
            float cost;
            uint32_t n_left;
            sah_sweep(bins + a * kBinsD * 7, lane, cost, n_left);
            // warp argmin, ties to the lower bin
            float bc = cost;
            int bb = lane;
            for (int o = 16; o > 0; o >>= 1) {
                const float oc = __shfl_xor_sync(0xffffffffu, bc, o);
                const int ob = __shfl_xor_sync(0xffffffffu, bb, o);
                if (oc < bc || (oc == bc && ob < bb)) { bc = oc; bb = ob; }
            }
            const uint32_t nlb = __shfl_sync(0xffffffffu, n_left, bb);
            if (bc < best) {
                best = bc;
                mode = 0;
                split_axis = uint32_t(a);
                split_bin = uint32_t(bb);
                nl = nlb;
            }
        }
    } else if (!degenerate) {
        // object median through the bins of the widest axis: the bin where half of the triangles is reached
        uint32_t c = uint32_t(bins[(axis * kBinsD + lane) * 7 + 6]), incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        const uint32_t ok = __ballot_sync(0xffffffffu, incl >= count / 2 && incl < count);
        if (ok) {
            const int bb = __ffs(ok) - 1;
            mode = 0;
            split_bin = uint32_t(bb);
            nl = __shfl_sync(0xffffffffu, incl, bb);
        }
    }
    if (nl == 0 || nl >= count) { mode = 1; nl = count / 2; }
    if (lane == 0) {
        B.tsplit[warp] = make_uint4(mode, split_axis, split_bin, nl);
        const uint32_t nr = count - nl;
        const uint32_t left = slot + 1, right = slot + 2 * nl;
        B.nlo[slot] = make_float4(lo[0], lo[1], lo[2], __uint_as_float(left));
        B.nhi[slot] = make_float4(hi[0], hi[1], hi[2], __uint_as_float(right));
        B.nrange[slot] = make_uint2(first, 0);
        atomicMax(&B.counters[3], depth + 1);
        const uint4 kids[2] = {make_uint4(first, nl, left, depth + 1), make_uint4(first + nl, nr, right, depth + 1)};
        for (int k = 0; k < 2; ++k) {
            if (kids[k].y > kSmall) {
                const uint32_t q = atomicAdd(&B.counters[0], 1u);
                B.tasks[cur ^ 1][q] = kids[k];
                atomicMax(&B.counters[2], kids[k].y);
            } else {
                const uint32_t q = atomicAdd(&B.counters[1], 1u);
                B.small[q] = kids[k];
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_task_partition(Build B, int cur) {
    const uint4 t = B.tasks[cur][blockIdx.y];
    const uint32_t first = t.x, count = t.y;
    const uint4 sp = B.tsplit[blockIdx.y];
    const int* tb = B.tbox + size_t(blockIdx.y) * 12;
    const int a = int(sp.y);
    const float clo = o2f(tb[6 + a]);
    const float ext = o2f(tb[9 + a]) - clo;
    const float k = ext > 0.0f ? float(kBinsD) * (1.0f - 1e-6f) / ext : 0.0f;
    const uint32_t begin = blockIdx.x * kChunk;
    if (begin >= count) return;
    const uint32_t end = min(count, begin + kChunk);
    const int lane = threadIdx.x & 31;
    for (uint32_t base = begin; base < end; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < end;
        uint32_t p = 0;
        bool left = false;
        if (valid) {
            p = B.idx[first + i];
            left = sp.x == 0 ? bin_of(centroid(B, p, a), clo, k) <= int(sp.z) : i < sp.w;
        }
        const uint32_t lm = __ballot_sync(0xffffffffu, valid && left), rm = __ballot_sync(0xffffffffu, valid && !left);
        uint32_t lb = 0, rb = 0;
        if (lane == 0) {
            if (lm) lb = atomicAdd(&B.tcursor[2 * blockIdx.y], __popc(lm));
            if (rm) rb = atomicAdd(&B.tcursor[2 * blockIdx.y + 1], __popc(rm));
        }
        lb = __shfl_sync(0xffffffffu, lb, 0);
        rb = __shfl_sync(0xffffffffu, rb, 0);
        const uint32_t below = (1u << lane) - 1u;
        if (valid) {
            const uint32_t dst = left ? first + lb + __popc(lm & below) : first + sp.w + rb + __popc(rm & below);
            B.idx_tmp[dst] = p;
        }
    }
}

__global__ void __launch_bounds__(256) k_task_copy_back(Build B, int cur) {
    const uint4 t = B.tasks[cur][blockIdx.y];
    const uint32_t first = t.x, count = t.y;
    const uint32_t begin = blockIdx.x * kChunk;
    if (begin >= count) return;
    const uint32_t end = min(count, begin + kChunk);
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) B.idx[first + i] = B.idx_tmp[first + i];
}

// ---------------------------------------------------------------------------------------------------
// Small subtrees: one warp each, depth first (the larger child waits on the stack, so it holds at most
// log2(kSmall) entries).
// ---------------------------------------------------------------------------------------------------
constexpr int kSmallWarps = 4;

__global__ void __launch_bounds__(32 * kSmallWarps) k_small(Build B) {
    __shared__ int sbins[kSmallWarps][3 * kBinsD * 7];
    __shared__ uint4 sstack[kSmallWarps][kWarpStack];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int* bins = sbins[w];
    uint4* stack = sstack[w];
    const uint32_t ntasks = B.counters[1];
    for (uint32_t task = blockIdx.x * kSmallWarps + w; task < ntasks; task += gridDim.x * kSmallWarps) {
        int sp = 0;
        uint4 t = B.small[task];
        for (;;) {
            const uint32_t first = t.x, count = t.y, slot = t.z, depth = t.w;
            float v[12];
            for (int k = 0; k < 12; ++k) v[k] = (k % 6) < 3 ? INFINITY : -INFINITY;
            for (uint32_t i = lane; i < count; i += 32) {
                const uint32_t p = B.idx[first + i];
                const float4 l = B.plo[p], h = B.phi[p];
                const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
                v[0] = fminf(v[0], l.x); v[1] = fminf(v[1], l.y); v[2] = fminf(v[2], l.z);
                v[3] = fmaxf(v[3], h.x); v[4] = fmaxf(v[4], h.y); v[5] = fmaxf(v[5], h.z);
                v[6] = fminf(v[6], c[0]); v[7] = fminf(v[7], c[1]); v[8] = fminf(v[8], c[2]);
                v[9] = fmaxf(v[9], c[0]); v[10] = fmaxf(v[10], c[1]); v[11] = fmaxf(v[11], c[2]);
            }
            for (int k = 0; k < 12; ++k)
                for (int o = 16; o > 0; o >>= 1) {
                    const float y = __shfl_xor_sync(0xffffffffu, v[k], o);
                    v[k] = (k % 6) < 3 ? fminf(v[k], y) : fmaxf(v[k], y);
                }
            if (lane == 0) atomicMax(&B.counters[3], depth + 1);
            bool leaf = count <= 1;
            uint32_t mode = 1, split_axis = 0, split_bin = 0, nl = count / 2;
            int axis = 0;
            for (int a = 1; a < 3; ++a)
                if (v[9 + a] - v[6 + a] > v[9 + axis] - v[6 + axis]) axis = a;
            split_axis = uint32_t(axis);
            const bool degenerate = !(v[9 + axis] > v[6 + axis]);
            if (!leaf && (degenerate || int(depth) >= kMedianDepthD)) {
                leaf = count <= B.max_leaf;  // otherwise split by position
            } else if (!leaf) {
                for (int i = lane; i < 3 * kBinsD * 7; i += 32) {
                    const int q = i % 7;
                    bins[i] = q < 3 ? f2o(INFINITY) : (q < 6 ? f2o(-INFINITY) : 0);
                }
                __syncwarp();
                float kk[3];
                for (int a = 0; a < 3; ++a) {
                    const float ext = v[9 + a] - v[6 + a];
                    kk[a] = ext > 0.0f ? float(kBinsD) * (1.0f - 1e-6f) / ext : 0.0f;
                }
                for (uint32_t i = lane; i < count; i += 32) {
                    const uint32_t p = B.idx[first + i];
                    const float4 l = B.plo[p], h = B.phi[p];
                    const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
                    const int lo[3] = {f2o(l.x), f2o(l.y), f2o(l.z)}, hi[3] = {f2o(h.x), f2o(h.y), f2o(h.z)};
                    for (int a = 0; a < 3; ++a) {
                        if (!(v[9 + a] > v[6 + a])) continue;
                        int* b = bins + (a * kBinsD + bin_of(c[a], v[6 + a], kk[a])) * 7;
                        for (int q = 0; q < 3; ++q) {
                            atomicMin(b + q, lo[q]);
                            atomicMax(b + 3 + q, hi[q]);
                        }
                        atomicAdd(b + 6, 1);
                    }
                }
                __syncwarp();
                float best = INFINITY;
                int best_axis = -1;
                for (int a = 0; a < 3; ++a) {
                    if (!(v[9 + a] > v[6 + a])) continue;
                    float cost;
                    uint32_t n_left;
                    sah_sweep(bins + a * kBinsD * 7, lane, cost, n_left);
                    float bc = cost;
                    int bb = lane;
                    for (int o = 16; o > 0; o >>= 1) {
                        const float oc = __shfl_xor_sync(0xffffffffu, bc, o);
                        const int ob = __shfl_xor_sync(0xffffffffu, bb, o);
                        if (oc < bc || (oc == bc && ob < bb)) { bc = oc; bb = ob; }
                    }
                    const uint32_t nlb = __shfl_sync(0xffffffffu, n_left, bb);
                    if (bc < best) {
                        best = bc;
                        best_axis = a;
                        split_bin = uint32_t(bb);
                        nl = nlb;
                    }
                }
                const float parent = box_area(make_float3(v[0], v[1], v[2]), make_float3(v[3], v[4], v[5]));
                const float leaf_cost = parent * float(count);
                const float split_cost = parent + best;
                if (count <= B.max_leaf && (best_axis < 0 || split_cost >= leaf_cost)) {
                    leaf = true;
                } else if (best_axis >= 0) {
                    mode = 0;
                    split_axis = uint32_t(best_axis);
                }
                __syncwarp();
            }
            if (!leaf && (nl == 0 || nl >= count)) { mode = 1; nl = count / 2; }
            if (leaf) {
                if (lane == 0) {
                    B.nlo[slot] = make_float4(v[0], v[1], v[2], __uint_as_float(0xffffffffu));
                    B.nhi[slot] = make_float4(v[3], v[4], v[5], __uint_as_float(0xffffffffu));
                    B.nrange[slot] = make_uint2(first, count);
                }
            } else {
                // stable partition into the scratch range, then back
                const float ext = v[9 + split_axis] - v[6 + split_axis];
                const float k = ext > 0.0f ? float(kBinsD) * (1.0f - 1e-6f) / ext : 0.0f;
                uint32_t lcount = 0, rcount = 0;
                for (uint32_t base = 0; base < count; base += 32) {
                    const uint32_t i = base + lane;
                    const bool valid = i < count;
                    uint32_t p = 0;
                    bool left = false;
                    if (valid) {
                        p = B.idx[first + i];
                        left = mode == 0 ? bin_of(centroid(B, p, int(split_axis)), v[6 + split_axis], k) <= int(split_bin)
                                         : i < nl;
                    }
                    const uint32_t lm = __ballot_sync(0xffffffffu, valid && left);
                    const uint32_t rm = __ballot_sync(0xffffffffu, valid && !left);
                    const uint32_t below = (1u << lane) - 1u;
                    if (valid) {
                        const uint32_t dst = left ? first + lcount + __popc(lm & below)
                                                  : first + nl + rcount + __popc(rm & below);
                        if (dst < first + count) B.idx_tmp[dst] = p;
                    }
                    lcount += __popc(lm);
                    rcount += __popc(rm);
                }
                __syncwarp();
                for (uint32_t i = lane; i < count; i += 32) B.idx[first + i] = B.idx_tmp[first + i];
                __syncwarp();
                const uint32_t nr = count - nl;
                const uint32_t left = slot + 1, right = slot + 2 * nl;
                if (lane == 0) {
                    B.nlo[slot] = make_float4(v[0], v[1], v[2], __uint_as_float(left));
                    B.nhi[slot] = make_float4(v[3], v[4], v[5], __uint_as_float(right));
                    B.nrange[slot] = make_uint2(first, 0);
                }
                const uint4 l4 = make_uint4(first, nl, left, depth + 1), r4 = make_uint4(first + nl, nr, right, depth + 1);
                const bool left_smaller = nl <= nr;
                if (sp >= kWarpStack) {  // cannot happen (depth-first on the smaller child): record, stop
                    if (lane == 0) atomicOr(&B.counters[4], kErrBuildStack);
                    break;
                }
                if (lane == 0) stack[sp] = left_smaller ? r4 : l4;
                __syncwarp();
                ++sp;
                t = left_smaller ? l4 : r4;
                continue;
            }
            if (sp == 0) break;
            --sp;
            __syncwarp();
            t = stack[sp];
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// Collapse to 8-wide nodes and quantisation, one level at a time.
// ---------------------------------------------------------------------------------------------------
struct Collapse {
    const uint2* level;   // (wide index, binary node)
    uint2* next;
    int* slots;           // per entry: 8 binary children in slot order (-1 empty)
    uint32_t* cnt_int;    // internal children per entry
    uint32_t* cnt_tri;    // leaf triangles per entry
    uint32_t* off_int;
    uint32_t* off_tri;
    WideNode* nodes;
    TriRecord* tris;
};

__device__ __forceinline__ bool is_leaf(const Build& B, int n) { return B.nrange[n].y > 0; }

__global__ void __launch_bounds__(128) k_collapse_gather(Build B, Collapse C, uint32_t count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int root = int(C.level[i].y);
    int children[8];
    int nc = 0;
    if (is_leaf(B, root)) {
        children[nc++] = root;
    } else {
        children[nc++] = int(__float_as_uint(B.nlo[root].w));
        children[nc++] = int(__float_as_uint(B.nhi[root].w));
        while (nc < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (int k = 0; k < nc; ++k) {
                if (is_leaf(B, children[k])) continue;
                const float4 l = B.nlo[children[k]], h = B.nhi[children[k]];
                const float a = box_area(make_float3(l.x, l.y, l.z), make_float3(h.x, h.y, h.z));
                if (a > best_area) { best_area = a; best = k; }
            }
            if (best < 0) break;
            const int opened = children[best];
            children[best] = int(__float_as_uint(B.nlo[opened].w));
            children[nc++] = int(__float_as_uint(B.nhi[opened].w));
        }
    }
    // slot assignment by octant direction (the host builder's rule): candidates (cost, child, slot) in
    // ascending cost, ties in (child, slot) order as a stable sort of child-major candidates leaves them
    float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float3 cen[8];
    for (int k = 0; k < nc; ++k) {
        const float4 l = B.nlo[children[k]], h = B.nhi[children[k]];
        nlo[0] = fminf(nlo[0], l.x); nlo[1] = fminf(nlo[1], l.y); nlo[2] = fminf(nlo[2], l.z);
        nhi[0] = fmaxf(nhi[0], h.x); nhi[1] = fmaxf(nhi[1], h.y); nhi[2] = fmaxf(nhi[2], h.z);
        cen[k] = make_float3(0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z));
    }
    const float pc[3] = {0.5f * (nlo[0] + nhi[0]), 0.5f * (nlo[1] + nhi[1]), 0.5f * (nlo[2] + nhi[2])};
    int slot_child[8];
    bool done[8] = {false, false, false, false, false, false, false, false};
    for (int s = 0; s < 8; ++s) slot_child[s] = -1;
    for (int round = 0; round < nc; ++round) {
        float best = INFINITY;
        int bc = -1, bs = -1;
        for (int k = 0; k < nc; ++k) {
            if (done[k]) continue;
            const float off[3] = {cen[k].x - pc[0], cen[k].y - pc[1], cen[k].z - pc[2]};
            for (int s = 0; s < 8; ++s) {
                if (slot_child[s] >= 0) continue;
                const float d = (s & 4 ? off[0] : -off[0]) + (s & 2 ? off[1] : -off[1]) + (s & 1 ? off[2] : -off[2]);
                const float cost = -d;
                if (cost < best) { best = cost; bc = k; bs = s; }
            }
        }
        if (bc < 0) break;
        slot_child[bs] = children[bc];
        done[bc] = true;
    }
    // A node's leaf children hold 32 records at most (the traversal's record mask).  With leaves of more than
    // 4 triangles eight of them can hold more: the largest leaf (the lowest slot among equals) then becomes an
    // internal child, a node of its own one level down whose single slot is that leaf, until the rest fit.
    // Such a demoted leaf is stored as -(child + 2) in the slot table.
    uint32_t nt = 0;
    for (int s = 0; s < 8; ++s)
        if (slot_child[s] >= 0 && is_leaf(B, slot_child[s])) nt += B.nrange[slot_child[s]].y;
    while (nt > kMaxNodeRecords) {
        int big = -1;
        for (int s = 0; s < 8; ++s)
            if (slot_child[s] >= 0 && is_leaf(B, slot_child[s]) &&
                (big < 0 || B.nrange[slot_child[s]].y > B.nrange[slot_child[big]].y))
                big = s;
        nt -= B.nrange[slot_child[big]].y;
        slot_child[big] = -(slot_child[big] + 2);
    }
    uint32_t ni = 0;
    for (int s = 0; s < 8; ++s) {
        C.slots[size_t(i) * 8 + s] = slot_child[s];
        if (slot_child[s] <= -2 || (slot_child[s] >= 0 && !is_leaf(B, slot_child[s]))) ++ni;
    }
    C.cnt_int[i] = ni;
    C.cnt_tri[i] = nt;
}

// Outward 8-bit quantisation of the child boxes on one axis (the host builder's rule, in double precision).
__device__ void quantise_axis(int a, float nlo, float nhi, const float* clo, const float* chi, const bool* present,
                              WideNode& node) {
    const double ext = double(nhi) - double(nlo);
    const double mag = fmax(fabs(double(nlo)), fabs(double(nhi)));
    const double min_q = fmax(ldexp(mag, -20), ldexp(1.0, -60));
    int e;
    frexp(fmax(ext / 250.0, min_q), &e);
    for (int guard = 0; guard < 2100; ++guard, ++e) {
        const double scale = ldexp(1.0, e);
        float p = float(double(nlo) - scale);
        if (double(p) > double(nlo) - scale) p = nextafterf(p, -INFINITY);
        bool ok = true;
        for (int s = 0; s < 8; ++s) {
            if (!present[s]) {
                node.qlo[a][s] = 255;
                node.qhi[a][s] = 0;
                continue;
            }
            double lo = floor((double(clo[s]) - p) / scale) - 1.0;
            double hi = ceil((double(chi[s]) - p) / scale) + 1.0;
            while (lo > 0.0 && double(p) + lo * scale > double(clo[s]) - 0.5 * scale) lo -= 1.0;
            while (double(p) + hi * scale < double(chi[s]) + 0.5 * scale) hi += 1.0;
            if (lo < 0.0 || hi > 255.0 || double(p) + lo * scale > double(clo[s]) - 0.5 * scale) {
                ok = false;
                break;
            }
            node.qlo[a][s] = uint8_t(lo);
            node.qhi[a][s] = uint8_t(hi);
        }
        if (ok) {
            node.p[a] = p;
            node.e[a] = uint8_t(e + 127);
            return;
        }
    }
}

__global__ void __launch_bounds__(128) k_collapse_emit(Build B, Collapse C, uint32_t count, uint32_t next_base,
                                                       uint32_t tri_base) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int slot_child[8];
    bool present[8];
    float lo[3][8], hi[3][8];
    float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    bool demoted[8];
    for (int s = 0; s < 8; ++s) {
        slot_child[s] = C.slots[size_t(i) * 8 + s];
        demoted[s] = slot_child[s] <= -2;
        if (demoted[s]) slot_child[s] = -slot_child[s] - 2;
        present[s] = slot_child[s] >= 0;
        if (!present[s]) continue;
        const float4 l = B.nlo[slot_child[s]], h = B.nhi[slot_child[s]];
        lo[0][s] = l.x; lo[1][s] = l.y; lo[2][s] = l.z;
        hi[0][s] = h.x; hi[1][s] = h.y; hi[2][s] = h.z;
        for (int a = 0; a < 3; ++a) { nlo[a] = fminf(nlo[a], lo[a][s]); nhi[a] = fmaxf(nhi[a], hi[a][s]); }
    }
    WideNode node;
    memset(&node, 0, sizeof(node));
    memset(node.meta, int(kLeafNone), sizeof(node.meta));
    for (int a = 0; a < 3; ++a) quantise_axis(a, nlo[a], nhi[a], lo[a], hi[a], present, node);
    node.child_base = next_base + C.off_int[i];
    node.tri_base = tri_base + C.off_tri[i];
    uint32_t ni = 0, offset = 0;
    for (int s = 0; s < 8; ++s) {
        const int c = slot_child[s];
        if (c < 0) continue;
        if (demoted[s] || !is_leaf(B, c)) {
            node.imask |= uint8_t(1u << s);
            C.next[C.off_int[i] + ni] = make_uint2(node.child_base + ni, uint32_t(c));
            ++ni;
            continue;
        }
        const uint2 r = B.nrange[c];
        node.meta[s] = uint8_t(((r.y - 1u) << 5) | offset);
        for (uint32_t k = 0; k < r.y; ++k) {
            const uint32_t tri = __float_as_uint(B.plo[B.idx[r.x + k]].w);
            const float4* src = B.soup + size_t(tri) * 3;
            float4* dst = reinterpret_cast<float4*>(C.tris + node.tri_base + offset + k);
            dst[0] = src[0];
            dst[1] = src[1];
            dst[2] = src[2];
        }
        offset += r.y;
    }
    C.nodes[C.level[i].x] = node;
}

template <typename T>
cudaError_t dalloc(T*& p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * (count ? count : 1));
}

}  // namespace

std::string build_wide_device(const std::vector<MeshInput>& meshes, uint32_t max_leaf, DeviceBuild& out) {
    if (max_leaf < 1 || max_leaf > kMaxLeafLimit) return "leaf size must lie in 1..8";
    std::vector<TriRecord> soup;
    size_t total = 0;
    for (const MeshInput& m : meshes) total += m.indices.size() / 3;
    if (total == 0) return "scene has no triangles";
    if (total > (size_t(1) << 30)) return "too many triangles";
    soup.reserve(total);
    for (const MeshInput& m : meshes) {
        const size_t nv = m.vertices.size() / 3;
        const size_t nt = m.indices.size() / 3;
        for (size_t t = 0; t < nt; ++t) {
            TriRecord r;
            float* dst[3] = {r.v0, r.v1, r.v2};
            for (int k = 0; k < 3; ++k) {
                const uint32_t vi = m.indices[3 * t + k];
                if (vi >= nv) return "triangle index out of range";
                std::memcpy(dst[k], &m.vertices[3 * size_t(vi)], 12);
                for (int a = 0; a < 3; ++a)
                    if (!std::isfinite(dst[k][a])) return "non-finite vertex";
            }
            r.prim = uint32_t(t);
            r.geom = m.geomID;
            r.kind = m.quads ? kTriQuadHalf : (m.curves ? kTriCurve : kTriPlain);
            soup.push_back(r);
        }
    }
    const uint32_t n = uint32_t(total);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t s = nullptr;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    const auto t0 = std::chrono::steady_clock::now();

    Build B;
    std::memset(&B, 0, sizeof(B));
    B.n = n;
    B.max_leaf = max_leaf;
    const uint32_t max_large = n / kSmall + 2;
    const size_t max_nodes = 2 * size_t(n);
    std::vector<void*> owned;
    cudaError_t e = cudaSuccess;
    auto take = [&](auto*& p, size_t count) {
        if (e == cudaSuccess) e = dalloc(p, count);
        if (e == cudaSuccess) owned.push_back(static_cast<void*>(p));
    };
    float4* soup_d = nullptr;
    take(soup_d, size_t(n) * 3);
    B.soup = soup_d;
    take(B.plo, n);
    take(B.phi, n);
    take(B.idx, n);
    take(B.idx_tmp, n);
    take(B.nlo, max_nodes);
    take(B.nhi, max_nodes);
    take(B.nrange, max_nodes);
    take(B.tasks[0], max_large);
    take(B.tasks[1], max_large);
    take(B.small, n);
    take(B.tbox, size_t(max_large) * 12);
    take(B.tbins, size_t(max_large) * 3 * kBinsD * 7);
    take(B.tsplit, max_large);
    take(B.tcursor, size_t(max_large) * 2);
    take(B.counters, 16);
    take(B.scene_box, 8);
    uint32_t* h_counters = nullptr;
    if (e == cudaSuccess) e = cudaMallocHost(&h_counters, 16 * sizeof(uint32_t));
    auto cleanup = [&]() {
        for (void* p : owned) cudaFree(p);
        if (h_counters) cudaFreeHost(h_counters);
        cudaStreamDestroy(s);
    };
    if (e != cudaSuccess) {
        cleanup();
        return std::string("device BVH build: ") + cudaGetErrorString(e);
    }
    e = cudaMemcpyAsync(soup_d, soup.data(), sizeof(TriRecord) * n, cudaMemcpyHostToDevice, s);
    k_init_counters<<<1, 32, 0, s>>>(B);
    k_prims<<<sms * 8, 256, 0, s>>>(B);
    const auto read_counters = [&]() {
        cudaMemcpyAsync(h_counters, B.counters, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        return cudaStreamSynchronize(s);
    };
    // root task
    const uint4 root = make_uint4(0, n, 0, 0);
    int cur = 0;
    uint32_t ntasks = 0, max_count = 0;
    if (n > kSmall) {
        cudaMemcpyAsync(B.tasks[0], &root, sizeof(root), cudaMemcpyHostToDevice, s);
        ntasks = 1;
        max_count = n;
    } else {
        cudaMemcpyAsync(B.small, &root, sizeof(root), cudaMemcpyHostToDevice, s);
        const uint32_t one = 1;
        cudaMemcpyAsync(B.counters + 1, &one, sizeof(one), cudaMemcpyHostToDevice, s);
    }
    while (ntasks > 0 && e == cudaSuccess) {
        if (ntasks > 65535) {  // one grid row per task
            cleanup();
            return "device BVH build: too many large tasks in one level (use the host builder)";
        }
        const dim3 grid((max_count + kChunk - 1) / kChunk, ntasks);
        k_task_init<<<sms * 4, 256, 0, s>>>(B, cur, ntasks);
        k_task_bounds<<<grid, 256, 0, s>>>(B, cur);
        k_task_bin<<<grid, 256, 0, s>>>(B, cur);
        cudaMemsetAsync(B.counters, 0, sizeof(uint32_t), s);      // next large tasks
        cudaMemsetAsync(B.counters + 2, 0, sizeof(uint32_t), s);  // their largest count
        k_task_split<<<(ntasks * 32 + 127) / 128, 128, 0, s>>>(B, cur, ntasks);
        k_task_partition<<<grid, 256, 0, s>>>(B, cur);
        k_task_copy_back<<<grid, 256, 0, s>>>(B, cur);
        e = read_counters();
        ntasks = h_counters[0];
        max_count = h_counters[2];
        cur ^= 1;
    }
    if (e == cudaSuccess) {
        k_small<<<sms * 8, 32 * kSmallWarps, 0, s>>>(B);
        e = read_counters();
    }
    if (e == cudaSuccess && h_counters[4]) e = cudaErrorUnknown;
    const uint32_t binary_depth = h_counters[3];

    // collapse, level by level
    std::vector<uint32_t> level_sizes;
    WideNode* nodes = nullptr;
    TriRecord* tris = nullptr;
    Collapse C;
    std::memset(&C, 0, sizeof(C));
    uint2 *lvl_a = nullptr, *lvl_b = nullptr;
    uint32_t* scan_tmp = nullptr;
    uint32_t *cnt_int = nullptr, *cnt_tri = nullptr, *off_int = nullptr, *off_tri = nullptr;
    int* slots = nullptr;
    // 8-wide nodes: each has at least two slots except the single-leaf nodes of demoted leaves (at most one per
    // five triangles, as only a leaf of five or more is demoted), so at most n + n / 5 + 1 of them
    const size_t max_wide = max_leaf > 4 ? n + n / 5 + 1 : n;
    take(nodes, max_wide);
    take(tris, n);
    take(lvl_a, max_wide);
    take(lvl_b, max_wide);
    take(slots, max_wide * 8);
    take(cnt_int, max_wide);
    take(cnt_tri, max_wide);
    take(off_int, max_wide + 1);
    take(off_tri, max_wide + 1);
    take(scan_tmp, scan_scratch_words(max_wide));
    std::string err;
    uint32_t node_count = 0, tri_count = 0, depth = 0;
    if (e == cudaSuccess) {
        const uint2 r = make_uint2(0, 0);
        cudaMemcpyAsync(lvl_a, &r, sizeof(r), cudaMemcpyHostToDevice, s);
        uint32_t count = 1, base = 0;
        while (count > 0 && e == cudaSuccess) {
            if (++depth > uint32_t(kWideStack)) {
                err = "8-wide BVH deeper than the traversal stack";
                break;
            }
            C.level = lvl_a;
            C.next = lvl_b;
            C.slots = slots;
            C.cnt_int = cnt_int;
            C.cnt_tri = cnt_tri;
            C.off_int = off_int;
            C.off_tri = off_tri;
            C.nodes = nodes;
            C.tris = tris;
            k_collapse_gather<<<(count + 127) / 128, 128, 0, s>>>(B, C, count);
            scan_exclusive(cnt_int, count, off_int, scan_tmp, s);
            scan_exclusive(cnt_tri, count, off_tri, scan_tmp, s);
            k_collapse_emit<<<(count + 127) / 128, 128, 0, s>>>(B, C, count, base + count, tri_count);
            uint32_t totals[2] = {0, 0};
            cudaMemcpyAsync(&totals[0], off_int + count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(&totals[1], off_tri + count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
            e = cudaStreamSynchronize(s);
            base += count;
            tri_count += totals[1];
            count = totals[0];
            std::swap(lvl_a, lvl_b);
        }
        node_count = base;
    }
    if (e == cudaSuccess && err.empty() && tri_count != n) err = "device BVH build lost triangles";
    if (e == cudaSuccess) e = cudaGetLastError();
    int box[8] = {0};
    if (e == cudaSuccess) {
        cudaMemcpyAsync(box, B.scene_box, 6 * sizeof(int), cudaMemcpyDeviceToHost, s);
        e = cudaStreamSynchronize(s);
    }
    const auto t1 = std::chrono::steady_clock::now();
    if (e != cudaSuccess || !err.empty()) {
        cleanup();
        return err.empty() ? std::string("device BVH build: ") + cudaGetErrorString(e) : err;
    }
    // hand the node and triangle arrays to the caller, free the rest
    out.d_nodes = nodes;
    out.d_tris = tris;
    for (void* p : owned)
        if (p != nodes && p != tris) cudaFree(p);
    cudaFreeHost(h_counters);
    cudaStreamDestroy(s);
    auto o2f_host = [](int i) {
        const int b = i >= 0 ? i : i ^ 0x7fffffff;
        float f;
        std::memcpy(&f, &b, 4);
        return f;
    };
    for (int a = 0; a < 3; ++a) {
        out.lo[a] = o2f_host(box[a]);
        out.hi[a] = o2f_host(box[3 + a]);
    }
    out.node_count = node_count;
    out.tri_count = tri_count;
    out.max_depth = depth;
    out.binary_depth = binary_depth;
    out.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    return "";
}

}  // namespace sel
