// Host interface of the vertex connection and merging integrator (vcm.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "graph.h"
#include "pt.h"

namespace sel {

// Per-pass constants (VCMCommon.cpp:91-112), computed on the host for a range of passes so that every
// pass launches the same kernels with the same arguments (a pass reads its row through a device counter).
struct VcmConsts {
    float radius, radius2;
    float vm_weight;  // pi r^2 N without merging turned off, else 0
    float vc_weight;  // 1 / (pi r^2 N)
    float vm_norm;    // 1 / (pi r^2 N)
    float n_paths;
    uint32_t pass;    // global pass index: random streams and the radius schedule
    uint32_t pad;
};

struct VcmSettings {
    uint32_t max_len;  // maximum path length in segments (MaxBounceCount_)
    uint64_t seed;
    int merging;       // 0: bidirectional path tracing (no merge term, no merge weights)
    uint32_t light_first, light_count;  // light set 0 within the scene's light array
    uint32_t trace_block;  // threads per traversal block: 256 or 128 (the 8-wide layout; the binary one: 128)
};

// Device scratch of one VCM pass for `paths` light and camera paths (paths = width * height): the light
// vertices, the wavefront path state and queues, the shadow queue and the hash grid.
struct VcmState {
    float4* verts;        // light vertices, 5 x float4 each, max_len - 1 slots per light path
    uint32_t* vcount;     // stored vertices per light path
    uint32_t* vpos;       // exclusive scan of vcount (+ total)
    // path state, one slot per path (slot = path index)
    float4* po;           // origin, dVCM
    float4* pd;           // direction, dVC
    float4* pt;           // throughput, dVM
    uint32_t* plen;       // path length in segments
    uint64_t* prng;       // PCG32 state (the stream is a function of the pass and the slot)
    float4* phit;         // t, u, v, triangle bits (all ones: miss)
    uint2* phinst;        // instances entered to the hit (scenes with instances: 1 + table index per level)
    uint32_t* queue[2];   // live path slots, ping-pong between bounces
    uint32_t* queue_sorted;  // the current queue ordered by material class (counting sort)
    uint32_t* cls;        // material class of each current queue entry
    float4* base;         // Ptex base colour (authored) of the path's current hit, filtered before shading
    // shadow queue: light tracing, next-event and connection segments with their contributions
    float4* so;           // origin, tnear
    float4* sd;           // direction, tfar
    float4* sc;           // contribution, pixel bits (zero contribution: null entry)
    uint32_t shadow_capacity;
    uint32_t* counters;   // [0],[1] queue lengths, [2] shadow entries, [3] extend cursor, [4] shadow cursor,
                          // [5] camera-vertex records, [6] connection pairs; [32..47] material-class counts,
                          // [48..63] their scatter cursors
    unsigned long long* rays;  // [0] closest-hit, [1] any-hit rays traced, running totals
    float4* cverts;       // camera-vertex records of the current bounce, 6 x float4 each
    uint2* pairs;         // (camera-vertex record, light-vertex index) connection pairs of the current bounce
    float4* spos;         // stored-vertex positions in cell order, slot bits in w
    uint32_t* keys[2];    // radix-sort ping-pong: cell of each stored vertex
    uint32_t* vals[2];    // ... and its slot
    uint32_t* cell_count; // vertices per cell
    uint32_t* cell_start; // exclusive scan of cell_count (+ total)
    uint32_t* hist;       // radix digit counts per tile (digit-major)
    uint32_t* hist_off;   // their exclusive scan
    uint32_t* scan_tmp;   // tile sums of the scans
    float* bounds_part;   // per-block bound partials
    float* grid;          // lo[3], hi[3], inv_cell, radius2
    uint32_t* iter;       // current row of the constants table
    VcmConsts* consts;    // constants table
    uint32_t paths, slots_per_path, consts_capacity;
};

size_t vcm_state_block_bytes(uint32_t paths, uint32_t max_len, uint32_t passes);
VcmState vcm_state_carve(void* block, uint32_t paths, uint32_t max_len, uint32_t passes);

// Camera model of the light-tracing strategy: the pixel-area image-plane distance width / (2 tan(fov/2)).
struct VcmCamera {
    PtCamera cam;
    float image_plane;
};

// Runs passes [first, first + passes).  Accumulates into d_accum ([height][width][3] doubles) the sum of
// the passes' images.
// Copies the constants of `passes` passes to the device table and restarts its row counter.
cudaError_t vcm_upload_constants(const VcmState& st, const VcmConsts* host_consts, uint32_t passes,
                                 cudaStream_t stream);
// Launches `passes` passes continuing from the current row of the constants table.  With `graphs`, one pass
// is captured as a CUDA graph (once per argument set) and replayed per pass.
cudaError_t vcm_run_passes(const PtScene& sc, const VcmCamera& cam, const VcmSettings& set, uint32_t passes,
                           const VcmState& st, double* d_accum, uint32_t* d_err, cudaStream_t stream,
                           GraphCache* graphs);
// Upload + run.

cudaError_t vcm_render(const PtScene& sc, const VcmCamera& cam, const VcmSettings& set, const VcmConsts* host_consts,
                       uint32_t passes, const VcmState& st, double* d_accum, uint32_t* d_err, cudaStream_t stream,
                       GraphCache* graphs);

}  // namespace sel
