// Wavefront unidirectional path tracer: the GB300 form of PathTracer::GenerateImage / EvaluatePath
// (Source/Applications/Selas/Source/PathTracer.cpp:142-258, 261-349).
//
// The wavefront is shared by up to kMaxPtJobs render jobs (scene, camera, spp, seed, accumulator) held in a
// device-resident job table: a batch takes up to `quota` paths from each job, every path carries its job
// slot, and each kernel reads the job's scene, camera and accumulator through it.  A single render is the
// one-job case.
//
// Per batch of paths: generate -> for each bounce: extend (closest hit) -> shade (surface setup, quad-light
// NEE, BSDF sampling, Russian roulette) -> shadow (any hit).  Queues hold path slots; appends are
// warp-aggregated (one atomic per warp).  Contributions go straight into an FP64 per-pixel accumulator
// (layer 0: first-bounce reflectance, layer 1: radiance, as the reference's two framebuffer layers), so
// the path state carries no per-path radiance.  Every path draws from its own PCG32 stream (stream id =
// global path index), consumed in the order the reference consumes its sampler: jitter x/y; per bounce
// [distance in a medium: 2], light pick + 2 for the light, BSDF lobe + 2..3, [medium scatter: 2],
// [Russian roulette after bounce 8: 1].
//
// A job may instead run the deferred path tracer (DeferredPathTracer.cpp:61-148, 151-279, 349-380): sample s of
// pixel p jitters by the correlated multi-jittered point cmj_point(s, m, m, p) (path index s * W * H + p, no
// draws), and per hit the stream gives light pick + 2, 2 for a background direction (drawn whatever the
// background), BSDF lobe + 2..3 and, from the 7th bounce on, one for Russian roulette.  Its shading emits up to
// two shadow rays (quad light with weight 1; background with the balance heuristic), both from tnear 0, and
// weights the BSDF continuation by the balance heuristic against the background density 1 / (4 pi).  Such a
// job accumulates one layer (radiance).
#include "pt.h"

#include <algorithm>
#include <cstring>

#include "capi_internal.h"
#include "cmj.cuh"
#include "graph.h"
#include "ibl.cuh"
#include "hitref.cuh"
#include "instance.cuh"
#include "ptex.cuh"
#include "ptex_quad.cuh"
#include "radix.cuh"
#include "scan.cuh"
#include "tex2d.cuh"
#include "shading.cuh"
#include "traverse.cuh"

namespace sel {

namespace {

constexpr int kBlock = 128;
constexpr float kFloatMax = 3.402823466e+38f;  // FloatMax_ (SystemLib/BasicTypes.h:31)

struct PtParams {
    PtState st;
    uint32_t* err;
};

__device__ __forceinline__ CameraDev camera_of(const PtCamera& c) {
    CameraDev d;
    d.x = make_float3(c.x[0], c.x[1], c.x[2]);
    d.y = make_float3(c.y[0], c.y[1], c.y[2]);
    d.z = make_float3(c.z[0], c.z[1], c.z[2]);
    d.position = make_float3(c.position[0], c.position[1], c.position[2]);
    d.width = float(c.width);
    d.height = float(c.height);
    return d;
}

// Warp-aggregated append: returns this lane's slot in a queue whose length lives at *count.
__device__ __forceinline__ uint32_t warp_append(uint32_t* count, bool want) {
    const uint32_t mask = __ballot_sync(__activemask(), want);
    if (!want) return 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void accumulate(double* accum, uint32_t npix, int layer, uint32_t pixel, float3 c) {
    double* p = accum + (size_t(layer) * npix + pixel) * 3;
    atomicAdd(p, double(c.x));
    atomicAdd(p + 1, double(c.y));
    atomicAdd(p + 2, double(c.z));
}

__device__ __forceinline__ Pcg32 load_rng(const PtState& st, uint32_t slot) {
    Pcg32 r;
    r.state = st.rng[slot];
    r.inc = (st.path_id[slot] << 1u) | 1u;
    return r;
}

// Batch set-up: each job slot contributes min(paths left, quota) paths; counts, prefix and the batch size are
// derived here from the device-resident control block, so every batch launches the same kernels with the
// same arguments and one batch can be captured as a graph and replayed.
__global__ void k_batch_begin(PtParams P) {
    PtControl& c = *P.st.control;
    const uint32_t lane = threadIdx.x;  // one warp
    uint32_t cnt = 0;
    if (lane < c.njobs && lane < kMaxPtJobs) {
        const uint64_t total = P.st.jobs[lane].total, next = c.next[lane];
        const uint64_t left = total > next ? total - next : 0;
        cnt = uint32_t(left < c.quota[lane] ? left : c.quota[lane]);
    }
    uint32_t incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= uint32_t(o)) incl += y;
    }
    const uint32_t batch = __shfl_sync(0xffffffffu, incl, 31);
    if (lane < kMaxPtJobs) {
        c.count[lane] = cnt;
        c.prefix[lane] = incl - cnt;
    }
    if (lane == 0) c.prefix[kMaxPtJobs] = batch;
    if (lane < kPtCounters) P.st.counters[lane] = lane == 0 ? batch : 0u;
    if (lane == kPtCounters) P.st.counters[kPtCounters] = batch;
}

__global__ void k_batch_end(PtParams P) {
    PtControl& c = *P.st.control;
    if (threadIdx.x < kMaxPtJobs) c.next[threadIdx.x] += c.count[threadIdx.x];
}

__global__ void k_bounce_reset(uint32_t* counters, int next) {
    // next queue length, shadow queue length and both fetch cursors restart each bounce
    if (threadIdx.x == 0) {
        counters[next] = 0u;
        counters[2] = 0u;
        counters[3] = 0u;
        counters[4] = 0u;
    }
}

__global__ void __launch_bounds__(kBlock) k_generate(PtParams P) {
    const PtControl& c = *P.st.control;
    const uint32_t batch = P.st.counters[kPtCounters];
    const uint32_t njobs = c.njobs < kMaxPtJobs ? c.njobs : kMaxPtJobs;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < batch; s += gridDim.x * blockDim.x) {
        uint32_t j = 0;
        while (j + 1 < njobs && s >= c.prefix[j + 1]) ++j;
        const PtJob& J = P.st.jobs[j];
        const uint64_t path = c.next[j] + (s - c.prefix[j]);
        const uint32_t width = J.cam.width;
        const uint32_t npix = width * J.cam.height;
        const uint32_t pixel = uint32_t(path % npix);
        Pcg32 rng = pcg_seed(J.seed, path);
        const uint32_t y = pixel / width, x = pixel - y * width;
        float vx, vy;
        if (J.mode == kPtModeDeferred) {  // JitteredCameraRay(camera, x, y, s, m, m, index) (Camera.cpp:77-86)
            const int32_t m = int32_t(J.samples_per_axis);
            const float2 j = cmj_point(int32_t(path / npix), m, m, int32_t(pixel));
            vx = float(x) + j.x;
            vy = float(y) + j.y;
        } else {  // JitteredCameraRay (Camera.cpp:63-74)
            vx = float(x) + pcg_float(rng);
            vy = float(y) + pcg_float(rng);
        }
        const CameraDev cam = camera_of(J.cam);
        const float3 d = camera_direction(cam, vx, vy);
        P.st.ray_o[s] = make_float4(cam.position.x, cam.position.y, cam.position.z, 0.0f);
        P.st.ray_d[s] = make_float4(d.x, d.y, d.z, kFloatMax);
        P.st.thr[s] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);  // w = isDeltaOnly
        P.st.medium[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // x = phase (0 vacuum, 1 isotropic)
        P.st.pixel[s] = pixel;
        P.st.job[s] = j;
        P.st.path_id[s] = path;
        P.st.rng[s] = rng.state;
        P.st.queue[0][s] = s;
    }
}

}  // namespace

// A scene whose hits may need Ptex (its own faces, or instances whose scenes may have some).
bool pt_scene_textured(const PtScene& sc) { return sc.ptex_face_count > 0 || sc.tex2d != 0 || sc.insts != nullptr; }

namespace {

// A hit's leaf record and shading data (hitref.cuh) for path slot s of the wavefront.
template <bool kInst>
__device__ __forceinline__ HitRef hit_ref(const PtState& st, const PtScene& S, uint32_t s, uint32_t tri) {
    return hit_ref_of<kInst>(S, kInst ? st.hinst[s] : make_uint2(0u, 0u), tri);
}

// Per-thread traversal stacks of a B-thread block in shared memory (entry k of thread t at k * B + t).  The
// instanced traversal's 40-entry stacks of a 256-thread block take 80 KB: they live in dynamic shared memory
// (launched with trace_stack_bytes<K, B>() bytes and the matching MaxDynamicSharedMemorySize attribute); every
// other stack is a static array.
template <int K, int B>
constexpr size_t trace_stack_bytes() {
    return size_t(Tracer<K>::kDepth) * B * sizeof(typename Tracer<K>::Entry);
}
template <int K, int B>
constexpr bool kDynamicStack = trace_stack_bytes<K, B>() > 48u * 1024u;

template <int K, int B>
__device__ __forceinline__ typename Tracer<K>::Entry* trace_stack() {
    if constexpr (kDynamicStack<K, B>) {
        extern __shared__ __align__(16) unsigned char pt_dynamic_stack[];
        return reinterpret_cast<typename Tracer<K>::Entry*>(pt_dynamic_stack);
    } else {
        __shared__ typename Tracer<K>::Entry stack_mem[Tracer<K>::kDepth * B];
        return stack_mem;
    }
}

// Closest hit for the queued paths.  Warps take 32-entry packets from the queue through an atomic cursor,
// so expensive and cheap rays balance across the GPU.  K = 2: the instanced traversal of the 8-wide layout.
template <int K, int B>
__global__ void __launch_bounds__(B, K == 2 ? 512 / B : 1024 / B) k_extend(PtParams P, int cur) {
    typename Tracer<K>::Entry* stack_mem = trace_stack<K, B>();
    const uint32_t n = P.st.counters[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(P.st.rays, (unsigned long long)n);
    const uint32_t* queue = P.st.queue[cur];
    uint32_t status = 0;
    for (;;) {
        uint32_t base = 0;
        if ((threadIdx.x & 31u) == 0) base = atomicAdd(&P.st.counters[3], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t e = base + (threadIdx.x & 31u);
        if (e < n) {
            const uint32_t s = queue[e];
            const float4 o = P.st.ray_o[s], d = P.st.ray_d[s];
            const float4 med = P.st.medium[s];
            float tfar = kFloatMax;
            if (med.x != 0.0f) {
                // Isotropic::SampleDistance (Shading/IsotropicScattering.cpp:18-47)
                Pcg32 rng = load_rng(P.st, s);
                const float ps = med.y + med.z + med.w;
                const float pr = med.y / ps, pg = med.z / ps, pb = med.w / ps;
                float c, p;
                const float r0 = pcg_float(rng);
                if (r0 < pr) { c = med.y; p = pr; }
                else if (r0 < pr + pg) { c = med.z; p = pg; }
                else { c = med.w; p = pb; }
                (void)p;
                tfar = -logf(pcg_float(rng)) / c;
                P.st.rng[s] = rng.state;
            }
            QueryRay q;
            q.ox = o.x; q.oy = o.y; q.oz = o.z; q.tnear = 0.0f;
            q.dx = d.x; q.dy = d.y; q.dz = d.z; q.tfar = tfar;
            const PtScene& sc = P.st.jobs[P.st.job[s]].scene;
            if constexpr (K == 2) {
                InstHit h;
                const bool found = trace_instanced<false>(static_cast<const uint4*>(sc.nodes), sc.tris, sc.insts, q,
                                                          h, stack_mem + threadIdx.x, B, status);
                P.st.hit[s] = found ? make_float4(h.t, h.u, h.v, __uint_as_float(h.tri))
                                    : make_float4(tfar, 0.0f, 0.0f, __uint_as_float(0xffffffffu));
                P.st.hinst[s] = found ? inst_indices(sc.insts, h) : make_uint2(0u, 0u);
            } else {
                QueryHit h;
                const bool found = Tracer<K>::template trace<false>(sc.nodes, sc.tris, q, h, stack_mem + threadIdx.x,
                                                                    B, status);
                P.st.hit[s] = found ? make_float4(h.t, h.u, h.v, __uint_as_float(h.tri))
                                    : make_float4(tfar, 0.0f, 0.0f, __uint_as_float(0xffffffffu));
            }
        }
    }
    if (status) atomicOr(P.err, status);
}

// Material class of a queued path's hit: 0 miss; else 1 + shader * 4 + 2 (Ptex) + 1 (transparent).  Paths
// are sorted by class before shading, so a warp shades one kind of surface.
__device__ __forceinline__ uint32_t class_of(const MaterialDev& m) {
    const uint32_t shader = uint32_t(m.shader) < 3u ? uint32_t(m.shader) : 0u;
    return 1u + shader * 4u + ((m.flags & kMaterialTextured) ? 2u : 0u) + ((m.flags & kMaterialTransparent) ? 1u : 0u);
}

template <bool kInst>
__device__ __forceinline__ uint32_t material_class(const PtParams& P, uint32_t s) {
    const uint32_t tri = __float_as_uint(P.st.hit[s].w);
    if (tri == 0xffffffffu) return 0u;
    const PtScene& S = P.st.jobs[P.st.job[s]].scene;
    const HitRef r = hit_ref<kInst>(P.st, S, s, tri);
    const uint32_t geom = __float_as_uint(__ldg(r.tp + 1).w);
    return class_of(r.mats[geom < r.mat_count ? geom : 0]);
}

__global__ void k_class_reset(uint32_t* counters) {
    if (threadIdx.x < 2 * kPtClasses) counters[32 + threadIdx.x] = 0u;
}

template <bool kInst>
__global__ void __launch_bounds__(kBlock) k_classify(PtParams P, int cur) {
    const uint32_t n = P.st.counters[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        const bool valid = e < n;
        const uint32_t c = valid ? material_class<kInst>(P, P.st.queue[cur][e]) : 0xffu;
        if (valid) P.st.cls[e] = c;
        const uint32_t peers = __match_any_sync(0xffffffffu, c);
        const uint32_t lane = threadIdx.x & 31u;
        if (valid && (__ffs(peers) - 1) == int(lane)) atomicAdd(&P.st.counters[32 + c], __popc(peers));
    }
}

__global__ void k_class_offsets(uint32_t* counters) {
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int c = 0; c < kPtClasses; ++c) {
            counters[48 + c] = run;
            run += counters[32 + c];
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_class_scatter(PtParams P, int cur) {
    const uint32_t n = P.st.counters[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        const bool valid = e < n;
        const uint32_t c = valid ? P.st.cls[e] : 0xffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, c);
        const uint32_t lane = threadIdx.x & 31u;
        const int leader = __ffs(peers) - 1;
        uint32_t at = 0;
        if (valid && leader == int(lane)) at = atomicAdd(&P.st.counters[48 + c], __popc(peers));
        at = __shfl_sync(0xffffffffu, at, leader);
        if (valid) P.st.queue_sorted[at + __popc(peers & ((1u << lane) - 1u))] = P.st.queue[cur][e];
    }
}

// Sort key of a queued hit in a textured scene: the material class (bits 20-23) above, for a Ptex-textured hit,
// its face modulo 2^17 (bits 3-19) and the edges its filter footprint crosses (bits 0-2).  Hits on one face sit together, as
// the reference's batcher orders hits by (instance, geometry, primitive) before shading
// (PathTracingBatcher.cpp:221-238,799-825), and hits whose footprints cross the same edges walk the same faces,
// so a warp's Ptex filter walks stay in step.  Three 8-bit radix passes order the queue by it.
// kCount: the classes are counted as k_classify counts them (per-shader shading kernels find their classes'
// ranges from the counts; a batch with one shader shades the whole queue and needs none).
template <bool kInst, bool kCount>
__global__ void __launch_bounds__(kBlock) k_sort_keys(PtParams P, int cur) {
    const uint32_t n = P.st.counters[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        const bool valid = e < n;
        const uint32_t s = valid ? P.st.queue[cur][e] : 0u;
        const float4 hit = valid ? P.st.hit[s] : make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xffffffffu));
        const uint32_t tri = __float_as_uint(hit.w);
        uint32_t key = 0u;
        if (tri != 0xffffffffu) {
            const PtScene& S = P.st.jobs[P.st.job[s]].scene;
            const HitRef r = hit_ref<kInst>(P.st, S, s, tri);
            const float4 p0 = __ldg(r.tp), p1 = __ldg(r.tp + 1);
            const uint32_t geom = __float_as_uint(p1.w);
            const MaterialDev& m = r.mats[geom < r.mat_count ? geom : 0];
            key = class_of(m) << 20;
            if (m.flags & kMaterialPtexQuad) {  // the quad's face; no footprint region
                const int face = int(m.ptex_base + (__float_as_uint(p0.w) >> 1));
                key |= (uint32_t(face) & 0x1ffffu) << 3;
            } else if (m.flags & kMaterialUsesPtex) {
                const int face = int(m.ptex_base + __float_as_uint(p0.w));
                key |= ((uint32_t(face) & 0x1ffffu) << 3) |
                       ptex_region(static_cast<const PtexFace*>(r.ptex_faces), int(r.ptex_count), face, hit.y, hit.z);
            }
        }
        if (valid) P.st.rkeys[0][e] = key;
        if constexpr (kCount) {
            const uint32_t c = valid ? key >> 20 : 0xffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, c);
            if (valid && (__ffs(peers) - 1) == int(threadIdx.x & 31u)) atomicAdd(&P.st.counters[32 + c], __popc(peers));
        }
    }
}

// Ptex base colour of the sorted paths whose hit material is textured (SurfaceParameters.cpp:196-206): a
// kernel of its own keeps the filter's code out of the shading kernel.
// kQuad: the batch has quad-mesh Ptex; without it the quad filter (a function call) stays out of the kernel, whose
// triangle filter would otherwise lose registers to the call.
template <bool kInst, bool kQuad>
__global__ void __launch_bounds__(kBlock) k_texture(PtParams P, int cur, const uint32_t* in_queue) {
    const uint32_t n = P.st.counters[cur];
    uint32_t status = 0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const uint32_t s = in_queue[e];
        const float4 hit = P.st.hit[s];
        const uint32_t tri = __float_as_uint(hit.w);
        if (tri == 0xffffffffu) continue;
        const PtScene& S = P.st.jobs[P.st.job[s]].scene;
        const HitRef r = hit_ref<kInst>(P.st, S, s, tri);
        const float4 p0 = __ldg(r.tp), p1 = __ldg(r.tp + 1);
        const uint32_t geom = __float_as_uint(p1.w);
        const MaterialDev& m = r.mats[geom < r.mat_count ? geom : 0];
        if (!(m.flags & kMaterialTextured)) continue;
        float3 base = ld3(m.base_color);
        if (m.flags & kMaterialUsesPtex) {
            uint32_t pstatus = 0;
            if (kQuad && (m.flags & kMaterialPtexQuad))
                ptex_material_eval(m, r.ptex_faces, int(r.ptex_count), static_cast<const __half*>(r.ptex_texels),
                                   __float_as_uint(p0.w), hit.y, hit.z, base, pstatus);
            else
                ptex_eval(static_cast<const PtexFace*>(r.ptex_faces), int(r.ptex_count),
                          static_cast<const __half*>(r.ptex_texels), int(m.ptex_base + __float_as_uint(p0.w)), hit.y,
                          hit.z, base, pstatus);
            status |= pstatus;
        } else {
            base = tex2d_base_colour(m, geom < r.attr_count ? r.attrs + geom : nullptr, __float_as_uint(p0.w), hit.y,
                                     hit.z);
        }
        P.st.base[s] = make_float4(base.x, base.y, base.z, 0.0f);
    }
    if (status) atomicOr(P.err, status);
}

// kModes: bit 0 path-tracer jobs, bit 1 deferred jobs in the batch (a single-mode batch compiles the other
// integrator out of the kernel).
// The path tracer's shading at most 96 registers (5 blocks per SM; a few bytes spill): 2 % faster renders of the
// room than 102 registers.  The deferred and mixed forms keep 4 blocks per SM (their bigger code would spill).
// kShader: the shader of every hit the kernel shades (-1: any).  classes = (c0, c1): the kernel shades the
// entries of material classes c0..c1 of the class-ordered queue (class counts in counters[32 + c]); c0 < 0: the
// whole queue.
template <uint32_t kModes, bool kInst, int kShader>
__global__ void __launch_bounds__(kBlock, kModes == 1u ? 5 : 4) k_shade(PtParams P, int cur, uint32_t bounce,
                                                                        const uint32_t* in_queue, int2 classes) {
    uint32_t lo = 0, hi = P.st.counters[cur];
    if (classes.x >= 0) {
        uint32_t before = 0, upto = 0;
        for (int c = 0; c < kPtClasses; ++c) {
            const uint32_t k = P.st.counters[32 + c];
            before += c < classes.x ? k : 0u;
            upto += c <= classes.y ? k : 0u;
        }
        lo = before;
        hi = upto;
    }
    const int next = cur ^ 1;
    for (uint32_t base = lo + blockIdx.x * blockDim.x; base < hi; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        const bool valid = e < hi;
        bool cont = false, shadow = false, shadow2 = false;
        uint32_t s = 0;
        float4 sh_o = make_float4(0, 0, 0, 0), sh_d = sh_o, sh_c = sh_o;
        float4 sh2_o = sh_o, sh2_d = sh_o, sh2_c = sh_o;  // deferred: the background's shadow ray
        if (valid) {
            s = in_queue[e];
            const uint32_t job = P.st.job[s];
            const PtJob& J = P.st.jobs[job];
            const PtScene& S = J.scene;
            const uint32_t npix = J.cam.width * J.cam.height;
            const bool deferred = kModes == 2u || (kModes == 3u && J.mode == kPtModeDeferred);
            const float4 o4 = P.st.ray_o[s], d4 = P.st.ray_d[s];
            const float3 o = f3(o4.x, o4.y, o4.z), d = f3(d4.x, d4.y, d4.z);
            float4 thr4 = P.st.thr[s];
            float3 thr = f3(thr4.x, thr4.y, thr4.z);
            float4 med = P.st.medium[s];
            const float4 hit = P.st.hit[s];
            const uint32_t tri = __float_as_uint(hit.w);
            const uint32_t pixel = P.st.pixel[s];
            Pcg32 rng = load_rng(P.st, s);
            float ray_distance = hit.x;
            float3 pos = f3(0.0f);
            if (tri != 0xffffffffu) {
                pos = f3(o.x + hit.x * d.x, o.y + hit.x * d.y, o.z + hit.x * d.z);
                ray_distance = length(pos - o);
            }
            if (med.x != 0.0f) {  // Isotropic::Transmission
                thr = thr * f3(expf(-med.y * ray_distance), expf(-med.z * ray_distance), expf(-med.w * ray_distance));
            }
            bool alive = true;
            if (tri != 0xffffffffu) {
                const HitRef hr = hit_ref<kInst>(P.st, S, s, tri);
                const float4 p0 = __ldg(hr.tp), p1 = __ldg(hr.tp + 1), p2 = __ldg(hr.tp + 2);
                const uint32_t geom = __float_as_uint(p1.w);
                const MaterialDev& m = hr.mats[geom < hr.mat_count ? geom : 0];
                const MeshAttrDev* attr = geom < hr.attr_count ? hr.attrs + geom : nullptr;
                float3 fn, ft, fb;
                float fsign;
                const float3 ng = kInst ? record_ng(hr.tp, p0, p1, p2, hr.rec0, hr.rec1, o, d, hit.x, hit.y)
                                        : triangle_ng(p0, p1, p2);
                shading_frame(attr, __float_as_uint(p0.w), hit.y, hit.z, ng,
                              [&](float3 x) { return kInst ? world_normal(hr, x) : x; }, fn, ft, fb, fsign);
                // RayPick error bound (PathTracer.cpp:134-136)
                const float err = 32.0f * 1.19209e-07f *
                                  fmaxf(fmaxf(fabsf(pos.x), fabsf(pos.y)), fmaxf(fabsf(pos.z), hit.x));
                float3 base = ld3(m.base_color);
                if (m.flags & kMaterialTextured) {  // filtered or sampled by k_texture for this hit
                    const float4 b = P.st.base[s];
                    base = f3(b.x, b.y, b.z);
                }
                const Surface sf = make_surface_frame(m, ft, fn, fb, -d, pow3(base, 2.2f));
                // Next-event estimation to the surface's light set (AreaLighting.cpp:353-373)
                LightSample ls;
                ls.radiance = f3(0.0f);
                if (m.light_set < S.light_set_count) {
                    const uint2 set = S.light_sets[m.light_set];
                    if (set.y > 0) {
                        const float p0u = pcg_float(rng);
                        uint32_t li = uint32_t(p0u * float(set.y));
                        li = li < set.y ? li : set.y - 1;
                        const float u = pcg_float(rng), v = pcg_float(rng);
                        sample_quad_light(S.lights[set.x + li], pos, sf.n, u, v, ls);
                        ls.pdf *= 1.0f / float(set.y);
                    }
                }
                const uint32_t tag = (job << 28) | pixel;
                if (dot(ls.radiance, f3(1.0f)) > 0.0f) {
                    float fpdf, rpdf;
                    const float3 refl = bsdf_evaluate_as<kShader>(sf, -d, ls.direction, fpdf, rpdf);
                    if (deferred) {
                        // weight 1 (DeferredPathTracer.cpp:65-88); the shadow ray starts at tnear 0
                        const float3 smp = 1.0f * refl * ls.radiance * (1.0f / ls.pdf);
                        if (dot(smp, f3(1.0f)) > 0.0f) {
                            const float3 so = offset_origin(pos, sf.n, err, ls.direction, 0.1f);
                            const float3 c = smp * thr;
                            sh_o = make_float4(so.x, so.y, so.z, 0.0f);
                            sh_d = make_float4(ls.direction.x, ls.direction.y, ls.direction.z, ls.distance);
                            sh_c = make_float4(c.x, c.y, c.z, __uint_as_float(tag));
                            shadow = true;
                        }
                    } else if (dot(refl, f3(1.0f)) > 0.0f) {
                        // OcclusionRay (PathTracer.cpp:71-92): origin offset 0.1 * error, tnear = error
                        const float3 so = offset_origin(pos, sf.n, err, ls.direction, 0.1f);
                        const float3 c = refl * ls.radiance * (1.0f / ls.pdf) * thr;
                        sh_o = make_float4(so.x, so.y, so.z, err);
                        sh_d = make_float4(ls.direction.x, ls.direction.y, ls.direction.z, ls.distance);
                        sh_c = make_float4(c.x, c.y, c.z, __uint_as_float(tag));
                        shadow = true;
                    }
                }
                if (deferred) {
                    // SampleBackground (AreaLighting.cpp:393-401): with an image DirectIblLightSample (:293-314),
                    // else BackgroundLightSample (:334-350), a uniform sphere direction whose density is recorded
                    // as 1; at distance 1e36; balance heuristic against the BSDF's density
                    // (DeferredPathTracer.cpp:90-111)
                    const float r0 = pcg_float(rng), r1 = pcg_float(rng);
                    float3 sdir, bg;
                    float spdf;
                    if (S.ibl) {
                        ibl_sample(*S.ibl, r0, r1, sdir, bg, spdf);
                    } else {
                        const float uu = 2.0f * r1 - 1.0f;
                        const float nn = sqrtf(fmaxf(0.0f, 1.0f - uu * uu));
                        const float th = kTwoPi * r0;
                        sdir = f3(nn * cosf(th), uu, nn * sinf(th));
                        bg = f3(S.background[0], S.background[1], S.background[2]);
                        spdf = 1.0f;
                    }
                    if (dot(bg, f3(1.0f)) > 0.0f) {
                        float fpdf, rpdf;
                        const float3 refl = bsdf_evaluate_as<kShader>(sf, -d, sdir, fpdf, rpdf);
                        const float mis = (1.0f * spdf) / (1.0f * spdf + 1.0f * fpdf);
                        const float3 smp = mis * refl * bg * (1.0f / spdf);
                        if (dot(smp, f3(1.0f)) > 0.0f) {
                            const float3 so = offset_origin(pos, sf.n, err, sdir, 0.1f);
                            const float3 c = smp * thr;
                            sh2_o = make_float4(so.x, so.y, so.z, 0.0f);
                            sh2_d = make_float4(sdir.x, sdir.y, sdir.z, 1e36f);
                            sh2_c = make_float4(c.x, c.y, c.z, __uint_as_float(tag));
                            shadow2 = true;
                        }
                    }
                }
                // BSDF sampling: draw ahead from a copy of the stream, then advance by what was used
                float u4[4];
                Pcg32 ahead = rng;
                for (int k = 0; k < 4; ++k) u4[k] = pcg_float(ahead);
                int used = 0;
                BsdfSampleOut bs;
                const bool ok = bsdf_sample_as<kShader>(sf, -d, u4, used, bs);
                for (int k = 0; k < used; ++k) pcg_next(rng);
                if (!ok) {
                    alive = false;
                } else if (deferred) {
                    // balance heuristic against the background density (BackgroundLightingPdf, AreaLighting.cpp:
                    // 404-413: the image's density, else 1 / (4 pi))
                    const float sky_pdf = S.ibl ? ibl_pdf(*S.ibl, bs.wi) : kInv4Pi;
                    const float mis = (1.0f * bs.forward_pdf) / (1.0f * bs.forward_pdf + 1.0f * sky_pdf);
                    if (!(bs.flags & kDiracEvent)) thr4.w = 0.0f;  // diracScatterOnly
                    const float3 t = mis * thr * bs.reflectance;
                    if (dot(t, t) == 0.0f) {
                        alive = false;
                    } else {
                        thr = t;
                        const float3 no = offset_origin(pos, sf.n, err, bs.wi, 1.0f);
                        P.st.ray_o[s] = make_float4(no.x, no.y, no.z, 0.0f);
                        P.st.ray_d[s] = make_float4(bs.wi.x, bs.wi.y, bs.wi.z, kFloatMax);
                    }
                } else {
                    if (!(bs.flags & kDiracEvent)) thr4.w = 0.0f;
                    if (bs.flags == kTransmissionEvent) {
                        if (med.x == 0.0f) med = make_float4(float(bs.medium_phase), bs.extinction.x, bs.extinction.y, bs.extinction.z);
                        else med = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    }
                    thr = 1.0f * thr * bs.reflectance;
                    const float3 no = offset_origin(pos, sf.n, err, bs.wi, 1.0f);
                    P.st.ray_o[s] = make_float4(no.x, no.y, no.z, 0.0f);
                    P.st.ray_d[s] = make_float4(bs.wi.x, bs.wi.y, bs.wi.z, kFloatMax);
                    if (bounce == 0) accumulate(J.accum, npix, 0, pixel, bs.reflectance);
                }
            } else if (!deferred && med.x != 0.0f) {
                // scatter inside the medium: Isotropic::SampleScatterDirection -> CSampler::UniformSphere
                const float3 no = o + ray_distance * d;
                const float r0 = pcg_float(rng), r1 = pcg_float(rng);
                const float uu = 2.0f * r1 - 1.0f;
                const float nn = sqrtf(fmaxf(0.0f, 1.0f - uu * uu));
                const float th = kTwoPi * r0;
                const float3 nd = f3(nn * cosf(th), uu, nn * sinf(th));
                P.st.ray_o[s] = make_float4(no.x, no.y, no.z, 0.0f);
                P.st.ray_d[s] = make_float4(nd.x, nd.y, nd.z, kFloatMax);
            } else {
                // miss: EvaluateBackgroundMiss for a camera ray or a pure specular chain, else EvaluateBackground
                // (AreaLighting.cpp:415-436): the image's miss / light texel, or the uniform background
                float3 bg = f3(S.background[0], S.background[1], S.background[2]);
                if (S.ibl) bg = thr4.w != 0.0f ? ibl_miss(*S.ibl, d) : ibl_radiance(*S.ibl, d);
                accumulate(J.accum, npix, deferred ? 0 : 1, pixel, bg * thr);
                alive = false;
            }
            if (alive) {
                const uint32_t nb = bounce + 1;
                if (deferred) {
                    if (bounce >= 7) {  // Russian roulette once MaxTrackedBounces_ = 7 are tracked
                        const float cp = fmaxf(fmaxf(thr.x, thr.y), thr.z);
                        if (pcg_float(rng) >= cp) alive = false;
                        else thr = thr * (1.0f / cp);
                    }
                } else if (nb > 8) {  // Russian roulette (PathTracer.cpp:248-254)
                    const float cp = fmaxf(fmaxf(thr.x, thr.y), thr.z);
                    if (pcg_float(rng) > cp) alive = false;
                    else thr = thr * (1.0f / cp);
                }
                cont = alive && nb < J.max_bounces;
            }
            P.st.thr[s] = make_float4(thr.x, thr.y, thr.z, thr4.w);
            P.st.medium[s] = med;
            P.st.rng[s] = rng.state;
        }
        const uint32_t qslot = warp_append(&P.st.counters[next], cont);
        if (cont) P.st.queue[next][qslot] = s;
        const uint32_t sslot = warp_append(&P.st.counters[2], shadow);
        if (shadow) {
            P.st.sh_o[sslot] = sh_o;
            P.st.sh_d[sslot] = sh_d;
            P.st.sh_c[sslot] = sh_c;
        }
        if ((kModes & 2u) && __any_sync(0xffffffffu, shadow2)) {  // the queue holds 2 records per path
            const uint32_t s2 = warp_append(&P.st.counters[2], shadow2);
            if (shadow2) {
                P.st.sh_o[s2] = sh2_o;
                P.st.sh_d[s2] = sh2_d;
                P.st.sh_c[s2] = sh2_c;
            }
        }
    }
}

template <int K, int B>
__global__ void __launch_bounds__(B, K == 2 ? 512 / B : 1024 / B) k_shadow(PtParams P) {
    typename Tracer<K>::Entry* stack_mem = trace_stack<K, B>();
    const uint32_t n = P.st.counters[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(P.st.rays + 1, (unsigned long long)n);
    uint32_t status = 0;
    for (;;) {
        uint32_t base = 0;
        if ((threadIdx.x & 31u) == 0) base = atomicAdd(&P.st.counters[4], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t e = base + (threadIdx.x & 31u);
        if (e < n) {
            const float4 o = P.st.sh_o[e], d = P.st.sh_d[e];
            const float4 c = P.st.sh_c[e];
            const uint32_t tag = __float_as_uint(c.w);
            const PtJob& J = P.st.jobs[tag >> 28];
            QueryRay q;
            q.ox = o.x; q.oy = o.y; q.oz = o.z; q.tnear = o.w;
            q.dx = d.x; q.dy = d.y; q.dz = d.z; q.tfar = d.w;
            bool blocked;
            if constexpr (K == 2) {
                InstHit h;
                blocked = trace_instanced<true>(static_cast<const uint4*>(J.scene.nodes), J.scene.tris, J.scene.insts,
                                                q, h, stack_mem + threadIdx.x, B, status);
            } else {
                QueryHit h;
                blocked = Tracer<K>::template trace<true>(J.scene.nodes, J.scene.tris, q, h, stack_mem + threadIdx.x, B,
                                                          status);
            }
            if (!blocked)
                accumulate(J.accum, J.cam.width * J.cam.height, J.mode == kPtModeDeferred ? 0 : 1, tag & 0x0fffffffu,
                           f3(c.x, c.y, c.z));
        }
    }
    if (status) atomicOr(P.err, status);
}

// Sort key of a continuing ray (the batcher's order, PathTracingBatcher.cpp:162-258): direction bin (dominant axis
// x 2 + sign, 3 bits) above a 12-bit Morton code of the origin in the job scene's bounds (4 bits per axis).
__device__ __forceinline__ uint32_t spread4(uint32_t x) {
    x &= 15u;
    x = (x | (x << 4)) & 0x0C3u;
    x = (x | (x << 2)) & 0x249u;
    return x;
}

__global__ void __launch_bounds__(kBlock) k_ray_keys(PtParams P, int next) {
    const uint32_t n = P.st.counters[next];
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const uint32_t s = P.st.queue[next][e];
        const float4 o = P.st.ray_o[s], d = P.st.ray_d[s];
        const PtScene& S = P.st.jobs[P.st.job[s]].scene;
        const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
        const uint32_t axis = (ax >= ay && ax >= az) ? 0u : (ay >= az ? 1u : 2u);
        const float dc = axis == 0 ? d.x : (axis == 1 ? d.y : d.z);
        const uint32_t bin = axis * 2u + (dc < 0.0f ? 1u : 0u);
        uint32_t q[3];
        const float oc[3] = {o.x, o.y, o.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float ext = S.hi[a] - S.lo[a];
            const float t = ext > 0.0f ? (oc[a] - S.lo[a]) / ext : 0.0f;
            q[a] = uint32_t(fminf(fmaxf(t * 16.0f, 0.0f), 15.0f));
        }
        P.st.rkeys[0][e] = (bin << 12) | spread4(q[0]) | (spread4(q[1]) << 1) | (spread4(q[2]) << 2);
    }
}

__global__ void k_resolve(const double* accum, uint32_t count, double scale, float* out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        out[i] = float(accum[i] * scale);
}

int grid_for(int sm_count, int blocks_per_sm) { return sm_count * blocks_per_sm; }

}  // namespace

// Carves the path state of `paths` slots out of one device block (the caller owns the block).
namespace {
template <typename Take>
void pt_layout(PtState& st, Take take, uint32_t paths) {
    st.ray_o = reinterpret_cast<float4*>(take(16ull * paths));
    st.ray_d = reinterpret_cast<float4*>(take(16ull * paths));
    st.thr = reinterpret_cast<float4*>(take(16ull * paths));
    st.medium = reinterpret_cast<float4*>(take(16ull * paths));
    st.hit = reinterpret_cast<float4*>(take(16ull * paths));
    st.hinst = reinterpret_cast<uint2*>(take(8ull * paths));
    st.pixel = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.job = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.path_id = reinterpret_cast<uint64_t*>(take(8ull * paths));
    st.rng = reinterpret_cast<uint64_t*>(take(8ull * paths));
    st.queue[0] = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.queue[1] = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.queue_sorted = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.cls = reinterpret_cast<uint32_t*>(take(4ull * paths));
    st.base = reinterpret_cast<float4*>(take(16ull * paths));
    st.sh_o = reinterpret_cast<float4*>(take(32ull * paths));
    st.sh_d = reinterpret_cast<float4*>(take(32ull * paths));
    st.sh_c = reinterpret_cast<float4*>(take(32ull * paths));
    st.counters = reinterpret_cast<uint32_t*>(take(64 * sizeof(uint32_t)));
    {
        const size_t ntiles = (size_t(paths) + kSortTile - 1) / kSortTile;
        st.rkeys[0] = reinterpret_cast<uint32_t*>(take(4ull * paths));
        st.rkeys[1] = reinterpret_cast<uint32_t*>(take(4ull * paths));
        st.rvals = reinterpret_cast<uint32_t*>(take(4ull * paths));
        st.rhist = reinterpret_cast<uint32_t*>(take(4 * 256 * ntiles));
        st.rhist_off = reinterpret_cast<uint32_t*>(take(4 * (256 * ntiles + 1)));
        st.rscan_tmp = reinterpret_cast<uint32_t*>(take(4 * ((256 * ntiles + 1 + kScanTile - 1) / kScanTile + 1)));
    }
    st.rays = reinterpret_cast<unsigned long long*>(take(2 * sizeof(unsigned long long)));
    st.control = reinterpret_cast<PtControl*>(take(sizeof(PtControl)));
    st.jobs = reinterpret_cast<PtJob*>(take(sizeof(PtJob) * kMaxPtJobs));
    st.capacity = paths;
}
}  // namespace

PtState pt_state_carve(void* block, uint32_t paths) {
    char* p = static_cast<char*>(block);
    PtState st;
    pt_layout(st, [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    }, paths);
    return st;
}

size_t pt_state_block_bytes(uint32_t paths) {
    size_t total = 0;
    PtState st;
    pt_layout(st, [&](size_t bytes) {
        total += (bytes + 255) & ~size_t(255);
        return static_cast<char*>(nullptr);
    }, paths);
    return total;
}

// Shader-specific kernels for the solid and Dirac shaders of single-integrator batches; thin surfaces and mixed
// batches take the kernel for every shader (each specialisation is compiled once per integrator and instancing).
template <uint32_t kModes, bool kInst>
void launch_shade_modes(int shader, int grid, cudaStream_t s, const PtParams& P, int cur, uint32_t b,
                        const uint32_t* q, int2 classes) {
    if constexpr (kModes != 3u) {
        if (shader == 1) {
            k_shade<kModes, kInst, 1><<<grid, kBlock, 0, s>>>(P, cur, b, q, classes);
            return;
        }
        if (shader == 2) {
            k_shade<kModes, kInst, 2><<<grid, kBlock, 0, s>>>(P, cur, b, q, classes);
            return;
        }
    }
    k_shade<kModes, kInst, -1><<<grid, kBlock, 0, s>>>(P, cur, b, q, classes);
}

void launch_shade(uint32_t modes, bool inst, int shader, int grid, cudaStream_t s, const PtParams& P, int cur,
                  uint32_t b, const uint32_t* q, int2 classes) {
    if (inst) {
        if (modes == 2u) launch_shade_modes<2, true>(shader, grid, s, P, cur, b, q, classes);
        else if (modes == 3u) launch_shade_modes<3, true>(shader, grid, s, P, cur, b, q, classes);
        else launch_shade_modes<1, true>(shader, grid, s, P, cur, b, q, classes);
    } else {
        if (modes == 2u) launch_shade_modes<2, false>(shader, grid, s, P, cur, b, q, classes);
        else if (modes == 3u) launch_shade_modes<3, false>(shader, grid, s, P, cur, b, q, classes);
        else launch_shade_modes<1, false>(shader, grid, s, P, cur, b, q, classes);
    }
}

cudaError_t pt_run_batches(int bvh_kind, uint32_t bounces, bool sort, const PtState& st, uint32_t* d_err,
                           uint64_t batches, cudaStream_t stream, GraphCache* graphs, int trace_block, uint32_t modes,
                           bool instanced, bool texture, bool ray_sort, uint64_t batch_paths, uint32_t shader_kinds,
                           bool quad_ptex) {
    const bool face_order = sort && texture && !instanced && batch_paths >= kFaceOrderPaths;
    // 256-thread traversal blocks for the 8-wide layout, flat (its 24-entry stacks fill 48 KB of static shared
    // memory) or instanced (40-entry stacks, 80 KB of dynamic shared memory); the binary layout's 64-entry
    // stacks stay at 128 threads
    const int tb = (trace_block == 256 && bvh_kind == 0) ? 256 : 128;
    constexpr size_t kInstStackBytes = trace_stack_bytes<2, 256>();
    if (instanced && tb == 256) {
        cudaError_t e = cudaFuncSetAttribute(k_extend<2, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(kInstStackBytes));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_shadow<2, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(kInstStackBytes));
        if (e != cudaSuccess) return e;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    PtParams P;
    std::memset(&P, 0, sizeof(P));
    P.st = st;
    P.err = d_err;
    const int trace_grid = grid_for(sms, 1024 / tb);
    const int shade_grid = grid_for(sms, 8);
    const int gen_grid = int((st.capacity + kBlock - 1) / kBlock);
    // the shading kernel (4 or 5 resident blocks per SM) runs one resident wave of grid-striding blocks, sized by
    // the occupancy calculator, as VCM's shading kernels do
    const void* shade_fn = instanced ? (modes == 2u ? reinterpret_cast<const void*>(&k_shade<2, true, -1>)
                                        : modes == 3u ? reinterpret_cast<const void*>(&k_shade<3, true, -1>)
                                                      : reinterpret_cast<const void*>(&k_shade<1, true, -1>))
                                     : (modes == 2u ? reinterpret_cast<const void*>(&k_shade<2, false, -1>)
                                        : modes == 3u ? reinterpret_cast<const void*>(&k_shade<3, false, -1>)
                                                      : reinterpret_cast<const void*>(&k_shade<1, false, -1>));
    // shading launches: one kernel for the jobs' single shader over the whole queue; with several shaders and the
    // class order, one per shader over its classes (1 + shader * 4 .. 4 + shader * 4; the misses, class 0, with
    // the thin shader's); else the kernel for every shader
    const uint32_t kinds = shader_kinds & 7u;
    const bool one_kind = kinds != 0u && (kinds & (kinds - 1u)) == 0u;
    const int single = one_kind ? __builtin_ctz(kinds) : -1;
    int shade_blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shade_blocks, shade_fn, kBlock, 0);
    const int wave_grid = sms * std::max(shade_blocks, 1);
    auto enqueue = [&](cudaStream_t s) {
        k_batch_begin<<<1, 32, 0, s>>>(P);
        k_generate<<<gen_grid, kBlock, 0, s>>>(P);
        for (uint32_t b = 0; b < bounces; ++b) {
            const int cur = int(b & 1u);
            k_bounce_reset<<<1, 32, 0, s>>>(st.counters, cur ^ 1);
            if (instanced && tb == 256) k_extend<2, 256><<<trace_grid, tb, kInstStackBytes, s>>>(P, cur);
            else if (instanced) k_extend<2, 128><<<trace_grid, tb, 0, s>>>(P, cur);
            else if (bvh_kind == 0 && tb == 256) k_extend<0, 256><<<trace_grid, tb, 0, s>>>(P, cur);
            else if (bvh_kind == 0) k_extend<0, 128><<<trace_grid, tb, 0, s>>>(P, cur);
            else k_extend<1, 128><<<trace_grid, tb, 0, s>>>(P, cur);
            if (face_order) {
                // textured scenes, large batches: order by (class, Ptex face, footprint region), three 8-bit
                // radix passes from the queue to queue_sorted (through rvals)
                if (one_kind) {
                    if (instanced) k_sort_keys<true, false><<<shade_grid, kBlock, 0, s>>>(P, cur);
                    else k_sort_keys<false, false><<<shade_grid, kBlock, 0, s>>>(P, cur);
                } else {
                    k_class_reset<<<1, 32, 0, s>>>(st.counters);
                    if (instanced) k_sort_keys<true, true><<<shade_grid, kBlock, 0, s>>>(P, cur);
                    else k_sort_keys<false, true><<<shade_grid, kBlock, 0, s>>>(P, cur);
                }
                const uint32_t ntiles = (st.capacity + kSortTile - 1) / kSortTile;
                uint32_t* kin = st.rkeys[0];
                uint32_t* kout = st.rkeys[1];
                const uint32_t* vin = st.queue[cur];
                for (int r = 0; r < 3; ++r) {
                    uint32_t* vout = (r & 1) ? st.rvals : st.queue_sorted;
                    k_radix_hist<<<ntiles, 256, 0, s>>>(kin, st.counters + cur, 8 * r, st.rhist, ntiles);
                    scan_exclusive(st.rhist, 256 * ntiles, st.rhist_off, st.rscan_tmp, s);
                    k_radix_scatter<<<ntiles, 256, 0, s>>>(kin, vin, kout, vout, st.counters + cur, 8 * r,
                                                           st.rhist_off, ntiles);
                    std::swap(kin, kout);
                    vin = vout;
                }
            } else if (sort) {
                k_class_reset<<<1, 32, 0, s>>>(st.counters);
                if (instanced) k_classify<true><<<shade_grid, kBlock, 0, s>>>(P, cur);
                else k_classify<false><<<shade_grid, kBlock, 0, s>>>(P, cur);
                k_class_offsets<<<1, 32, 0, s>>>(st.counters);
                k_class_scatter<<<shade_grid, kBlock, 0, s>>>(P, cur);
            }
            // Ptex base colours of the hits (the shading kernel reads them), in shading order
            const uint32_t* q = sort ? st.queue_sorted : st.queue[cur];
            if (texture && instanced && quad_ptex) k_texture<true, true><<<shade_grid, kBlock, 0, s>>>(P, cur, q);
            else if (texture && instanced) k_texture<true, false><<<shade_grid, kBlock, 0, s>>>(P, cur, q);
            else if (texture && quad_ptex) k_texture<false, true><<<shade_grid, kBlock, 0, s>>>(P, cur, q);
            else if (texture) k_texture<false, false><<<shade_grid, kBlock, 0, s>>>(P, cur, q);
            const int2 whole = make_int2(-1, -1);
            if (one_kind) {
                launch_shade(modes, instanced, single, wave_grid, s, P, cur, b, q, whole);
            } else if (sort) {
                launch_shade(modes, instanced, -1, wave_grid, s, P, cur, b, q, make_int2(0, 4));
                if (kinds & 2u) launch_shade(modes, instanced, 1, wave_grid, s, P, cur, b, q, make_int2(5, 8));
                if (kinds & 4u) launch_shade(modes, instanced, 2, wave_grid, s, P, cur, b, q, make_int2(9, 12));
            } else {
                launch_shade(modes, instanced, -1, wave_grid, s, P, cur, b, q, whole);
            }
            if (instanced && tb == 256) k_shadow<2, 256><<<trace_grid, tb, kInstStackBytes, s>>>(P);
            else if (instanced) k_shadow<2, 128><<<trace_grid, tb, 0, s>>>(P);
            else if (bvh_kind == 0 && tb == 256) k_shadow<0, 256><<<trace_grid, tb, 0, s>>>(P);
            else if (bvh_kind == 0) k_shadow<0, 128><<<trace_grid, tb, 0, s>>>(P);
            else k_shadow<1, 128><<<trace_grid, tb, 0, s>>>(P);
            if (ray_sort && b + 1 < bounces) {
                // order the next bounce's queue by (direction bin, origin cell): two 8-bit radix passes, the
                // queue ping-ponging through rvals
                const int next = cur ^ 1;
                k_ray_keys<<<shade_grid, kBlock, 0, s>>>(P, next);
                const uint32_t ntiles = (st.capacity + kSortTile - 1) / kSortTile;
                uint32_t* kin = st.rkeys[0];
                uint32_t* kout = st.rkeys[1];
                uint32_t* vin = st.queue[next];
                uint32_t* vout = st.rvals;
                for (int r = 0; r < 2; ++r) {
                    k_radix_hist<<<ntiles, 256, 0, s>>>(kin, st.counters + next, 8 * r, st.rhist, ntiles);
                    scan_exclusive(st.rhist, 256 * ntiles, st.rhist_off, st.rscan_tmp, s);
                    k_radix_scatter<<<ntiles, 256, 0, s>>>(kin, vin, kout, vout, st.counters + next, 8 * r,
                                                           st.rhist_off, ntiles);
                    std::swap(kin, kout);
                    std::swap(vin, vout);
                }
            }
        }
        k_batch_end<<<1, 32, 0, s>>>(P);
    };
    struct Key {
        PtParams P;
        int kind, sms;
        uint32_t bounces, sort;
        int tb;
        uint32_t modes, instanced, texture, ray_sort, face_order, kinds, quad_ptex;
    } key;
    std::memset(&key, 0, sizeof(key));
    std::memcpy(&key.P, &P, sizeof(P));
    key.kind = bvh_kind;
    key.sms = sms;
    key.bounces = bounces;
    key.sort = sort ? 1u : 0u;
    key.tb = tb;
    key.modes = modes;
    key.instanced = instanced ? 1u : 0u;
    key.texture = texture ? 1u : 0u;
    key.ray_sort = ray_sort ? 1u : 0u;
    key.face_order = face_order ? 1u : 0u;
    key.kinds = kinds;
    key.quad_ptex = quad_ptex ? 1u : 0u;
    return replay(graphs, &key, sizeof(key), stream, batches, enqueue);
}

cudaError_t pt_render(const PtScene& sc, const PtCamera& cam, const PtSettings& set, const PtState& st, double* d_accum,
                      uint32_t* d_err, cudaStream_t stream, GraphCache* graphs, int trace_block) {
    PtJob job;
    std::memset(&job, 0, sizeof(job));
    job.scene = sc;
    job.cam = cam;
    job.max_bounces = set.max_bounces;
    job.mode = set.mode;
    job.samples_per_axis = set.samples_per_axis;
    job.seed = set.seed;
    job.total = uint64_t(cam.width) * cam.height * set.spp;
    job.accum = d_accum;
    PtControl ctl;
    std::memset(&ctl, 0, sizeof(ctl));
    ctl.quota[0] = st.capacity;
    ctl.njobs = 1;
    cudaError_t e = cudaMemcpyAsync(st.jobs, &job, sizeof(job), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st.control, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    const uint64_t batches = (job.total + st.capacity - 1) / st.capacity;
    return pt_run_batches(sc.bvh_kind, set.max_bounces, sc.sort_hint != 0, st, d_err, batches, stream, graphs,
                          trace_block, set.mode == kPtModeDeferred ? 2u : 1u, sc.insts != nullptr,
                          pt_scene_textured(sc), sc.ray_sort != 0, std::min<uint64_t>(job.total, st.capacity),
                          sc.shader_kinds, sc.ptex_quads != 0);
}

cudaError_t pt_resolve(const double* d_accum, uint32_t values, double scale, float* d_out, cudaStream_t stream) {
    k_resolve<<<1024, 256, 0, stream>>>(d_accum, values, scale, d_out);
    return cudaGetLastError();
}

}  // namespace sel
