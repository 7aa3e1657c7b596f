// Render server: continuous batching of path-tracer and VCM jobs on one GPU (include/selas.h,
// sel_server_*).  No reference counterpart: the reference renders one hard-coded image per process
// (Source/Applications/Selas/Source/main.cpp:82-127).
//
// One worker thread per server runs rounds:
//   admit   pending jobs in arrival order while a job slot and the device-byte budget allow; a job's
//           accumulator (and VCM state) is allocated with the stream-ordered allocator, so admission and
//           retirement never synchronise the device;
//   PT      one batch of the shared path-tracer wavefront, filled shortest-remaining-work first and one scene
//           at a time (the job with the fewest paths left, the other jobs on its scene, then the rest); the
//           batch is a replayed CUDA graph, the job table and quotas go up from pinned buffers (two rounds in
//           flight);
//   VCM     one pass of every admitted VCM job on the job's own stream (at most two passes queued per job);
//           streams carry CUDA priorities, highest for the shared path-tracer batches and then by a VCM job's
//           work (pixels x passes, smaller first), so short jobs are not held behind long passes;
//   retire  jobs whose last work finished: resolve, copy the image to host memory, free the device memory.
// A path's random stream depends only on its job and index, so a job renders the same image alone and in
// any mix (up to the order of FP64 additions).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "capi_internal.h"
#include "pt.h"
#include "vcm.h"

using namespace sel;
using Clock = std::chrono::steady_clock;

namespace {

constexpr int kRing = 2;
constexpr uint32_t kMaxVcmPasses = 65536;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Job {
    uint64_t id = 0;
    SelJob desc{};
    enum State { kPending, kActive, kDone } state = kPending;
    int status = SEL_OK;
    Clock::time_point t_submit, t_admit, t_done;
    size_t values = 0;  // floats of the result
    size_t bytes = 0;   // device bytes held while admitted
    void* d_block = nullptr;
    double* accum = nullptr;
    float* resolved = nullptr;
    double scale = 1.0;
    std::vector<float> result;
    cudaEvent_t done_ev = nullptr;
    bool issued_all = false;
    cudaStream_t alloc_stream = nullptr;
    // path tracer
    int slot = -1;
    uint64_t total = 0, issued = 0;
    // VCM
    cudaStream_t stream = nullptr;
    VcmState vst{};
    VcmSettings vset{};
    VcmCamera vcam{};
    PtScene scene{};
    std::unique_ptr<GraphCache> graph;
    uint32_t passes = 0, passes_issued = 0;
    cudaEvent_t pass_ev[kRing] = {nullptr, nullptr};
};

size_t result_floats(const SelJob& j) {
    const size_t px = size_t(j.camera.width) * j.camera.height;
    return j.integrator == SEL_INTEGRATOR_PT ? 2 * px * 3 : px * 3;  // deferred and VCM: one layer
}

}  // namespace

struct SelServerTy {
    SelDeviceTy* dev = nullptr;
    SelServerConfig cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
    std::vector<Job*> active;
    uint64_t next_id = 1;
    bool stop = false;
    std::thread worker;
    // shared path-tracer wavefront
    void* pt_block = nullptr;
    PtState pst{};
    cudaStream_t pt_stream = nullptr, retire_stream = nullptr;
    GraphCache pt_graph;
    Job* slots[kMaxPtJobs] = {};
    PtJob* h_jobs = nullptr;     // pinned: kRing tables of kMaxPtJobs entries
    PtControl* h_ctl = nullptr;  // pinned: kRing control blocks
    cudaEvent_t pt_ev[kRing] = {};
    bool pt_ev_used[kRing] = {};
    uint64_t pt_rounds = 0;
    unsigned long long* h_rays = nullptr;  // pinned scratch for counter reads
    uint64_t vcm_rays = 0;
    uint64_t held_bytes = 0;
    int prio_least = 0, prio_greatest = 0;  // cudaDeviceGetStreamPriorityRange
    SelServerStats stats{};
};

namespace {

int worker_error(SelServerTy* S, Job* j, cudaError_t e) {
    (void)S;
    j->status = SEL_ERR_CUDA;
    return cuda_fail(e, "render server");
}

// Device bytes a job holds while admitted.
size_t job_bytes(const SelServerTy* S, const Job& j) {
    (void)S;
    const size_t acc = j.values * sizeof(double), res = j.values * sizeof(float);
    size_t b = ((acc + 255) & ~size_t(255)) + ((res + 255) & ~size_t(255));
    if (j.desc.integrator == SEL_INTEGRATOR_VCM)
        b += vcm_state_block_bytes(j.desc.camera.width * j.desc.camera.height, j.desc.vcm.maxPathLength, j.desc.vcm.passes);
    return b;
}

bool budget_allows(SelServerTy* S, size_t need) {
    if (S->cfg.hbm_budget_bytes) return S->held_bytes + need <= S->cfg.hbm_budget_bytes;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
    return need + S->cfg.hbm_reserve_bytes <= free_b;
}

// Allocates and initialises an admitted job's device state.  Called by the worker with S->mu held.
bool admit_one(SelServerTy* S, Job* j) {
    const SelJob& d = j->desc;
    int slot = -1;
    if (d.integrator != SEL_INTEGRATOR_VCM) {
        for (int k = 0; k < kMaxPtJobs; ++k)
            if (!S->slots[k]) { slot = k; break; }
        if (slot < 0) return false;
    }
    if (!budget_allows(S, j->bytes)) return false;
    cudaStream_t s = S->pt_stream;
    if (d.integrator == SEL_INTEGRATOR_VCM) {
        // priority by work: one level per factor 16 of pixels x passes above 2^20, the largest jobs lowest
        const double work = double(d.camera.width) * d.camera.height * d.vcm.passes;
        int level = 0;
        for (double w = work; w > double(1 << 20) && level < 8; w /= 16.0) ++level;
        int prio = S->prio_greatest + 1 + level;  // numerically larger = lower priority
        if (prio > S->prio_least) prio = S->prio_least;
        if (prio < S->prio_greatest) prio = S->prio_greatest;
        if (cudaStreamCreateWithPriority(&j->stream, cudaStreamNonBlocking, prio) != cudaSuccess) return false;
        s = j->stream;
    }
    j->alloc_stream = s;
    if (cudaMallocAsync(&j->d_block, j->bytes, s) != cudaSuccess) {
        cudaGetLastError();
        if (j->stream) cudaStreamDestroy(j->stream);
        j->stream = nullptr;
        j->d_block = nullptr;
        return false;
    }
    char* p = static_cast<char*>(j->d_block);
    j->accum = reinterpret_cast<double*>(p);
    p += (j->values * sizeof(double) + 255) & ~size_t(255);
    j->resolved = reinterpret_cast<float*>(p);
    p += (j->values * sizeof(float) + 255) & ~size_t(255);
    cudaMemsetAsync(j->accum, 0, j->values * sizeof(double), s);
    cudaEventCreateWithFlags(&j->done_ev, cudaEventDisableTiming);
    SelSceneTy* sc = d.scene;
    j->scene = scene_view(sc);
    if (d.integrator != SEL_INTEGRATOR_VCM) {
        j->slot = slot;
        S->slots[slot] = j;
        j->total = uint64_t(d.camera.width) * d.camera.height * d.pt.samplesPerPixel;
        j->issued = 0;
        j->scale = 1.0 / double(d.pt.samplesPerPixel);
    } else {
        const uint32_t paths = d.camera.width * d.camera.height;
        j->passes = d.vcm.passes;
        j->vst = vcm_state_carve(p, paths, d.vcm.maxPathLength, d.vcm.passes);
        init_camera(d.camera, j->vcam.cam);
        const float hlen = std::tan(d.camera.fovDegrees * (3.141592653589793f / 180.0f) * 0.5f);
        j->vcam.image_plane = float(d.camera.width) / (2.0f * hlen);
        j->vset.max_len = d.vcm.maxPathLength;
        j->vset.seed = d.vcm.seed;
        j->vset.merging = d.vcm.disableMerging ? 0 : 1;
        j->vset.trace_block = sc->tuned_trace_block;
        vcm_lights(sc, j->vset);
        const float r0 = d.vcm.radius != 0.0f ? d.vcm.radius : vcm_default_radius(sc);
        std::vector<VcmConsts> consts(d.vcm.passes);
        for (uint32_t k = 0; k < d.vcm.passes; ++k)
            vcm_constants(r0, d.vcm.radiusAlpha, paths, j->vset.merging != 0, d.vcm.firstPass + k, consts[k]);
        // pageable upload: the job's fresh stream has nothing queued but this job's set-up
        vcm_upload_constants(j->vst, consts.data(), d.vcm.passes, s);
        cudaMemsetAsync(j->vst.rays, 0, 2 * sizeof(unsigned long long), s);
        j->graph.reset(new GraphCache());
        for (auto& ev : j->pass_ev) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        j->scale = 1.0 / double(d.vcm.passes);
    }
    j->state = Job::kActive;
    j->t_admit = Clock::now();
    S->held_bytes += j->bytes;
    S->active.push_back(j);
    S->stats.peak_jobs = std::max<uint64_t>(S->stats.peak_jobs, S->active.size());
    S->stats.peak_bytes = std::max<uint64_t>(S->stats.peak_bytes, S->held_bytes);
    return true;
}

// Returns true when jobs finished without running (they can never be admitted).
bool admit(SelServerTy* S) {
    bool failed = false;
    while (!S->pending.empty() && S->active.size() < S->cfg.max_jobs) {
        Job* j = S->pending.front();
        if (!admit_one(S, j)) {
            // arrival order: the head waits for memory or a slot, unless nothing runs that could free any
            if (!S->active.empty()) break;
            j->status = SEL_ERR_OUT_OF_MEMORY;
            j->state = Job::kDone;
            j->t_admit = j->t_done = Clock::now();
            ++S->stats.completed;
            failed = true;
        }
        S->pending.pop_front();
    }
    return failed;
}

// One batch of the shared path-tracer wavefront.  Returns true when work was queued.
bool pt_round(SelServerTy* S) {
    int n = 0, njobs = 0;
    for (int k = 0; k < kMaxPtJobs; ++k) {
        Job* j = S->slots[k];
        if (j && j->issued < j->total) ++n;
        if (j) njobs = k + 1;
    }
    if (n == 0) return false;
    const int par = int(S->pt_rounds % kRing);
    if (S->pt_ev_used[par]) cudaEventSynchronize(S->pt_ev[par]);  // round k-2 done: its pinned buffers are free
    PtControl& c = S->h_ctl[par];
    std::memset(&c, 0, sizeof(c));
    PtJob* table = S->h_jobs + size_t(par) * kMaxPtJobs;
    // shortest remaining work first, one scene at a time: the batch takes the paths of the job with the
    // fewest left, then of the other jobs on the same scene, and only then fills up from other scenes,
    // so a batch's traversal mostly stays in one scene's BVH and textures
    std::vector<std::pair<uint64_t, int>> left;
    for (int k = 0; k < kMaxPtJobs; ++k) {
        Job* j = S->slots[k];
        if (j && j->issued < j->total) left.push_back({j->total - j->issued, k});
    }
    std::sort(left.begin(), left.end());
    uint64_t cap = S->pst.capacity;
    const SelSceneTy* lead = S->slots[left.front().second]->desc.scene;
    for (int pass = 0; pass < 2 && cap > 0; ++pass)
        for (const auto& lk : left) {
            const bool same = S->slots[lk.second]->desc.scene == lead;
            if ((pass == 0) != same || cap == 0) continue;
            const uint64_t q = std::min(lk.first, cap);
            c.quota[lk.second] = uint32_t(q);
            cap -= q;
        }
    c.njobs = uint32_t(njobs);
    uint32_t bounces = 1;
    for (int k = 0; k < kMaxPtJobs; ++k) {
        Job* j = S->slots[k];
        std::memset(&table[k], 0, sizeof(PtJob));
        if (!j) continue;
        c.next[k] = j->issued;
        PtJob& t = table[k];
        t.scene = j->scene;
        init_camera(j->desc.camera, t.cam);
        t.max_bounces = j->desc.pt.maxBounces;
        if (j->desc.integrator == SEL_INTEGRATOR_DEFERRED) {
            t.mode = kPtModeDeferred;
            t.samples_per_axis = deferred_axis(j->desc.pt);
        }
        t.seed = j->desc.pt.seed;
        bounces = std::max(bounces, t.max_bounces);
        t.total = j->total;
        t.accum = j->accum;
    }
    cudaMemcpyAsync(S->pst.jobs, table, sizeof(PtJob) * kMaxPtJobs, cudaMemcpyHostToDevice, S->pt_stream);
    cudaMemcpyAsync(S->pst.control, &c, sizeof(PtControl), cudaMemcpyHostToDevice, S->pt_stream);
    bool sort = false, instanced = false, texture = false, ray_sort = false, quad_ptex = false;
    uint32_t modes = 0, shader_kinds = 0;
    for (int k = 0; k < kMaxPtJobs; ++k)
        if (S->slots[k]) {
            sort |= S->slots[k]->scene.sort_hint != 0;
            instanced |= S->slots[k]->scene.insts != nullptr;
            texture |= pt_scene_textured(S->slots[k]->scene);
            ray_sort |= S->slots[k]->scene.ray_sort != 0;
            shader_kinds |= S->slots[k]->scene.shader_kinds;
            quad_ptex |= S->slots[k]->scene.ptex_quads != 0;
            modes |= S->slots[k]->desc.integrator == SEL_INTEGRATOR_DEFERRED ? 2u : 1u;
        }
    // rounds per batch: the largest maxBounces of the jobs in the slots (at most config.max_bounces)
    uint64_t batch_paths = 0;
    for (int k = 0; k < kMaxPtJobs; ++k) batch_paths += c.quota[k];
    cudaError_t e = pt_run_batches(0, bounces, sort, S->pst, S->dev->d_err, 1, S->pt_stream, &S->pt_graph, 128,
                                   modes, instanced, texture, ray_sort, batch_paths, shader_kinds, quad_ptex);
    for (int k = 0; k < kMaxPtJobs; ++k) {
        Job* j = S->slots[k];
        if (!j || c.quota[k] == 0) continue;
        j->issued += c.quota[k];
        if (e != cudaSuccess) j->status = SEL_ERR_CUDA;
        if (j->issued >= j->total && !j->issued_all) {
            cudaEventRecord(j->done_ev, S->pt_stream);
            j->issued_all = true;
        }
    }
    cudaEventRecord(S->pt_ev[par], S->pt_stream);
    S->pt_ev_used[par] = true;
    ++S->pt_rounds;
    return true;
}

// One pass of the admitted VCM jobs with the least work left (pixels x passes, shortest first) whose pixels
// together stay within the wavefront capacity, each only while it has fewer than kRing passes queued.  The
// job with the least work always advances; the others wait for the GPU the shorter jobs leave.
bool vcm_round(SelServerTy* S, const std::vector<Job*>& act) {
    std::vector<std::pair<double, Job*>> order;
    for (Job* j : act)
        if (j->desc.integrator == SEL_INTEGRATOR_VCM && j->passes_issued < j->passes)
            order.push_back({double(j->desc.camera.width) * j->desc.camera.height * (j->passes - j->passes_issued), j});
    std::sort(order.begin(), order.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    bool queued = false;
    uint64_t pixels = 0;
    for (size_t r = 0; r < order.size(); ++r) {
        Job* j = order[r].second;
        const uint64_t px = uint64_t(j->desc.camera.width) * j->desc.camera.height;
        if (r > 0 && pixels + px > S->cfg.paths_in_flight) break;
        pixels += px;
        const int par = int(j->passes_issued % kRing);
        if (j->passes_issued >= uint32_t(kRing) && cudaEventQuery(j->pass_ev[par]) == cudaErrorNotReady) continue;
        cudaError_t e = vcm_run_passes(j->scene, j->vcam, j->vset, 1, j->vst, j->accum, S->dev->d_err, j->stream,
                                       j->graph.get());
        if (e != cudaSuccess) j->status = SEL_ERR_CUDA;
        cudaEventRecord(j->pass_ev[par], j->stream);
        ++j->passes_issued;
        if (j->passes_issued == j->passes) {
            cudaEventRecord(j->done_ev, j->stream);
            j->issued_all = true;
        }
        queued = true;
    }
    return queued;
}

// Result to host memory, device memory back to the pool.  Called without S->mu.
void finish(SelServerTy* S, Job* j) {
    cudaStreamWaitEvent(S->retire_stream, j->done_ev, 0);
    cudaError_t e = pt_resolve(j->accum, uint32_t(j->values), j->scale, j->resolved, S->retire_stream);
    j->result.resize(j->values);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(j->result.data(), j->resolved, j->values * sizeof(float), cudaMemcpyDeviceToHost,
                            S->retire_stream);
    if (j->desc.integrator == SEL_INTEGRATOR_VCM && e == cudaSuccess)
        e = cudaMemcpyAsync(S->h_rays, j->vst.rays, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            S->retire_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S->retire_stream);
    if (e != cudaSuccess) worker_error(S, j, e);
    if (j->desc.integrator == SEL_INTEGRATOR_VCM) S->vcm_rays += S->h_rays[0] + S->h_rays[1];
    cudaFreeAsync(j->d_block, S->retire_stream);
    j->d_block = nullptr;
    if (j->stream) {
        cudaStreamSynchronize(j->stream);
        cudaStreamDestroy(j->stream);
        j->stream = nullptr;
    }
    for (auto& ev : j->pass_ev)
        if (ev) { cudaEventDestroy(ev); ev = nullptr; }
    cudaEventDestroy(j->done_ev);
    j->done_ev = nullptr;
    j->graph.reset();
}

void worker_main(SelServerTy* S) {
    cudaSetDevice(S->dev->cuda_device);
    for (;;) {
        std::vector<Job*> act;
        {
            std::unique_lock<std::mutex> lock(S->mu);
            if (admit(S)) S->cv_done.notify_all();
            if (S->active.empty()) {
                if (S->stop && S->pending.empty()) break;
                S->cv_work.wait_for(lock, std::chrono::milliseconds(50));
                continue;
            }
            act = S->active;
        }
        bool progressed = pt_round(S);
        progressed |= vcm_round(S, act);
        std::vector<Job*> done;
        for (Job* j : act)
            if (j->issued_all && cudaEventQuery(j->done_ev) == cudaSuccess) done.push_back(j);
        for (Job* j : done) {
            finish(S, j);
            std::lock_guard<std::mutex> lock(S->mu);
            if (j->slot >= 0) S->slots[j->slot] = nullptr;
            S->held_bytes -= j->bytes;
            S->active.erase(std::find(S->active.begin(), S->active.end(), j));
            j->state = Job::kDone;
            j->t_done = Clock::now();
            ++S->stats.completed;
            progressed = true;
        }
        if (!done.empty()) S->cv_done.notify_all();
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

}  // namespace

extern "C" {

int sel_server_config_defaults(SelServerConfig* out) {
    if (!out) return fail(SEL_ERR_INVALID_ARGUMENT, "out is null");
    std::memset(out, 0, sizeof(*out));
    out->hbm_reserve_bytes = uint64_t(2) << 30;
    out->max_jobs = kMaxPtJobs;
    out->paths_in_flight = 1u << 22;
    out->max_bounces = 8;
    return SEL_OK;
}

int sel_server_new(SelDevice device, const SelServerConfig* config, SelServer* out_server) {
    if (!device || !out_server) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    *out_server = nullptr;
    SelServerConfig cfg;
    sel_server_config_defaults(&cfg);
    if (config) cfg = *config;
    if (cfg.max_jobs == 0 || cfg.max_jobs > uint32_t(kMaxPtJobs))
        return fail(SEL_ERR_INVALID_ARGUMENT, "max_jobs must lie in 1..16");
    if (cfg.paths_in_flight == 0) cfg.paths_in_flight = 1u << 22;
    if (cfg.max_bounces == 0 || cfg.max_bounces > 64) return fail(SEL_ERR_INVALID_ARGUMENT, "max_bounces must lie in 1..64");
    if (int rc = set_device(device)) return rc;
    std::unique_ptr<SelServerTy> S(new SelServerTy());
    S->dev = device;
    S->cfg = cfg;
    cudaError_t e = cudaMalloc(&S->pt_block, pt_state_block_bytes(cfg.paths_in_flight));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(server path state)");
    S->pst = pt_state_carve(S->pt_block, cfg.paths_in_flight);
    e = cudaMemset(S->pst.rays, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&S->prio_least, &S->prio_greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&S->pt_stream, cudaStreamNonBlocking, S->prio_greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->retire_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_jobs, sizeof(PtJob) * kMaxPtJobs * kRing);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_ctl, sizeof(PtControl) * kRing);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_rays, 2 * sizeof(unsigned long long));
    for (int k = 0; e == cudaSuccess && k < kRing; ++k) e = cudaEventCreateWithFlags(&S->pt_ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaFree(S->pt_block);
        return cuda_fail(e, "render server set-up");
    }
    SelServerTy* raw = S.release();
    raw->worker = std::thread(worker_main, raw);
    *out_server = raw;
    return SEL_OK;
}

int sel_server_result_floats(const SelJob* job, size_t* out_floats) {
    if (!job || !out_floats) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    *out_floats = result_floats(*job);
    return SEL_OK;
}

int sel_server_submit(SelServer server, const SelJob* job, uint64_t* out_job_id) {
    if (!server || !job || !out_job_id) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    SelSceneTy* sc = job->scene;
    if (job->integrator == SEL_INTEGRATOR_PT || job->integrator == SEL_INTEGRATOR_DEFERRED) {
        if (int rc = job->integrator == SEL_INTEGRATOR_PT ? check_render_args(sc, &job->camera, &job->pt)
                                                          : check_deferred_args(sc, &job->camera, &job->pt))
            return rc;
        if (sc->info.bvh_kind != SEL_BVH_WIDE8_Q8)
            return fail(SEL_ERR_INVALID_OPERATION, "served path-tracer jobs need SEL_BVH_WIDE8_Q8 scenes");
        if (job->pt.maxBounces == 0 || job->pt.maxBounces > server->cfg.max_bounces)
            return fail(SEL_ERR_INVALID_ARGUMENT, "maxBounces must lie in 1..config.max_bounces");
    } else if (job->integrator == SEL_INTEGRATOR_VCM) {
        if (int rc = check_vcm_args(sc, &job->camera, &job->vcm)) return rc;
        if (job->vcm.passes > kMaxVcmPasses) return fail(SEL_ERR_INVALID_ARGUMENT, "served VCM jobs take at most 65536 passes");
    } else {
        return fail(SEL_ERR_INVALID_ARGUMENT, "unknown integrator");
    }
    {
        std::lock_guard<std::mutex> lock(sc->mu);
        if (int rc = set_device(sc->dev)) return rc;
        if (int rc = sync_shading(sc)) return rc;
        if (job->integrator == SEL_INTEGRATOR_VCM)
            if (int rc = check_vcm_materials(sc)) return rc;
    }
    std::unique_ptr<Job> j(new Job());
    j->desc = *job;
    j->values = result_floats(*job);
    j->bytes = job_bytes(server, *j);
    j->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lock(server->mu);
        if (server->stop) return fail(SEL_ERR_INVALID_OPERATION, "server is stopping");
        j->id = server->next_id++;
        *out_job_id = j->id;
        server->pending.push_back(j.get());
        server->jobs[j->id] = std::move(j);
        ++server->stats.submitted;
    }
    server->cv_work.notify_one();
    return SEL_OK;
}

int sel_server_poll(SelServer server, uint64_t job_id, int* out_done) {
    if (!server || !out_done) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(server->mu);
    auto it = server->jobs.find(job_id);
    if (it == server->jobs.end()) return fail(SEL_ERR_INVALID_ARGUMENT, "unknown job id");
    *out_done = it->second->state == Job::kDone ? 1 : 0;
    return SEL_OK;
}

int sel_server_wait(SelServer server, uint64_t job_id, float* out, size_t out_floats, SelJobStats* stats) {
    if (!server) return fail(SEL_ERR_INVALID_ARGUMENT, "server is null");
    std::unique_ptr<Job> j;
    {
        std::unique_lock<std::mutex> lock(server->mu);
        auto it = server->jobs.find(job_id);
        if (it == server->jobs.end()) return fail(SEL_ERR_INVALID_ARGUMENT, "unknown job id");
        Job* raw = it->second.get();
        if (out && out_floats < raw->values) return fail(SEL_ERR_INVALID_ARGUMENT, "out is smaller than the result");
        server->cv_done.wait(lock, [&] { return raw->state == Job::kDone; });
        j = std::move(it->second);
        server->jobs.erase(it);
    }
    if (out) {
        if (j->status == SEL_OK && j->result.size() == j->values)
            std::memcpy(out, j->result.data(), j->values * sizeof(float));
        else
            std::memset(out, 0, j->values * sizeof(float));
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->queue_ms = ms_between(j->t_submit, j->t_admit);
        stats->run_ms = ms_between(j->t_admit, j->t_done);
        stats->latency_ms = ms_between(j->t_submit, j->t_done);
        stats->device_bytes = j->bytes;
        stats->status = j->status;
    }
    if (j->status != SEL_OK)
        return fail(j->status, j->status == SEL_ERR_OUT_OF_MEMORY ? "render job does not fit the device-byte budget"
                                                                   : "render job failed");
    return SEL_OK;
}

int sel_server_stats(SelServer server, SelServerStats* out) {
    if (!server || !out) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    if (int rc = set_device(server->dev)) return rc;
    unsigned long long pt_rays[2] = {0, 0};
    cudaError_t e = cudaMemcpyAsync(pt_rays, server->pst.rays, sizeof(pt_rays), cudaMemcpyDeviceToHost,
                                    server->retire_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(server->retire_stream);
    if (e != cudaSuccess) return cuda_fail(e, "server statistics");
    std::lock_guard<std::mutex> lock(server->mu);
    *out = server->stats;
    out->rays = pt_rays[0] + pt_rays[1] + server->vcm_rays;
    out->graph_captures = server->pt_graph.captures;
    return SEL_OK;
}

int sel_server_release(SelServer server) {
    if (!server) return fail(SEL_ERR_INVALID_ARGUMENT, "server is null");
    {
        std::lock_guard<std::mutex> lock(server->mu);
        server->stop = true;
    }
    server->cv_work.notify_all();
    if (server->worker.joinable()) server->worker.join();
    set_device(server->dev);
    cudaStreamSynchronize(server->pt_stream);
    cudaStreamSynchronize(server->retire_stream);
    server->pt_graph.reset();
    for (auto& ev : server->pt_ev)
        if (ev) cudaEventDestroy(ev);
    cudaStreamDestroy(server->pt_stream);
    cudaStreamDestroy(server->retire_stream);
    cudaFree(server->pt_block);
    cudaFreeHost(server->h_jobs);
    cudaFreeHost(server->h_ctl);
    cudaFreeHost(server->h_rays);
    delete server;
    return SEL_OK;
}

}  // extern "C"
