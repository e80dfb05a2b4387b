// Host side of the wavefront engine: the wave buffers, the resident scene
// table, job staging and CUDA-graph replay; the renderer's wavefront mode,
// the batch API and the request server are built on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "device_guard.cuh"
#include "engine.h"
#include "internal.h"
#include "kernels.h"

namespace cvx {

static int32_t cuda_err(cudaError_t e, const char* what) {
    return set_error(CVX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define ECK(call, what)                                     \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_err(e_, what);   \
    } while (0)

template <class T>
static int32_t alloc(T** p, size_t n, std::vector<void*>& owned) {
    *p = nullptr;
    if (injected_allocation_failure())
        return set_error(CVX_ERR_CAPACITY, "cudaMalloc for the wave buffers: out of memory (injected)");
    cudaError_t e = cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(e == cudaErrorMemoryAllocation ? CVX_ERR_CAPACITY : CVX_ERR_CUDA,
                         std::string("cudaMalloc for the wave buffers: ") + cudaGetErrorString(e));
    }
    owned.push_back(*p);
    return CVX_OK;
}

uint32_t groups_of(uint32_t w, uint32_t h) { return 8u * ((w + 15u) / 16u) * ((h + 3u) / 4u); }

WaveEngine::~WaveEngine() {
    for (auto& g : graphs_) cudaGraphExecDestroy(g.exec);
    for (void* p : owned_) cudaFree(p);
    if (h_jobs_) cudaFreeHost(h_jobs_);
    if (h_hdr_) cudaFreeHost(h_hdr_);
    if (h_read_) cudaFreeHost(h_read_);
    if (h_job_rays_) cudaFreeHost(h_job_rays_);
    if (e0_) cudaEventDestroy(e0_);
    if (e1_) cudaEventDestroy(e1_);
}

int32_t WaveEngine::init(uint32_t max_groups, uint32_t max_jobs, bool packet, bool use_graph,
                         uint32_t blocks_per_sm, uint32_t refill_mode, bool fused) {
    refill_mode_ = refill_mode;
    refill_from_ = refill_from(refill_mode);
    max_groups_ = max_groups;
    max_jobs_ = max_jobs;
    packet_ = packet;
    use_graph_ = use_graph;
    blocks_per_sm_ = blocks_per_sm;
    fused_ = fused;
    int32_t st = 0;
    if (!fused) {  // the fused kernel keeps a path's state in registers: no ray queues
        size_t L = (size_t)max_groups * 8;
        float** f[] = {&st_.ox, &st_.oy, &st_.oz, &st_.dx, &st_.dy, &st_.dz, &st_.cr, &st_.cg, &st_.cb,
                       &st_.ht, &st_.hu, &st_.hv};
        for (float** p : f)
            if ((st = alloc(p, L, owned_))) return st;
        if ((st = alloc(&st_.rng, L, owned_))) return st;
        if ((st = alloc(&st_.gbuf, L, owned_))) return st;
        if ((st = alloc(&st_.flags, L, owned_))) return st;
        if ((st = alloc(&st_.htri, L, owned_))) return st;
        if ((st = alloc(&st_.group_job, max_groups, owned_))) return st;
        if ((st = alloc(&st_.queue[0], max_groups, owned_))) return st;
        if ((st = alloc(&st_.queue[1], max_groups, owned_))) return st;
        if ((st = alloc(&st_.counts, 16, owned_))) return st;
    }
    if ((st = alloc(&d_jobs_, max_jobs, owned_))) return st;
    if ((st = alloc(&d_hdr_, 1, owned_))) return st;
    if ((st = alloc(&d_rays_, 1, owned_))) return st;
    if ((st = alloc(&d_job_rays_, max_jobs, owned_))) return st;
    if ((st = alloc(&d_err_, 2, owned_))) return st;  // [0] status, [1] group counter of the fused kernel
    ECK(cudaMallocHost((void**)&h_jobs_, max_jobs * sizeof(Job)), "pinned job staging");
    ECK(cudaMallocHost((void**)&h_hdr_, sizeof(WaveHeader)), "pinned job staging");
    ECK(cudaMallocHost((void**)&h_read_, sizeof(Readback)), "pinned readback");
    ECK(cudaMallocHost((void**)&h_job_rays_, max_jobs * sizeof(unsigned long long)), "pinned readback");
    ECK(cudaEventCreate(&e0_), "cudaEventCreate");
    ECK(cudaEventCreate(&e1_), "cudaEventCreate");
    return CVX_OK;
}

int32_t WaveEngine::set_scenes(cvx_scene* const* scenes, uint32_t n) {
    std::vector<DeviceScene> v(n);
    for (uint32_t i = 0; i < n; i++) v[i] = scene_view(scenes[i]);
    if (n > scene_cap_) {
        if (d_scenes_) {
            cudaFree(d_scenes_);
            owned_.erase(std::remove(owned_.begin(), owned_.end(), (void*)d_scenes_), owned_.end());
        }
        int32_t st = alloc(&d_scenes_, n, owned_);
        if (st) return st;
        scene_cap_ = n;
        for (auto& g : graphs_) cudaGraphExecDestroy(g.exec);
        graphs_.clear();
    }
    ECK(cudaMemcpy(d_scenes_, v.data(), n * sizeof(DeviceScene), cudaMemcpyHostToDevice), "upload scene table");
    n_scenes_ = n;
    scene_depth_.resize(n);
    for (uint32_t i = 0; i < n; i++) scene_depth_[i] = v[i].depth;
    return CVX_OK;
}

static bool same_out(const WaveOutputs& a, const WaveOutputs& b) { return std::memcmp(&a, &b, sizeof a) == 0; }

static cudaError_t launch_any(bool fused, const Job* jobs, const WaveHeader* hdr, const DeviceScene* scenes,
                              const WaveState& st, const WaveOutputs& out, bool packet, uint32_t bps,
                              uint32_t refill_from, bool deep, cudaStream_t stream) {
    return fused ? launch_wave_fused(jobs, hdr, scenes, out, packet, bps, deep, stream)
                 : launch_wave(jobs, hdr, scenes, st, out, packet, bps, refill_from, deep, stream);
}

// deep: a scene of this wave is deeper than 40 levels (the traversal's claim
// threshold; captured graphs are kept per value).
int32_t WaveEngine::launch(const WaveOutputs& out, bool deep, cudaStream_t stream) {
    if (!use_graph_) {
        ECK(launch_any(fused_, d_jobs_, d_hdr_, d_scenes_, st_, out, packet_, blocks_per_sm_, refill_from_, deep, stream),
            "wave launch");
        return CVX_OK;
    }
    for (auto& g : graphs_)
        if (same_out(g.out, out) && g.deep == deep) {
            ECK(cudaGraphLaunch(g.exec, stream), "graph launch");
            return CVX_OK;
        }
    cudaGraph_t graph;
    ECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t e =
        launch_any(fused_, d_jobs_, d_hdr_, d_scenes_, st_, out, packet_, blocks_per_sm_, refill_from_, deep, stream);
    cudaError_t e2 = cudaStreamEndCapture(stream, &graph);
    if (e != cudaSuccess) return cuda_err(e, "capture wave");
    if (e2 != cudaSuccess) return cuda_err(e2, "end capture");
    cudaGraphExec_t exec;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_err(e, "instantiate graph");
    if (graphs_.size() >= 4) {
        cudaGraphExecDestroy(graphs_.front().exec);
        graphs_.erase(graphs_.begin());
    }
    graphs_.push_back(Graph{out, deep, exec});
    ECK(cudaGraphLaunch(exec, stream), "graph launch");
    return CVX_OK;
}

int32_t WaveEngine::submit(const std::vector<Job>& jobs_in, WaveOutputs out, cudaStream_t stream,
                           bool want_job_rays) {
    last_jobs_ = 0;
    last_want_ = want_job_rays;
    if (jobs_in.size() > max_jobs_) return set_error(CVX_ERR_CAPACITY, "too many jobs for one wave");
    uint64_t total = 0, deep_total = 0;
    uint32_t depth = 0;
    for (size_t i = 0; i < jobs_in.size(); i++) {
        Job j = jobs_in[i];
        if (j.scene >= n_scenes_) return set_error(CVX_ERR_INVALID, "job scene outside the scene table");
        if (j.w == 0 || j.h == 0 || j.w > kMaxImageSide || j.h > kMaxImageSide)
            return set_error(CVX_ERR_INVALID, "job image size out of range");
        const uint32_t dj = scene_depth_[j.scene];
        depth = dj > depth ? dj : depth;
        j.n_groups = groups_of(j.w, j.h);
        if (dj >= kRefillMinDepth) deep_total += j.n_groups;
        if (total + j.n_groups > max_groups_) return set_error(CVX_ERR_CAPACITY, "wave exceeds the ray-queue capacity");
        j.group_base = (uint32_t)total;
        total += j.n_groups;
        h_jobs_[i] = j;
    }
    const uint32_t groups = (uint32_t)total, deep_groups = (uint32_t)deep_total;
    h_hdr_->n_jobs = (uint32_t)jobs_in.size();
    h_hdr_->n_groups = groups;
    if (jobs_in.empty()) return CVX_OK;
    last_jobs_ = (uint32_t)jobs_in.size();
    out.rays = d_rays_;
    out.job_rays = want_job_rays ? d_job_rays_ : nullptr;
    out.err = d_err_;
    const bool deep = depth > 40;
    // Single-ray fused waves that take paths per lane (path_refill_wave):
    // one counter word per group of the wave, grown on demand, zeroed per wave.
    // (Waves of kMaxRefillGroups groups or more keep the octet form.)
    out.group_em = nullptr;
    if (fused_ && !packet_ && groups < kMaxRefillGroups && path_refill_wave(refill_mode_, deep_groups, groups)) {
        if (groups > group_em_cap_) {
            uint64_t twice = 2ull * group_em_cap_;
            uint32_t cap = (uint64_t)groups > twice ? groups : (uint32_t)(twice < kMaxRefillGroups ? twice : kMaxRefillGroups);
            if (d_group_em_) {
                cudaFree(d_group_em_);
                owned_.erase(std::remove(owned_.begin(), owned_.end(), (void*)d_group_em_), owned_.end());
                d_group_em_ = nullptr;
                group_em_cap_ = 0;
            }
            int32_t st = alloc(&d_group_em_, cap, owned_);
            if (st) return st;
            group_em_cap_ = cap;
        }
        out.group_em = d_group_em_;
        ECK(cudaMemsetAsync(d_group_em_, 0, (size_t)groups * 4, stream), "reset group counters");
    }
    if (out.samples && !out.group_em) return set_error(CVX_ERR_INVALID, "sample slots need a path-refill wave");
    ECK(cudaMemcpyAsync(d_jobs_, h_jobs_, jobs_in.size() * sizeof(Job), cudaMemcpyHostToDevice, stream),
        "upload jobs");
    ECK(cudaMemcpyAsync(d_hdr_, h_hdr_, sizeof(WaveHeader), cudaMemcpyHostToDevice, stream), "upload jobs");
    ECK(cudaMemsetAsync(d_rays_, 0, 8, stream), "reset counters");
    ECK(cudaMemsetAsync(d_err_, 0, 8, stream), "reset status");
    if (want_job_rays) ECK(cudaMemsetAsync(d_job_rays_, 0, jobs_in.size() * 8, stream), "reset counters");
    ECK(cudaEventRecord(e0_, stream), "event");
    int32_t st = launch(out, deep, stream);
    if (st) return st;
    ECK(cudaEventRecord(e1_, stream), "event");
    ECK(cudaMemcpyAsync(&h_read_->rays, d_rays_, 8, cudaMemcpyDeviceToHost, stream), "read counters");
    ECK(cudaMemcpyAsync(&h_read_->err, d_err_, 4, cudaMemcpyDeviceToHost, stream), "read status");
    if (want_job_rays)
        ECK(cudaMemcpyAsync(h_job_rays_, d_job_rays_, jobs_in.size() * 8, cudaMemcpyDeviceToHost, stream),
            "read counters");
    return CVX_OK;
}

int32_t WaveEngine::collect(cudaStream_t stream, uint64_t* rays, std::vector<uint64_t>* job_rays, float* ms) {
    if (last_jobs_ == 0) {
        if (rays) *rays = 0;
        if (ms) *ms = 0.0f;
        if (job_rays) job_rays->clear();
        return CVX_OK;
    }
    ECK(cudaStreamSynchronize(stream), "wave");
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0_, e1_);
    if (ms) *ms = t;
    if (rays) *rays = h_read_->rays;
    if (job_rays) job_rays->assign(h_job_rays_, h_job_rays_ + (last_want_ ? last_jobs_ : 0));
    if (job_rays && !last_want_) job_rays->assign(last_jobs_, 0);
    if (h_read_->err) return set_error(CVX_ERR_DEVICE, "traversal stack overflow reported by the kernel");
    return CVX_OK;
}

int32_t WaveEngine::run(const std::vector<Job>& jobs, WaveOutputs out, cudaStream_t stream, uint64_t* rays,
                        std::vector<uint64_t>* job_rays, float* ms) {
    int32_t st = submit(jobs, out, stream, job_rays != nullptr);
    if (st) return st;
    return collect(stream, rays, job_rays, ms);
}

}  // namespace cvx

using namespace cvx;

// ---------------------------------------------------------------------------
// Batch API

// Kernel organisation of a scene in batches and in the server: the fused
// kernel for shallow BVHs, the wavefront form (ray refill) for deep or large
// ones, where long traversals benefit most from refill.
static uint32_t default_scene_mode(const cvx_scene* s) {
    DeviceScene v = scene_view(s);
    return (scene_depth(s) > 40 || v.n_tris > 200000) ? 1u : 0u;
}

// The device of a batch's or server's scenes, which must all be on one.
static int32_t common_device(cvx_scene* const* scenes, uint32_t n, int* dev) {
    *dev = scene_device(scenes[0]);
    for (uint32_t i = 1; i < n; i++)
        if (scene_device(scenes[i]) != *dev)
            return set_error(CVX_ERR_INVALID, "the scenes of a batch or server must be on one device");
    return CVX_OK;
}

struct cvx_batch {
    int device = 0;  // its scenes'
    std::vector<cvx_scene*> scenes;
    std::vector<uint32_t> mode;  // per scene: 0 fused, 1 wavefront
    WaveEngine engine;           // wavefront
    WaveEngine fused;
    cudaStream_t stream2 = nullptr;
    uint64_t max_pixels = 0;
    float* d_accum = nullptr;
    uint32_t* d_rgba = nullptr;
    ResolveItem* d_items = nullptr;
    uint32_t max_items = 0;
    cudaStream_t stream = nullptr;
    ~cvx_batch() {
        cudaFree(d_accum);
        cudaFree(d_rgba);
        cudaFree(d_items);
        if (stream) cudaStreamDestroy(stream);
        if (stream2) cudaStreamDestroy(stream2);
    }
};

extern "C" int32_t cvx_batch_create(cvx_scene* const* scenes, uint32_t n_scenes, uint32_t max_groups,
                                    uint64_t max_pixels, const cvx_render_config* cfg, cvx_batch** out) {
    if (!scenes || !n_scenes || !out || !max_groups || !max_pixels)
        return set_error(CVX_ERR_INVALID, "bad batch arguments");
    cvx_render_config c{};
    if (cfg) c = *cfg;
    for (uint32_t i = 0; i < n_scenes; i++)
        if (!scenes[i] || scene_num_lights(scenes[i]) == 0)
            return set_error(CVX_ERR_INVALID, "every batch scene needs a direct-sample triangle");
    int dev = 0;
    int32_t st = common_device(scenes, n_scenes, &dev);
    if (st) return st;
    CVX_ON_DEVICE(dev);
    std::unique_ptr<cvx_batch> b(new cvx_batch());
    b->device = dev;
    b->scenes.assign(scenes, scenes + n_scenes);
    b->max_pixels = max_pixels;
    ECK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    ECK(cudaStreamCreateWithFlags(&b->stream2, cudaStreamNonBlocking), "cudaStreamCreate");
    st = b->engine.init(max_groups, 4096, c.traversal == CVX_TRAVERSE_PACKET, c.use_graph != 0,
                                c.blocks_per_sm, c.refill_mode);
    if (st) return st;
    if ((st = b->fused.init(0xffffffffu, 4096, c.traversal == CVX_TRAVERSE_PACKET, c.use_graph != 0, 0,
                            c.refill_mode, true)))
        return st;
    if ((st = b->engine.set_scenes(scenes, n_scenes))) return st;
    if ((st = b->fused.set_scenes(scenes, n_scenes))) return st;
    for (uint32_t i = 0; i < n_scenes; i++)
        b->mode.push_back(c.mode == CVX_MODE_WAVEFRONT ? 1u : c.mode == CVX_MODE_MEGAKERNEL ? 0u
                                                                                         : default_scene_mode(scenes[i]));
    std::vector<void*> owned;
    if ((st = alloc(&b->d_accum, max_pixels * 3, owned))) return st;
    if ((st = alloc(&b->d_rgba, max_pixels, owned))) return st;
    b->max_items = 4096;
    if ((st = alloc(&b->d_items, b->max_items, owned))) return st;
    *out = b.release();
    return CVX_OK;
}

extern "C" int32_t cvx_batch_render(cvx_batch* b, const cvx_view* views, uint32_t n, uint32_t* const* rgba,
                                    uint64_t* rays_out, float* ms_out) {
    if (!b || (!views && n)) return set_error(CVX_ERR_INVALID, "null argument");
    CVX_ON_DEVICE(b->device);
    if (n > b->max_items) return set_error(CVX_ERR_CAPACITY, "too many views in one batch call");
    std::vector<uint64_t> offset(n);
    uint64_t total = 0;
    uint32_t max_spp = 0;
    for (uint32_t i = 0; i < n; i++) {
        const cvx_view& v = views[i];
        if (v.scene >= b->scenes.size() || v.width == 0 || v.height == 0 || v.spp == 0 ||
            v.width > kMaxImageSide || v.height > kMaxImageSide)
            return set_error(CVX_ERR_INVALID, "bad view");
        if (b->mode[v.scene] == 1 && groups_of(v.width, v.height) > b->engine.max_groups())
            return set_error(CVX_ERR_CAPACITY, "a view is larger than the ray-queue capacity");
        offset[i] = total;
        total += (uint64_t)v.width * v.height;
        max_spp = std::max(max_spp, v.spp);
    }
    if (total > b->max_pixels) return set_error(CVX_ERR_CAPACITY, "views exceed the batch framebuffer");
    StreamSync sync(b->stream, b->stream2);
    ECK(cudaMemsetAsync(b->d_accum, 0, total * 12, b->stream), "clear accumulator");
    uint64_t rays = 0;
    float ms = 0.0f;
    WaveOutputs out{};
    out.accum = b->d_accum;
    // Sample s of every view goes into wave s; a wave's jobs are split by
    // their scene's kernel organisation, and the two halves run concurrently
    // (disjoint pixels) on two streams. A wave larger than the ray-queue
    // capacity is split into several.
    for (uint32_t s = 0; s < max_spp; s++) {
        std::vector<Job> jobs[2];
        uint32_t groups = 0;
        auto flush = [&]() -> int32_t {
            uint64_t r[2] = {0, 0};
            float t[2] = {0.0f, 0.0f};
            int32_t st = b->fused.submit(jobs[0], out, b->stream2, false);
            if (!st) st = b->engine.submit(jobs[1], out, b->stream, false);
            int32_t st0 = b->fused.collect(b->stream2, &r[0], nullptr, &t[0]);
            int32_t st1 = b->engine.collect(b->stream, &r[1], nullptr, &t[1]);
            rays += r[0] + r[1];
            ms += t[0] > t[1] ? t[0] : t[1];
            jobs[0].clear();
            jobs[1].clear();
            groups = 0;
            return st ? st : (st0 ? st0 : st1);
        };
        for (uint32_t i = 0; i < n; i++) {
            const cvx_view& v = views[i];
            if (v.spp <= s) continue;
            uint32_t m = b->mode[v.scene];
            uint32_t g = groups_of(v.width, v.height);
            if ((m == 1 && groups + g > b->engine.max_groups()) || jobs[m].size() == b->engine.max_jobs()) {
                int32_t st = flush();
                if (st) return st;
            }
            Job j{};
            std::memcpy(&j.cam, &v.camera, sizeof(cvx_camera));
            j.scene = v.scene;
            j.w = v.width;
            j.h = v.height;
            j.frame = v.frame_base + s;
            j.out_offset = offset[i];
            jobs[m].push_back(j);
            if (m == 1) groups += g;
        }
        if (!jobs[0].empty() || !jobs[1].empty()) {
            int32_t st = flush();
            if (st) return st;
        }
    }
    std::vector<ResolveItem> items(n);
    for (uint32_t i = 0; i < n; i++)
        items[i] = ResolveItem{offset[i], views[i].width * views[i].height, 1.0f / (float)views[i].spp};
    ECK(cudaMemcpyAsync(b->d_items, items.data(), n * sizeof(ResolveItem), cudaMemcpyHostToDevice, b->stream),
        "upload resolve list");
    ECK(launch_resolve_multi(b->d_items, n, b->d_accum, b->d_rgba, b->stream), "resolve");
    if (rgba)
        for (uint32_t i = 0; i < n; i++)
            if (rgba[i])
                ECK(cudaMemcpyAsync(rgba[i], b->d_rgba + offset[i], (size_t)items[i].npx * 4, cudaMemcpyDeviceToHost,
                                    b->stream),
                    "copy image");
    ECK(cudaStreamSynchronize(b->stream), "batch");
    if (rays_out) *rays_out = rays;
    if (ms_out) *ms_out = ms;
    return CVX_OK;
}

extern "C" int32_t cvx_batch_set_scene_mode(cvx_batch* b, uint32_t scene, uint32_t mode) {
    if (!b || scene >= b->scenes.size() || mode > 1) return set_error(CVX_ERR_INVALID, "bad scene mode");
    b->mode[scene] = mode;
    return CVX_OK;
}

extern "C" void cvx_batch_destroy(cvx_batch* b) {
    if (!b) return;
    DeviceGuard g(b->device);
    delete b;
}

// ---------------------------------------------------------------------------
// Request server

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id = 0;
    cvx_request r{};
    uint32_t* host_rgba = nullptr;
    uint64_t npx = 0;
    uint32_t groups = 0;
    uint64_t offset = 0;  // pixel offset in the framebuffer pool
    uint32_t next_sample = 0;
    uint32_t wave_k = 1, wave_job = 0;  // samples in its current wave, and the first one's job index
    int eng = -1;            // engine it is rendered on: 0 single-launch, 1 and 2 wavefront
    bool in_flight = false;  // a sample of it is on the GPU
    bool admitted = false, finished = false, cancelled = false;
    cvx_request_result res{};
};

// First-fit allocator over pixel ranges of the framebuffer pool.
struct RangeAlloc {
    std::map<uint64_t, uint64_t> free_;  // offset -> length
    void init(uint64_t n) { free_ = {{0, n}}; }
    bool take(uint64_t n, uint64_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= n) {
                *off = it->first;
                uint64_t rest = it->second - n, at = it->first + n;
                free_.erase(it);
                if (rest) free_[at] = rest;
                return true;
            }
        return false;
    }
    void give(uint64_t off, uint64_t n) {
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

}  // namespace

struct cvx_server {
    int device = 0;  // its scenes'; the worker thread selects it
    std::vector<cvx_scene*> scenes;
    std::vector<uint32_t> mode;  // per scene: 0 fused, 1 wavefront
    cvx_server_config cfg{};
    WaveEngine engine;  // wavefront
    // further wavefront engines (wavefront_streams > 1): their waves fill the
    // first one's bounce tails
    static constexpr int kMaxEngines = 5;  // the single-launch engine and up to 4 wavefront engines
    WaveEngine extra_wf[kMaxEngines - 2];
    cudaStream_t extra_stream[kMaxEngines - 2] = {nullptr, nullptr, nullptr};
    int n_wf = 1;
    WaveEngine fused;
    cudaStream_t stream2 = nullptr;
    float* d_accum = nullptr;
    uint32_t* d_rgba = nullptr;
    ResolveItem* d_items = nullptr;
    // cfg.samples_per_wave > 1: colour slots of the samples after a request's
    // first in a wave, one region of slot_region_px pixels per engine (an
    // engine has one wave on the GPU at a time), and their reduction lists
    float* d_samples = nullptr;
    uint64_t slot_region_px = 0;
    SlotItem* d_slot_items = nullptr;
    uint64_t pool_px = 0;
    RangeAlloc pool;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::condition_variable cv, done_cv;
    std::deque<std::shared_ptr<Request>> pending;
    std::vector<std::shared_ptr<Request>> admitted;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> all;
    uint64_t next_id = 1;
    uint32_t eng_groups[kMaxEngines] = {};  // ray-queue groups admitted per engine
    uint32_t eng_jobs[kMaxEngines] = {};
    uint64_t admitted_px = 0;  // pixels of the admitted requests (cfg.max_inflight_pixels)
    uint64_t arrivals = 0;  // bumped by submissions, cancellations and finished waves
    bool stop = false;
    std::thread worker;
    Clock::time_point t0 = Clock::now();
    std::atomic<uint64_t> waves{0}, rays{0};
    double busy_s = 0.0;
    double busy_fused_s = 0.0, busy_wavefront_s = 0.0;  // per engine (the two overlap)
    int32_t fatal = CVX_OK;
    std::string fatal_msg;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    void finish(const std::shared_ptr<Request>& q, int32_t status) {
        q->finished = true;
        q->res.status = status;
        q->res.done_s = now();
        if (q->admitted) {
            pool.give(q->offset, q->npx);
            admitted_px -= q->npx;
            eng_groups[q->eng] -= q->groups;
            eng_jobs[q->eng]--;
            q->admitted = false;
        }
    }

    // The engines and their streams: 0 single-launch (low priority), 1 .. n_wf
    // wavefront (high priority).
    WaveEngine* eng_of(int e) { return e == 0 ? &fused : e == 1 ? &engine : &extra_wf[e - 2]; }
    cudaStream_t stream_of(int e) const { return e == 0 ? stream2 : e == 1 ? stream : extra_stream[e - 2]; }

    // Under mu. Admits pending requests in FIFO order while they fit; a
    // request is bound to one engine, so its samples run in order.
    void admit() {
        while (!pending.empty()) {
            auto& q = pending.front();
            if (cfg.sequential && !admitted.empty()) break;
            // Pixel cap: in overload, requests then finish in arrival order
            // instead of all advancing together; the oldest pending request
            // is admitted whenever none is.
            if (cfg.max_inflight_pixels && !admitted.empty() && admitted_px + q->npx > cfg.max_inflight_pixels)
                break;
            int e = 0;
            if (mode[q->r.scene] != 0) {  // the wavefront engine with the fewest admitted groups
                e = 1;
                for (int k = 2; k <= n_wf; k++)
                    if (eng_groups[k] < eng_groups[e]) e = k;
            }
            uint32_t qg = e ? q->groups : 0u;
            uint64_t off = 0;
            if (eng_groups[e] + qg > eng_of(e)->max_groups() || eng_jobs[e] >= eng_of(e)->max_jobs() ||
                !pool.take(q->npx, &off))
                break;
            q->offset = off;
            q->admitted = true;
            admitted_px += q->npx;
            q->eng = e;
            q->res.start_s = now();
            q->groups = qg;
            eng_groups[e] += qg;
            eng_jobs[e]++;
            admitted.push_back(q);
            pending.pop_front();
        }
    }

    // Queues the next sample of each request in `reqs` as one wave on engine
    // e; with cfg.samples_per_wave > 1 and an engine that takes sample slots,
    // up to that many of its next samples, while the engine's jobs, its slot
    // region and the wave's path numbers last. The first adds to the
    // accumulator in the wave, the others write slots that
    // k_accumulate_slots adds after it, in sample order.
    int32_t submit_wave(int e, const std::vector<std::shared_ptr<Request>>& reqs) {
        std::vector<Job> jobs;
        std::vector<SlotItem> items;
        jobs.reserve(reqs.size());
        cudaStream_t st = stream_of(e);
        WaveEngine* eng = eng_of(e);
        const uint64_t region = slot_region_px * (uint64_t)e;
        uint64_t used = 0, groups = 0;
        for (auto& q : reqs) groups += groups_of(q->r.width, q->r.height);
        // The wave's groups stay within the engine's ray-queue capacity (which
        // admission checked for one sample of each request) and below
        // kMaxRefillGroups (from there a wave takes the octet form).
        const uint64_t max_groups = std::min<uint64_t>(eng->max_groups(), kMaxRefillGroups - 1);
        const bool slots = cfg.samples_per_wave > 1 && d_samples && eng->takes_sample_slots() &&
                           groups <= max_groups;
        for (size_t i = 0; i < reqs.size(); i++) {
            auto& q = reqs[i];
            uint32_t k = 1;
            if (slots) {
                const uint32_t g = groups_of(q->r.width, q->r.height);
                uint64_t fit = std::min<uint64_t>(q->r.spp - q->next_sample, cfg.samples_per_wave);
                // every later request keeps its first sample's job
                fit = std::min<uint64_t>(fit, 1 + (eng->max_jobs() - jobs.size() - (reqs.size() - i)));
                fit = std::min<uint64_t>(fit, 1 + (slot_region_px - used) / q->npx);
                fit = std::min<uint64_t>(fit, 1 + (max_groups - groups) / g);
                k = (uint32_t)fit;
                groups += (uint64_t)(k - 1) * g;
            }
            q->wave_job = (uint32_t)jobs.size();
            q->wave_k = k;
            for (uint32_t smp = 0; smp < k; smp++) {
                Job j{};
                std::memcpy(&j.cam, &q->r.camera, sizeof(cvx_camera));
                j.scene = q->r.scene;
                j.w = q->r.width;
                j.h = q->r.height;
                j.frame = q->r.frame_base + q->next_sample + smp;
                j.out_offset = q->offset;
                j.slot = smp == 0 ? kNoSlot : region + used + (uint64_t)(smp - 1) * q->npx;
                jobs.push_back(j);
            }
            if (k > 1) {
                items.push_back(SlotItem{q->offset, region + used, (uint32_t)q->npx, k - 1});
                used += (uint64_t)(k - 1) * q->npx;
            }
            // a request's accumulator starts at zero with its first sample
            if (q->next_sample == 0) cudaMemsetAsync(d_accum + 3 * q->offset, 0, q->npx * 12, st);
        }
        WaveOutputs out{};
        out.accum = d_accum;
        if (!items.empty()) out.samples = d_samples;
        int32_t r = eng->submit(jobs, out, st, true);
        if (r || items.empty()) return r;
        SlotItem* di = d_slot_items + 1024 * e;
        ECK(cudaMemcpyAsync(di, items.data(), items.size() * sizeof(SlotItem), cudaMemcpyHostToDevice, st),
            "upload slot list");
        ECK(launch_accumulate_slots(di, (uint32_t)items.size(), d_accum, d_samples, st), "add sample slots");
        return CVX_OK;
    }

    // Engine e's wave over `reqs` has ended with status st: account for it,
    // resolve and copy out the requests that have all their samples.
    void complete(int e, const std::vector<std::shared_ptr<Request>>& reqs, int32_t st) {
        uint64_t r = 0;
        float ms = 0.0f;
        std::vector<uint64_t> jr;
        int32_t cst = eng_of(e)->collect(stream_of(e), &r, &jr, &ms);
        if (!st) st = cst;
        std::vector<std::shared_ptr<Request>> done;
        std::vector<ResolveItem> items;
        {
            std::lock_guard<std::mutex> lk(mu);
            waves++;
            rays += r;
            (e == 0 ? busy_fused_s : busy_wavefront_s) += ms * 1e-3;
            for (size_t i = 0; i < reqs.size(); i++) {
                auto& q = reqs[i];
                q->in_flight = false;
                if (st) {
                    if (!q->finished) {
                        finish(q, st);
                        admitted.erase(std::find(admitted.begin(), admitted.end(), q));
                    }
                    continue;
                }
                for (uint32_t k = 0; k < q->wave_k; k++)
                    q->res.rays += q->wave_job + k < jr.size() ? jr[q->wave_job + k] : 0;
                q->next_sample += q->wave_k;
                if (q->next_sample == q->r.spp && !q->cancelled) {
                    done.push_back(q);
                    items.push_back(ResolveItem{q->offset, (uint32_t)q->npx, 1.0f / (float)q->r.spp});
                }
            }
            if (st) {
                char buf[256];
                cvx_last_error(buf, sizeof buf);
                fatal_msg = buf;
            }
            arrivals++;  // the loop re-checks admission: memory or queue space may have freed
        }
        if (!done.empty()) {
            cudaStream_t rs = stream_of(e);
            ResolveItem* di = d_items + 1024 * e;  // each engine resolves through its own item list
            cudaError_t ce = cudaMemcpyAsync(di, items.data(), items.size() * sizeof(ResolveItem),
                                             cudaMemcpyHostToDevice, rs);
            if (ce == cudaSuccess) ce = launch_resolve_multi(di, (uint32_t)items.size(), d_accum, d_rgba, rs);
            for (auto& q : done)
                if (ce == cudaSuccess && q->host_rgba)
                    ce = cudaMemcpyAsync(q->host_rgba, d_rgba + q->offset, q->npx * 4, cudaMemcpyDeviceToHost, rs);
            // Wait even after a failed enqueue: copies queued before it still
            // write into the requests' buffers, which their callers may free
            // once the requests are finished.
            cudaError_t se = cudaStreamSynchronize(rs);
            if (ce == cudaSuccess) ce = se;
            std::lock_guard<std::mutex> lk(mu);
            for (auto& q : done) {
                finish(q, ce == cudaSuccess ? CVX_OK : CVX_ERR_CUDA);
                admitted.erase(std::find(admitted.begin(), admitted.end(), q));
            }
        }
        std::lock_guard<std::mutex> lk(mu);
        done_cv.notify_all();
    }

    // The request loop. Each engine has at most one wave on the GPU; an
    // engine whose wave ends starts its next one at once, without waiting
    // for the others, so the engines run out of phase and each fills SMs the
    // others leave idle (bounce tails, the gaps between launches). The host
    // waits by polling completion events (no GPU-side waiting).
    void loop() {
        struct Flight {
            bool busy = false;
            std::vector<std::shared_ptr<Request>> reqs;
            cudaEvent_t done = nullptr;
        } fl[kMaxEngines];
        // The thread starts on device 0: take the server's device. (If that
        // fails, every wave fails and its requests end with the error.)
        cudaSetDevice(device);
        for (auto& f : fl) cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
        int n_busy = 0;
        double busy_from = 0.0;
        uint64_t seen = 0;
        for (;;) {
            std::vector<std::shared_ptr<Request>> start[kMaxEngines];
            {
                std::unique_lock<std::mutex> lk(mu);
                if (n_busy == 0) cv.wait(lk, [&] { return stop || !pending.empty() || !admitted.empty(); });
                if (stop) break;
                seen = arrivals;
                admit();
                for (auto it = admitted.begin(); it != admitted.end();) {
                    if ((*it)->cancelled && !(*it)->in_flight) {
                        finish(*it, CVX_ERR_CANCELLED);
                        it = admitted.erase(it);
                    } else {
                        ++it;
                    }
                }
                done_cv.notify_all();
                for (int e = 0; e <= n_wf; e++)
                    if (!fl[e].busy)
                        for (auto& q : admitted)
                            if (q->eng == e && !q->in_flight) {
                                q->in_flight = true;
                                start[e].push_back(q);
                            }
            }
            for (int e = 0; e <= n_wf; e++) {
                if (start[e].empty()) continue;
                int32_t st = submit_wave(e, start[e]);
                if (st) {
                    complete(e, start[e], st);
                    continue;
                }
                cudaEventRecord(fl[e].done, stream_of(e));
                fl[e].busy = true;
                fl[e].reqs = std::move(start[e]);
                if (n_busy++ == 0) busy_from = now();
            }
            if (n_busy == 0) continue;
            // Wait for an engine to finish, or for new work an idle engine could take.
            for (;;) {
                bool ready = false;
                for (auto& f : fl)
                    if (f.busy && cudaEventQuery(f.done) != cudaErrorNotReady) ready = true;
                if (ready) break;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    if (stop || arrivals != seen) break;
                }
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            }
            for (int e = 0; e <= n_wf; e++) {
                if (!fl[e].busy || cudaEventQuery(fl[e].done) == cudaErrorNotReady) continue;
                fl[e].busy = false;
                complete(e, fl[e].reqs, CVX_OK);
                fl[e].reqs.clear();
                if (--n_busy == 0) {
                    std::lock_guard<std::mutex> lk(mu);
                    busy_s += now() - busy_from;
                }
            }
        }
        for (int e = 0; e <= n_wf; e++)
            if (fl[e].busy) cudaStreamSynchronize(stream_of(e));
        for (auto& f : fl) cudaEventDestroy(f.done);
    }

    ~cvx_server() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        if (worker.joinable()) worker.join();
        cudaFree(d_accum);
        cudaFree(d_rgba);
        cudaFree(d_items);
        cudaFree(d_samples);
        cudaFree(d_slot_items);
        if (stream) cudaStreamDestroy(stream);
        if (stream2) cudaStreamDestroy(stream2);
        for (cudaStream_t x : extra_stream)
            if (x) cudaStreamDestroy(x);
    }
};

extern "C" int32_t cvx_server_create(cvx_scene* const* scenes, uint32_t n_scenes, const cvx_server_config* cfg,
                                     cvx_server** out) {
    if (!scenes || !n_scenes || !cfg || !out) return set_error(CVX_ERR_INVALID, "null argument");
    if (cfg->max_groups == 0 || cfg->framebuffer_bytes < 16) return set_error(CVX_ERR_INVALID, "empty budget");
    for (uint32_t i = 0; i < n_scenes; i++)
        if (!scenes[i] || scene_num_lights(scenes[i]) == 0)
            return set_error(CVX_ERR_INVALID, "every served scene needs a direct-sample triangle");
    int dev = 0;
    int32_t st = common_device(scenes, n_scenes, &dev);
    if (st) return st;
    CVX_ON_DEVICE(dev);
    std::unique_ptr<cvx_server> s(new cvx_server());
    s->device = dev;
    s->scenes.assign(scenes, scenes + n_scenes);
    s->cfg = *cfg;
    // The wavefront waves (deep scenes) are the longer part of a wave: their
    // stream gets the highest priority, so that their bounce kernels take SMs
    // ahead of the single-launch waves running beside them.
    int least = 0, greatest = 0;
    ECK(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
    ECK(cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, greatest), "cudaStreamCreate");
    ECK(cudaStreamCreateWithPriority(&s->stream2, cudaStreamNonBlocking, least), "cudaStreamCreate");
    const bool deep_fused = cfg->deep_single_launch != 0;
    st = s->engine.init(cfg->max_groups, 1024, cfg->traversal == CVX_TRAVERSE_PACKET, cfg->use_graph != 0,
                                cfg->blocks_per_sm, cfg->refill_mode, deep_fused);
    if (st) return st;
    if ((st = s->fused.init(0xffffffffu, 1024, cfg->traversal == CVX_TRAVERSE_PACKET, cfg->use_graph != 0,
                            cfg->fused_blocks_per_sm, cfg->refill_mode, true)))
        return st;
    if ((st = s->engine.set_scenes(scenes, n_scenes))) return st;
    if ((st = s->fused.set_scenes(scenes, n_scenes))) return st;
    if (cfg->wavefront_streams > (uint32_t)cvx_server::kMaxEngines - 1)
        return set_error(CVX_ERR_INVALID, "at most 4 wavefront streams");
    for (uint32_t k = 1; k < cfg->wavefront_streams; k++) {
        ECK(cudaStreamCreateWithPriority(&s->extra_stream[k - 1], cudaStreamNonBlocking, greatest),
            "cudaStreamCreate");
        if ((st = s->extra_wf[k - 1].init(cfg->max_groups, 1024, cfg->traversal == CVX_TRAVERSE_PACKET,
                                          cfg->use_graph != 0, cfg->blocks_per_sm, cfg->refill_mode, deep_fused)))
            return st;
        if ((st = s->extra_wf[k - 1].set_scenes(scenes, n_scenes))) return st;
        s->n_wf = (int)k + 1;
    }
    for (uint32_t i = 0; i < n_scenes; i++)
        s->mode.push_back(cfg->kernel_mode == 1 ? 0u : cfg->kernel_mode == 2 ? 1u : default_scene_mode(scenes[i]));
    s->pool_px = cfg->framebuffer_bytes / 16;  // 12 B accumulator + 4 B RGBA per pixel
    std::vector<void*> owned;
    if ((st = alloc(&s->d_accum, s->pool_px * 3, owned))) return st;
    if ((st = alloc(&s->d_rgba, s->pool_px, owned))) return st;
    if ((st = alloc(&s->d_items, (size_t)cvx_server::kMaxEngines * 1024, owned))) return st;
    if (cfg->samples_per_wave > 1) {
        const uint64_t bytes = cfg->sample_buffer_bytes ? cfg->sample_buffer_bytes : cfg->framebuffer_bytes;
        s->slot_region_px = bytes / 12 / (uint64_t)(s->n_wf + 1);
        if (s->slot_region_px == 0) return set_error(CVX_ERR_INVALID, "sample buffer too small");
        if ((st = alloc(&s->d_samples, s->slot_region_px * 3 * (uint64_t)(s->n_wf + 1), owned))) return st;
        if ((st = alloc(&s->d_slot_items, (size_t)cvx_server::kMaxEngines * 1024, owned))) return st;
    }
    s->pool.init(s->pool_px);
    s->worker = std::thread([p = s.get()] { p->loop(); });
    *out = s.release();
    return CVX_OK;
}

extern "C" int32_t cvx_server_submit(cvx_server* s, const cvx_request* req, uint32_t* rgba, uint64_t* id) {
    if (!s || !req || !id) return set_error(CVX_ERR_INVALID, "null argument");
    if (req->scene >= s->scenes.size() || req->width == 0 || req->height == 0 || req->spp == 0 ||
        req->width > kMaxImageSide || req->height > kMaxImageSide)
        return set_error(CVX_ERR_INVALID, "bad request");
    auto q = std::make_shared<Request>();
    q->r = *req;
    q->host_rgba = rgba;
    q->npx = (uint64_t)req->width * req->height;
    q->groups = groups_of(req->width, req->height);
    {
        // The scene's mode is read under the lock: cvx_server_set_scene_mode
        // writes it under the same lock.
        std::lock_guard<std::mutex> lk(s->mu);
        if (q->npx > s->pool_px || (s->mode[req->scene] == 1 && q->groups > s->engine.max_groups()))
            return set_error(CVX_ERR_CAPACITY, "request larger than the server's framebuffer or ray-queue budget");
        q->id = s->next_id++;
        q->res.submit_s = s->now();
        s->pending.push_back(q);
        s->all[q->id] = q;
        s->arrivals++;
        *id = q->id;
    }
    s->cv.notify_all();
    return CVX_OK;
}

extern "C" int32_t cvx_server_wait(cvx_server* s, uint64_t id, uint32_t timeout_ms, cvx_request_result* result) {
    if (!s) return set_error(CVX_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return set_error(CVX_ERR_NOT_FOUND, "unknown request id");
    auto q = it->second;
    if (!q->finished)
        s->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return q->finished; });
    if (!q->finished) return set_error(CVX_ERR_TIMEOUT, "request not finished");
    if (result) *result = q->res;
    s->all.erase(id);
    return CVX_OK;
}

extern "C" int32_t cvx_server_cancel(cvx_server* s, uint64_t id) {
    if (!s) return set_error(CVX_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return set_error(CVX_ERR_NOT_FOUND, "unknown request id");
    auto q = it->second;
    if (q->finished) return CVX_OK;
    q->cancelled = true;
    s->arrivals++;
    auto p = std::find(s->pending.begin(), s->pending.end(), q);
    if (p != s->pending.end()) {
        s->pending.erase(p);
        s->finish(q, CVX_ERR_CANCELLED);
        s->done_cv.notify_all();
    }
    s->cv.notify_all();
    return CVX_OK;
}

extern "C" int32_t cvx_server_stats(cvx_server* s, double* now_s, uint64_t* waves, uint64_t* rays, double* busy_s) {
    if (!s) return set_error(CVX_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (now_s) *now_s = s->now();
    if (waves) *waves = s->waves;
    if (rays) *rays = s->rays;
    if (busy_s) *busy_s = s->busy_s;
    return CVX_OK;
}

extern "C" int32_t cvx_server_engine_stats(cvx_server* s, double* fused_busy_s, double* wavefront_busy_s) {
    if (!s) return set_error(CVX_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (fused_busy_s) *fused_busy_s = s->busy_fused_s;
    if (wavefront_busy_s) *wavefront_busy_s = s->busy_wavefront_s;
    return CVX_OK;
}

extern "C" int32_t cvx_server_set_scene_mode(cvx_server* s, uint32_t scene, uint32_t mode) {
    if (!s || scene >= s->scenes.size() || mode > 1) return set_error(CVX_ERR_INVALID, "bad scene mode");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->admitted.empty() || !s->pending.empty())
        return set_error(CVX_ERR_INVALID, "scene modes can change only while the server is idle");
    s->mode[scene] = mode;
    return CVX_OK;
}

extern "C" void cvx_server_destroy(cvx_server* s) {
    if (!s) return;
    DeviceGuard g(s->device);
    delete s;
}
