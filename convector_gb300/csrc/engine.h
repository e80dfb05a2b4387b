// Host class of the wavefront engine (engine.cu).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/convector_gpu.h"
#include "layout.cuh"
#include "wavefront.cuh"

namespace cvx {

DeviceScene scene_view(const cvx_scene* s);
cudaStream_t scene_stream(const cvx_scene* s);
uint32_t scene_depth(const cvx_scene* s);
uint32_t scene_num_lights(const cvx_scene* s);
int scene_device(const cvx_scene* s);  // the device the scene was created on
// Resident blocks per SM of the scene's nearest-hit queries (0: default;
// cvx_scene_set_query_launch).
uint32_t scene_query_blocks_per_sm(const cvx_scene* s);
// Stack entries per lane the nearest-hit query keeps in shared memory
// (cvx_scene_set_query_stack).
uint32_t scene_query_stack(const cvx_scene* s);
// Loads the module of cvx_intersect_nearest_noalloc's static scratch array on
// the current device and caches its address (noalloc.cu); scene creation
// calls it once per scene, so the no-allocation query loads and allocates
// nothing itself.
int32_t noalloc_setup_device();
// Largest image width and height of a renderer, batch view or server request
// (an image of 16384 x 16384 is 2^25 groups, so group and path indices of
// one image stay far inside 32 bits).
constexpr uint32_t kMaxImageSide = CVX_MAX_IMAGE_SIDE;
// Waves with per-lane path refill hold fewer groups than this: path ids and
// the path counter are 32-bit, and the counter runs past the last path by at
// most one claim per lane of the grid.
constexpr uint32_t kMaxRefillGroups = 1u << 28;
uint32_t groups_of(uint32_t w, uint32_t h);
// First bounce of a wavefront wave whose traversal refills rays, for a
// CVX_REFILL_* mode.
inline uint32_t refill_from(uint32_t refill_mode) { return refill_mode == 1 ? 0u : refill_mode == 2 ? 5u : 1u; }

class WaveEngine {
   public:
    ~WaveEngine();
    // max_groups: ray-queue capacity (8-pixel groups) of one wave. fused: run
    // waves as one persistent fused kernel (no ray queues) instead of the
    // wavefront kernels; refill_mode: CVX_REFILL_* (wavefront: which bounces
    // refill; fused: path_refill_frames with the wave's deepest scene).
    int32_t init(uint32_t max_groups, uint32_t max_jobs, bool packet, bool use_graph, uint32_t blocks_per_sm,
                 uint32_t refill_mode = CVX_REFILL_AFTER_CAMERA, bool fused = false);
    int32_t set_scenes(cvx_scene* const* scenes, uint32_t n);
    // Queues one wave on `stream` (asynchronous); group_base / n_groups of the
    // jobs are filled in here. collect() waits for it and reads its counters.
    int32_t submit(const std::vector<Job>& jobs, WaveOutputs out, cudaStream_t stream, bool want_job_rays);
    int32_t collect(cudaStream_t stream, uint64_t* rays, std::vector<uint64_t>* job_rays, float* ms);
    // submit + collect. rays, job_rays and ms may be null.
    int32_t run(const std::vector<Job>& jobs, WaveOutputs out, cudaStream_t stream, uint64_t* rays,
                std::vector<uint64_t>* job_rays, float* ms);
    uint32_t max_groups() const { return max_groups_; }
    uint32_t max_jobs() const { return max_jobs_; }
    bool fused() const { return fused_; }
    // Its waves take paths per lane whatever their scenes, so they accept
    // sample slots (Job::slot, WaveOutputs::samples).
    bool takes_sample_slots() const { return fused_ && !packet_ && refill_mode_ == CVX_REFILL_ALL; }

   private:
    int32_t launch(const WaveOutputs& out, bool deep, cudaStream_t stream);
    struct Readback {
        unsigned long long rays;
        uint32_t err;
    };
    Readback* h_read_ = nullptr;
    unsigned long long* h_job_rays_ = nullptr;
    uint32_t last_jobs_ = 0;
    bool last_want_ = false, fused_ = false;
    struct Graph {
        WaveOutputs out;
        bool deep;
        cudaGraphExec_t exec;
    };
    WaveState st_{};
    Job* d_jobs_ = nullptr;
    Job* h_jobs_ = nullptr;
    WaveHeader* d_hdr_ = nullptr;
    WaveHeader* h_hdr_ = nullptr;
    DeviceScene* d_scenes_ = nullptr;
    unsigned long long* d_rays_ = nullptr;
    unsigned long long* d_job_rays_ = nullptr;
    uint32_t* d_err_ = nullptr;
    uint32_t* d_group_em_ = nullptr;  // per group of a wave: the path refill's emitter counts
    uint32_t group_em_cap_ = 0;
    std::vector<uint32_t> scene_depth_;
    uint32_t n_scenes_ = 0, scene_cap_ = 0, max_groups_ = 0, max_jobs_ = 0, blocks_per_sm_ = 0, refill_from_ = 1,
             refill_mode_ = 0;
    bool packet_ = false, use_graph_ = false;
    std::vector<void*> owned_;
    std::vector<Graph> graphs_;
    cudaEvent_t e0_ = nullptr, e1_ = nullptr;
};

}  // namespace cvx
