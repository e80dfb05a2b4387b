// Wavefront form of the path loop (renderer.rs:413-468): ray generation,
// traversal and shading kernels over structure-of-arrays ray queues.
//
// A wave is a list of jobs; a job is one sample of one image of one resident
// scene (its own camera, size, frame number and output slot). All groups of
// all jobs of a wave share the queues, so images of different scenes and
// sizes fill the same launches. Every group uses the per-group RNG order, so
// a job's pixels do not depend on which other jobs share its wave.
#pragma once
#include <cstdint>

#include "layout.cuh"

namespace cvx {

struct Job {
    DeviceCamera cam;
    uint32_t scene;       // index into the wave's scene table
    uint32_t w, h, frame;
    uint32_t group_base;  // first wave-global group index of this job
    uint32_t n_groups;    // 8 * ceil(w/16) * ceil(h/4)
    uint64_t out_offset;  // first pixel of this image in the output buffers
    // Waves with WaveOutputs::samples (path refill only): kNoSlot, or the
    // first pixel of this job's colour slot there; the job then writes its
    // colours to the slot instead of the outputs, and a pass after the wave
    // adds the slots to the accumulator in sample order (several samples of
    // one image in one wave).
    uint64_t slot;
};
constexpr uint64_t kNoSlot = ~0ull;

// A request's samples 1 .. count of one wave, added after it: accum pixels
// from accum_offset, count slots of npx pixels each from slot.
struct SlotItem {
    uint64_t accum_offset;
    uint64_t slot;
    uint32_t npx;
    uint32_t count;
};

struct WaveHeader {
    uint32_t n_jobs;
    uint32_t n_groups;
};

// Per-lane state, lane = group * 8 + k.
struct WaveState {
    float *ox, *oy, *oz, *dx, *dy, *dz;
    float *cr, *cg, *cb;
    uint64_t* rng;
    uint32_t* gbuf;     // gbuffer word of bounce 0
    uint32_t* flags;    // bit 0: active, bit 1: last hit emissive
    float *ht, *hu, *hv;
    int32_t* htri;
    uint32_t* group_job;
    uint32_t* queue[2];  // group queues, alternating between bounces
    uint32_t* counts;    // [b]: groups alive before bounce b (0..5); [6 + b]: refill ray counter of
                         // bounce b; [11 + b]: octet traversal's queue-entry counter of bounce b
};

struct WaveOutputs {
    uint32_t* rgba;
    uint32_t* gbuf;
    float* color;
    float* accum;
    unsigned long long* rays;      // all rays of the wave
    unsigned long long* job_rays;  // per job of the wave, or null
    uint32_t* err;
    // one word per group of the wave, zero at launch: given, a single-ray
    // fused wave takes paths per lane (k_wave_refill)
    uint32_t* group_em;
    // colour slots of the jobs' Job::slot (3 floats per pixel), or null
    float* samples;
};

// One image to resolve from the accumulator (renderer.rs:378-410).
struct ResolveItem {
    uint64_t offset;
    uint32_t npx;
    float factor;
};

}  // namespace cvx
