// Launchers of the device kernels (kernels.cu), used by the C-ABI (capi.cu).
#pragma once
#include <cuda_runtime.h>

#include "../../include/convector_gpu.h"
#include "layout.cuh"
#include "wavefront.cuh"

namespace cvx {

// SM count of the calling thread's current device (cached per device).
int sm_count();
// The traversal stack limit (traverse.cuh c_stack_limit) on the current
// device, for the kernels of kernels.cu and of wavefront.cu.
cudaError_t set_stack_limit(int entries);
cudaError_t set_stack_limit_wave(int entries);
cudaError_t upload_tables(const uint16_t* rcp, const uint16_t* rsqrt);
cudaError_t upload_tables_wave(const uint16_t* rcp, const uint16_t* rsqrt);
cudaError_t launch_prep_geom(const cvx_triangle* tris, uint32_t n, float4* geom, TriShade* shade, cudaStream_t st);
cudaError_t launch_prep_lights(const cvx_triangle* tris, const uint32_t* ds, uint32_t n, float4* lights,
                               cudaStream_t st);
// The six ray components of a nearest-hit query (origin x, y, z, direction
// x, y, z), each an array of n floats. The pointers may be device memory or,
// where the device shares the host's page tables, host memory read in place.
struct RayCols {
    const float* c[6];
};
inline RayCols soa_cols(const float* rays, uint32_t n) {  // one (6, n) device array
    RayCols r;
    for (int k = 0; k < 6; k++) r.c[k] = rays + (size_t)k * n;
    return r;
}

// shared_stack: stack entries of each lane kept in shared memory by the
// select-form single-ray kernel at 8 blocks per SM (0, 4, 8 or 12; other
// launch shapes keep 8).
cudaError_t launch_intersect(const DeviceScene& s, const RayCols& rays, uint32_t n, float far_dist, bool packet,
                             float* t_out, int32_t* tri_out, uint32_t* counters, uint32_t* err, uint32_t block,
                             uint32_t blocks_per_sm, cudaStream_t st, uint32_t shared_stack = 8);
// Single-launch form of single-ray frames and waves in the per-group RNG
// order: paths per lane with ray refill (k_render_refill, k_wave_refill), or
// one octet per 8-pixel group (k_render_group, k_wave_fused). CVX_REFILL_ALL
// and CVX_REFILL_NONE choose; by default the depth of the frame's scene
// decides, and for a wave whether at least half of its groups belong to scenes
// that deep. Measured at 1280x736 (octet against refill, ms per frame): the
// 19-level room 0.82 / 0.73, the 28-level icosphere 1.87 / 1.45, the 70-level
// tube 5.36 / 3.14; 256 scenes of 11 to 23 levels (median 16), batched: 53 / 66
// ms, one at a time: 2,808 / 2,546 Mrays/s. Refill wins clearly from the
// icosphere's depth on; the shallow open scenes, whose paths are mostly one or
// two rays, keep warps of neighbouring camera rays together.
constexpr uint32_t kRefillMinDepth = 25;
inline bool path_refill_frames(uint32_t refill_mode, uint32_t depth) {
    return refill_mode == CVX_REFILL_ALL || (refill_mode == CVX_REFILL_AFTER_CAMERA && depth >= kRefillMinDepth);
}
// deep_groups of a wave's groups belong to scenes of kRefillMinDepth levels or more.
inline bool path_refill_wave(uint32_t refill_mode, uint32_t deep_groups, uint32_t groups) {
    return refill_mode == CVX_REFILL_ALL ||
           (refill_mode == CVX_REFILL_AFTER_CAMERA && 2ull * deep_groups >= (uint64_t)groups && groups > 0);
}

// group_em: one word per 8-pixel group; given, a single-ray frame in the
// per-group RNG order takes the per-lane path refill form (k_render_refill),
// else one octet per group (k_render_group). work (3 words, zeroed by the
// caller; needs group_em): the counting form of k_render_refill adds the
// frame's boxes tested, triangles tested and light-PDF shading steps.
cudaError_t launch_render(const DeviceScene& s, const DeviceCamera& cam, uint32_t w, uint32_t h, uint32_t frame,
                          bool packet, bool patch_order, uint32_t* rgba, uint32_t* gbuf, float* color, float* accum,
                          unsigned long long* rays, uint32_t* err, uint32_t block, bool debug, cudaStream_t st, uint32_t patch = 32,
                          const uint32_t* patches = nullptr, uint32_t n_patches = 0, uint32_t* group_em = nullptr,
                          unsigned long long* work = nullptr, uint32_t samples = 1, float* sample_color = nullptr);
// Frames with the per-lane path refill (group_em set, single-ray traversal,
// per-group RNG order) may render `samples` > 1 frames, frame .. frame +
// samples - 1, in one launch, accumulating them into `accum` in frame order
// (bit-identical to one launch per frame); color and gbuf then hold the last
// frame's values, and sample_color holds 3 * w * h * (samples - 1) floats.
// Other forms take samples == 1 only.
cudaError_t launch_resolve(const float* accum, uint32_t npx, float factor, uint32_t* rgba, cudaStream_t st);
// refill_from: first bounce whose single-ray traversal uses ray refill (the
// earlier ones traverse one octet per group); packet traversal ignores it.
cudaError_t launch_wave(const Job* jobs, const WaveHeader* hdr, const DeviceScene* scenes, const WaveState& st,
                        const WaveOutputs& out, bool packet, uint32_t blocks_per_sm, uint32_t refill_from, bool deep,
                        cudaStream_t stream);
// The fused (megakernel) form of a wave: one persistent launch.
// deep: a scene of the wave is deeper than 40 levels (claim threshold 8, else 16)
cudaError_t launch_wave_fused(const Job* jobs, const WaveHeader* hdr, const DeviceScene* scenes,
                              const WaveOutputs& out, bool packet, uint32_t blocks_per_sm, bool deep,
                              cudaStream_t stream);
cudaError_t launch_resolve_multi(const ResolveItem* items, uint32_t n_items, const float* accum, uint32_t* rgba,
                                 cudaStream_t stream);
// After a wave with sample slots (WaveOutputs::samples): adds each item's
// slots to its accumulator pixels in sample order.
cudaError_t launch_accumulate_slots(const SlotItem* items, uint32_t n_items, float* accum, const float* samples,
                                    cudaStream_t stream);

}  // namespace cvx
