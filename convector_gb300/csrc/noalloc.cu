// cvx_intersect_nearest_noalloc: the nearest-hit query of cvx_intersect_nearest
// for callers that must not allocate device memory. Every byte it needs beyond
// the scene and the caller's host buffers lives in one file-scope static
// device array. The array's module is loaded, and its device address looked
// up, when the first scene is created on a device (cvx_scene_create calls
// cvx::noalloc_setup_device, and scene creation allocates anyway), so the
// query itself neither loads a module nor allocates.
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "device_guard.cuh"
#include "engine.h"
#include "internal.h"
#include "kernels.h"

namespace {

// Largest batch of rays one call accepts.
constexpr uint32_t kNoAllocMaxRays = 1u << 19;  // 524,288 rays
// Layout: [0, 256) status word and ray counter; then 6 ray arrays of n floats,
// n distances and n triangle indices, each region sized for kNoAllocMaxRays.
constexpr size_t kHeaderBytes = 256;
constexpr size_t kRayBytes = (size_t)kNoAllocMaxRays * 6 * sizeof(float);
constexpr size_t kTBytes = (size_t)kNoAllocMaxRays * sizeof(float);
constexpr size_t kTriBytes = (size_t)kNoAllocMaxRays * sizeof(int32_t);
constexpr size_t kScratchBytes = kHeaderBytes + kRayBytes + kTBytes + kTriBytes;  // 16 MiB + 256 B

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
std::vector<unsigned char*> g_scratch_by_device;

// Device address of the scratch array on the current device, looked up once
// per device with that device current. In host code `g_noalloc_scratch` is
// only a host-side stand-in for the symbol, never a device address.
int32_t scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cvx::set_error(CVX_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_scratch_by_device.size() <= dev) g_scratch_by_device.resize(dev + 1, nullptr);
    if (!g_scratch_by_device[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return cvx::set_error(CVX_ERR_CUDA,
                                  std::string("cudaGetSymbolAddress of the static scratch: ") + cudaGetErrorString(e));
        g_scratch_by_device[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_by_device[dev];
    return CVX_OK;
}

}  // namespace

// Looks up the scratch array's address on the current device (loading the
// module that holds it, which reserves the array there) unless that was
// done before. Called by cvx_scene_create with the scene's device current.
int32_t cvx::noalloc_setup_device() {
    unsigned char* p = nullptr;
    return scratch_address(&p);
}

namespace {

int32_t fail(cudaError_t e, const char* what) {
    return cvx::set_error(CVX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" int32_t cvx_intersect_nearest_noalloc(cvx_scene* scene, const float* ox, const float* oy, const float* oz,
                                                 const float* dx, const float* dy, const float* dz, uint32_t n,
                                                 float far_dist, uint32_t traversal, float* t_out,
                                                 int32_t* tri_out) {
    if (!scene) return cvx::set_error(CVX_ERR_INVALID, "null scene");
    if (n == 0) return CVX_OK;
    if (!ox || !oy || !oz || !dx || !dy || !dz || !t_out || !tri_out)
        return cvx::set_error(CVX_ERR_INVALID, "null buffer");
    if (traversal > 1) return cvx::set_error(CVX_ERR_INVALID, "unknown traversal variant");
    CVX_ON_DEVICE(cvx::scene_device(scene));
    if (n > kNoAllocMaxRays)
        return cvx::set_error(CVX_ERR_INVALID, "cvx_intersect_nearest_noalloc takes at most " +
                                                   std::to_string(kNoAllocMaxRays) + " rays per call, got " +
                                                   std::to_string(n));
    unsigned char* base = nullptr;
    int32_t st = scratch_address(&base);  // set up when the scene was created: a cached lookup
    if (st) return st;
    uint32_t* status = reinterpret_cast<uint32_t*>(base);  // [0] status, [1] ray counter
    float* rays = reinterpret_cast<float*>(base + kHeaderBytes);
    float* t_dev = reinterpret_cast<float*>(base + kHeaderBytes + kRayBytes);
    int32_t* tri_dev = reinterpret_cast<int32_t*>(base + kHeaderBytes + kRayBytes + kTBytes);
    cudaStream_t stream = cvx::scene_stream(scene);
    uint32_t err = 0;
    cvx::StreamSync sync(stream);
    cudaError_t e;
    // The array keeps the previous call's contents: the status word must start at zero.
    if ((e = cudaMemsetAsync(status, 0, 2 * sizeof(uint32_t), stream)) != cudaSuccess) return fail(e, "clear status");
    const float* src[6] = {ox, oy, oz, dx, dy, dz};
    for (int k = 0; k < 6; k++)
        if ((e = cudaMemcpyAsync(rays + (size_t)k * n, src[k], (size_t)n * sizeof(float), cudaMemcpyHostToDevice,
                                 stream)) != cudaSuccess)
            return fail(e, "copy rays");
    if ((e = cvx::launch_intersect(cvx::scene_view(scene), cvx::soa_cols(rays, n), n, far_dist,
                                   traversal == CVX_TRAVERSE_PACKET, t_dev, tri_dev, nullptr, status, 0,
                                   cvx::scene_query_blocks_per_sm(scene), stream, cvx::scene_query_stack(scene))) !=
        cudaSuccess)
        return fail(e, "intersect launch");
    if ((e = cudaMemcpyAsync(t_out, t_dev, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
        return fail(e, "copy distances");
    if ((e = cudaMemcpyAsync(tri_out, tri_dev, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, stream)) !=
        cudaSuccess)
        return fail(e, "copy indices");
    if ((e = cudaMemcpyAsync(&err, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
        return fail(e, "copy status");
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return fail(e, "intersect");
    if (err) return cvx::set_error(CVX_ERR_DEVICE, "traversal stack overflow reported by the kernel");
    return CVX_OK;
}
