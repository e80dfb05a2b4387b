// L2 read bandwidth of this GPU, measured: the roofline denominator for the
// traversal kernels, whose node and triangle data stay in L2 (the scene is
// far smaller than the 126 MB L2) while HBM only carries rays and images.
// No counterpart in the reference. Built as its own library
// (libconvector_l2probe.so): the render path never calls it.
//
// Every thread of a grid sized to fill the GPU reads 16-byte words of an
// L2-resident buffer in grid-stride order with ld.global.cg (cached in L2,
// not L1), pass after pass; the sum of the words is kept so that no load is
// dropped. achieved = passes * buffer bytes / the launch's CUDA-event time.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

__global__ void __launch_bounds__(256) k_l2_read(const float4* __restrict__ buf, uint32_t n4, uint32_t passes,
                                                 float* __restrict__ sink) {
    const uint32_t stride = gridDim.x * blockDim.x, tid = blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.0f;
    for (uint32_t p = 0; p < passes; p++) {
        // four independent loads in flight per thread
        uint32_t i = tid;
        for (; i + 3u * stride < n4; i += 4u * stride) {
            float4 a = __ldcg(buf + i), b = __ldcg(buf + i + stride), c = __ldcg(buf + i + 2u * stride),
                   d = __ldcg(buf + i + 3u * stride);
            acc += (a.x + b.y) + (c.z + d.w);
        }
        for (; i < n4; i += stride) acc += __ldcg(buf + i).x;
    }
    if (acc == 1.0e30f) sink[tid] = acc;  // never true for the zeroed buffer, but the compiler cannot know
}

}  // namespace

extern "C" {

// Reads a `bytes`-byte device buffer (a multiple of 16, at most 1 GiB)
// `passes` times in each of `launches` timed launches after one warm-up
// launch; returns the best launch's rate in GB/s (1e9 bytes/s). 0 = OK,
// 1 = bad argument, 2 = CUDA error.
int32_t cvx_probe_l2_read_gbs(uint64_t bytes, uint32_t passes, uint32_t launches, double* gbs) {
    if (!gbs || bytes < 16 || (bytes & 15u) || bytes > (1ull << 30) || passes == 0 || launches == 0) return 1;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        return 2;
    float4* buf = nullptr;
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const uint32_t threads = 256, blocks = (uint32_t)sms * 8u;
    int32_t rc = 2;
    double best = 0.0;
    if (cudaMalloc(&buf, bytes) != cudaSuccess || cudaMalloc(&sink, (size_t)blocks * threads * 4) != cudaSuccess ||
        cudaMemset(buf, 0, bytes) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess)
        goto done;
    k_l2_read<<<blocks, threads>>>(buf, (uint32_t)(bytes / 16), passes, sink);
    for (uint32_t k = 0; k < launches; k++) {
        cudaEventRecord(e0);
        k_l2_read<<<blocks, threads>>>(buf, (uint32_t)(bytes / 16), passes, sink);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) goto done;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double rate = (double)bytes * passes / (ms * 1e-3) / 1e9;
        if (rate > best) best = rate;
    }
    if (cudaGetLastError() == cudaSuccess) {
        *gbs = best;
        rc = 0;
    }
done:
    cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(sink);
    return rc;
}

}  // extern "C"
