// The reference's display post-process (src/gpu/*.glsl, driven by
// Window::display_buffer, ui.rs:313-364) restated as CUDA kernels over
// headless device buffers, since OpenGL is not available here:
//   gbuffer pass  gbuffer.glsl:18-42  texture composite with the Fresnel factor
//   blend         blend.glsl:22-34    mean of the last 8 gbuffer-pass frames
//   median        median.glsl:16-75   5-tap "+" median in CIE XYZ
//   display       the sRGB framebuffer (ui.rs:246, with_srgb) encodes to sRGB
// GL behaviour that the shaders leave to the driver is fixed here as:
// unorm8 textures read as byte/255; render targets store round(clamp(x)*255);
// the material textures are sRGB-decoded and sampled bilinearly with repeat
// wrapping; the median's neighbours clamp at the frame edge. sRGB decode and
// encode go through host-computed tables, so the oracle restatement gives the
// same bytes. Arithmetic is unfused (-fmad=false), written out in shader order.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "device_guard.cuh"
#include "internal.h"

namespace {

struct PostTables {
    float srgb_decode[256];  // sRGB byte -> linear
    float srgb_encode[255];  // linear threshold of sRGB byte k+1 (byte = count of thresholds <= x)
};

__device__ __forceinline__ float unorm(uint32_t w, int c) { return (float)((w >> (8 * c)) & 0xffu) * (1.0f / 255.0f); }

__device__ __forceinline__ uint32_t quant(float x) {  // unorm8 render target: round(clamp(x) * 255)
    x = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
    return (uint32_t)__float2int_rn(x * 255.0f);
}

__device__ __forceinline__ uint32_t pack4(float r, float g, float b, float a) {
    return quant(r) | (quant(g) << 8) | (quant(b) << 16) | (quant(a) << 24);
}

struct Tex {
    const uint8_t* rgb;  // sRGB bytes, row-major
    uint32_t w, h;
};

// Bilinear sample with repeat wrapping of an sRGB RGB8 texture at (u, v).
__device__ __forceinline__ void sample(const Tex& t, const float* dec, float u, float v, float out[4]) {
    float x = u * (float)t.w - 0.5f, y = v * (float)t.h - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy;
    int xs[2] = {((x0 % (int)t.w) + (int)t.w) % (int)t.w, (((x0 + 1) % (int)t.w) + (int)t.w) % (int)t.w};
    int ys[2] = {((y0 % (int)t.h) + (int)t.h) % (int)t.h, (((y0 + 1) % (int)t.h) + (int)t.h) % (int)t.h};
    for (int c = 0; c < 3; c++) {
        float p00 = dec[t.rgb[3 * ((size_t)ys[0] * t.w + xs[0]) + c]];
        float p10 = dec[t.rgb[3 * ((size_t)ys[0] * t.w + xs[1]) + c]];
        float p01 = dec[t.rgb[3 * ((size_t)ys[1] * t.w + xs[0]) + c]];
        float p11 = dec[t.rgb[3 * ((size_t)ys[1] * t.w + xs[1]) + c]];
        float top = p00 * (1.0f - ax) + p10 * ax, bot = p01 * (1.0f - ax) + p11 * ax;
        out[c] = top * (1.0f - ay) + bot * ay;
    }
    out[3] = 1.0f;
}

// gbuffer.glsl:18-42, writing frames[slot].
__global__ void k_post_gbuffer(const uint32_t* __restrict__ frame, const uint32_t* __restrict__ gbuf, uint32_t npx,
                               Tex t1, Tex t2, const PostTables* __restrict__ tab, uint32_t* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x) {
        uint32_t fw = frame[i], gw = gbuf[i];
        float color[4] = {unorm(fw, 0), unorm(fw, 1), unorm(fw, 2), unorm(fw, 3)};
        float data[4] = {unorm(gw, 0), unorm(gw, 1), unorm(gw, 2), unorm(gw, 3)};
        float fresnel = data[2];
        for (int k = 1; k <= 2; k++) {
            if (data[3] == (float)k / 255.0f) {
                float tex[4];
                sample(k == 1 ? t1 : t2, tab->srgb_decode, data[0], data[1], tex);
                for (int c = 0; c < 4; c++) {
                    float surface = 1.0f * fresnel + tex[c] * (1.0f - fresnel);
                    color[c] = color[c] * surface;
                }
            }
        }
        out[i] = pack4(color[0], color[1], color[2], color[3]);
    }
}

// blend.glsl:22-34 over the 8 ring slots (or 8 times one slot: draw_single).
__global__ void k_post_blend(const uint32_t* __restrict__ ring, uint32_t npx, int only_slot,
                             uint32_t* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x) {
        float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int f = 0; f < 8; f++) {
            uint32_t w = ring[(size_t)(only_slot >= 0 ? only_slot : f) * npx + i];
            for (int c = 0; c < 4; c++) s[c] = f == 0 ? unorm(w, c) : s[c] + unorm(w, c);
        }
        out[i] = pack4(s[0] * 0.125f, s[1] * 0.125f, s[2] * 0.125f, 1.0f);
    }
}

__device__ __forceinline__ void rgb_to_xyz(float c[4]) {  // median.glsl:35-41 (column-major mat3)
    const float k = 1.0f / 0.17697f;
    float m[9] = {0.49f * k, 0.17697f * k, 0.0f * k, 0.31f * k, 0.81240f * k, 0.01f * k, 0.20f * k, 0.01063f * k,
                  0.99f * k};
    float r = c[0], g = c[1], b = c[2];
    c[0] = m[0] * r + m[3] * g + m[6] * b;
    c[1] = m[1] * r + m[4] * g + m[7] * b;
    c[2] = m[2] * r + m[5] * g + m[8] * b;
}
__device__ __forceinline__ void xyz_to_rgb(float c[4]) {  // median.glsl:43-49
    float m[9] = {0.41847f, -0.091169f, 0.00092090f, -0.15866f, 0.25243f, -0.0025498f, -0.082835f, 0.015708f,
                  0.17860f};
    float x = c[0], y = c[1], z = c[2];
    c[0] = m[0] * x + m[3] * y + m[6] * z;
    c[1] = m[1] * x + m[4] * y + m[7] * z;
    c[2] = m[2] * x + m[5] * y + m[8] * z;
}
__device__ __forceinline__ void sort2(float a[4], float b[4]) {
    for (int c = 0; c < 4; c++) {
        float lo = fminf(a[c], b[c]), hi = fmaxf(a[c], b[c]);
        a[c] = lo;
        b[c] = hi;
    }
}

__device__ __forceinline__ uint32_t srgb_byte(float x, const float* enc) {
    uint32_t lo = 0, hi = 255;  // count thresholds <= x
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (enc[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// median.glsl:51-75, or the identity (id.glsl) when disabled; then the sRGB
// framebuffer's encode.
__global__ void k_post_median(const uint32_t* __restrict__ in, uint32_t w, uint32_t h, int enable,
                              const PostTables* __restrict__ tab, uint32_t* __restrict__ out) {
    uint32_t npx = w * h;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x) {
        int x = (int)(i % w), y = (int)(i / w);
        float res[4];
        if (!enable) {
            for (int c = 0; c < 4; c++) res[c] = unorm(in[i], c);
        } else {
            const int dx[5] = {0, 1, 0, -1, 0}, dy[5] = {0, 0, 1, 0, -1};
            float c5[5][4];
            for (int t = 0; t < 5; t++) {
                int xx = min(max(x + dx[t], 0), (int)w - 1), yy = min(max(y + dy[t], 0), (int)h - 1);
                uint32_t wd = in[(size_t)yy * w + xx];
                for (int c = 0; c < 4; c++) c5[t][c] = unorm(wd, c);
                rgb_to_xyz(c5[t]);
            }
            sort2(c5[0], c5[1]);
            sort2(c5[3], c5[4]);
            sort2(c5[0], c5[2]);
            sort2(c5[1], c5[2]);
            sort2(c5[0], c5[3]);
            sort2(c5[2], c5[3]);
            sort2(c5[1], c5[4]);
            sort2(c5[1], c5[2]);
            sort2(c5[3], c5[4]);
            for (int c = 0; c < 4; c++) res[c] = c5[2][c] * 0.667f + c5[1][c] * 0.1666f + c5[3][c] * 0.1666f;
            xyz_to_rgb(res);
        }
        out[i] = srgb_byte(res[0], tab->srgb_encode) | (srgb_byte(res[1], tab->srgb_encode) << 8) |
                 (srgb_byte(res[2], tab->srgb_encode) << 16) | (quant(res[3]) << 24);
    }
}

}  // namespace

struct cvx_display {
    int device = 0;  // current at creation
    uint32_t w = 0, h = 0, slot = 0;
    uint32_t *d_frame = nullptr, *d_gbuf = nullptr, *d_ring = nullptr, *d_scratch = nullptr, *d_out = nullptr;
    uint8_t *d_tex1 = nullptr, *d_tex2 = nullptr;
    uint32_t tw = 1, th = 1;
    PostTables* d_tab = nullptr;
    cudaStream_t stream = nullptr;
    ~cvx_display() {
        cudaFree(d_frame);
        cudaFree(d_gbuf);
        cudaFree(d_ring);
        cudaFree(d_scratch);
        cudaFree(d_out);
        cudaFree(d_tex1);
        cudaFree(d_tex2);
        cudaFree(d_tab);
        if (stream) cudaStreamDestroy(stream);
    }
};

static int32_t cerr(cudaError_t e, const char* what) {
    return cvx::set_error(CVX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define PCK(call, what)                                   \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cerr(e_, what);     \
    } while (0)

// sRGB transfer tables, computed in double on the host.
static void make_tables(PostTables* t) {
    for (int i = 0; i < 256; i++) {
        double s = i / 255.0;
        double l = s <= 0.04045 ? s / 12.92 : std::pow((s + 0.055) / 1.055, 2.4);
        t->srgb_decode[i] = (float)l;
    }
    for (int k = 1; k <= 255; k++) {  // linear value at which the encoded byte reaches k
        double s = (k - 0.5) / 255.0;
        double l = s <= 0.04045 ? s / 12.92 : std::pow((s + 0.055) / 1.055, 2.4);
        t->srgb_encode[k - 1] = (float)l;
    }
}

extern "C" {

int32_t cvx_display_create(uint32_t width, uint32_t height, const uint8_t* tex1_rgb, const uint8_t* tex2_rgb,
                           uint32_t tex_w, uint32_t tex_h, cvx_display** out) {
    if (!out || !width || !height || !tex1_rgb || !tex2_rgb || !tex_w || !tex_h)
        return cvx::set_error(CVX_ERR_INVALID, "bad display arguments");
    // Pixel and texel indices are 32-bit in the kernels.
    if (width > CVX_MAX_IMAGE_SIDE || height > CVX_MAX_IMAGE_SIDE || tex_w > CVX_MAX_IMAGE_SIDE ||
        tex_h > CVX_MAX_IMAGE_SIDE)
        return cvx::set_error(CVX_ERR_INVALID, "display and texture sides are limited to 16384 pixels");
    std::unique_ptr<cvx_display> d(new cvx_display());
    d->device = cvx::current_device();
    if (d->device < 0) return cvx::set_error(CVX_ERR_CUDA, "no CUDA device available");
    d->w = width;
    d->h = height;
    d->tw = tex_w;
    d->th = tex_h;
    size_t npx = (size_t)width * height, tb = (size_t)tex_w * tex_h * 3;
    PCK(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    PCK(cudaMalloc(&d->d_frame, npx * 4), "cudaMalloc");
    PCK(cudaMalloc(&d->d_gbuf, npx * 4), "cudaMalloc");
    PCK(cudaMalloc(&d->d_ring, npx * 4 * 8), "cudaMalloc");
    PCK(cudaMalloc(&d->d_scratch, npx * 4), "cudaMalloc");
    PCK(cudaMalloc(&d->d_out, npx * 4), "cudaMalloc");
    PCK(cudaMalloc(&d->d_tex1, tb), "cudaMalloc");
    PCK(cudaMalloc(&d->d_tex2, tb), "cudaMalloc");
    PCK(cudaMalloc(&d->d_tab, sizeof(PostTables)), "cudaMalloc");
    PostTables t;
    make_tables(&t);
    PCK(cudaMemcpy(d->d_tab, &t, sizeof t, cudaMemcpyHostToDevice), "upload tables");
    PCK(cudaMemcpy(d->d_tex1, tex1_rgb, tb, cudaMemcpyHostToDevice), "upload texture");
    PCK(cudaMemcpy(d->d_tex2, tex2_rgb, tb, cudaMemcpyHostToDevice), "upload texture");
    PCK(cudaMemset(d->d_ring, 0, npx * 4 * 8), "clear frames");  // black_bitmap (ui.rs:232-239)
    *out = d.release();
    return CVX_OK;
}

int32_t cvx_display_frame(cvx_display* d, const uint32_t* rgba, const uint32_t* gbuffer, uint32_t enable_blend,
                          uint32_t enable_median, uint32_t* out_srgb) {
    if (!d || !rgba || !gbuffer || !out_srgb) return cvx::set_error(CVX_ERR_INVALID, "null argument");
    CVX_ON_DEVICE(d->device);
    cvx::StreamSync sync(d->stream);
    uint32_t npx = d->w * d->h;
    PCK(cudaMemcpyAsync(d->d_frame, rgba, (size_t)npx * 4, cudaMemcpyHostToDevice, d->stream), "upload frame");
    PCK(cudaMemcpyAsync(d->d_gbuf, gbuffer, (size_t)npx * 4, cudaMemcpyHostToDevice, d->stream), "upload gbuffer");
    d->slot = (d->slot + 1) % 8;  // ui.rs:330
    uint32_t blocks = (npx + 255) / 256;
    if (blocks > 2048) blocks = 2048;
    Tex t1{d->d_tex1, d->tw, d->th}, t2{d->d_tex2, d->tw, d->th};
    k_post_gbuffer<<<blocks, 256, 0, d->stream>>>(d->d_frame, d->d_gbuf, npx, t1, t2, d->d_tab,
                                                 d->d_ring + (size_t)d->slot * npx);
    k_post_blend<<<blocks, 256, 0, d->stream>>>(d->d_ring, npx, enable_blend ? -1 : (int)d->slot, d->d_scratch);
    k_post_median<<<blocks, 256, 0, d->stream>>>(d->d_scratch, d->w, d->h, enable_median ? 1 : 0, d->d_tab,
                                                d->d_out);
    PCK(cudaGetLastError(), "post-process launch");
    PCK(cudaMemcpyAsync(out_srgb, d->d_out, (size_t)npx * 4, cudaMemcpyDeviceToHost, d->stream), "copy output");
    PCK(cudaStreamSynchronize(d->stream), "post-process");
    return CVX_OK;
}

void cvx_display_destroy(cvx_display* d) {
    if (!d) return;
    cvx::DeviceGuard g(d->device);
    delete d;
}

}  // extern "C"
