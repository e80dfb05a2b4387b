// Device-side arithmetic with the semantics of the x86 AVX instructions that
// the reference path tracer is written in (simd.rs). Every kernel that
// includes this header is compiled with -fmad=false: a plain `a * b + c`
// rounds twice, as an unfused AVX mul and add do, and every fused
// multiply-add the reference asks for (mul_add, mul_sub, neg_mul_add,
// simd.rs:82-94) is an explicit fmaf.
#pragma once
#include <cstdint>

#include "x86_approx_tables.h"

namespace cvx {

// 12-bit mantissa fragments (bits 22..11) of the VRCPPS / VRSQRTPS results;
// bits 10..0 of every entry are zero and the exponent is always 126.
struct ApproxTables {
    uint16_t rcp[2048];
    uint16_t rsqrt[2048];
};

__device__ __forceinline__ uint32_t fb(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float bf(uint32_t u) { return __uint_as_float(u); }

// _mm256_rcp_ps (recip_fast, simd.rs:254-256), bit-exact.
__device__ __forceinline__ float x_rcp(float x, const ApproxTables& t) {
    uint32_t u = fb(x), s = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    int ne = 253 - (int)e;
    uint32_t r = s | ((uint32_t)ne << 23) | ((uint32_t)t.rcp[m >> 12] << 11);
    r = ne <= 0 ? s : r;
    r = e == 0u ? (s | 0x7f800000u) : r;
    r = e == 255u ? (m ? (u | 0x00400000u) : s) : r;
    return bf(r);
}

// _mm256_rsqrt_ps (simd.rs:309-311), bit-exact.
__device__ __forceinline__ float x_rsqrt(float x, const ApproxTables& t) {
    uint32_t u = fb(x), s = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    int k = (int)e - 127, odd = k & 1, half = (k - odd) >> 1;
    uint32_t r = ((uint32_t)(126 - half) << 23) | ((uint32_t)t.rsqrt[(odd << 10) | (m >> 13)] << 11);
    r = (e == 255u) ? (m ? (u | 0x00400000u) : 0u) : r;
    r = (s && !(e == 255u && m) && e != 0u) ? 0xffc00000u : r;
    r = e == 0u ? (s | 0x7f800000u) : r;
    return bf(r);
}

// Sign bit as the AVX mask instructions read it. x86 arithmetic generates only
// the default NaN 0xffc00000 (sign set) and no NaN enters as input, so a NaN
// counts as negative here; the GPU's own NaNs are positive.
__device__ __forceinline__ bool sneg(float x) { return (int32_t)fb(x) < 0 || x != x; }
__device__ __forceinline__ float xmin(float a, float b) { return a < b ? a : b; }  // _mm256_min_ps
__device__ __forceinline__ float xmax(float a, float b) { return a > b ? a : b; }  // _mm256_max_ps
__device__ __forceinline__ bool geq(float a, float b) { return !(a < b); }          // cmp NLT_UQ
__device__ __forceinline__ float fmsub(float a, float b, float c) { return fmaf(a, b, -c); }
__device__ __forceinline__ float fnmadd(float a, float b, float c) { return fmaf(-a, b, c); }
__device__ __forceinline__ float neg0(float x) { return 0.0f - x; }  // Neg for Mf32 is 0 - x
__device__ __forceinline__ float fabs_bits(float x) { return bf(fb(x) & 0x7fffffffu); }

// _mm256_cvtps_epi32: nearest-even; NaN and out of range give 0x80000000.
__device__ __forceinline__ int32_t x_cvtps(float x) {
    bool ok = x >= -2147483648.0f && x < 2147483648.0f;
    return ok ? __float2int_rn(x) : INT32_MIN;
}

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 mulk(F3 a, float k) { return f3(a.x * k, a.y * k, a.z * k); }
__device__ __forceinline__ F3 vneg0(F3 a) { return f3(neg0(a.x), neg0(a.y), neg0(a.z)); }
// MVector3::dot is the naive, unfused form (vector3.rs:202-217).
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// MVector3::cross is cross_fma (vector3.rs:186-199).
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
    return f3(fmsub(a.y, b.z, a.z * b.y), fmsub(a.z, b.x, a.x * b.z), fmsub(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ F3 vfma(F3 a, float k, F3 b) {
    return f3(fmaf(a.x, k, b.x), fmaf(a.y, k, b.y), fmaf(a.z, k, b.z));
}
__device__ __forceinline__ F3 normalized(F3 a, const ApproxTables& t) {
    float r = x_rsqrt(dot(a, a), t);
    return f3(a.x * r, a.y * r, a.z * r);
}

// Polynomial sine and cosine of the reference (simd.rs:190-239).
__device__ __forceinline__ float poly_cos(float x) {
    float x2 = x * x, x4 = x2 * x2, x6 = x2 * x4;
    return fmaf(x6, -0.000966231179636657107f, fmaf(x4, 0.0392596924214f, fmaf(x2, -0.496000299455f, 1.0f)));
}
__device__ __forceinline__ float poly_sin(float x) {
    float x2 = x * x, x3 = x * x2, x5 = x3 * x2;
    return fmaf(x5, 0.00533738081738135917f, fmaf(x3, -0.152175915294f, x * 0.982006669405f));
}

constexpr float kPi = 3.14159265358979323846f;

}  // namespace cvx
