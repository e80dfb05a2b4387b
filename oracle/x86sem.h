// ORACLE / TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py may load anything under oracle/.
//
// Scalar restatement of the x86 AVX semantics that the reference path tracer
// relies on (simd.rs). Portable C++: no intrinsics, so it builds and gives the
// same results on x86-64 and aarch64. Compile with -ffp-contract=off; every
// fused multiply-add below is an explicit std::fma, as in the reference
// (simd.rs:82-94 mul_add / mul_sub / neg_mul_add).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "x86_approx_tables.h"

namespace orc {

static const uint32_t kRcpMant[2048] = CVX_RCP_TABLE_INIT;
static const uint32_t kRsqrtMant[2048] = CVX_RSQRT_TABLE_INIT;

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// _mm256_rcp_ps (simd.rs:254-256 `recip_fast`), emulated bit-exactly from the
// table of the hardware's results. Zero and denormal inputs give a signed
// infinity, infinities give a signed zero, results below the normal range are
// flushed to a signed zero, NaNs are quieted.
inline float rcp(float x) {
    uint32_t u = fbits(x), s = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    if (e == 255u) return bitsf(m ? (u | 0x00400000u) : s);
    if (e == 0u) return bitsf(s | 0x7f800000u);
    int ne = 126 - ((int)e - 127);
    if (ne <= 0) return bitsf(s);
    return bitsf(s | ((uint32_t)ne << 23) | kRcpMant[m >> 12]);
}

// _mm256_rsqrt_ps (simd.rs:309-311 `rsqrt`), emulated bit-exactly. Negative
// non-zero inputs give the x86 default NaN 0xffc00000.
inline float rsqrt(float x) {
    uint32_t u = fbits(x), s = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    if (e == 255u && m) return bitsf(u | 0x00400000u);
    if (e == 0u) return bitsf(s | 0x7f800000u);
    if (s) return bitsf(0xffc00000u);
    if (e == 255u) return 0.0f;
    int k = (int)e - 127, odd = k & 1, half = (k - odd) / 2;
    return bitsf(((uint32_t)(126 - half) << 23) | kRsqrtMant[(odd << 10) | (m >> 13)]);
}

// Sign bit as the AVX mask instructions see it (blendv, testc, movemask).
// Every NaN that x86 arithmetic generates is the default NaN 0xffc00000,
// whose sign bit is set; no NaN enters the path as input. So a NaN counts as
// negative here, whatever sign the host's own arithmetic gave it.
inline bool sneg(float x) { return (fbits(x) >> 31) != 0u || x != x; }

// _mm256_min_ps / _mm256_max_ps: `a < b ? a : b` / `a > b ? a : b`, so the
// second operand wins when either is NaN (simd.rs:318-326).
inline float xmin(float a, float b) { return a < b ? a : b; }
inline float xmax(float a, float b) { return a > b ? a : b; }

// _mm256_cmp_ps(a, b, 21): not-less-than, unordered is true (simd.rs:329-333).
inline bool geq(float a, float b) { return !(a < b); }

inline float fmadd(float a, float b, float c) { return std::fma(a, b, c); }    // a*b + c
inline float fmsub(float a, float b, float c) { return std::fma(a, b, -c); }   // a*b - c
inline float fnmadd(float a, float b, float c) { return std::fma(-a, b, c); }  // c - a*b

// `Neg for Mf32` is `0 - x` (simd.rs:578-592): -(+0) and -(-0) are both +0.
inline float neg(float x) { return 0.0f - x; }
inline float fabs_bits(float x) { return bitsf(fbits(x) & 0x7fffffffu); }

// _mm256_cvtps_epi32: round to nearest even; NaN and out-of-range inputs give
// the integer indefinite value 0x80000000.
inline int32_t cvtps(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)std::nearbyint(x);
}

// Polynomial cosine and sine (simd.rs:190-239).
inline float poly_cos(float x) {
    const float a = -0.496000299455f, b = 0.0392596924214f, c = -0.000966231179636657107f;
    float x2 = x * x, x4 = x2 * x2, x6 = x2 * x4;
    return fmadd(x6, c, fmadd(x4, b, fmadd(x2, a, 1.0f)));
}
inline float poly_sin(float x) {
    const float a = 0.982006669405f, b = -0.152175915294f, c = 0.00533738081738135917f;
    float x2 = x * x, x3 = x * x2, x5 = x3 * x2;
    return fmadd(x5, c, fmadd(x3, b, x * a));
}
// Rational inverse cosines (simd.rs:105-178); not on the render path.
inline float poly_acos_fast(float x) {
    const float z = 1.57079632679489661923f;
    const float a = -1.010967650783108321215466002435f, b = 0.7187490034089083954058416974792f,
                c = -0.8139678312270743216751354761334f;
    float x2 = x * x, x3 = x * x2;
    float numer = fmadd(x3, b, a * x), denom = fmadd(x2, c, 1.0f);
    return fmadd(numer, rcp(denom), z);
}
inline float poly_acos(float x) {
    const float z = 1.57079632679489661923f;
    const float a = -0.939115566365855f, b = 0.9217841528914573f, c = -1.2845906244690837f,
                d = 0.295624144969963174f;
    float x2 = x * x, x3 = x * x2, x4 = x2 * x2;
    float numer = fmadd(x3, b, a * x), denom = fmadd(x4, d, fmadd(x2, c, 1.0f));
    return fmadd(numer, rcp(denom), z);
}
// simd.rs:266-269
inline float recip_precise(float x) {
    float x0 = rcp(x);
    return fnmadd(x, x0 * x0, x0 + x0);
}

const float kPi = 3.14159265358979323846f;

}  // namespace orc
