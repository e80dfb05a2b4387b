/*
 * Generates x86_approx_tables.h: the results of the x86 approximate
 * reciprocal (VRCPPS, `_mm256_rcp_ps`) and approximate reciprocal square root
 * (VRSQRTPS, `_mm256_rsqrt_ps`) on the host CPU, for every input that the
 * result depends on.
 *
 * The reference path tracer calls these two instructions through
 * `Mf32::recip_fast` (simd.rs:254-256) and `Mf32::rsqrt` (simd.rs:309-311).
 * On Intel CPUs their result for a normal input depends only on the top 11
 * mantissa bits (rcp) or on the top 10 mantissa bits plus the parity of the
 * exponent (rsqrt); the exponent of the result then follows from the input
 * exponent. This program records the results for inputs in [1, 2) (rcp) and
 * [1, 4) (rsqrt), then checks the table-driven emulation against the hardware
 * on a stride of all 2^32 inputs (pass --exhaustive to check every input).
 *
 * x86-64 only: it is a generator and a check, not part of the build.
 * Build: gcc -O2 -mavx2 gen_x86_approx_tables.c -o gen && ./gen > x86_approx_tables.h
 */
#include <immintrin.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static uint32_t rcp_mant[2048];
static uint32_t rsqrt_mant[2048];

static uint32_t hw_rcp(uint32_t x) {
    float f; memcpy(&f, &x, 4);
    __m256 v = _mm256_rcp_ps(_mm256_set1_ps(f));
    float o[8]; _mm256_storeu_ps(o, v);
    uint32_t r; memcpy(&r, &o[0], 4); return r;
}
static uint32_t hw_rsqrt(uint32_t x) {
    float f; memcpy(&f, &x, 4);
    __m256 v = _mm256_rsqrt_ps(_mm256_set1_ps(f));
    float o[8]; _mm256_storeu_ps(o, v);
    uint32_t r; memcpy(&r, &o[0], 4); return r;
}

/* The emulation, written the same way the product and the oracle use it. */
static uint32_t em_rcp(uint32_t x) {
    uint32_t s = x & 0x80000000u, e = (x >> 23) & 0xffu, m = x & 0x7fffffu;
    if (e == 255u) return m ? (x | 0x00400000u) : s;
    if (e == 0u) return s | 0x7f800000u;
    int ne = 126 - ((int)e - 127);
    if (ne <= 0) return s;
    return s | ((uint32_t)ne << 23) | rcp_mant[m >> 12];
}
static uint32_t em_rsqrt(uint32_t x) {
    uint32_t s = x & 0x80000000u, e = (x >> 23) & 0xffu, m = x & 0x7fffffu;
    if (e == 255u && m) return x | 0x00400000u;
    if (e == 0u) return s | 0x7f800000u;
    if (s) return 0xffc00000u;
    if (e == 255u) return 0u;
    int k = (int)e - 127, odd = k & 1, half = (k - odd) / 2;
    return ((uint32_t)(126 - half) << 23) | rsqrt_mant[(odd << 10) | (m >> 13)];
}

int main(int argc, char** argv) {
    int exhaustive = argc > 1 && strcmp(argv[1], "--exhaustive") == 0;
    for (uint32_t i = 0; i < 2048; i++) {
        uint32_t r = hw_rcp(0x3f800000u | (i << 12));
        if (((r >> 23) & 0xffu) != 126u || (r >> 31)) { fprintf(stderr, "unexpected rcp exponent\n"); return 1; }
        rcp_mant[i] = r & 0x7fffffu;
    }
    for (uint32_t p = 0; p < 2; p++)
        for (uint32_t i = 0; i < 1024; i++) {
            uint32_t r = hw_rsqrt(((127u + p) << 23) | (i << 13));
            if (((r >> 23) & 0xffu) != 126u || (r >> 31)) { fprintf(stderr, "unexpected rsqrt exponent\n"); return 1; }
            rsqrt_mant[(p << 10) | i] = r & 0x7fffffu;
        }
    uint64_t step = exhaustive ? 1 : 97, bad = 0, n = 0;
    for (uint64_t x = 0; x < (1ull << 32); x += step, n++) {
        uint32_t u = (uint32_t)x;
        if (hw_rcp(u) != em_rcp(u) || hw_rsqrt(u) != em_rsqrt(u)) bad++;
    }
    if (bad) { fprintf(stderr, "emulation mismatch on %llu of %llu inputs\n", (unsigned long long)bad, (unsigned long long)n); return 1; }
    fprintf(stderr, "emulation matches hardware on %llu inputs\n", (unsigned long long)n);

    printf("/* Generated by gen_x86_approx_tables.c on an x86-64 host: mantissas of the\n"
           " * VRCPPS / VRSQRTPS results for inputs in [1,2) (rcp, index = top 11\n"
           " * mantissa bits) and [1,4) (rsqrt, index = exponent parity << 10 | top 10\n"
           " * mantissa bits). Every result has biased exponent 126. Do not edit. */\n");
    printf("#ifndef CVX_X86_APPROX_TABLES_H\n#define CVX_X86_APPROX_TABLES_H\n#include <stdint.h>\n");
    printf("#define CVX_RCP_TABLE_INIT {");
    for (int i = 0; i < 2048; i++) printf("%s0x%06xu", i ? (i % 8 ? "," : ",\\\n  ") : "\\\n  ", rcp_mant[i]);
    printf("}\n#define CVX_RSQRT_TABLE_INIT {");
    for (int i = 0; i < 2048; i++) printf("%s0x%06xu", i ? (i % 8 ? "," : ",\\\n  ") : "\\\n  ", rsqrt_mant[i]);
    printf("}\n#endif\n");
    return 0;
}
