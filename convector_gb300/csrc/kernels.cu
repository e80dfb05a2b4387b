// Kernels of the render hot path and their launchers (declared in kernels.h).
// Compiled with -fmad=false (see x86sem.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "kernels.h"
#include "path_refill.cuh"
#include "shade.cuh"

namespace cvx {

__device__ ApproxTables g_tables;

// Copies the 8 KB approximation tables into shared memory.
__device__ __forceinline__ void load_tables(ApproxTables& sm) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&g_tables);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&sm);
    for (int i = threadIdx.x; i < (int)(sizeof(ApproxTables) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Scene preparation

__global__ void k_prep_geom(const cvx_triangle* __restrict__ tris, uint32_t n, float4* __restrict__ geom,
                            TriShade* __restrict__ shade) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const cvx_triangle& t = tris[i];
        F3 v0 = f3(t.v0[0], t.v0[1], t.v0[2]), v1 = f3(t.v1[0], t.v1[1], t.v1[2]), v2 = f3(t.v2[0], t.v2[1], t.v2[2]);
        F3 e1 = sub(v0, v2), e2 = sub(v1, v0);
        F3 n = cross(e1, e2);
        geom[3 * i] = make_float4(v0.x, v0.y, v0.z, n.x);
        geom[3 * i + 1] = make_float4(e1.x, e1.y, e1.z, n.y);
        geom[3 * i + 2] = make_float4(e2.x, e2.y, e2.z, n.z);
        TriShade s;
        s.uv[0] = t.uv0[0];
        s.uv[1] = t.uv0[1];
        s.uv[2] = t.uv1[0];
        s.uv[3] = t.uv1[1];
        s.uv[4] = t.uv2[0];
        s.uv[5] = t.uv2[1];
        s.material = t.material;
        s.pad = 0u;
        shade[i] = s;
    }
}

// LightRec (5 x float4): v0 area | e1 rnorm | e2 - | n - | normal -
__global__ void k_prep_lights(const cvx_triangle* __restrict__ tris, const uint32_t* __restrict__ ds, uint32_t n,
                              float4* __restrict__ lights) {
    __shared__ ApproxTables tab;
    load_tables(tab);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const cvx_triangle& t = tris[ds[i]];
        F3 v0 = f3(t.v0[0], t.v0[1], t.v0[2]), v1 = f3(t.v1[0], t.v1[1], t.v1[2]), v2 = f3(t.v2[0], t.v2[1], t.v2[2]);
        F3 e1 = sub(v0, v2), e2 = sub(v1, v0);
        F3 nn = cross(e1, e2);
        float rnorm = x_rsqrt(dot(nn, nn), tab);
        float area = 0.5f * x_rcp(rnorm, tab);
        F3 normal = mulk(nn, rnorm);
        lights[5 * i] = make_float4(v0.x, v0.y, v0.z, area);
        lights[5 * i + 1] = make_float4(e1.x, e1.y, e1.z, rnorm);
        lights[5 * i + 2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
        lights[5 * i + 3] = make_float4(nn.x, nn.y, nn.z, 0.0f);
        lights[5 * i + 4] = make_float4(normal.x, normal.y, normal.z, 0.0f);
    }
}

// ---------------------------------------------------------------------------
// Nearest hit over SoA rays (Bvh::intersect_nearest, bvh.rs:659). The packet
// form (k_intersect<true>: eight consecutive rays are one reference packet)
// is the reference's traversal exactly; the single-ray form is
// k_intersect_refill below.

// Next unit (group or packet) index for the calling octet (one atomic by its lane 0).
__device__ __forceinline__ uint32_t octet_claim(uint32_t* counter, unsigned omask, int k) {
    uint32_t g = 0;
    if (k == 0) g = atomicAdd(counter, 1u);
    return __shfl_sync(omask, g, (int)(threadIdx.x & 24u));
}

template <bool PACKET>
__global__ void __launch_bounds__(256) k_intersect(DeviceScene s, const RayCols rays, uint32_t n,
                                                   float far_dist, float* __restrict__ t_out,
                                                   int32_t* __restrict__ tri_out, uint32_t* __restrict__ counters,
                                                   uint32_t* __restrict__ err) {
    __shared__ ApproxTables tab;
    load_tables(tab);
    const unsigned omask = 0xffu << (threadIdx.x & 24u);
    const int k = threadIdx.x & 7;
    const uint32_t npk = (n + 7u) >> 3;
    // Packets (8 consecutive rays, one per octet) claimed one at a time from err[1].
    for (uint32_t pk = octet_claim(err + 1, omask, k); pk < npk; pk = octet_claim(err + 1, omask, k)) {
        uint32_t i = pk * 8u + (uint32_t)k;
        bool active = i < n;
        uint32_t src = active ? i : (i & ~7u);
        F3 o = f3(__ldg(rays.c[0] + src), __ldg(rays.c[1] + src), __ldg(rays.c[2] + src));
        F3 d = f3(__ldg(rays.c[3] + src), __ldg(rays.c[4] + src), __ldg(rays.c[5] + src));
        Hit h{far_dist, 0.0f, 0.0f, -1};
        Counters c{0u, 0u};
        bool ok = true;
        // The select-form slab test for a packet whose 8 rays all allow it,
        // decided once per packet outside the traversal loop (4M random rays:
        // 3.05 -> 2.92 ms; the same results).
        const bool sel = PACKET && s.slab_sel && !counters &&
                         oct_all(omask, select_form_ray(f3(x_rcp(d.x, tab), x_rcp(d.y, tab), x_rcp(d.z, tab))));
        if (sel) ok = traverse<true, true>(s, o, d, active, omask, h, tab, nullptr);
        else if (PACKET || active) ok = traverse<PACKET>(s, o, d, active, omask, h, tab, counters ? &c : nullptr);
        if (!ok) atomicOr(err, kErrStackOverflow);
        if (active) {
            t_out[i] = h.t;
            tri_out[i] = h.tri;
            if (counters) {
                counters[i] = c.aabb;
                counters[n + i] = c.tri;
            }
        }
    }
}

constexpr int32_t kDeferredRay = -2;  // never a hit index: -1 is the miss

// Ray source of the isolated nearest-hit query: SoA rays in, (t, index) out.
struct SoaRays {
    const float4* nodes;
    const float4* geom;
    RayCols rays;
    uint32_t n;
    float far_dist;
    float* t_out;
    int32_t* tri_out;
    uint32_t* counters;
    __device__ __forceinline__ bool load(uint32_t r, F3& o, F3& d, float& far, const float4*& nd,
                                         const float4*& gm) const {
        nd = nodes;
        gm = geom;
        o = f3(__ldg(rays.c[0] + r), __ldg(rays.c[1] + r), __ldg(rays.c[2] + r));
        d = f3(__ldg(rays.c[3] + r), __ldg(rays.c[4] + r), __ldg(rays.c[5] + r));
        far = far_dist;
        return true;
    }
    // A ray left to k_intersect_deferred (its index word holds kDeferredRay).
    __device__ __forceinline__ void defer(uint32_t r) const { tri_out[r] = kDeferredRay; }
    __device__ __forceinline__ void store(uint32_t r, const Hit& h, uint32_t na, uint32_t nt) const {
        t_out[r] = h.t;
        tri_out[r] = h.tri;
        if (counters) {
            counters[r] = na;
            counters[n + r] = nt;
        }
    }
};

// Staged ray supply of the isolated query: a warp claims 32 consecutive rays
// at a time and copies them into shared memory with cp.async, one batch ahead
// of use. A lane that finishes a ray takes the next one from shared memory, so
// neither the claim's atomic nor the ray's DRAM load stalls the warp.
struct StagedSoaClaim {
    const SoaRays& src;
    uint32_t* next_ray;
    float (*buf)[6][32];  // this warp's two batches: [batch][component][slot]
    uint32_t base_cur, base_nxt, used;
    int cur;

    __device__ __forceinline__ uint32_t claim32(int lane) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(next_ray, 32u);
        return __shfl_sync(0xffffffffu, b, 0);
    }
    __device__ __forceinline__ void issue(int which, uint32_t base, int lane) {
        uint32_t r = base + (uint32_t)lane;
        if (r < src.n)
            for (int c = 0; c < 6; c++) cp_async4(&buf[which][c][lane], src.rays.c[c] + r);
        cp_async_commit();
    }
    __device__ __forceinline__ void init(int lane) {
        base_cur = claim32(lane);
        issue(0, base_cur, lane);
        base_nxt = claim32(lane);
        issue(1, base_nxt, lane);
        cp_async_wait_one_pending();
        __syncwarp();
        cur = 0;
        used = 0;
    }
    __device__ __forceinline__ int claim(unsigned b, bool want, int lane, uint32_t& r, RayIn& in) {
        uint32_t k = (uint32_t)__popc(b);
        if (used + k > 32u) {  // some lanes take from the next batch: it must have landed
            cp_async_wait_all();
            __syncwarp();
        }
        int res = kClaimNone;
        if (want) {
            uint32_t t = used + (uint32_t)__popc(b & ((1u << lane) - 1u));
            int which = t < 32u ? cur : cur ^ 1;
            uint32_t slot = t & 31u;
            r = (t < 32u ? base_cur : base_nxt) + slot;
            if (r < src.n) {
                in.o = f3(buf[which][0][slot], buf[which][1][slot], buf[which][2][slot]);
                in.d = f3(buf[which][3][slot], buf[which][4][slot], buf[which][5][slot]);
                in.far = src.far_dist;
                in.nodes = src.nodes;
                in.geom = src.geom;
                res = kClaimRay;
            } else {
                res = kClaimDone;
            }
        }
        used += k;
        if (used >= 32u) {  // the current batch is used up: the next one becomes current
            __syncwarp();    // every read of the old batch is done
            used -= 32u;
            cur ^= 1;
            base_cur = base_nxt;
            cp_async_wait_all();
            __syncwarp();
            base_nxt = claim32(lane);
            issue(cur ^ 1, base_nxt, lane);
        }
        return res;
    }
};

// MINB: resident blocks per SM the register allocation must allow (8: the
// compiler's choice, 64 registers; 10 and 12 cap registers for occupancy).
// CLAIM: lanes without a ray wait until this many want one. Short traversals
// (shallow trees) gain from large batches of claims, long ones lose more to
// the waiting: 16 for trees up to 40 levels, 8 beyond (measured on the
// 82k-triangle icosphere and on the 70-level tube).
// The first entries of each lane's traversal stack live in shared memory,
// the deeper ones in local memory. Pops of local entries missed L1 about a
// third of the time (68.7 % hit rate); measured on 4M rays: 0.905 ms with none
// shared, 0.890 with 4, 0.878 with 8, 0.883 with 12. (The wavefront and the
// path-refill traversals, whose larger working sets need the L1 that the
// carve-out takes, measured no gain or a loss.)
// Traversal steps a lane takes per round of the warp's claim votes: 1, 3, 4
// -> 0.798, 0.784, 0.777 ms per 4M rays of the 28-level icosphere (12 shared
// stack entries) and 1.538, 1.503, 1.499 ms on the 70-level tube (medians of
// three runs each; six steps: 0.774-0.778 and 1.474-1.482, within noise). The
// claim thresholds, swept again at four steps, stay at 16 (12, 16, 20 on the
// icosphere: 0.774-0.780, 0.776-0.778, 0.792-0.796 ms) and 8 for trees deeper
// than 40 levels (6, 8, 12 on the tube: 1.499, 1.489-1.513, 1.493 ms). A leaf
// reached from a pair tested in the same step (the frame kernels' form) is
// slower here at 2, 3 and 4 steps: 0.84, 0.82-0.84, 0.82 ms on the icosphere.
constexpr int kQuerySteps = 4;
// The default; a scene may choose 0, 4 or 12 instead (cvx_scene_set_query_stack,
// which the query autotuner sets per scene).
constexpr int kQueryStackShared = 8;

// SELECT: the select-form slab test for the rays that meet its conditions
// (on scenes that do); the others are marked kDeferredRay and traced by
// k_intersect_deferred. Measured on 4M rays: 0.844 against 0.877 ms.
// SHARED: stack entries of each lane in shared memory (the rest in local).
template <int MINB, bool COUNT, int CLAIM, bool SELECT, int SHARED = kQueryStackShared>
__global__ void __launch_bounds__(128, MINB) k_intersect_refill(SoaRays src, uint32_t* __restrict__ next_ray,
                                                                uint32_t* __restrict__ err) {
    // The reciprocal table is read three times per ray: from global memory
    // (L1-resident), which leaves the shared-memory carve-out to L1.
    __shared__ float stage[4][2][6][32];
    __shared__ uint2 sstack[4][SHARED > 0 ? SHARED : 1][32];
    StagedSoaClaim claim{src, next_ray, stage[threadIdx.x >> 5], 0u, 0u, 0u, 0};
    claim.init(threadIdx.x & 31);
    bool ok = traverse_refill<COUNT, false, CLAIM, SHARED, SELECT, kQuerySteps>(
        src, claim, g_tables, &sstack[threadIdx.x >> 5][0][threadIdx.x & 31]);
    if (!ok) atomicOr(err, kErrStackOverflow);
}

// After k_intersect_refill<SELECT>: the rays it left (index word kDeferredRay:
// a reciprocal infinite or below 0.75 in magnitude) with the x86-form slab
// test. Such rays are rare (axis-parallel or very long directions), so the
// scan over the index words is most of the work: each thread reads
// kDeferredScan words spread over the whole array, independent coalesced loads
// in one round (a grid-stride loop of dependent loads took 16 us per 4M rays).
constexpr uint32_t kDeferredScan = 4;
__global__ void __launch_bounds__(256) k_intersect_deferred(SoaRays src, uint32_t* __restrict__ err) {
    const uint32_t stride = gridDim.x * blockDim.x, t = blockIdx.x * blockDim.x + threadIdx.x;
    int32_t w[kDeferredScan];
#pragma unroll
    for (uint32_t k = 0; k < kDeferredScan; k++) {
        const uint64_t r = (uint64_t)t + (uint64_t)k * stride;
        w[k] = r < src.n ? __ldg(src.tri_out + r) : 0;
    }
    bool ok = true;
#pragma unroll 1
    for (uint32_t k = 0; k < kDeferredScan; k++) {
        if (w[k] != kDeferredRay) continue;
        const uint32_t r = t + k * stride;
        F3 o, d;
        float far;
        const float4 *nodes, *geom;
        src.load(r, o, d, far, nodes, geom);
        RefillRay ray;
        uint2 local_stack[kStackDepth];
        LocalStack stack{local_stack};
        ray.top = make_uint2(0u, 0u);
        ray.start(o, d, far, nodes, geom, g_tables);
        bool overflow = false;
        while (!ray.step<false, false>(stack, overflow)) {
        }
        ok &= !overflow;
        src.store(r, ray.h, 0u, 0u);
    }
    if (!ok) atomicOr(err, kErrStackOverflow);
}

// ---------------------------------------------------------------------------
// Frame rendering: one octet renders one 8-pixel group (RNG_GROUP), or walks
// the 128 groups of one 32x32 patch in the reference's order (RNG_PATCH).

struct FrameArgs {
    DeviceScene s;
    DeviceCamera cam;
    uint32_t w, h, frame;
    uint32_t* rgba;
    uint32_t* gbuf;
    float* color;
    float* accum;
    unsigned long long* rays;
    uint32_t* err;
    uint32_t debug;  // Renderer::toggle_debug_view (renderer.rs:150-152)
    // patch order: patch width (a multiple of 16) and the patch origins
    // (x, y pairs; null: every patch of the frame, column by column)
    uint32_t patch;
    const uint32_t* patches;
    uint32_t n_patches;
    // per-lane path refill (k_render_refill): one word per 8-pixel group,
    // zero at launch
    uint32_t* group_em;
    // the counting form of k_render_refill: totals of boxes and triangles
    // tested and of light-PDF shading steps (3 words, zero at launch)
    unsigned long long* work;
    // k_render_refill: samples rendered by the launch (frames frame ..
    // frame + samples - 1, their paths claimed sample after sample). The last
    // sample writes the frame buffers as a one-sample launch does (without the
    // accumulator); sample s < samples - 1 writes its linear colour to
    // sample_color + 3 * w * h * s, for k_accumulate_samples.
    uint32_t samples;
    float* sample_color;
};

// Screen x (or y) of lane k of group g of the 16x4 block at (xb, yb), before
// jitter (renderer.rs:171-198).
__device__ __forceinline__ void block_coord(uint32_t w, uint32_t h, uint32_t xb, uint32_t yb, int g, int k,
                                            float* x, float* y, float* scale_out) {
    float scale = 2.0f / (float)w;
    float s2 = 2.0f * scale, s4 = 4.0f * scale, s8 = 8.0f * scale, s12 = 12.0f * scale;
    float bx = scale * ((float)(k & 3) + ((float)xb - (float)w * 0.5f));
    float by = scale * ((float)(k >> 2) + ((float)yb - (float)h * 0.5f));
    int col = g >> 1;
    float gx = col == 0 ? bx : col == 1 ? bx + s4 : col == 2 ? bx + s8 : bx + s12;
    float gy = (g & 1) ? by + s2 : by;
    *x = gx;
    *y = gy;
    *scale_out = scale;
}

__device__ __forceinline__ void store_pixel(const FrameArgs& a, uint32_t px, uint32_t py, const PixelOut& p) {
    if (px >= a.w || py >= a.h) return;
    size_t idx = (size_t)py * a.w + px;
    if (a.rgba) a.rgba[idx] = pack_color(p.color);
    if (a.gbuf) a.gbuf[idx] = pack_gbuffer(p);
    if (a.color) {
        a.color[3 * idx] = p.color.x;
        a.color[3 * idx + 1] = p.color.y;
        a.color[3 * idx + 2] = p.color.z;
    }
    if (a.accum) {
        a.accum[3 * idx] += p.color.x;
        a.accum[3 * idx + 1] += p.color.y;
        a.accum[3 * idx + 2] += p.color.z;
    }
}

__device__ __forceinline__ void flush_rays(const FrameArgs& a, uint32_t rays) {
    unsigned long long v = rays;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31u) == 0u && v) atomicAdd(a.rays, v);
}

template <bool PACKET>
__global__ void __launch_bounds__(128, 8) k_render_group(FrameArgs a) {
    __shared__ ApproxTables tab;
    load_tables(tab);
    const int k = threadIdx.x & 7;
    const unsigned omask = 0xffu << (threadIdx.x & 24u);
    const uint32_t bw = (a.w + 15u) / 16u, bh = (a.h + 3u) / 4u;
    const uint32_t ngroups = bw * bh * 8u;
    uint32_t rays = 0;
    bool ok = true;
    // Octet index runs through the 8 groups of a 16x4 block, then blocks in
    // row-major order, so a warp covers half a block.
    // Groups are claimed one at a time by each octet (a counter in a.err[1]):
    // paths end after 1 to 5 bounces, so a fixed share of groups per octet
    // leaves some octets working long after the others (room scene frame
    // 0.815 against 0.874 ms with a grid-stride share).
    for (uint32_t gi = octet_claim(a.err + 1, omask, k); gi < ngroups; gi = octet_claim(a.err + 1, omask, k)) {
        uint32_t blk = gi >> 3;
        int g = (int)(gi & 7u);
        uint32_t xb = (blk % bw) * 16u, yb = (blk / bw) * 4u;
        uint32_t gx = xb + 4u * (uint32_t)(g >> 1), gy = yb + 2u * (uint32_t)(g & 1);
        if (gx >= a.w || gy >= a.h) continue;  // whole group outside the frame (octet-uniform)
        float x, y, scale;
        block_coord(a.w, a.h, xb, yb, g, k, &x, &y, &scale);
        LaneRng rng;
        rng.seed(gx, gy, a.frame, k);
        x = fmaf(unit_from(rng.next()), scale, x);
        y = fmaf(unit_from(rng.next()), scale, y);
        PixelOut p;
        if (a.debug) ok &= render_pixels_debug<PACKET>(a.s, a.cam, x, y, omask, tab, p, rays);
        else ok &= render_pixels<PACKET>(a.s, a.cam, x, y, rng, omask, tab, p, rays);
        store_pixel(a, gx + (uint32_t)(k & 3), gy + (uint32_t)(k >> 2), p);
    }
    if (!ok) atomicOr(a.err, kErrStackOverflow);
    flush_rays(a, rays);
}

// Pixel of path p (lane p & 7 of group p >> 3; groups numbered as in
// k_render_group) and its group's origin.
__device__ __forceinline__ void path_pixel(uint32_t p, uint32_t bw, uint32_t& gx, uint32_t& gy, uint32_t& px,
                                           uint32_t& py) {
    uint32_t gi = p >> 3, blk = gi >> 3, g = gi & 7u, k = p & 7u;
    uint32_t xb = (blk % bw) * 16u, yb = (blk / bw) * 4u;
    gx = xb + 4u * (g >> 1);
    gy = yb + 2u * (g & 1u);
    px = gx + (k & 3u);
    py = gy + (k >> 2);
}

// The paths of a launch for path_refill. One sample (MULTI false): path p is
// lane p & 7 of group p >> 3, groups numbered as in k_render_group. MULTI:
// a.samples samples, claimed one after the other: claim number p is path
// p mod per of sample p / per, per being the paths of one sample (a multiple
// of 64, so both numbers share their lane and group-in-block bits). The two
// forms are separate instantiations: the sample logic in the one-sample
// kernel's loop slowed it by 6-7 % (tube 2.945 -> 3.12 ms, room 0.705 ->
// 0.759 ms). The reference keeps the sample, so that only the path's start
// divides (tube 2.356 -> 2.248 ms per sample with 16 per launch, room 0.620 ->
// 0.588 ms).
template <bool MULTI>
struct FramePaths {
    struct PathRef {
        uint32_t path;  // within its sample
        uint32_t smp;
    };
    const FrameArgs& a;
    uint32_t bw, bh, rays;

    __device__ __forceinline__ uint32_t per() const { return bw * bh * 64u; }
    __device__ __forceinline__ uint32_t n_paths() const { return MULTI ? per() * a.samples : per(); }
    __device__ __forceinline__ uint32_t claim(uint32_t n) { return atomicAdd(a.err + 1, n); }
    __device__ __forceinline__ bool begin(uint32_t p, PathRef& r, F3& o, F3& d, LaneRng& rng,
                                          const ApproxTables& tab) {
        const uint32_t smp = MULTI ? p / per() : 0u;
        p -= smp * per();
        uint32_t gx, gy, px, py;
        path_pixel(p, bw, gx, gy, px, py);
        if (gx >= a.w || gy >= a.h) return false;
        r.path = p;
        r.smp = smp;
        const int k = (int)(p & 7u);
        float x, y, scale;
        block_coord(a.w, a.h, gx & ~15u, gy & ~3u, (int)((p >> 3) & 7u), k, &x, &y, &scale);
        rng.seed(gx, gy, a.frame + smp, k);
        x = fmaf(unit_from(rng.next()), scale, x);
        y = fmaf(unit_from(rng.next()), scale, y);
        camera_ray(a.cam, x, y, unit_from(rng.next()), tab, o, d);
        return true;
    }
    __device__ __forceinline__ DeviceScene scene(const PathRef&) const { return a.s; }
    __device__ __forceinline__ bool last(const PathRef& r) const { return !MULTI || r.smp + 1u == a.samples; }
    __device__ __forceinline__ void gbuffer(const PathRef& r, uint32_t word) {
        if (!a.gbuf || !last(r)) return;
        uint32_t gx, gy, px, py;
        path_pixel(r.path, bw, gx, gy, px, py);
        if (px < a.w && py < a.h) a.gbuf[(size_t)py * a.w + px] = word;
    }
    __device__ __forceinline__ void mark_emitter(const PathRef& r) {
        if (!a.gbuf || !last(r)) return;
        atomicOr(a.group_em + (r.path >> 3), 1u << (r.path & 7u));
    }
    __device__ __forceinline__ void store(const PathRef& r, F3 c) {
        uint32_t gx, gy, px, py;
        path_pixel(r.path, bw, gx, gy, px, py);
        if (px >= a.w || py >= a.h) return;
        const size_t idx = (size_t)py * a.w + px;
        if (!last(r)) {
            float* out = a.sample_color + (size_t)3 * a.w * a.h * r.smp + 3 * idx;
            out[0] = c.x;
            out[1] = c.y;
            out[2] = c.z;
            return;
        }
        if (a.rgba) a.rgba[idx] = pack_color(c);
        if (a.color) {
            a.color[3 * idx] = c.x;
            a.color[3 * idx + 1] = c.y;
            a.color[3 * idx + 2] = c.z;
        }
        if (a.accum) {
            a.accum[3 * idx] += c.x;
            a.accum[3 * idx + 1] += c.y;
            a.accum[3 * idx + 2] += c.z;
        }
    }
    __device__ __forceinline__ void count_ray(const PathRef&) { rays++; }
    __device__ __forceinline__ void finish(const PathRef&) { flush_rays(a, rays); }
    __device__ __forceinline__ void work(uint64_t boxes, uint64_t tris, uint64_t shades) {
        unsigned long long v[3] = {boxes, tris, shades};
        for (int k = 0; k < 3; k++) {
            for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
            if ((threadIdx.x & 31u) == 0u && v[k]) atomicAdd(a.work + k, v[k]);
        }
    }
};

// Launch shape and loop form of the per-lane path refill, each measured on the
// room (5k triangles), the 82k-triangle icosphere and the 870k-triangle tube at
// 1280x736: 7 resident blocks per SM (72 registers, no spill; 8 blocks spill
// and lose 2-7 %), and a leaf reached from a pair tested in the same step.
// Trees up to 40 levels: claim threshold 16 and three traversal steps per
// round of votes, swept with the select-form rounds in place (room 0.711 ->
// 0.701-0.704 ms, icosphere 1.42 -> 1.40-1.41 ms against two steps; four
// steps 0.733 and 1.46; claim 12 or 20 at three steps: room 0.751 or 0.694,
// icosphere 1.412 or 1.432). Deeper trees: below (kDeepFrame*).
constexpr int kRefillFrameBlocksPerSm = 7;
constexpr int kRefillFrameSteps = 3;

// COUNT: the same frame, also counting its work (FrameArgs::work); the
// counters cost registers, so frames are rendered without them.
// Trees deeper than 40 levels (the CLAIM_MIN 8 instantiation) keep the first
// 16 stack entries of each lane in shared memory and read the approximation
// tables from global memory instead (the 16 KB of entries per block take the
// room the tables would); shallower trees keep the whole stack local. Measured
// on the 870k-triangle tube (70 levels), ms per 1280x736 sample: local stack
// 3.07-3.11; 4, 8 entries 3.11, 3.03; 8, 12, 16 with the tables in global
// memory 3.10, 3.04, 2.99 (20, 24, 32: 2.96, 3.00, 3.19). On the 19-level room
// the same entries cost 3-4 %.
constexpr int kDeepFrameStackShared = 16;

// Deep trees: claim threshold 8 and three traversal steps per round of votes
// (tube, ms per sample: claim 6, 8, 10, 12 -> 3.01, 2.98, 2.97, 2.99 at two
// steps; steps 1, 2, 3, 4 -> 3.15, 2.98, 2.93, 3.07 at claim 8; 6 and 8
// resident blocks per SM instead of 7 -> 3.07 and 2.97, the latter with 64
// registers and a 76-byte spill).
constexpr int kDeepFrameClaim = 8;
constexpr int kDeepFrameSteps = 3;
// DEEP: a tree deeper than 40 levels (shared stack entries, the constants above).
// MULTI: a.samples samples in one launch (FramePaths<true>).
template <bool DEEP, bool COUNT, bool MULTI = false>
__global__ void __launch_bounds__(128, kRefillFrameBlocksPerSm) k_render_refill(FrameArgs a) {
    FramePaths<MULTI> P{a, (a.w + 15u) / 16u, (a.h + 3u) / 4u, 0u};
    bool ok;
    if constexpr (DEEP) {
        __shared__ uint2 sstack[4][kDeepFrameStackShared][32];
        ok = path_refill<kDeepFrameClaim, kDeepFrameSteps, COUNT, true, kDeepFrameStackShared>(
            P, g_tables, &sstack[threadIdx.x >> 5][0][threadIdx.x & 31]);
    } else {
        __shared__ ApproxTables tab;
        load_tables(tab);
        ok = path_refill<16, kRefillFrameSteps, COUNT, true>(P, tab);
    }
    if (!ok) atomicOr(a.err, kErrStackOverflow);
}

// After k_render_refill: a group whose 8 lanes all hit an emitter at bounce 0
// leaves the reference's path loop before its gbuffer values are taken
// (renderer.rs:413-468), so its gbuffer words are 0.
__global__ void __launch_bounds__(256) k_emitter_groups(const uint32_t* __restrict__ mask, uint32_t ngroups,
                                                       uint32_t w, uint32_t h, uint32_t* __restrict__ gbuf) {
    const uint32_t bw = (w + 15u) / 16u;
    for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngroups; gi += gridDim.x * blockDim.x) {
        if (mask[gi] != 0xffu) continue;
        uint32_t gx, gy, px, py;
        path_pixel(gi << 3, bw, gx, gy, px, py);
        for (uint32_t q = 0; q < 8u; q++) {
            uint32_t qx = gx + (q & 3u), qy = gy + (q >> 2);
            if (qx < w && qy < h) gbuf[(size_t)qy * w + qx] = 0u;
        }
    }
}

// After a k_render_refill launch of n > 1 samples: adds each pixel's sample
// colours to the accumulator in sample order (samples 0 .. n - 2 from
// `samples`, the last from the frame's colour buffer). These are the additions
// one launch per frame makes (renderer.rs:339-410 accumulates a frame at a
// time), in the same order, so the accumulator gets the same bits.
__global__ void __launch_bounds__(256) k_accumulate_samples(float* __restrict__ accum,
                                                           const float* __restrict__ samples,
                                                           const float* __restrict__ last, size_t nf, uint32_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf; i += (size_t)gridDim.x * blockDim.x) {
        float v = accum[i];
        for (uint32_t s = 0; s + 1u < n; s++) v += __ldg(samples + (size_t)s * nf + i);
        accum[i] = v + last[i];
    }
}

// One resident block per SM is all the launch bound asks: the frame's few
// hundred chains leave most warp slots empty, so registers are free, and with
// the bound of 128 threads alone the compiler capped the kernel at 64
// registers and spilled 48 bytes (packet 32) on the chains' critical path.
// Without the cap (118 and 100 registers, no spill): room frame 17.49 ->
// 17.01 ms, icosphere 26.52 -> 26.00 ms. (The packet traversal's stack top
// held in registers, as in the refill step, measured slower: packet query
// 2.92 -> 3.03 ms, packet frame 1.21 -> 1.32 ms.)
template <bool PACKET>
__global__ void __launch_bounds__(128, 1) k_render_patch(FrameArgs a) {
    __shared__ ApproxTables tab;
    load_tables(tab);
    const int k = threadIdx.x & 7;
    const unsigned omask = 0xffu << (threadIdx.x & 24u);
    const uint32_t pw = (a.w + a.patch - 1u) / a.patch, ph = (a.h + a.patch - 1u) / a.patch;
    const uint32_t n = a.patches ? a.n_patches : pw * ph;
    const uint32_t wb = a.patch / 16u, hb = a.patch / 4u;  // 16x4 blocks across and up a patch
    // One octet per warp: a patch is one long serial chain, so its octet gets a
    // scheduler slot of its own instead of sharing a warp (and diverging) with
    // three other patches, and the few hundred chains of a frame spread over
    // every SM.
    if ((threadIdx.x & 31u) >= 8u) return;
    const uint32_t octets = (gridDim.x * blockDim.x) >> 5;
    uint32_t rays = 0;
    bool ok = true;
    for (uint32_t pi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; pi < n; pi += octets) {
        uint32_t x0 = a.patches ? a.patches[2 * pi] : (pi / ph) * a.patch;
        uint32_t y0 = a.patches ? a.patches[2 * pi + 1] : (pi % ph) * a.patch;
        LaneRng rng;
        rng.seed(x0, y0, a.frame, k);
        for (uint32_t i = 0; i < wb; i++) {
            for (uint32_t j = 0; j < hb; j++) {
                uint32_t xb = x0 + i * 16u, yb = y0 + j * 4u;
                float jx[8], jy[8];
                for (int q = 0; q < 8; q++) jx[q] = unit_from(rng.next());
                for (int q = 0; q < 8; q++) jy[q] = unit_from(rng.next());
#pragma unroll 1
                for (int g = 0; g < 8; g++) {
                    float x, y, scale;
                    block_coord(a.w, a.h, xb, yb, g, k, &x, &y, &scale);
                    x = fmaf(jx[g], scale, x);
                    y = fmaf(jy[g], scale, y);
                    PixelOut p;
                    if (a.debug) ok &= render_pixels_debug<PACKET>(a.s, a.cam, x, y, omask, tab, p, rays);
                    else ok &= render_pixels<PACKET>(a.s, a.cam, x, y, rng, omask, tab, p, rays);
                    store_pixel(a, xb + 4u * (uint32_t)(g >> 1) + (uint32_t)(k & 3),
                                yb + 2u * (uint32_t)(g & 1) + (uint32_t)(k >> 2), p);
                }
            }
        }
    }
    if (!ok) atomicOr(a.err, kErrStackOverflow);
    // only the warp's first octet is alive here: reduce over it alone
    unsigned long long v = rays;
    for (int off = 4; off > 0; off >>= 1) v += __shfl_down_sync(0xffu, v, off, 8);
    if (k == 0 && v) atomicAdd(a.rays, v);
}

__global__ void k_resolve(const float* __restrict__ accum, uint32_t npx, float factor, uint32_t* __restrict__ rgba) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x) {
        F3 c = f3(accum[3 * i] * factor, accum[3 * i + 1] * factor, accum[3 * i + 2] * factor);
        rgba[i] = pack_color(c);
    }
}

// ---------------------------------------------------------------------------
// Launchers

// SM count of the calling thread's current device, looked up once per device.
// Threads may call this concurrently and devices may differ in SM count, so
// each device has its own atomic slot (a racing first lookup stores the same
// value twice).
constexpr int kMaxCachedDevices = 64;
static std::atomic<int> g_sm_count[kMaxCachedDevices];
int sm_count() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    if (dev >= 0 && dev < kMaxCachedDevices) {
        const int v = g_sm_count[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 1;
    }
    if (dev >= 0 && dev < kMaxCachedDevices) g_sm_count[dev].store(n, std::memory_order_relaxed);
    return n;
}
static int num_sms() { return sm_count(); }

cudaError_t set_stack_limit(int entries) {
    return cudaMemcpyToSymbol(c_stack_limit, &entries, sizeof entries);
}

cudaError_t upload_tables(const uint16_t* rcp, const uint16_t* rsqrt) {
    ApproxTables t;
    for (int i = 0; i < 2048; i++) {
        t.rcp[i] = rcp[i];
        t.rsqrt[i] = rsqrt[i];
    }
    return cudaMemcpyToSymbol(g_tables, &t, sizeof t);
}

cudaError_t launch_prep_geom(const cvx_triangle* tris, uint32_t n, float4* geom, TriShade* shade, cudaStream_t st) {
    uint32_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (blocks == 0) blocks = 1;
    k_prep_geom<<<blocks, 256, 0, st>>>(tris, n, geom, shade);
    return cudaGetLastError();
}

cudaError_t launch_prep_lights(const cvx_triangle* tris, const uint32_t* ds, uint32_t n, float4* lights,
                               cudaStream_t st) {
    uint32_t blocks = (n + 127) / 128;
    if (blocks > 1024) blocks = 1024;
    if (blocks == 0) blocks = 1;
    k_prep_lights<<<blocks, 128, 0, st>>>(tris, ds, n, lights);
    return cudaGetLastError();
}

// The select-form query with CLAIM at 8 blocks per SM and `shared` stack
// entries in shared memory (0, 4, 8 or 12).
template <int CLAIM>
static void launch_select_stack(uint32_t shared, uint32_t blocks, const SoaRays& src, uint32_t* err,
                                cudaStream_t st) {
    switch (shared) {
        case 0: k_intersect_refill<8, false, CLAIM, true, 0><<<blocks, 128, 0, st>>>(src, err + 1, err); break;
        case 4: k_intersect_refill<8, false, CLAIM, true, 4><<<blocks, 128, 0, st>>>(src, err + 1, err); break;
        case 12: k_intersect_refill<8, false, CLAIM, true, 12><<<blocks, 128, 0, st>>>(src, err + 1, err); break;
        default: k_intersect_refill<8, false, CLAIM, true, 8><<<blocks, 128, 0, st>>>(src, err + 1, err); break;
    }
}

cudaError_t launch_intersect(const DeviceScene& s, const RayCols& rays, uint32_t n, float far_dist, bool packet,
                             float* t_out, int32_t* tri_out, uint32_t* counters, uint32_t* err, uint32_t block,
                             uint32_t blocks_per_sm, cudaStream_t st, uint32_t shared_stack) {
    if (!packet) {
        // persistent ray-refill kernel; err[1] is its ray counter
        cudaError_t e = cudaMemsetAsync(err + 1, 0, 4, st);
        if (e != cudaSuccess) return e;
        uint32_t bps = blocks_per_sm ? blocks_per_sm : 8;
        uint32_t blocks = (uint32_t)num_sms() * bps;
        uint32_t need = (n + 127u) / 128u;
        if (blocks > need) blocks = need;
        SoaRays src{s.nodes, s.geom, rays, n, far_dist, t_out, tri_out, counters};
        bool deep = s.depth > 40;
        const bool sel = s.slab_sel != 0u && !counters;
        if (counters) k_intersect_refill<8, true, 16, false><<<blocks, 128, 0, st>>>(src, err + 1, err);
        else if (!sel) {  // x86-form slab test throughout
            if (deep) k_intersect_refill<8, false, 8, false><<<blocks, 128, 0, st>>>(src, err + 1, err);
            else k_intersect_refill<8, false, 16, false><<<blocks, 128, 0, st>>>(src, err + 1, err);
        } else if (deep) {
            if (bps >= 12) k_intersect_refill<12, false, 8, true><<<blocks, 128, 0, st>>>(src, err + 1, err);
            else if (bps >= 10) k_intersect_refill<10, false, 8, true><<<blocks, 128, 0, st>>>(src, err + 1, err);
            else launch_select_stack<8>(shared_stack, blocks, src, err, st);
        } else {
            if (bps >= 12) k_intersect_refill<12, false, 16, true><<<blocks, 128, 0, st>>>(src, err + 1, err);
            else if (bps >= 10) k_intersect_refill<10, false, 16, true><<<blocks, 128, 0, st>>>(src, err + 1, err);
            else launch_select_stack<16>(shared_stack, blocks, src, err, st);
        }
        if (sel) {
            const uint32_t per_block = 256u * kDeferredScan;
            k_intersect_deferred<<<(n + per_block - 1u) / per_block, 256, 0, st>>>(src, err);
        }
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(err + 1, 0, 4, st);  // packet counter
    if (e != cudaSuccess) return e;
    if (block == 0) block = 128;
    if (blocks_per_sm == 0) blocks_per_sm = 8;
    uint32_t need = ((n + 7u) & ~7u) / block + 1u;
    uint32_t blocks = (uint32_t)num_sms() * blocks_per_sm;
    if (blocks > need) blocks = need;
    k_intersect<true><<<blocks, block, 0, st>>>(s, rays, n, far_dist, t_out, tri_out, counters, err);
    return cudaGetLastError();
}

cudaError_t launch_render(const DeviceScene& s, const DeviceCamera& cam, uint32_t w, uint32_t h, uint32_t frame,
                          bool packet, bool patch_order, uint32_t* rgba, uint32_t* gbuf, float* color, float* accum,
                          unsigned long long* rays, uint32_t* err, uint32_t block, bool debug, cudaStream_t st,
                          uint32_t patch, const uint32_t* patches, uint32_t n_patches, uint32_t* group_em,
                          unsigned long long* work, uint32_t samples, float* sample_color) {
    if (patch == 0) patch = 32;
    if (samples == 0) samples = 1;
    if (samples > 1 && (!accum || !color || !sample_color)) return cudaErrorInvalidValue;
    FrameArgs a{s,      cam,     w,         h,       frame, rgba, gbuf, color, samples > 1 ? nullptr : accum,
                rays,   err,     debug ? 1u : 0u, patch, patches, n_patches, group_em, work, samples, sample_color};
    if (block == 0) block = 128;
    if (group_em && !packet && !patch_order && !debug) {
        uint32_t ngroups = ((w + 15u) / 16u) * ((h + 3u) / 4u) * 8u;
        cudaError_t e = cudaMemsetAsync(group_em, 0, (size_t)ngroups * 4u, st);
        if (e != cudaSuccess) return e;
        uint32_t need = (uint32_t)(((uint64_t)ngroups * 8u * samples + 127u) / 128u),
                 blocks = (uint32_t)num_sms() * kRefillFrameBlocksPerSm;
        if (blocks > need) blocks = need;
        if (work) {
            if (samples > 1) return cudaErrorInvalidValue;
            if (s.depth > 40) k_render_refill<true, true><<<blocks, 128, 0, st>>>(a);
            else k_render_refill<false, true><<<blocks, 128, 0, st>>>(a);
        } else if (samples > 1) {
            if (s.depth > 40) k_render_refill<true, false, true><<<blocks, 128, 0, st>>>(a);
            else k_render_refill<false, false, true><<<blocks, 128, 0, st>>>(a);
        } else if (s.depth > 40) {
            k_render_refill<true, false><<<blocks, 128, 0, st>>>(a);
        } else {
            k_render_refill<false, false><<<blocks, 128, 0, st>>>(a);
        }
        if (gbuf) {
            uint32_t fb = (ngroups + 255u) / 256u, cap = (uint32_t)num_sms() * 8u;
            k_emitter_groups<<<fb < cap ? fb : cap, 256, 0, st>>>(group_em, ngroups, w, h, gbuf);
        }
        if (samples > 1 && accum) {
            const size_t nf = (size_t)3 * w * h;
            const uint32_t cap = (uint32_t)num_sms() * 8u;
            const uint32_t fb = (uint32_t)std::min<size_t>((nf + 255u) / 256u, cap);
            k_accumulate_samples<<<fb, 256, 0, st>>>(accum, sample_color, color, nf, samples);
        }
        return cudaGetLastError();
    }
    if (samples != 1) return cudaErrorInvalidValue;
    if (patch_order) {
        uint32_t units = patches ? n_patches : ((w + patch - 1) / patch) * ((h + patch - 1) / patch);
        uint32_t blocks = (units * 32 + block - 1) / block;  // one warp per patch
        if (packet) k_render_patch<true><<<blocks, block, 0, st>>>(a);
        else k_render_patch<false><<<blocks, block, 0, st>>>(a);
    } else {
        uint32_t units = ((w + 15) / 16) * ((h + 3) / 4) * 8;
        uint32_t need = (units * 8 + block - 1) / block;
        uint32_t blocks = (uint32_t)num_sms() * 16u;
        if (blocks > need) blocks = need;
        if (packet) k_render_group<true><<<blocks, block, 0, st>>>(a);
        else k_render_group<false><<<blocks, block, 0, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_resolve(const float* accum, uint32_t npx, float factor, uint32_t* rgba, cudaStream_t st) {
    uint32_t blocks = (npx + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (blocks == 0) blocks = 1;
    k_resolve<<<blocks, 256, 0, st>>>(accum, npx, factor, rgba);
    return cudaGetLastError();
}

}  // namespace cvx
