// Wavefront kernels (see wavefront.cuh). All three are persistent: a fixed
// grid walks the queue whose length it reads from device memory, so the whole
// bounce loop of a wave is a fixed sequence of launches that a CUDA graph can
// replay. Compiled with -fmad=false (x86sem.cuh).
#include <cuda_runtime.h>

#include "kernels.h"
#include "path_refill.cuh"
#include "shade.cuh"
#include "wavefront.cuh"

namespace cvx {

// This translation unit's copy of the approximation tables (device globals
// are per translation unit without relocatable device code).
__device__ ApproxTables g_tables_wf;

// Traversal steps per round of the refill traversal's claim votes (1, 2, 3 ->
// 4.48, 4.42, 4.35 ms per tube sample with the graph).
constexpr int kWaveTraverseSteps = 3;
cudaError_t upload_tables_wave(const uint16_t* rcp, const uint16_t* rsqrt) {
    ApproxTables t;
    for (int i = 0; i < 2048; i++) {
        t.rcp[i] = rcp[i];
        t.rsqrt[i] = rsqrt[i];
    }
    return cudaMemcpyToSymbol(g_tables_wf, &t, sizeof t);
}

__device__ __forceinline__ void load_tables_wf(ApproxTables& sm) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&g_tables_wf);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&sm);
    for (int i = threadIdx.x; i < (int)(sizeof(ApproxTables) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
}

// Appends `gi` for every octet leader whose `keep` is set; one atomic per
// converged set of threads.
__device__ __forceinline__ void enqueue_octets(bool leader_keep, uint32_t gi, uint32_t* queue, uint32_t* count) {
    unsigned m = __activemask();
    unsigned b = __ballot_sync(m, leader_keep);
    if (!b) return;
    int lane = threadIdx.x & 31;
    int first = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == first) base = atomicAdd(count, (uint32_t)__popc(b));
    base = __shfl_sync(m, base, first);
    if (leader_keep) queue[base + __popc(b & ((1u << lane) - 1u))] = gi;
}

__device__ __forceinline__ uint32_t find_job(const Job* jobs, uint32_t n_jobs, uint32_t gi) {
    uint32_t lo = 0, hi = n_jobs;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&jobs[mid].group_base) <= gi) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Next group index for the calling octet (one atomic by its lane 0).
__device__ __forceinline__ uint32_t octet_claim_wf(uint32_t* counter, unsigned omask, int k) {
    uint32_t g = 0;
    if (k == 0) g = atomicAdd(counter, 1u);
    return __shfl_sync(omask, g, (int)(threadIdx.x & 24u));
}

// Pixel origin of group `local` of a job (octet order of k_render_group).
__device__ __forceinline__ void group_origin(const Job& j, uint32_t local, uint32_t* xb, uint32_t* yb, int* g,
                                             uint32_t* gx, uint32_t* gy) {
    uint32_t bw = (j.w + 15u) / 16u, blk = local >> 3;
    *g = (int)(local & 7u);
    *xb = (blk % bw) * 16u;
    *yb = (blk / bw) * 4u;
    *gx = *xb + 4u * (uint32_t)(*g >> 1);
    *gy = *yb + 2u * (uint32_t)(*g & 1);
}

__device__ __forceinline__ void block_coord_wf(uint32_t w, uint32_t h, uint32_t xb, uint32_t yb, int g, int k,
                                               float* x, float* y, float* scale_out) {
    float scale = 2.0f / (float)w;
    float s2 = 2.0f * scale, s4 = 4.0f * scale, s8 = 8.0f * scale, s12 = 12.0f * scale;
    float bx = scale * ((float)(k & 3) + ((float)xb - (float)w * 0.5f));
    float by = scale * ((float)(k >> 2) + ((float)yb - (float)h * 0.5f));
    int col = g >> 1;
    *x = col == 0 ? bx : col == 1 ? bx + s4 : col == 2 ? bx + s8 : bx + s12;
    *y = (g & 1) ? by + s2 : by;
    *scale_out = scale;
}

__global__ void __launch_bounds__(128) k_wf_raygen(const Job* __restrict__ jobs, const WaveHeader* __restrict__ hdr,
                                                   WaveState st) {
    __shared__ ApproxTables tab;
    load_tables_wf(tab);
    const int k = threadIdx.x & 7;
    const uint32_t n_groups = hdr->n_groups, n_jobs = hdr->n_jobs;
    const uint32_t octets = (gridDim.x * blockDim.x) >> 3;
    for (uint32_t gi = (blockIdx.x * blockDim.x + threadIdx.x) >> 3; gi < n_groups; gi += octets) {
        uint32_t ji = find_job(jobs, n_jobs, gi);
        const Job& j = jobs[ji];
        uint32_t xb, yb, gx, gy;
        int g;
        group_origin(j, gi - j.group_base, &xb, &yb, &g, &gx, &gy);
        bool inside = gx < j.w && gy < j.h;
        if (inside) {
            float x, y, scale;
            block_coord_wf(j.w, j.h, xb, yb, g, k, &x, &y, &scale);
            LaneRng rng;
            rng.seed(gx, gy, j.frame, k);
            x = fmaf(unit_from(rng.next()), scale, x);
            y = fmaf(unit_from(rng.next()), scale, y);
            F3 o, d;
            camera_ray(j.cam, x, y, unit_from(rng.next()), tab, o, d);
            size_t l = (size_t)gi * 8 + k;
            st.ox[l] = o.x;
            st.oy[l] = o.y;
            st.oz[l] = o.z;
            st.dx[l] = d.x;
            st.dy[l] = d.y;
            st.dz[l] = d.z;
            st.cr[l] = 1.0f;
            st.cg[l] = 1.0f;
            st.cb[l] = 1.0f;
            st.rng[l] = rng.s;
            st.gbuf[l] = 0u;
            st.flags[l] = 1u;
            if (k == 0) st.group_job[gi] = ji;
        }
        enqueue_octets(k == 0 && inside, gi, st.queue[0], &st.counts[0]);
    }
}

// One octet per queued group: decisions over the octet (PACKET) or each lane
// over its own ray (single, without refill: suits the coherent camera rays,
// whose adjacent pixels share a warp).
template <bool PACKET>
__global__ void __launch_bounds__(128, 8) k_wf_traverse_octet(const Job* __restrict__ jobs,
                                                           const DeviceScene* __restrict__ scenes, WaveState st,
                                                           int bounce, WaveOutputs out) {
    __shared__ ApproxTables tab;
    load_tables_wf(tab);
    const int k = threadIdx.x & 7;
    const unsigned omask = 0xffu << (threadIdx.x & 24u);
    const uint32_t n = st.counts[bounce];
    const uint32_t* queue = st.queue[bounce & 1];
    bool ok = true;
    // Queue entries claimed one at a time by each octet (counter counts[11 + bounce]).
    uint32_t* next = &st.counts[11 + bounce];
    for (uint32_t qi = octet_claim_wf(next, omask, k); qi < n; qi = octet_claim_wf(next, omask, k)) {
        uint32_t gi = queue[qi];
        size_t l = (size_t)gi * 8 + k;
        const DeviceScene s = scenes[jobs[st.group_job[gi]].scene];
        bool active = (st.flags[l] & 1u) != 0u;
        F3 o = f3(st.ox[l], st.oy[l], st.oz[l]), d = f3(st.dx[l], st.dy[l], st.dz[l]);
        Hit h{1.0e5f, 0.0f, 0.0f, -1};
        if (PACKET || active) ok &= traverse<PACKET>(s, o, d, active, omask, h, tab, nullptr);
        st.ht[l] = h.t;
        st.hu[l] = h.u;
        st.hv[l] = h.v;
        st.htri[l] = h.tri;
    }
    if (!ok) atomicOr(out.err, kErrStackOverflow);
}

// Single-ray traversal over the lanes of the queued groups, with ray refill
// (traverse_refill): ray r is lane r % 8 of queue entry r / 8. The claim
// hands the traversal the lane slot l = group * 8 + k as the ray's index, so
// its result is stored without reading the queue again.
struct QueueStore {
    WaveState st;
    __device__ __forceinline__ void store(uint32_t l, const Hit& h, uint32_t, uint32_t) const {
        st.ht[l] = h.t;
        st.hu[l] = h.u;
        st.hv[l] = h.v;
        st.htri[l] = h.tri;
    }
};

struct QueueClaim {
    const Job* jobs;
    const DeviceScene* scenes;
    WaveState st;
    const uint32_t* queue;
    uint32_t n;
    uint32_t* next_ray;
    __device__ __forceinline__ int claim(unsigned b, bool want, int lane, uint32_t& r_out, RayIn& in) {
        uint32_t base = 0;
        int first = __ffs(b) - 1;
        if (lane == first) base = atomicAdd(next_ray, (uint32_t)__popc(b));
        base = __shfl_sync(0xffffffffu, base, first);
        if (!want) return kClaimNone;
        uint32_t r = base + __popc(b & ((1u << lane) - 1u));
        if (r >= n) return kClaimDone;
        uint32_t gi = queue[r >> 3];
        uint32_t l = gi * 8u + (r & 7u);
        if (!(st.flags[l] & 1u)) {  // inactive lane: its result is the miss
            st.ht[l] = 1.0e5f;
            st.hu[l] = 0.0f;
            st.hv[l] = 0.0f;
            st.htri[l] = -1;
            return kClaimNone;
        }
        const DeviceScene* s = scenes + jobs[st.group_job[gi]].scene;
        in.nodes = s->nodes;
        in.geom = s->geom;
        in.o = f3(st.ox[l], st.oy[l], st.oz[l]);
        in.d = f3(st.dx[l], st.dy[l], st.dz[l]);
        in.far = 1.0e5f;
        r_out = l;
        return kClaimRay;
    }
};

// 10 resident blocks per SM (48 registers): measured on the 870k-triangle
// tube, 4.17 ms per sample against 4.56 (56 registers, 9 blocks), 4.69 (12) and 5.46 (16).
// CLAIM: lanes without a ray wait until this many want one; 16 for waves of
// shallow trees, 8 when a scene is deeper than 40 levels (room scene frame
// 1.013 against 1.063 ms at 8; tube sample 4.23 against 4.33 ms at 16).
template <int CLAIM>
__global__ void __launch_bounds__(128, 10) k_wf_traverse_single(const Job* __restrict__ jobs,
                                                            const DeviceScene* __restrict__ scenes, WaveState st,
                                                            int bounce, WaveOutputs out) {
    QueueStore store{st};
    QueueClaim claim{jobs, scenes, st, st.queue[bounce & 1], st.counts[bounce] * 8u, &st.counts[6 + bounce]};
    if (!traverse_refill<false, true, CLAIM, 0, false, kWaveTraverseSteps>(store, claim, g_tables_wf))
        atomicOr(out.err, kErrStackOverflow);
}

__device__ __forceinline__ void finalize(const Job& j, uint32_t gi, int k, F3 color, F3 d, bool hit_em,
                                         uint32_t gword, const WaveOutputs& out) {
    uint32_t xb, yb, gx, gy;
    int g;
    group_origin(j, gi - j.group_base, &xb, &yb, &g, &gx, &gy);
    uint32_t px = gx + (uint32_t)(k & 3), py = gy + (uint32_t)(k >> 2);
    if (px >= j.w || py >= j.h) return;
    F3 em = sky_intensity(d);
    F3 c = f3(color.x * em.x, color.y * em.y, color.z * em.z);
    c = hit_em ? c : f3(0.0f, 0.0f, 0.0f);
    size_t idx = (size_t)j.out_offset + (size_t)py * j.w + px;
    if (out.rgba) out.rgba[idx] = pack_color(c);
    if (out.gbuf) out.gbuf[idx] = gword;
    if (out.color) {
        out.color[3 * idx] = c.x;
        out.color[3 * idx + 1] = c.y;
        out.color[3 * idx + 2] = c.z;
    }
    if (out.accum) {
        out.accum[3 * idx] += c.x;
        out.accum[3 * idx + 1] += c.y;
        out.accum[3 * idx + 2] += c.z;
    }
}

// 8 resident blocks per SM (64 registers, down from 96): room scene
// wavefront frame 1.02 against 1.12 ms with the octet kernel below.
__global__ void __launch_bounds__(128, 8) k_wf_shade(const Job* __restrict__ jobs, const DeviceScene* __restrict__ scenes,
                                                  WaveState st, int bounce, WaveOutputs out) {
    __shared__ ApproxTables tab;
    load_tables_wf(tab);
    const int k = threadIdx.x & 7;
    const unsigned omask = 0xffu << (threadIdx.x & 24u);
    const uint32_t n = st.counts[bounce];
    const uint32_t* queue = st.queue[bounce & 1];
    uint32_t* next_q = st.queue[(bounce + 1) & 1];
    uint32_t* next_n = &st.counts[bounce + 1];
    const uint32_t octets = (gridDim.x * blockDim.x) >> 3;
    uint32_t rays = 0;
    for (uint32_t qi = (blockIdx.x * blockDim.x + threadIdx.x) >> 3; qi < n; qi += octets) {
        uint32_t gi = queue[qi];
        size_t l = (size_t)gi * 8 + k;
        const Job& j = jobs[st.group_job[gi]];
        const DeviceScene s = scenes[j.scene];
        uint32_t flags = st.flags[l];
        bool active = (flags & 1u) != 0u;
        F3 o = f3(st.ox[l], st.oy[l], st.oz[l]), d = f3(st.dx[l], st.dy[l], st.dz[l]);
        Hit h{st.ht[l], st.hu[l], st.hv[l], st.htri[l]};
        Isect I = make_isect(s, h, o, d, tab);
        bool hit_em = (I.mat >> 31) != 0u;
        F3 color = f3(st.cr[l], st.cg[l], st.cb[l]);
        unsigned traced = __popc(__ballot_sync(omask, active) & omask);  // rays this group traced this bounce
        rays += traced;
        if (out.job_rays && k == 0 && traced) atomicAdd(&out.job_rays[st.group_job[gi]], (unsigned long long)traced);
        bool keep = false;
        if (oct_all(omask, hit_em)) {
            finalize(j, gi, k, color, d, hit_em, st.gbuf[l], out);
        } else {
            LaneRng rng;
            rng.resume(st.rng[l], k);
            F3 cm;
            float fr;
            continue_path(s, o, d, active, I, rng, bounce == 0, tab, cm, fr);
            color = f3(color.x * cm.x, color.y * cm.y, color.z * cm.z);
            uint32_t gword = st.gbuf[l];
            if (bounce == 0) {
                PixelOut p;
                p.tex = ((int32_t)I.mat >> 24) & 3;
                p.tu = I.tu;
                p.tv = I.tv;
                p.fresnel = fr;
                gword = pack_gbuffer(p);
            }
            if (bounce == 4) {
                finalize(j, gi, k, color, d, hit_em, gword, out);
            } else {
                st.ox[l] = o.x;
                st.oy[l] = o.y;
                st.oz[l] = o.z;
                st.dx[l] = d.x;
                st.dy[l] = d.y;
                st.dz[l] = d.z;
                st.cr[l] = color.x;
                st.cg[l] = color.y;
                st.cb[l] = color.z;
                st.rng[l] = rng.s;
                st.gbuf[l] = gword;
                st.flags[l] = active ? 1u : 0u;
                keep = true;
            }
        }
        enqueue_octets(k == 0 && keep, gi, next_q, next_n);
    }
    // each octet counted its rays on all 8 lanes: keep lane 0's
    unsigned long long v = (threadIdx.x & 7u) == 0u ? rays : 0u;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31u) == 0u && v) atomicAdd(out.rays, v);
}

static int sms() { return sm_count(); }

cudaError_t set_stack_limit_wave(int entries) {
    return cudaMemcpyToSymbol(c_stack_limit, &entries, sizeof entries);
}

// The fused form over a wave: every octet renders whole groups of any job
// (camera ray, bounce loop and shading in registers), walking the wave's
// groups with a grid-stride loop. Same per-group RNG order and outputs as the
// wavefront kernels.
template <bool PACKET>
// 8 resident blocks per SM (64 registers, small spill): batches of small
// scenes render 12 % faster than at the compiler's 80 registers (6 blocks).
__global__ void __launch_bounds__(128, 8) k_wave_fused(const Job* __restrict__ jobs, const WaveHeader* __restrict__ hdr,
                                                    const DeviceScene* __restrict__ scenes, WaveOutputs out) {
    __shared__ ApproxTables tab;
    load_tables_wf(tab);
    const int k = threadIdx.x & 7;
    const unsigned omask = 0xffu << (threadIdx.x & 24u);
    const uint32_t n_groups = hdr->n_groups, n_jobs = hdr->n_jobs;
    uint32_t rays = 0;
    bool ok = true;
    // Groups are claimed one at a time by each octet (a counter in
    // out.err[1]), which balances paths of 1 to 5 bounces across octets
    // (256-scene batch: 9.0 against 7.7 Grays/s with a grid-stride share).
    for (uint32_t gi = octet_claim_wf(out.err + 1, omask, k); gi < n_groups;
         gi = octet_claim_wf(out.err + 1, omask, k)) {
        uint32_t ji = find_job(jobs, n_jobs, gi);
        const Job& j = jobs[ji];
        uint32_t xb, yb, gx, gy;
        int g;
        group_origin(j, gi - j.group_base, &xb, &yb, &g, &gx, &gy);
        if (gx >= j.w || gy >= j.h) continue;  // whole group outside the frame (octet-uniform)
        const DeviceScene s = scenes[j.scene];
        float x, y, scale;
        block_coord_wf(j.w, j.h, xb, yb, g, k, &x, &y, &scale);
        LaneRng rng;
        rng.seed(gx, gy, j.frame, k);
        x = fmaf(unit_from(rng.next()), scale, x);
        y = fmaf(unit_from(rng.next()), scale, y);
        PixelOut p;
        uint32_t r = 0;
        ok &= render_pixels<PACKET>(s, j.cam, x, y, rng, omask, tab, p, r);
        rays += r;
        if (out.job_rays) {
            uint32_t tot = r;
            for (int off = 4; off > 0; off >>= 1) tot += __shfl_down_sync(omask, tot, off, 8);
            if (k == 0 && tot) atomicAdd(&out.job_rays[ji], (unsigned long long)tot);
        }
        uint32_t px = gx + (uint32_t)(k & 3), py = gy + (uint32_t)(k >> 2);
        if (px < j.w && py < j.h) {
            size_t idx = (size_t)j.out_offset + (size_t)py * j.w + px;
            if (out.rgba) out.rgba[idx] = pack_color(p.color);
            if (out.gbuf) out.gbuf[idx] = pack_gbuffer(p);
            if (out.color) {
                out.color[3 * idx] = p.color.x;
                out.color[3 * idx + 1] = p.color.y;
                out.color[3 * idx + 2] = p.color.z;
            }
            if (out.accum) {
                out.accum[3 * idx] += p.color.x;
                out.accum[3 * idx + 1] += p.color.y;
                out.accum[3 * idx + 2] += p.color.z;
            }
        }
    }
    if (!ok) atomicOr(out.err, kErrStackOverflow);
    unsigned long long v = rays;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31u) == 0u && v) atomicAdd(out.rays, v);
}

// The paths of a wave for path_refill: path p is lane p & 7 of wave group
// p >> 3, which belongs to the job whose group range holds it. Ray counts per
// job are kept per lane for the job of its current path (the path reference's
// job) and added to the job's total when the lane moves to another job, and at
// the end. SLOTS: the wave carries sample slots (WaveOutputs::samples), and a
// job with one writes its colours there (a separate instantiation, so that
// waves without slots run the loop they ran before).
template <bool SLOTS>
struct WavePaths {
    struct PathRef {
        uint32_t path, job;
    };
    const Job* __restrict__ jobs;
    const DeviceScene* __restrict__ scenes;
    const WaveOutputs& out;
    uint32_t n_jobs, n_groups;
    uint32_t rays, job_acc;

    __device__ __forceinline__ uint32_t n_paths() const { return n_groups * 8u; }
    __device__ __forceinline__ uint32_t claim(uint32_t n) { return atomicAdd(out.err + 1, n); }
    __device__ __forceinline__ void origin(const PathRef& r, const Job& j, uint32_t& gx, uint32_t& gy, uint32_t& px,
                                           uint32_t& py) const {
        uint32_t xb, yb;
        int g;
        group_origin(j, (r.path >> 3) - j.group_base, &xb, &yb, &g, &gx, &gy);
        px = gx + (r.path & 3u);
        py = gy + ((r.path >> 2) & 1u);
    }
    __device__ __forceinline__ bool begin(uint32_t p, PathRef& r, F3& o, F3& d, LaneRng& rng,
                                          const ApproxTables& tab) {
        // Paths are claimed in order, so the next one is mostly in the job of
        // the last: search the job table only when it is not.
        const uint32_t gi = p >> 3;
        uint32_t ji = r.job;
        if (ji >= n_jobs || gi - __ldg(&jobs[ji].group_base) >= __ldg(&jobs[ji].n_groups))
            ji = find_job(jobs, n_jobs, gi);
        const Job& j = jobs[ji];
        uint32_t xb, yb, gx, gy;
        int g;
        group_origin(j, gi - j.group_base, &xb, &yb, &g, &gx, &gy);
        if (gx >= j.w || gy >= j.h) return false;
        if (ji != r.job) {  // job_acc counts the rays of the previous path's job
            if (out.job_rays && job_acc) atomicAdd(&out.job_rays[r.job], (unsigned long long)job_acc);
            job_acc = 0;
        }
        r.path = p;
        r.job = ji;
        const int k = (int)(p & 7u);
        float x, y, scale;
        block_coord_wf(j.w, j.h, xb, yb, g, k, &x, &y, &scale);
        rng.seed(gx, gy, j.frame, k);
        x = fmaf(unit_from(rng.next()), scale, x);
        y = fmaf(unit_from(rng.next()), scale, y);
        camera_ray(j.cam, x, y, unit_from(rng.next()), tab, o, d);
        return true;
    }
    __device__ __forceinline__ DeviceScene scene(const PathRef& r) const { return scenes[__ldg(&jobs[r.job].scene)]; }
    __device__ __forceinline__ void gbuffer(const PathRef& r, uint32_t word) {
        if (!out.gbuf) return;
        const Job& j = jobs[r.job];
        uint32_t gx, gy, px, py;
        origin(r, j, gx, gy, px, py);
        if (px < j.w && py < j.h) out.gbuf[(size_t)j.out_offset + (size_t)py * j.w + px] = word;
    }
    __device__ __forceinline__ void mark_emitter(const PathRef& r) {
        if (out.gbuf) atomicOr(out.group_em + (r.path >> 3), 1u << (r.path & 7u));
    }
    __device__ __forceinline__ void store(const PathRef& r, F3 c) {
        const Job& j = jobs[r.job];
        uint32_t gx, gy, px, py;
        origin(r, j, gx, gy, px, py);
        if (px >= j.w || py >= j.h) return;
        if (SLOTS) {
            const uint64_t slot = j.slot;
            if (slot != kNoSlot) {
                float* o = out.samples + 3 * (slot + (size_t)py * j.w + px);
                o[0] = c.x;
                o[1] = c.y;
                o[2] = c.z;
                return;
            }
        }
        const size_t idx = (size_t)j.out_offset + (size_t)py * j.w + px;
        if (out.rgba) out.rgba[idx] = pack_color(c);
        if (out.color) {
            out.color[3 * idx] = c.x;
            out.color[3 * idx + 1] = c.y;
            out.color[3 * idx + 2] = c.z;
        }
        if (out.accum) {
            out.accum[3 * idx] += c.x;
            out.accum[3 * idx + 1] += c.y;
            out.accum[3 * idx + 2] += c.z;
        }
    }
    __device__ __forceinline__ void count_ray(const PathRef&) {
        rays++;
        job_acc++;
    }
    __device__ __forceinline__ void finish(const PathRef& r) {
        if (out.job_rays && job_acc) atomicAdd(&out.job_rays[r.job], (unsigned long long)job_acc);
        unsigned long long v = rays;
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31u) == 0u && v) atomicAdd(out.rays, v);
    }
};

// A fused wave in per-lane path refill form (path_refill); launch shape and
// loop form as the frame kernel's (k_render_refill).
// 7 resident blocks per SM (72 registers and a small spill): 6 (80 registers,
// no spill) served the 415-request mix at 2,014 against 2,083 Mrays/s.
constexpr int kRefillWaveBlocksPerSm = 7;
// As the frame kernel: waves whose trees are deeper than 40 levels keep the
// first 16 stack entries of each lane in shared memory and read the tables
// from global memory (4 tube views of 1280x736, 2 samples: 21.5 -> 20.3 ms;
// 12 entries 20.5 ms; three or four steps per round 20.3, 22.5 ms).
constexpr int kDeepWaveStackShared = 16;
template <int CLAIM_MIN, bool SLOTS = false>
__global__ void __launch_bounds__(128, kRefillWaveBlocksPerSm) k_wave_refill(const Job* __restrict__ jobs,
                                                                          const WaveHeader* __restrict__ hdr,
                                                                          const DeviceScene* __restrict__ scenes,
                                                                          WaveOutputs out) {
    constexpr int kShared = CLAIM_MIN == 8 ? kDeepWaveStackShared : 0;
    WavePaths<SLOTS> P{jobs, scenes, out, hdr->n_jobs, hdr->n_groups, 0u, 0u};
    bool ok;
    if constexpr (kShared > 0) {
        __shared__ uint2 sstack[4][kShared][32];
        ok = path_refill<CLAIM_MIN, 2, false, false, kShared>(P, g_tables_wf,
                                                               &sstack[threadIdx.x >> 5][0][threadIdx.x & 31]);
    } else {
        __shared__ ApproxTables tab;
        load_tables_wf(tab);
        ok = path_refill<CLAIM_MIN, 2>(P, tab);  // three steps: room waves 5.24 -> 5.34 ms
    }
    if (!ok) atomicOr(out.err, kErrStackOverflow);
}

// After k_wave_refill: the groups of the wave whose 8 lanes all hit an
// emitter at bounce 0 get gbuffer words 0 (as k_emitter_groups for a frame).
__global__ void __launch_bounds__(256) k_wave_emitter_groups(const Job* __restrict__ jobs,
                                                            const WaveHeader* __restrict__ hdr, WaveOutputs out) {
    const uint32_t n_groups = hdr->n_groups, n_jobs = hdr->n_jobs;
    for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < n_groups; gi += gridDim.x * blockDim.x) {
        if (out.group_em[gi] != 0xffu) continue;
        const Job& j = jobs[find_job(jobs, n_jobs, gi)];
        uint32_t xb, yb, gx, gy;
        int g;
        group_origin(j, gi - j.group_base, &xb, &yb, &g, &gx, &gy);
        for (uint32_t q = 0; q < 8u; q++) {
            uint32_t qx = gx + (q & 3u), qy = gy + (q >> 2);
            if (qx < j.w && qy < j.h) out.gbuf[(size_t)j.out_offset + (size_t)qy * j.w + qx] = 0u;
        }
    }
}

cudaError_t launch_wave_fused(const Job* jobs, const WaveHeader* hdr, const DeviceScene* scenes,
                              const WaveOutputs& out, bool packet, uint32_t blocks_per_sm, bool deep,
                              cudaStream_t stream) {
    if (!packet && out.group_em) {
        uint32_t grid = (uint32_t)sms() * kRefillWaveBlocksPerSm;
        if (out.samples) {  // sample slots: no gbuffer (several samples of an image share the wave)
            if (out.gbuf) return cudaErrorInvalidValue;
            if (deep) k_wave_refill<8, true><<<grid, 128, 0, stream>>>(jobs, hdr, scenes, out);
            else k_wave_refill<16, true><<<grid, 128, 0, stream>>>(jobs, hdr, scenes, out);
            return cudaGetLastError();
        }
        if (deep) k_wave_refill<8><<<grid, 128, 0, stream>>>(jobs, hdr, scenes, out);
        else k_wave_refill<16><<<grid, 128, 0, stream>>>(jobs, hdr, scenes, out);
        if (out.gbuf) k_wave_emitter_groups<<<(uint32_t)sms() * 4u, 256, 0, stream>>>(jobs, hdr, out);
        return cudaGetLastError();
    }
    if (out.samples) return cudaErrorInvalidValue;  // slots need the path-refill wave
    if (blocks_per_sm == 0) blocks_per_sm = 16;
    uint32_t grid = (uint32_t)sms() * blocks_per_sm;
    if (packet) k_wave_fused<true><<<grid, 128, 0, stream>>>(jobs, hdr, scenes, out);
    else k_wave_fused<false><<<grid, 128, 0, stream>>>(jobs, hdr, scenes, out);
    return cudaGetLastError();
}

__global__ void k_resolve_multi(const ResolveItem* __restrict__ items, uint32_t n_items, const float* __restrict__ accum,
                                uint32_t* __restrict__ rgba) {
    for (uint32_t it = blockIdx.y; it < n_items; it += gridDim.y) {
        ResolveItem r = items[it];
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < r.npx; i += gridDim.x * blockDim.x) {
            size_t p = (size_t)r.offset + i;
            F3 c = f3(accum[3 * p] * r.factor, accum[3 * p + 1] * r.factor, accum[3 * p + 2] * r.factor);
            rgba[p] = pack_color(c);
        }
    }
}

// After a wave with sample slots: each item's slots added to its accumulator
// in sample order, after the sample the wave added directly. These are the
// additions one wave per sample makes, in the same order.
__global__ void k_accumulate_slots(const SlotItem* __restrict__ items, uint32_t n_items, float* __restrict__ accum,
                                   const float* __restrict__ samples) {
    for (uint32_t it = blockIdx.y; it < n_items; it += gridDim.y) {
        const SlotItem r = items[it];
        const size_t nf = (size_t)3 * r.npx;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf; i += (size_t)gridDim.x * blockDim.x) {
            float v = accum[3 * r.accum_offset + i];
            for (uint32_t k = 0; k < r.count; k++) v += __ldg(samples + 3 * r.slot + (size_t)k * nf + i);
            accum[3 * r.accum_offset + i] = v;
        }
    }
}

cudaError_t launch_accumulate_slots(const SlotItem* items, uint32_t n_items, float* accum, const float* samples,
                                    cudaStream_t stream) {
    if (n_items == 0) return cudaSuccess;
    dim3 grid(64, n_items < 1024 ? n_items : 1024);
    k_accumulate_slots<<<grid, 256, 0, stream>>>(items, n_items, accum, samples);
    return cudaGetLastError();
}

cudaError_t launch_resolve_multi(const ResolveItem* items, uint32_t n_items, const float* accum, uint32_t* rgba,
                                 cudaStream_t stream) {
    if (n_items == 0) return cudaSuccess;
    dim3 grid(64, n_items < 1024 ? n_items : 1024);
    k_resolve_multi<<<grid, 256, 0, stream>>>(items, n_items, accum, rgba);
    return cudaGetLastError();
}

cudaError_t launch_wave(const Job* jobs, const WaveHeader* hdr, const DeviceScene* scenes, const WaveState& st,
                        const WaveOutputs& out, bool packet, uint32_t blocks_per_sm, uint32_t refill_from,
                        bool deep, cudaStream_t stream) {
    if (blocks_per_sm == 0) blocks_per_sm = 12;
    uint32_t grid = (uint32_t)sms() * blocks_per_sm;
    // counts[0..5]: queue lengths per bounce; counts[6..10]: ray counters of
    // the refill traversal, one per bounce; counts[11..15]: queue-entry
    // counters of the octet traversal, one per bounce
    cudaError_t e = cudaMemsetAsync(st.counts, 0, 16 * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    k_wf_raygen<<<grid, 128, 0, stream>>>(jobs, hdr, st);
    for (int b = 0; b < 5; b++) {
        if (packet) k_wf_traverse_octet<true><<<grid, 128, 0, stream>>>(jobs, scenes, st, b, out);
        else if ((uint32_t)b < refill_from) k_wf_traverse_octet<false><<<grid, 128, 0, stream>>>(jobs, scenes, st, b, out);
        else if (deep) k_wf_traverse_single<8><<<grid, 128, 0, stream>>>(jobs, scenes, st, b, out);
        else k_wf_traverse_single<16><<<grid, 128, 0, stream>>>(jobs, scenes, st, b, out);
        k_wf_shade<<<grid, 128, 0, stream>>>(jobs, scenes, st, b, out);
    }
    return cudaGetLastError();
}

}  // namespace cvx
