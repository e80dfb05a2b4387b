// The path loop (renderer.rs:413-468) in per-lane refill form, for the
// per-group RNG order and the single-ray traversal, shared by the frame
// kernel (one Renderer frame) and the wave kernel (a batch or server wave of
// many images and scenes).
//
// Each lane takes one path at a time from a counter (path p is lane p & 7 of
// group p >> 3) and carries it through its bounces; every round a lane tracing
// a ray processes up to STEPS node pairs or leaves of it (RefillRay). A lane
// whose ray is finished waits until CLAIM_MIN lanes of its warp are in that
// state (or none is tracing); those lanes then shade together: the hit record,
// continue_path, and either the next bounce's ray or the pixel's store and a
// new path with its camera ray. Warps thus stay busy while paths of 1 to 5
// bounces and rays of different lengths finish, and the long shading code runs
// with many lanes at once.
//
// A lane's results depend only on its own path: lane k of a group draws from
// its own 64-bit generator state (LaneRng), a lane that hits an emitter keeps
// its colour and ray from then on (material.rs:327-411: cm = 1), and the bounce
// limit holds per lane. The one coupling in the reference is the group's exit
// when all 8 lanes hit an emitter at bounce 0, before the gbuffer values are
// taken: that group's gbuffer words are 0. Every lane writes its own word; a
// lane that hits an emitter at bounce 0 also sets its bit in its group's mask,
// and a pass after the kernel writes 0 over the groups whose mask is full.
// Such a lane ends there, so it computes only the Fresnel value of its
// gbuffer word (the sampled direction, not the light PDFs or the BRDF).
//
// Paths provides, for a path reference `PathRef` it fills in:
//   uint32_t n_paths() const, uint32_t claim(uint32_t n)  (first of n paths)
//   bool begin(uint32_t p, PathRef&, F3& o, F3& d, LaneRng&, const ApproxTables&)
//       (false: the path's group lies outside its image; take another)
//   DeviceScene scene(const PathRef&) const  (a copy: its fields stay in
//       registers through the shading code, which stores to the images)
//   void gbuffer(const PathRef&, uint32_t word), void mark_emitter(const PathRef&)
//   void store(const PathRef&, F3 colour)
//   void count_ray(const PathRef&), void finish(const PathRef& last)  (finish: whole warp)
//   COUNT only: void work(uint64_t boxes, uint64_t triangles, uint64_t shades)
//       (whole warp): this lane's totals of the boxes and triangles its rays
//       tested (bvh.rs:604-651 counters) and of the shading steps that
//       evaluated every light's PDF (material.rs:281-320)
#pragma once
#include "shade.cuh"
#include "traverse.cuh"

namespace cvx {

// SELECT_ROUNDS: each round's traversal steps take the select-form slab test
// when every tracing lane's ray allows it (a warp-uniform choice, so neither
// form's code runs for the other's lanes), the x86 form otherwise. Measured
// for the frame kernel: 1280x736 tube 3.11 -> 3.08 ms, room 0.714 -> 0.704 ms,
// icosphere 1.44 -> 1.42 ms (the wave kernel, whose scene table costs
// registers, would spill 10 bytes more).
template <int CLAIM_MIN, int STEPS, bool COUNT = false, bool SELECT_ROUNDS = false, int SHARED_STACK = 0,
          class Paths>
__device__ __forceinline__ bool path_refill(Paths& P, const ApproxTables& tab, uint2* shared_stack = nullptr) {
    typedef typename Paths::PathRef PathRef;
    const int lane = threadIdx.x & 31;
    const uint32_t npaths = P.n_paths();
    RefillRay ray;
    uint2 local_stack[kStackDepth];
    typename std::conditional<SHARED_STACK == 0, LocalStack, SharedLocalStack<SHARED_STACK>>::type stack =
        make_stack<SHARED_STACK>(shared_stack, local_stack);
    ray.top = make_uint2(0u, 0u);
    ray.sp = 0;
    ray.cur = RefillRay::kNone;
    ray.na = ray.nt = 0;
    ray.nodes = ray.geom = nullptr;
    ray.o = ray.d = ray.inv = f3(0, 0, 0);
    ray.h = Hit{0.0f, 0.0f, 0.0f, -1};
    LaneRng rng;
    rng.s = rng.f = 0ull;
    rng.hi = 0u;
    PathRef ref{};
    F3 color = f3(1.0f, 1.0f, 1.0f);
    uint32_t bounce = 0;
    bool tracing = false, has_path = false, done = false, overflow = false;
    bool ray_sel = false;  // the current ray allows the select-form slab test (SELECT_ROUNDS)
    uint64_t work_boxes = 0, work_tris = 0, work_shades = 0;
    for (;;) {
        bool want = !tracing && !done;
        unsigned b = __ballot_sync(0xffffffffu, want);
        if (CLAIM_MIN > 1 && b && __popc(b) < CLAIM_MIN && __any_sync(0xffffffffu, tracing)) b = 0u;
        want = want && b;
        if (want && has_path) {
            // Shade the finished ray of this bounce.
            if constexpr (COUNT) {
                work_boxes += ray.na;
                work_tris += ray.nt;
            }
            const DeviceScene s = P.scene(ref);
            Isect I = make_isect(s, ray.h, ray.o, ray.d, tab);
            const bool em = (I.mat >> 31) != 0u;
            const bool ends = em || bounce == 4u;
            // continue_path (material.rs:327-411), split so that a lane that
            // ends at an emitter on bounce 0 stops after the Fresnel value of
            // its gbuffer word (its colour modulation is 1).
            NextRay n{ray.o, ray.d, false};
            float fr = 0.0f;
            if (bounce == 0u || !ends) n = sample_next(s, I, rng, tab);
            if (em) {
                F3 h;
                if (bounce == 0u) fr = fresnel_term(n.d, ray.d, h, tab);
            } else if (!ends) {
                if constexpr (COUNT) work_shades++;
                F3 cm = path_modulation(s, I, n, ray.d, bounce == 0u, tab, fr);
                color = f3(color.x * cm.x, color.y * cm.y, color.z * cm.z);
            }
            if (bounce == 0u) {
                PixelOut g0;
                g0.tex = ((int32_t)I.mat >> 24) & 3;
                g0.tu = I.tu;
                g0.tv = I.tv;
                g0.fresnel = fr;
                P.gbuffer(ref, pack_gbuffer(g0));
                if (em) P.mark_emitter(ref);
            }
            if (ends) {
                F3 sky = sky_intensity(ray.d);
                P.store(ref, em ? f3(color.x * sky.x, color.y * sky.y, color.z * sky.z) : f3(0.0f, 0.0f, 0.0f));
                has_path = false;
            } else {
                bounce++;
                ray.start(n.o, n.d, 1.0e5f, s.nodes, s.geom, tab);
                ray_sel = SELECT_ROUNDS && s.slab_sel && select_form_ray(ray.inv);
                tracing = true;
                P.count_ray(ref);
            }
        }
        // Lanes without a path take the next ones (one atomic per warp).
        const bool need = want && !has_path;
        const unsigned nb = __ballot_sync(0xffffffffu, need);
        if (nb) {
            uint32_t base = 0;
            const int first = __ffs(nb) - 1;
            if (lane == first) base = P.claim((uint32_t)__popc(nb));
            base = __shfl_sync(0xffffffffu, base, first);
            if (need) {
                const uint32_t p = base + (uint32_t)__popc(nb & ((1u << lane) - 1u));
                if (p >= npaths) {
                    done = true;
                } else {
                    F3 o, d;
                    if (P.begin(p, ref, o, d, rng, tab)) {  // else: a group outside its image; take another path
                        const DeviceScene s = P.scene(ref);
                        ray.start(o, d, 1.0e5f, s.nodes, s.geom, tab);
                        ray_sel = SELECT_ROUNDS && s.slab_sel && select_form_ray(ray.inv);
                        color = f3(1.0f, 1.0f, 1.0f);
                        bounce = 0u;
                        has_path = true;
                        tracing = true;
                        P.count_ray(ref);
                    }
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (SELECT_ROUNDS && __all_sync(0xffffffffu, !tracing || ray_sel)) {
            for (int st = 0; st < STEPS && tracing; st++)
                if (ray.step<COUNT, true, SELECT_ROUNDS>(stack, overflow)) tracing = false;
        } else {
            for (int st = 0; st < STEPS && tracing; st++)
                if (ray.step<COUNT, true>(stack, overflow)) tracing = false;
        }
    }
    if constexpr (COUNT) P.work(work_boxes, work_tris, work_shades);
    P.finish(ref);
    return !overflow;
}

}  // namespace cvx
