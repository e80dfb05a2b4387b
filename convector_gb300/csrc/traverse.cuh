// Nearest-hit BVH traversal (bvh.rs:589-657) with the reference's box test
// (aabb.rs:105-141) and triangle test (triangle.rs:59-148), bit-exact.
//
// Two variants share the arithmetic:
//  * PACKET: the 8 threads of an octet (lanes 8k..8k+7 of a warp) are one
//    reference ray packet. Every decision the reference takes over the packet
//    (child order by should_try_before, push by any_masked, cull by
//    is_further_away_than) is a warp vote over the octet, so all 8 threads walk
//    the same node sequence as the reference's packet, node fetches are
//    broadcast loads, and the result is the reference's lane for lane.
//  * SINGLE: each thread walks its own ray with the same decisions taken over
//    itself alone. Results equal the packet traversal except where two
//    triangles tie in t, or where the approximate-reciprocal box test is not
//    conservative for a grazing ray.
#pragma once
#include <type_traits>

#include "layout.cuh"
#include "x86sem.cuh"

namespace cvx {

// Stack entries a traversal may hold before it reports kErrStackOverflow:
// kStackDepth, unless lowered to test that error path
// (cvx_set_traversal_stack_limit). Every stack array keeps kStackDepth
// entries, so any limit up to that keeps all accesses in bounds. Each
// translation unit that traverses has its own copy; set_stack_limit (in
// kernels.cu and wavefront.cu) writes each.
static __constant__ int c_stack_limit = kStackDepth;

struct Hit {
    float t, u, v;
    int32_t tri;
};

struct BoxT {
    float tmin, tmax;
    bool mask;
};

__device__ __forceinline__ BoxT box_test(float lx, float ly, float lz, float hx, float hy, float hz, F3 o, F3 inv) {
    float tx1 = (lx - o.x) * inv.x, tx2 = (hx - o.x) * inv.x;
    float ty1 = (ly - o.y) * inv.y, ty2 = (hy - o.y) * inv.y;
    float tz1 = (lz - o.z) * inv.z, tz2 = (hz - o.z) * inv.z;
    float tmin = xmax(xmin(tx1, tx2), xmax(xmin(ty1, ty2), xmin(tz1, tz2)));
    float tmax = xmin(xmax(tx1, tx2), xmin(xmax(ty1, ty2), xmax(tz1, tz2)));
    return BoxT{tmin, tmax, geq(tmax, tmin)};
}

// The slab test in select form: the near and far plane of each axis are
// picked by the sign of the ray's reciprocal instead of by the x86 min/max of
// the two plane distances (one select for each compare-and-select). It gives
// the bits of box_test when every bound is finite, lo <= hi and no bound is -0
// (DeviceScene::slab_sel), and the reciprocals are finite with |1/d| >= 0.75
// (select_form_ray). With a positive reciprocal, rounding keeps
// (lo - o) / d <= (hi - o) / d; x86 min takes the first and max the second, and
// on equal values the second, which then has the same bits: a zero difference
// is +0 without -0 bounds, and a non-zero one does not round to a zero at
// |1/d| >= 0.75. A negative reciprocal swaps the two.
__device__ __forceinline__ BoxT box_test_sel(float lx, float ly, float lz, float hx, float hy, float hz, F3 o,
                                             F3 inv) {
    const bool px = inv.x > 0.0f, py = inv.y > 0.0f, pz = inv.z > 0.0f;
    float tx1 = (lx - o.x) * inv.x, tx2 = (hx - o.x) * inv.x;
    float ty1 = (ly - o.y) * inv.y, ty2 = (hy - o.y) * inv.y;
    float tz1 = (lz - o.z) * inv.z, tz2 = (hz - o.z) * inv.z;
    float nx = px ? tx1 : tx2, fx = px ? tx2 : tx1;
    float ny = py ? ty1 : ty2, fy = py ? ty2 : ty1;
    float nz = pz ? tz1 : tz2, fz = pz ? tz2 : tz1;
    float tmin = xmax(nx, xmax(ny, nz));
    float tmax = xmin(fx, xmin(fy, fz));
    return BoxT{tmin, tmax, geq(tmax, tmin)};
}
__device__ __forceinline__ bool select_form_ray(F3 inv) {
    return isfinite(inv.x) && isfinite(inv.y) && isfinite(inv.z) && fabsf(inv.x) >= 0.75f &&
           fabsf(inv.y) >= 0.75f && fabsf(inv.z) >= 0.75f;
}

// One triangle against one lane; updates the hit when the reference would
// pick the new intersection (triangle.rs:122-147).
__device__ __forceinline__ void tri_test(const float4* __restrict__ geom, uint32_t i, F3 o, F3 d, bool active,
                                         Hit& h) {
    float4 A = __ldg(geom + 3 * i), B = __ldg(geom + 3 * i + 1), C = __ldg(geom + 3 * i + 2);
    F3 v0 = f3(A.x, A.y, A.z), e1 = f3(B.x, B.y, B.z), e2 = f3(C.x, C.y, C.z), n = f3(A.w, B.w, C.w);
    F3 fr = sub(v0, o);
    float denom = 1.0f / dot(d, n);
    float t = dot(fr, n) * denom;
    F3 c = cross(d, fr);
    float u = dot(c, e2) * denom;
    float v = dot(c, e1) * denom;
    float w = (1.0f - u) - v;
    bool reject = sneg(t) | sneg(u) | sneg(v) | sneg(w) | !active | geq(t, h.t);
    if (!reject) {
        h.t = t;
        h.u = u;
        h.v = v;
        h.tri = (int32_t)i;
    }
}

// Node references: the two children's entries in a node pair's last float4
// (q3.x, q3.y), as the scene upload writes them and the traversal stacks hold
// them. (index << 5) | len: len 0 is an internal node (index = its first
// child), len 1..30 a leaf of len triangles at index; len 31 escapes larger
// leaves, index being the slot of their (index, len) in the float4 at
// nodes[-1 - slot]. Indices are below 2^27 (checked at scene creation).
// The escape is marked unlikely: as an ordinary branch in the packet
// traversal's pop loop it made that traversal up to 1.6x slower, even never
// taken (with the hint, and the stack holding references, the room frame runs
// 0.823 against 0.840 ms with (index, len) pairs on the stack).
__device__ __forceinline__ void leaf_range(const float4* __restrict__ nodes, uint32_t& idx, uint32_t& len) {
    if (__builtin_expect(len == 31u, 0)) {
        const float4 e = __ldg(nodes - 1 - (size_t)idx);
        idx = __float_as_uint(e.x);
        len = __float_as_uint(e.y);
    }
}

__device__ __forceinline__ bool oct_all(unsigned m, bool p) { return (__ballot_sync(m, p) & m) == m; }
__device__ __forceinline__ bool oct_any(unsigned m, bool p) { return (__ballot_sync(m, p) & m) != 0u; }

struct Counters {
    uint32_t aabb, tri;
};

// omask: the octet's lanes in the warp (PACKET) or the calling lane (SINGLE).
// In SINGLE mode an inactive lane must not call this. Returns false on stack
// overflow (the hit is then incomplete). SELECT: the select-form slab test
// (box_test_sel), for a scene with DeviceScene::slab_sel and rays whose
// reciprocals meet select_form_ray (in PACKET mode: all 8 lanes').
template <bool PACKET, bool SELECT = false>
__device__ __forceinline__ bool traverse(const DeviceScene& s, F3 o, F3 d, bool active, unsigned omask, Hit& h,
                                         const ApproxTables& tab, Counters* cnt) {
    F3 inv = f3(x_rcp(d.x, tab), x_rcp(d.y, tab), x_rcp(d.z, tab));
    uint32_t st_ref[kStackDepth];  // node references (leaf_range)
    float st_t[kStackDepth];
    int sp = 0;
    uint32_t na = 2, nt = 0;
    bool ok = true;

    uint32_t pair = 0;
    for (;;) {
        // Test the two children of a pair and push them in the reference order.
        const float4* np = s.nodes + 4 * pair;
        float4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3);
        BoxT b0, b1;
        if constexpr (SELECT) {
            b0 = box_test_sel(q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, o, inv);
            b1 = box_test_sel(q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, o, inv);
        } else {
            b0 = box_test(q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, o, inv);
            b1 = box_test(q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, o, inv);
        }
        bool first0 = !sneg(b0.tmin - b1.tmin);
        bool hit0 = b0.mask & active & !sneg(b0.tmax);
        bool hit1 = b1.mask & active & !sneg(b1.tmax);
        if (PACKET) {
            first0 = oct_all(omask, first0);
            hit0 = oct_any(omask, hit0);
            hit1 = oct_any(omask, hit1);
        }
        // Lanes outside the box never block a cull (aabb.rs:171-177): +inf.
        float c0 = b0.mask ? b0.tmin : __int_as_float(0x7f800000);
        float c1 = b1.mask ? b1.tmin : __int_as_float(0x7f800000);
        const uint32_t r0 = __float_as_uint(q3.x), r1 = __float_as_uint(q3.y);
        int need = (int)hit0 + (int)hit1;
        if (sp + need > c_stack_limit) {
            ok = false;
            break;
        }
        if (first0) {
            if (hit0) { st_ref[sp] = r0; st_t[sp] = c0; sp++; }
            if (hit1) { st_ref[sp] = r1; st_t[sp] = c1; sp++; }
        } else {
            if (hit1) { st_ref[sp] = r1; st_t[sp] = c1; sp++; }
            if (hit0) { st_ref[sp] = r0; st_t[sp] = c0; sp++; }
        }
        // Pop until an internal node whose children must be tested.
        bool descend = false;
        while (sp > 0) {
            sp--;
            uint32_t idx = st_ref[sp] >> 5, len = st_ref[sp] & 31u;
            bool skip = !active | geq(st_t[sp], h.t);
            if (PACKET) skip = oct_all(omask, skip);
            if (skip) continue;
            if (len == 0u) {
                na += 2;
                pair = idx >> 1;
                descend = true;
                break;
            }
            leaf_range(s.nodes, idx, len);
            for (uint32_t i = idx; i < idx + len; i++) tri_test(s.geom, i, o, d, active, h);
            nt += len;
        }
        if (!descend) break;
    }
    if (cnt) {
        cnt->aabb = na;
        cnt->tri = nt;
    }
    return ok;
}

// Asynchronous global-to-shared copies (cp.async) for staging rays.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(__cvta_generic_to_global(gmem)));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one_pending() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Ray supply of the refill traversal. claim() is called by the whole warp in
// an iteration in which the lanes of `b` want a ray; for a wanting lane it
// returns kClaimRay with the ray's data, kClaimDone when the rays are used up,
// or kClaimNone when the ray it took needs no tracing (the source then stored
// that ray's result itself).
enum : int { kClaimNone = 0, kClaimRay = 1, kClaimDone = 2 };

struct RayIn {
    F3 o, d;
    float far;
    const float4* nodes;
    const float4* geom;
};

// Where a refill traversal keeps the stack entries below its top. LocalStack:
// a local array. SharedLocalStack<N>: the first N entries in shared memory,
// in this lane's column of a warp's [N][32] block (no bank conflicts, and pops
// of those never miss the cache), the deeper ones in the local array.
struct LocalStack {
    uint2 (&a)[kStackDepth];
    __device__ __forceinline__ uint2 load(int i) const { return a[i]; }
    __device__ __forceinline__ void store(int i, uint2 v) { a[i] = v; }
};
template <int N>
struct SharedLocalStack {
    uint2* sm;  // entry i at sm[32 * i]
    uint2 (&a)[kStackDepth];
    __device__ __forceinline__ uint2 load(int i) const { return i < N ? sm[32 * i] : a[i]; }
    __device__ __forceinline__ void store(int i, uint2 v) {
        if (i < N) sm[32 * i] = v;
        else a[i] = v;
    }
};

// One lane's single-ray traversal in the refill form. step() does one
// iteration: one node pair (and, LEAF_AFTER_PAIR, the leaf it leads to) or one
// leaf. Decisions and their order are exactly those of traverse<false>: after a
// pair test the child the reference would pop next is processed at once (its
// cull test sees the same hit distance the pop would), the other one is
// pushed, and culled entries are popped within the same iteration.
struct RefillRay {
    static constexpr uint32_t kNone = 0xffffffffu;
    const float4* nodes;
    const float4* geom;
    F3 o, d, inv;
    Hit h;
    // The stack holds (ref, entry distance bits) entries. Its top entry lives
    // in `top`, the entries below it in the caller's local array: a pop takes
    // `top` at once and reloads the next one from memory, so that load's
    // latency hides behind the work on the popped node.
    uint2 top;
    int sp;
    uint32_t cur;  // ref of the node to process; kNone: pop
    uint32_t na, nt;

    __device__ __forceinline__ void start(F3 o_, F3 d_, float far, const float4* nodes_, const float4* geom_,
                                          const ApproxTables& tab) {
        o = o_;
        d = d_;
        nodes = nodes_;
        geom = geom_;
        inv = f3(x_rcp(d.x, tab), x_rcp(d.y, tab), x_rcp(d.z, tab));
        h = Hit{far, 0.0f, 0.0f, -1};
        sp = 0;
        na = 2;
        nt = 0;
        cur = 0;  // the root pair: internal ref with index 0
    }

    // The leaf loops are not unrolled: len is bounded by its 5 bits, and the
    // compiler's unrolled copies of tri_test cost more in instruction fetch
    // than the loop (4M-ray query 0.825 -> 0.808 ms, tube frame 3.24 -> 3.11 ms).
    //
    // Returns true when the ray is finished (its stack is empty): h is then
    // its nearest hit. Sets `overflow` (and finishes the ray) when the stack
    // would overflow. SELECT: the slab test in select form (box_test_sel; the
    // scene and the ray must meet its conditions).
    template <bool COUNT, bool LEAF_AFTER_PAIR, bool SELECT = false, class Stack>
    __device__ __forceinline__ bool step(Stack& stack, bool& overflow) {
        if (cur == kNone) {
            // Pop until an entry survives the cull test (aabb.rs:171-177).
            while (sp > 0) {
                uint2 e = top;
                if (--sp > 0) top = stack.load(sp - 1);
                if (!geq(__uint_as_float(e.y), h.t)) {
                    cur = e.x;
                    break;
                }
            }
            if (cur == kNone) return true;
        }
        uint32_t len = cur & 31u, idx = cur >> 5;
        if (!LEAF_AFTER_PAIR && len != 0u) {  // a popped leaf; the pair loop continues next iteration
            leaf_range(nodes, idx, len);
#pragma unroll 1
            for (uint32_t i = idx; i < idx + len; i++) tri_test(geom, i, o, d, true, h);
            if (COUNT) nt += len;
            cur = kNone;
            return false;
        }
        if (len == 0u) {
            // An internal node: test its two children.
            if (COUNT && cur != 0u) na += 2;  // every pair but the root pair (bvh.rs:604-634)
            // The reference of an internal node is its first child's index (even:
            // checked at scene creation) times 32, which is the byte offset of
            // the child pair (64 bytes per pair).
            const float4* np = reinterpret_cast<const float4*>(reinterpret_cast<const char*>(nodes) + cur);
            float4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3);
            BoxT b0, b1;
            if constexpr (SELECT) {
                b0 = box_test_sel(q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, o, inv);
                b1 = box_test_sel(q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, o, inv);
            } else {
                b0 = box_test(q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, o, inv);
                b1 = box_test(q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, o, inv);
            }
            bool first0 = !sneg(b0.tmin - b1.tmin);
            bool hit0 = b0.mask & !sneg(b0.tmax);
            bool hit1 = b1.mask & !sneg(b1.tmax);
            const uint32_t r0 = __float_as_uint(q3.x), r1 = __float_as_uint(q3.y);
            // The reference pushes `first` then `second` and pops `second` first.
            bool hit_first = first0 ? hit0 : hit1, hit_second = first0 ? hit1 : hit0;
            uint32_t ref_first = first0 ? r0 : r1, ref_second = first0 ? r1 : r0;
            float t_first = first0 ? b0.tmin : b1.tmin, t_second = first0 ? b1.tmin : b0.tmin;
            if (sp + (int)hit_first + (int)hit_second > c_stack_limit) {
                overflow = true;
                sp = 0;
                cur = kNone;
                return false;
            }
            if (hit_first) {
                if (sp > 0) stack.store(sp - 1, top);
                top = make_uint2(ref_first, __float_as_uint(t_first));
                sp++;
            }
            cur = (hit_second && !geq(t_second, h.t)) ? ref_second : kNone;
            if (!LEAF_AFTER_PAIR || cur == kNone) return false;
            len = cur & 31u;
            idx = cur >> 5;
        }
        // LEAF_AFTER_PAIR: a leaf, popped or reached from the pair just tested
        // (the reference would pop it next with no decision in between).
        if (len != 0u) {
            leaf_range(nodes, idx, len);
#pragma unroll 1
            for (uint32_t i = idx; i < idx + len; i++) tri_test(geom, i, o, d, true, h);
            if (COUNT) nt += len;
            cur = kNone;
        }
        return false;
    }
};

template <int N>
__device__ __forceinline__ typename std::conditional<N == 0, LocalStack, SharedLocalStack<N>>::type make_stack(
    uint2* sm, uint2 (&a)[kStackDepth]) {
    if constexpr (N == 0) return LocalStack{a};
    else return SharedLocalStack<N>{sm, a};
}

// Persistent single-ray traversal with ray refill over the rays of `claim`.
// Every iteration each lane processes one node pair or one leaf (RefillRay);
// a lane whose ray is finished takes the next unclaimed ray, so warps stay
// full while rays of different lengths finish.
// The whole warp must call this. `src` provides
//   void store(r, const Hit&, uint32_t boxes, uint32_t triangles)
// (box and triangle counts when COUNT, else 0). LEAF_AFTER_PAIR: a lane whose
// pair test leads to a leaf tests that leaf in the same iteration (fewer
// iterations for deep trees; the order of decisions is the same either way).
// CLAIM_MIN: lanes without a ray wait until that many want one; results do
// not depend on it (each ray's traversal is independent of when it starts).
// Returns false if a ray overflowed the stack (its hit is then incomplete).
// SELECT: every ray whose reciprocals meet select_form_ray is traversed with
// the select-form slab test; the others are handed to src.defer(r) untraced
// (the caller traces them afterwards with the x86 form). STEPS: traversal
// steps per round of the warp's votes (a lane whose ray ends within a round
// waits for the next round's claim).
template <bool COUNT, bool LEAF_AFTER_PAIR, int CLAIM_MIN, int SHARED_STACK = 0, bool SELECT = false, int STEPS = 1,
          class Src, class Claim>
__device__ __forceinline__ bool traverse_refill(const Src& src, Claim& claim, const ApproxTables& tab,
                                                uint2* shared_stack = nullptr) {
    const int lane = threadIdx.x & 31;
    RefillRay ray;
    uint2 local_stack[kStackDepth];
    typename std::conditional<SHARED_STACK == 0, LocalStack, SharedLocalStack<SHARED_STACK>>::type stack =
        make_stack<SHARED_STACK>(shared_stack, local_stack);
    ray.top = make_uint2(0u, 0u);
    ray.sp = 0;
    ray.cur = 0;
    ray.na = ray.nt = 0;
    ray.nodes = ray.geom = nullptr;
    ray.o = ray.d = ray.inv = f3(0, 0, 0);
    ray.h = Hit{0.0f, 0.0f, 0.0f, -1};
    uint32_t r_id = 0;
    bool have = false, done = false, overflow = false;
    for (;;) {
        bool want = !have && !done;
        unsigned b = __ballot_sync(0xffffffffu, want);
        // Claim only when CLAIM_MIN lanes want a ray (or none has work): the
        // claim path then runs with many lanes at once instead of with one or
        // two lanes in nearly every iteration.
        if (CLAIM_MIN > 1 && b && __popc(b) < CLAIM_MIN && __any_sync(0xffffffffu, have)) b = 0u;
        want = want && b;
        if (b) {
            uint32_t r = 0;
            RayIn in;
            int got = claim.claim(b, want, lane, r, in);
            if (want) {
                if (got == kClaimRay) {
                    r_id = r;
                    ray.start(in.o, in.d, in.far, in.nodes, in.geom, tab);
                    have = true;
                    if constexpr (SELECT) {
                        if (!select_form_ray(ray.inv)) {
                            src.defer(r);
                            have = false;
                        }
                    }
                } else if (got == kClaimDone) {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        for (int st = 0; st < STEPS && have; st++) {
            if (ray.step<COUNT, LEAF_AFTER_PAIR, SELECT>(stack, overflow)) {
                src.store(r_id, ray.h, ray.na, ray.nt);
                have = false;
            }
        }
    }
    return !overflow;
}

}  // namespace cvx
