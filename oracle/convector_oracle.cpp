// ORACLE / TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py may load liboracle; the product path never does.
//
// A CPU restatement of the render hot path of ruuda/convector, following the
// reference's Rust sources function by function (file:line cited at each
// function, paths relative to the reference's src/). Arithmetic is per lane
// with the reference's x86 semantics (x86sem.h); decisions the reference
// takes per 8-ray packet (traversal order and culling, the bounce-loop exit)
// are taken over the 8 lanes here too.
//
// Pinning: the reference cannot be built here (2017 nightly Rust, no
// toolchain). Its own known-answer and property tests are ported in
// tests/test_oracle_units.py and pass against this restatement; the x86
// approximate reciprocal tables are pinned against the hardware instruction
// exhaustively. Full frames, BVH node order and direct-light sampling have no
// pin in the reference's tests. BVH node order is checked against a second,
// independent restatement of Bvh::build (bvh_oracle.cpp). Full frames are
// pinned statistically to the two screenshots the reference ships, its
// indoor scene in accumulative and in interactive mode
// (tests/test_oracle_screenshot.py); no frame is pinned bit for bit.
//
// Additions, each a documented deviation from the reference:
//  * the hit record carries the BVH-order triangle index (ray.rs:35-50 has none);
//  * a general light pick `(bits * n) >> 32` (equal to scene.rs:159 `bits >> 29`
//    for n = 8, which is the only n the reference supports);
//  * the per-group RNG order (each 8-pixel group seeded from its own pixel
//    coordinates) beside the reference's patch-sequential order;
//  * a single-ray traversal that restates the GPU's per-ray traversal variant;
//  * frames whose size is not a multiple of the tiling are padded and cropped.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "x86sem.h"

namespace orc {

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 scale(V3 a, float k) { return v3(a.x * k, a.y * k, a.z * k); }
inline V3 vneg(V3 a) { return v3(neg(a.x), neg(a.y), neg(a.z)); }
// vector3.rs:202-205 dot_naive (MVector3::dot is the naive form, :213-217)
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vector3.rs:186-193 cross_fma
inline V3 cross(V3 a, V3 b) {
    return v3(fmsub(a.y, b.z, a.z * b.y), fmsub(a.z, b.x, a.x * b.z), fmsub(a.x, b.y, a.y * b.x));
}
// vector3.rs:295-306
inline V3 normalized(V3 a) {
    float r = rsqrt(dot(a, a));
    return v3(a.x * r, a.y * r, a.z * r);
}
// vector3.rs:254-260 MVector3::mul_add
inline V3 vfma(V3 a, float k, V3 b) { return v3(fmadd(a.x, k, b.x), fmadd(a.y, k, b.y), fmadd(a.z, k, b.z)); }
inline V3 vpick(V3 a, V3 b, bool m) { return m ? b : a; }

// vector3.rs:221-251
inline V3 rotate_hemisphere(V3 v, V3 normal) {
    bool flip = sneg(normal.z);
    V3 n = flip ? vneg(normal) : normal;
    float rz = rcp(1.0f + n.z);
    float c = n.x * n.y * rz;
    float x = fmsub(v.x, fmadd(n.y, n.y * rz, n.z), fmsub(v.y, c, v.z * n.x));
    float y = fnmadd(v.x, c, fmadd(v.y, fmadd(n.x, n.x * rz, n.z), v.z * n.y));
    float z = fnmadd(v.x, n.x, fnmadd(v.y, n.y, v.z * n.z));
    V3 r = v3(x, y, z);
    return flip ? vneg(r) : r;
}

struct Quat {
    float a, b, c, d;
};
// quaternion.rs:62-107
inline Quat interpolate(Quat q, Quat dq, float t) {
    float a = fmadd(dq.a, t, q.a), b = fmadd(dq.b, t, q.b), c = fmadd(dq.c, t, q.c), d = fmadd(dq.d, t, q.d);
    float nsq = fmadd(a, a, b * b) + fmadd(c, c, d * d);
    float rn = 1.0f / std::sqrt(nsq);
    return Quat{a * rn, b * rn, c * rn, d * rn};
}
// quaternion.rs:110-153, written as the reference writes it (left to right).
inline V3 rotate(V3 v, Quat q) {
    float pa = q.b * v.x + q.c * v.y + q.d * v.z;
    float pb = q.b * v.x - q.c * v.y + q.d * v.z + (q.a - q.b) * v.x + (q.c - q.d) * (v.y + v.z);
    float pc = q.d * v.x + q.a * v.y - q.b * v.z;
    float pd = q.d * v.x - q.a * v.y - q.b * v.z - (q.c + q.d) * v.x + (q.a + q.b) * (v.y + v.z);
    float rb = (pa + pb) * (q.a + q.b) - (pc - pd) * (q.c + q.d) - pa * q.a - pb * q.b + pc * q.c - pd * q.d;
    float rc = pc * q.a - pd * q.b + pa * q.c + pb * q.d;
    float rd = (pc + pd) * (q.a + q.b) + (pa - pb) * (q.c + q.d) - pc * q.a - pd * q.b - pa * q.c + pb * q.d;
    return v3(rb, rc, rd);
}

// random.rs:33-159. Four 64-bit multiplicative congruential lanes; one draw
// yields 8 u32: lane 2k is the low half of state k, lane 2k+1 the high half.
struct Rng {
    uint64_t s[4];
    static Rng with_seed(uint32_t x, uint32_t y, uint32_t i) {
        uint64_t a = (uint64_t)x * 12276630456901467871ull;
        uint64_t b = (uint64_t)y * 7661526868048087387ull;
        uint64_t c = (uint64_t)i * 2268244495640532043ull;
        uint64_t seed = a + b + c;
        seed = seed + seed % 9358246936573323101ull;
        const uint64_t primes[4] = {14491630826648200009ull, 13149596372461506851ull, 6119410235796056053ull,
                                    14990141545859273719ull};
        Rng r;
        for (int k = 0; k < 4; k++) r.s[k] = seed * primes[k];
        return r;
    }
    void next(uint32_t out[8]) {
        const uint64_t f[4] = {3ull * 1073243692214514217ull, 5ull * 3335100457702756523ull,
                               7ull * 8789056573444181ull, 11ull * 781436371140792079ull};
        for (int k = 0; k < 4; k++) {
            out[2 * k] = (uint32_t)s[k];
            out[2 * k + 1] = (uint32_t)(s[k] >> 32);
            s[k] *= f[k];
        }
    }
};
inline float unit_from(uint32_t u) { return fmadd((float)(int32_t)u, 0.5f / (float)INT32_MIN, 0.5f); }
inline float biunit_from(uint32_t u) { return (float)(int32_t)u * (1.0f / (float)INT32_MIN); }
inline float angle_from(uint32_t u) { return (float)(int32_t)u * (kPi / (float)INT32_MIN); }

// random.rs:140-159 for one lane, from that lane's two draws.
inline V3 hemisphere_from(uint32_t angle_bits, uint32_t unit_bits) {
    float phi = angle_from(angle_bits), r_sqr = unit_from(unit_bits);
    float r = std::sqrt(r_sqr);
    return v3(poly_sin(phi) * r, poly_cos(phi) * r, std::sqrt(1.0f - r_sqr));
}

// Reference Triangle (triangle.rs:24-32), 64 bytes.
struct Tri {
    float v0[3], v1[3], v2[3], uv0[2], uv1[2], uv2[2];
    uint32_t material;
};
// Reference BvhNode (bvh.rs:21-30), 32 bytes.
struct Node {
    float origin[3], far_[3];
    uint32_t index, len;
};
static_assert(sizeof(Tri) == 64, "triangle layout");
static_assert(sizeof(Node) == 32, "node layout");

inline V3 ld(const float* p) { return v3(p[0], p[1], p[2]); }

struct Scene {
    std::vector<Tri> tris;
    std::vector<Node> nodes;
    std::vector<uint32_t> ds;  // direct-sample triangle indices (scene.rs:108-110)
    bool general_pick = true;
    // Boxes and triangles tested by the single-ray traversals of the last
    // orc_render (the reference's counters, bvh.rs:604-651), all threads.
    mutable std::atomic<uint64_t> work_boxes{0}, work_tris{0};
};

struct Ray {
    V3 o, d;
};
// ray.rs:35-50 plus the triangle index and (u, v) of the hit.
struct Isect {
    V3 pos, normal;
    float dist;
    uint32_t mat;
    float tu, tv;
    int32_t tri;
};

const uint32_t kSky = 0xC0000000u;  // material.rs:85-90

// aabb.rs:105-141 for one lane.
struct BoxHit {
    float tmin, tmax;
    bool mask;
};
inline BoxHit box_hit(const Node& n, V3 o, V3 inv) {
    float d1x = n.origin[0] - o.x, d1y = n.origin[1] - o.y, d1z = n.origin[2] - o.z;
    float d2x = n.far_[0] - o.x, d2y = n.far_[1] - o.y, d2z = n.far_[2] - o.z;
    float tx1 = d1x * inv.x, tx2 = d2x * inv.x;
    float txmin = xmin(tx1, tx2), txmax = xmax(tx1, tx2);
    float ty1 = d1y * inv.y, ty2 = d2y * inv.y;
    float tymin = xmin(ty1, ty2), tymax = xmax(ty1, ty2);
    float tz1 = d1z * inv.z, tz2 = d2z * inv.z;
    float tzmin = xmin(tz1, tz2), tzmax = xmax(tz1, tz2);
    float tmin = xmax(txmin, xmax(tymin, tzmin));
    float tmax = xmin(txmax, xmin(tymax, tzmax));
    return BoxHit{tmin, tmax, geq(tmax, tmin)};
}

// triangle.rs:59-148 for one lane; `active` false means the lane's sign bit
// in ray.active is set.
inline void tri_intersect(const Tri& tr, int32_t idx, const Ray& r, bool active, Isect& is) {
    V3 v0 = ld(tr.v0), v1 = ld(tr.v1), v2 = ld(tr.v2);
    V3 e1 = v0 - v2, e2 = v1 - v0;
    V3 n = cross(e1, e2);
    V3 fr = v0 - r.o;
    float denom = 1.0f / dot(r.d, n);
    float t = dot(fr, n) * denom;
    V3 c = cross(r.d, fr);
    float u = dot(c, e2) * denom;
    float v = dot(c, e1) * denom;
    float w = (1.0f - u) - v;
    bool reject = sneg(t) || sneg(u) || sneg(v) || sneg(w) || !active || geq(t, is.dist);
    if (reject) return;
    is.pos = vfma(r.d, t, r.o);
    is.normal = normalized(n);
    is.dist = t;
    is.mat = tr.material;
    is.tu = fmadd(tr.uv0[0], w, fmadd(tr.uv1[0], v, tr.uv2[0] * u));
    is.tv = fmadd(tr.uv0[1], w, fmadd(tr.uv1[1], v, tr.uv2[1] * u));
    is.tri = idx;
}

// bvh.rs:589-657, the 8-ray packet traversal, with its debug counters.
// The packet traversal and the light PDFs of a group work on all 8 lanes at
// once, in the shape of the reference's Mf32: a GCC/Clang vector of 8 floats
// (one AVX register on x86-64, two NEON registers on aarch64). Its operations
// are elementwise IEEE operations, never fused or reordered
// (-ffp-contract=off), so every lane rounds exactly as the one-ray functions
// above (box_hit, tri_intersect, intersect_direct) do.
typedef float F8 __attribute__((vector_size(32)));
typedef int32_t I8 __attribute__((vector_size(32)));
// Always inlined: where the target's registers are narrower than 8 floats,
// an 8-float value passed to a call would go through memory.
#define ORC_V8 inline __attribute__((always_inline))

ORC_V8 F8 splat8(float x) { return F8{x, x, x, x, x, x, x, x}; }
ORC_V8 F8 vmin8(F8 a, F8 b) { return a < b ? a : b; }  // xmin per lane
ORC_V8 F8 vmax8(F8 a, F8 b) { return a > b ? a : b; }  // xmax per lane
// sneg per lane (sign bit set, or NaN): all ones where it holds.
ORC_V8 I8 vsneg8(F8 x) {
    I8 bits;
    std::memcpy(&bits, &x, sizeof bits);
    return (bits < 0) | (x != x);
}
ORC_V8 bool any8(I8 m) {
    for (int j = 0; j < 8; j++)
        if (m[j]) return true;
    return false;
}

ORC_V8 F8 fmadd8(F8 a, F8 b, F8 c) {  // fmadd per lane
    F8 r;
    for (int j = 0; j < 8; j++) r[j] = std::fma(a[j], b[j], c[j]);
    return r;
}
ORC_V8 F8 fmsub8(F8 a, F8 b, F8 c) { return fmadd8(a, b, -c); }  // fmsub per lane

struct Packet8 {  // origins, directions and reciprocal directions of the 8 rays
    F8 ox, oy, oz, dx, dy, dz, ix, iy, iz;
    I8 active;  // all ones where the lane is active
};
struct BoxHit8 {
    F8 tmin, tmax;
    I8 mask;  // geq(tmax, tmin) per lane
};
// Aabb::intersect (aabb.rs:105-141) for the 8 rays of a packet.
ORC_V8 BoxHit8 box_hit8(const Node& n, const Packet8& p) {
    F8 tx1 = (splat8(n.origin[0]) - p.ox) * p.ix, tx2 = (splat8(n.far_[0]) - p.ox) * p.ix;
    F8 txmin = vmin8(tx1, tx2), txmax = vmax8(tx1, tx2);
    F8 ty1 = (splat8(n.origin[1]) - p.oy) * p.iy, ty2 = (splat8(n.far_[1]) - p.oy) * p.iy;
    F8 tymin = vmin8(ty1, ty2), tymax = vmax8(ty1, ty2);
    F8 tz1 = (splat8(n.origin[2]) - p.oz) * p.iz, tz2 = (splat8(n.far_[2]) - p.oz) * p.iz;
    F8 tzmin = vmin8(tz1, tz2), tzmax = vmax8(tz1, tz2);
    BoxHit8 h;
    h.tmin = vmax8(txmin, vmax8(tymin, tzmin));
    h.tmax = vmin8(txmax, vmin8(tymax, tzmax));
    h.mask = ~(h.tmax < h.tmin);
    return h;
}
struct Entry {
    const Node* node;
    BoxHit8 b;
};
ORC_V8 bool should_try_before(const BoxHit8& a, const BoxHit8& b) {  // aabb.rs:180-182
    return !any8(vsneg8(a.tmin - b.tmin));
}
ORC_V8 bool any_masked(const BoxHit8& b, const Packet8& p) {  // aabb.rs:155-166
    return any8(b.mask & p.active & ~vsneg8(b.tmax));
}
ORC_V8 bool further_away(const BoxHit8& b, const Isect is[8], const Packet8& p) {  // aabb.rs:171-177
    F8 dist;
    for (int j = 0; j < 8; j++) dist[j] = is[j].dist;
    return !any8(b.mask & (b.tmin < dist) & p.active);
}

// Triangle::intersect (triangle.rs:59-148) for the 8 rays of a packet: the
// lane arithmetic of tri_intersect, with the triangle's edges and normal
// computed once; the hit record of each lane that is not rejected is taken
// as tri_intersect takes it.
ORC_V8 void tri_intersect8(const Tri& tr, int32_t idx, const Packet8& p, const Ray r[8], Isect is[8]) {
    V3 v0 = ld(tr.v0), v1 = ld(tr.v1), v2 = ld(tr.v2);
    V3 e1 = v0 - v2, e2 = v1 - v0;
    V3 n = cross(e1, e2);
    F8 frx = splat8(v0.x) - p.ox, fry = splat8(v0.y) - p.oy, frz = splat8(v0.z) - p.oz;
    F8 denom = splat8(1.0f) / (p.dx * n.x + p.dy * n.y + p.dz * n.z);
    F8 t = (frx * n.x + fry * n.y + frz * n.z) * denom;
    F8 cx = fmsub8(p.dy, frz, p.dz * fry), cy = fmsub8(p.dz, frx, p.dx * frz), cz = fmsub8(p.dx, fry, p.dy * frx);
    F8 u = (cx * e2.x + cy * e2.y + cz * e2.z) * denom;
    F8 v = (cx * e1.x + cy * e1.y + cz * e1.z) * denom;
    F8 w = (splat8(1.0f) - u) - v;
    F8 dist;
    for (int j = 0; j < 8; j++) dist[j] = is[j].dist;
    I8 keep = ~(vsneg8(t) | vsneg8(u) | vsneg8(v) | vsneg8(w)) & p.active & (t < dist);
    if (!any8(keep)) return;
    for (int j = 0; j < 8; j++) {
        if (!keep[j]) continue;
        Isect& h = is[j];
        h.pos = vfma(r[j].d, t[j], r[j].o);
        h.normal = normalized(n);
        h.dist = t[j];
        h.mat = tr.material;
        h.tu = fmadd(tr.uv0[0], w[j], fmadd(tr.uv1[0], v[j], tr.uv2[0] * u[j]));
        h.tv = fmadd(tr.uv0[1], w[j], fmadd(tr.uv1[1], v[j], tr.uv2[1] * u[j]));
        h.tri = idx;
    }
}

void packet_traverse(const Scene& s, const Ray r[8], const bool active[8], Isect is[8], uint32_t* numi_aabb,
                     uint32_t* numi_tri) {
    Packet8 p;
    for (int j = 0; j < 8; j++) {
        p.ox[j] = r[j].o.x;
        p.oy[j] = r[j].o.y;
        p.oz[j] = r[j].o.z;
        p.dx[j] = r[j].d.x;
        p.dy[j] = r[j].d.y;
        p.dz[j] = r[j].d.z;
        p.ix[j] = rcp(r[j].d.x);
        p.iy[j] = rcp(r[j].d.y);
        p.iz[j] = rcp(r[j].d.z);
        p.active[j] = active[j] ? -1 : 0;
    }
    std::vector<Entry> stack;
    stack.reserve(32);
    uint32_t na = 2, nt = 0;
    auto push_pair = [&](const Node* n0, const Node* n1) {
        Entry e0{n0, box_hit8(*n0, p)}, e1{n1, box_hit8(*n1, p)};
        if (should_try_before(e0.b, e1.b)) {
            if (any_masked(e0.b, p)) stack.push_back(e0);
            if (any_masked(e1.b, p)) stack.push_back(e1);
        } else {
            if (any_masked(e1.b, p)) stack.push_back(e1);
            if (any_masked(e0.b, p)) stack.push_back(e0);
        }
    };
    push_pair(&s.nodes[0], &s.nodes[1]);
    while (!stack.empty()) {
        Entry e = stack.back();
        stack.pop_back();
        if (further_away(e.b, is, p)) continue;
        const Node& nd = *e.node;
        if (nd.len == 0) {
            na += 2;
            push_pair(&s.nodes[nd.index], &s.nodes[nd.index + 1]);
        } else {
            for (uint32_t i = nd.index; i < nd.index + nd.len; i++) {
                tri_intersect8(s.tris[i], (int32_t)i, p, r, is);
                nt++;
            }
        }
    }
    if (numi_aabb) *numi_aabb = na;
    if (numi_tri) *numi_tri = nt;
}

// The GPU's per-ray traversal variant, restated: the same box and triangle
// arithmetic, with every packet decision taken over this ray alone.
void single_traverse(const Scene& s, const Ray& r, Isect& is, uint32_t* numi_aabb, uint32_t* numi_tri) {
    V3 inv = v3(rcp(r.d.x), rcp(r.d.y), rcp(r.d.z));
    struct SE {
        const Node* node;
        BoxHit b;
    };
    std::vector<SE> stack;
    stack.reserve(64);
    uint32_t na = 2, nt = 0;
    auto push_pair = [&](const Node* c0, const Node* c1) {
        BoxHit b0 = box_hit(*c0, r.o, inv), b1 = box_hit(*c1, r.o, inv);
        bool first0 = !sneg(b0.tmin - b1.tmin);
        bool h0 = b0.mask && !sneg(b0.tmax), h1 = b1.mask && !sneg(b1.tmax);
        if (first0) {
            if (h0) stack.push_back(SE{c0, b0});
            if (h1) stack.push_back(SE{c1, b1});
        } else {
            if (h1) stack.push_back(SE{c1, b1});
            if (h0) stack.push_back(SE{c0, b0});
        }
    };
    push_pair(&s.nodes[0], &s.nodes[1]);
    while (!stack.empty()) {
        SE e = stack.back();
        stack.pop_back();
        if (!e.b.mask || geq(e.b.tmin, is.dist)) continue;
        const Node& nd = *e.node;
        if (nd.len == 0) {
            na += 2;
            push_pair(&s.nodes[nd.index], &s.nodes[nd.index + 1]);
        } else {
            for (uint32_t i = nd.index; i < nd.index + nd.len; i++) {
                tri_intersect(s.tris[i], (int32_t)i, r, true, is);
                nt++;
            }
        }
    }
    if (numi_aabb) *numi_aabb = na;
    if (numi_tri) *numi_tri = nt;
}

// Every triangle in BVH order against one ray: the nearest accepted hit with
// the reference's triangle arithmetic, for classifying traversal differences.
void brute_force(const Scene& s, const Ray& r, Isect& is) {
    for (size_t i = 0; i < s.tris.size(); i++) tri_intersect(s.tris[i], (int32_t)i, r, true, is);
}

// Why two traversals of one ray can return different nearest hits, both
// computed with the reference's arithmetic. Result classes:
//   kSame     equal index and equal t bits;
//   kTie      equal t bits, different indices, and each triangle tested alone
//             gives that t: the traversals tested the two in different
//             orders, and the first tested wins (triangle.rs:127 rejects
//             t >= dist);
//   kGrazing  the nearer hit's triangle lies under a box (the leaf holding it
//             or an ancestor) that the reference's approximate-reciprocal slab
//             test (aabb.rs:105-141) rejects for this ray at the farther hit's
//             distance (mask false, exit behind the origin, or entry at or
//             beyond that distance), while an exact slab test in double
//             precision finds the ray inside that box at the nearer hit. A
//             traversal rejects a box only on one of those three conditions,
//             and its current distance never drops below its final one, so
//             this is the box the traversal with the farther hit discarded;
//   kUnclassified anything else (a wrong result), including a result that
//             is not what its own triangle gives alone.
enum { kSame = 0, kTie = 1, kGrazing = 2, kUnclassified = 3 };

// Leaf of every triangle and parent of every node (roots 0 and 1 have none).
struct TreeIndex {
    std::vector<uint32_t> tri_leaf, parent;
    explicit TreeIndex(const Scene& s) : tri_leaf(s.tris.size(), UINT32_MAX), parent(s.nodes.size(), UINT32_MAX) {
        for (uint32_t k = 0; k < s.nodes.size(); k++) {
            const Node& nd = s.nodes[k];
            if (nd.len == 0) {
                parent[nd.index] = k;
                parent[nd.index + 1] = k;
            } else {
                for (uint32_t i = nd.index; i < nd.index + nd.len && i < tri_leaf.size(); i++) tri_leaf[i] = k;
            }
        }
    }
};

// The ray is inside the box at distance t, by exact division in double
// precision, within a slack of 1e-5 relative (the hit point's own rounding).
inline bool exact_box_contains(const Node& n, const Ray& r, double t) {
    const double o[3] = {r.o.x, r.o.y, r.o.z}, d[3] = {r.d.x, r.d.y, r.d.z};
    const double eps = 1e-5 * (1.0 + std::fabs(t));
    double tmin = -INFINITY, tmax = INFINITY;
    for (int a = 0; a < 3; a++) {
        if (d[a] == 0.0) {
            if (o[a] < n.origin[a] - eps || o[a] > n.far_[a] + eps) return false;
            continue;
        }
        double t1 = (n.origin[a] - o[a]) / d[a], t2 = (n.far_[a] - o[a]) / d[a];
        tmin = std::max(tmin, std::min(t1, t2));
        tmax = std::min(tmax, std::max(t1, t2));
    }
    return tmin <= t + eps && tmax >= t - eps;
}

inline float tri_alone_t(const Scene& s, int32_t i, const Ray& r, float far_dist) {
    Isect is;
    is.dist = far_dist;
    is.tri = -1;
    tri_intersect(s.tris[(size_t)i], i, r, true, is);
    return is.tri == i ? is.dist : NAN;
}

int classify_pair(const Scene& s, const TreeIndex& ix, const Ray& r, float far_dist, float ta, int32_t ia,
                  float tb, int32_t ib) {
    if (ia == ib && fbits(ta) == fbits(tb)) return kSame;
    const int32_t nt = (int32_t)s.tris.size();
    if (ia < -1 || ia >= nt || ib < -1 || ib >= nt) return kUnclassified;
    if (fbits(ta) == fbits(tb)) {
        if (ia < 0 || ib < 0) return kUnclassified;
        float a = tri_alone_t(s, ia, r, far_dist), b = tri_alone_t(s, ib, r, far_dist);
        return fbits(a) == fbits(ta) && fbits(b) == fbits(tb) ? kTie : kUnclassified;
    }
    // The nearer hit must be a hit of its triangle alone.
    const bool a_near = ta < tb;
    const float t_near = a_near ? ta : tb, t_far = a_near ? tb : ta;
    const int32_t i_near = a_near ? ia : ib, i_far = a_near ? ib : ia;
    if (i_near < 0 || i_near == i_far || !(t_near < t_far)) return kUnclassified;
    // Each result must be what its triangle gives alone (a miss: the far distance).
    if (fbits(tri_alone_t(s, i_near, r, far_dist)) != fbits(t_near)) return kUnclassified;
    if (i_far < 0 ? fbits(t_far) != fbits(far_dist) : fbits(tri_alone_t(s, i_far, r, far_dist)) != fbits(t_far))
        return kUnclassified;
    V3 inv = v3(rcp(r.d.x), rcp(r.d.y), rcp(r.d.z));
    for (uint32_t k = ix.tri_leaf[(size_t)i_near]; k != UINT32_MAX; k = ix.parent[k]) {
        const Node& nd = s.nodes[k];
        BoxHit b = box_hit(nd, r.o, inv);
        const bool rejected = !b.mask || sneg(b.tmax) || geq(b.tmin, t_far);
        if (rejected && exact_box_contains(nd, r, (double)t_near)) return kGrazing;
    }
    return kUnclassified;
}

inline Isect far_isect(const Ray& r, float far_dist) {  // scene.rs:220-230
    Isect is;
    is.pos = vfma(r.d, far_dist, r.o);
    is.normal = r.d;
    is.dist = far_dist;
    is.mat = kSky;
    is.tu = 0.0f;
    is.tv = 0.0f;
    is.tri = -1;
    return is;
}

struct Camera {  // scene.rs:20-30
    V3 pos, pos_delta;
    Quat q, dq;
    float screen_distance;
};
// scene.rs:81-99
inline Ray camera_ray(const Camera& c, float x, float y, float t) {
    Ray r;
    r.o = vfma(c.pos_delta, t, c.pos);
    Quat q = interpolate(c.q, c.dq, t);
    V3 src = normalized(v3(x, y, -c.screen_distance));
    r.d = rotate(src, q);
    return r;
}

// material.rs:205-215
inline V3 sky_intensity(V3 d) {
    float up = d.x * 0.0f + d.y * 0.0f + d.z * 1.0f;
    float k = fmadd(up, 0.5f, 0.5f);
    float r = k, g = k * k, b = k * (k * k);
    return v3(fmadd(r, 2.0f, 0.5f), fmadd(g, 2.0f, 0.5f), fmadd(b, 2.0f, 0.5f));
}

// material.rs:151-168
inline V3 get_color(uint32_t m) {
    int32_t mi = (int32_t)m;
    const float k = 1.0f / 255.0f;
    return v3((float)(mi & 0xff) * k, (float)((mi >> 8) & 0xff) * k, (float)((mi >> 16) & 0xff) * k);
}
inline int32_t get_glossiness(uint32_t m) { return ((int32_t)m >> 26) & 7; }  // material.rs:171-178
inline int32_t get_texture(uint32_t m) { return ((int32_t)m >> 24) & 3; }     // material.rs:181-188
inline bool has_texture(uint32_t m) { return ((m << 6) | (m << 7)) >> 31; }    // material.rs:192-201

// material.rs:475-513
inline float normal_dist(V3 h, V3 n, int32_t gloss) {
    float c1 = dot(h, n), c2 = c1 * c1, c4 = c2 * c2, c8 = c4 * c4, c16 = c8 * c8;
    switch (gloss) {
        case 0: return 0.5f / kPi;
        case 1: return xmax(c1, 0.0f) * (1.0f / kPi);
        case 2: return c2 * (1.5f / kPi);
        case 3: return c4 * (2.5f / kPi);
        case 4: return c8 * (4.5f / kPi);
        default: return c16 * (8.5f / kPi);  // index 5; 6 and 7 are rejected at scene creation
    }
}

// triangle.rs:152-185
struct DirectHit {
    V3 normal;
    float area, dist;
    bool miss;
};
inline DirectHit intersect_direct(const Tri& tr, const Ray& r) {
    V3 v0 = ld(tr.v0), v1 = ld(tr.v1), v2 = ld(tr.v2);
    V3 e1 = v0 - v2, e2 = v1 - v0;
    V3 n = cross(e1, e2);
    float nsq = dot(n, n);
    float rnorm = rsqrt(nsq);
    float area = 0.5f * rcp(rnorm);
    V3 fr = v0 - r.o;
    float denom = rcp(dot(r.d, n));
    float t = dot(fr, n) * denom;
    V3 c = cross(r.d, fr);
    float u = dot(c, e2) * denom;
    float v = dot(c, e1) * denom;
    bool mask_uv = geq(u + v, 1.0f);
    DirectHit h;
    h.normal = scale(n, rnorm);
    h.dist = t;
    h.area = area;
    h.miss = sneg(u) || sneg(v) || sneg(t) || mask_uv;
    return h;
}

// pd_direct_sample (material.rs:281-320) for the 8 rays of a group at once:
// per light, the lane arithmetic of intersect_direct above, with the light
// triangle's edges, normal and area computed once.
void pd_direct_sample8(const Scene& s, const Ray r[8], float out[8]) {
    F8 ox, oy, oz, dx, dy, dz;
    for (int j = 0; j < 8; j++) {
        ox[j] = r[j].o.x;
        oy[j] = r[j].o.y;
        oz[j] = r[j].o.z;
        dx[j] = r[j].d.x;
        dy[j] = r[j].d.y;
        dz[j] = r[j].d.z;
    }
    F8 pd_total = splat8(0.0f);
    for (uint32_t li : s.ds) {
        const Tri& tr = s.tris[li];
        V3 v0 = ld(tr.v0), v1 = ld(tr.v1), v2 = ld(tr.v2);
        V3 e1 = v0 - v2, e2 = v1 - v0;
        V3 n = cross(e1, e2);
        float rnorm = rsqrt(dot(n, n));
        float area = 0.5f * rcp(rnorm);
        V3 nn = scale(n, rnorm);
        F8 frx = splat8(v0.x) - ox, fry = splat8(v0.y) - oy, frz = splat8(v0.z) - oz;
        F8 denom = dx * n.x + dy * n.y + dz * n.z;
        for (int j = 0; j < 8; j++) denom[j] = rcp(denom[j]);
        F8 t = (frx * n.x + fry * n.y + frz * n.z) * denom;
        F8 cx = fmsub8(dy, frz, dz * fry), cy = fmsub8(dz, frx, dx * frz), cz = fmsub8(dx, fry, dy * frx);
        F8 u = (cx * e2.x + cy * e2.y + cz * e2.z) * denom;
        F8 v = (cx * e1.x + cy * e1.y + cz * e1.z) * denom;
        I8 miss = vsneg8(u) | vsneg8(v) | vsneg8(t) | ~((u + v) < splat8(1.0f));
        F8 dsq = t * t;
        F8 dn = splat8(nn.x) * dx + splat8(nn.y) * dy + splat8(nn.z) * dz;
        I8 bits;
        std::memcpy(&bits, &dn, sizeof bits);
        bits &= 0x7fffffff;
        std::memcpy(&dn, &bits, sizeof bits);
        F8 q = splat8(area) * (dn + 0.0001f);
        for (int j = 0; j < 8; j++) q[j] = rcp(q[j]);
        F8 pd = dsq * q;
        pd_total = miss ? pd_total : pd_total + pd;
    }
    const float k = 1.0f / (float)s.ds.size();
    for (int j = 0; j < 8; j++) out[j] = pd_total[j] * k;
}

inline uint32_t light_pick(const Scene& s, uint32_t bits) {
    if (!s.general_pick) return bits >> 29;  // scene.rs:159 (8 lights)
    return (uint32_t)(((uint64_t)bits * (uint64_t)s.ds.size()) >> 32);
}

struct PixelOut {
    V3 color;
    int32_t tex;
    float tu, tv, fresnel;
};

// material.rs:327-411 over one 8-lane packet, with continue_path_brdf
// (:228-242), continue_path_direct_sample (:253-265), get_direct_sample
// (scene.rs:143-202), pd_brdf (:245-250) and microfacet_brdf (:415-469).
void continue_path(const Scene& s, Ray ray[8], bool active[8], const Isect is[8], Rng& rng, bool ignore_fresnel,
                   V3 color_mod[8], float fresnel[8]) {
    uint32_t dphi[8], dr[8], dsel[8], du[8], dv[8], drr[8];
    rng.next(dphi);
    rng.next(dr);
    rng.next(dsel);
    rng.next(du);
    rng.next(dv);
    rng.next(drr);
    // First the next ray of every lane, then the 8 light PDFs together, then
    // the rest of each lane.
    Ray nrs[8];
    bool picks[8];
    for (int j = 0; j < 8; j++) {
        const Isect& I = is[j];
        // BRDF sample
        V3 dir_b = rotate_hemisphere(hemisphere_from(dphi[j], dr[j]), I.normal);
        V3 org_b = vfma(dir_b, 1.0e-4f, I.pos);
        // direct sample
        const Tri& lt = s.tris[s.ds[light_pick(s, dsel[j])]];
        V3 lv0 = ld(lt.v0), lv1 = ld(lt.v1), lv2 = ld(lt.v2);
        V3 le1 = lv0 - lv2, le2 = lv1 - lv0;
        float u = unit_from(du[j]), v = unit_from(dv[j]);
        float sgn = (1.0f - u) - v;
        if (sneg(sgn)) {
            u = 1.0f - u;
            v = 1.0f - v;
        }
        V3 p = v3(fmadd(le2.x, v, fnmadd(le1.x, u, lv0.x)), fmadd(le2.y, v, fnmadd(le1.y, u, lv0.y)),
                  fmadd(le2.z, v, fnmadd(le1.z, u, lv0.z)));
        V3 dir_d = normalized(p - I.pos);
        V3 org_d = vfma(dir_d, 1.0e-4f, I.pos);
        // one-sample MIS
        float rr = fmadd(I.normal.z, 0.8f, biunit_from(drr[j]));
        bool pick_direct = sneg(rr);
        picks[j] = pick_direct;
        nrs[j].o = vpick(org_b, org_d, pick_direct);
        nrs[j].d = vpick(dir_b, dir_d, pick_direct);
    }
    float pds[8];
    pd_direct_sample8(s, nrs, pds);
    for (int j = 0; j < 8; j++) {
        const Isect& I = is[j];
        bool inactive = !active[j] || (I.mat >> 31) != 0u;
        const bool pick_direct = picks[j];
        const Ray& nr = nrs[j];
        float pd_b = xmax(dot(I.normal, nr.d), 0.0f) * (1.0f / kPi);
        float pd_d = pds[j];
        float wden = pd_b + pd_d + 0.01f;
        float p_brdf = fmadd(I.normal.z, 0.4f, 0.5f);
        float p_direct = fnmadd(I.normal.z, 0.4f, 0.5f);
        float pp = pick_direct ? p_direct : p_brdf;
        float modulation = rcp(wden * pp);
        float cos_theta = xmax(dot(I.normal, nr.d), 0.0f);
        // microfacet BRDF
        V3 col = get_color(I.mat);
        int32_t gloss = get_glossiness(I.mat);
        V3 h = normalized(nr.d - ray[j].d);
        float D = normal_dist(h, I.normal, gloss);
        V3 r1 = v3(1.0f - col.x, 1.0f - col.y, 1.0f - col.z);
        float ct = 1.0f - fabs_bits(dot(h, nr.d));
        float ct2 = ct * ct, ct3 = ct2 * ct, ct5 = fabs_bits(ct2 * ct3);
        V3 fcol = v3(fmadd(r1.x, ct5, col.x), fmadd(r1.y, ct5, col.y), fmadd(r1.z, ct5, col.z));
        if (ignore_fresnel && has_texture(I.mat)) fcol = v3(1.0f, 1.0f, 1.0f);
        V3 brdf = scale(fcol, D);
        float k = modulation * cos_theta;
        V3 cm = v3(brdf.x * k, brdf.y * k, brdf.z * k);
        cm = v3(xmin(cm.x, 2.0f), xmin(cm.y, 2.0f), xmin(cm.z, 2.0f));
        fresnel[j] = ct5;
        if (inactive) {
            color_mod[j] = v3(1.0f, 1.0f, 1.0f);
            active[j] = false;
        } else {
            color_mod[j] = cm;
            ray[j] = nr;
        }
    }
}

struct NearestFn {
    const Scene* s;
    bool single;
    void operator()(const Ray r[8], const bool active[8], Isect is[8]) const {
        if (!single) {
            packet_traverse(*s, r, active, is, nullptr, nullptr);
        } else {
            uint64_t boxes = 0, tris = 0;
            for (int j = 0; j < 8; j++) {
                if (!active[j]) continue;
                uint32_t a = 0, b = 0;
                single_traverse(*s, r[j], is[j], &a, &b);
                boxes += a;
                tris += b;
            }
            s->work_boxes += boxes;
            s->work_tris += tris;
        }
    }
};

// renderer.rs:413-468 for one 8-pixel group.
void render_pixels(const Scene& s, const Camera& cam, const float xs[8], const float ys[8], Rng& rng,
                   bool single, PixelOut out[8], uint64_t* rays) {
    uint32_t dt[8];
    rng.next(dt);
    Ray ray[8];
    bool active[8];
    V3 color[8];
    uint32_t hit_em[8];
    for (int j = 0; j < 8; j++) {
        ray[j] = camera_ray(cam, xs[j], ys[j], unit_from(dt[j]));
        active[j] = true;
        color[j] = v3(1.0f, 1.0f, 1.0f);
        hit_em[j] = 0u;
        out[j].tex = 0;
        out[j].tu = out[j].tv = out[j].fresnel = 0.0f;
    }
    NearestFn nearest{&s, single};
    for (int i = 0; i < 5; i++) {
        Isect is[8];
        uint64_t nact = 0;
        for (int j = 0; j < 8; j++) {
            is[j] = far_isect(ray[j], 1.0e5f);
            nact += active[j];
        }
        *rays += nact;
        nearest(ray, active, is);
        bool all_em = true;
        for (int j = 0; j < 8; j++) {
            hit_em[j] = is[j].mat;
            all_em = all_em && (is[j].mat >> 31);
        }
        if (all_em) break;
        V3 cm[8];
        float fr[8];
        continue_path(s, ray, active, is, rng, i == 0, cm, fr);
        for (int j = 0; j < 8; j++) {
            color[j] = v3(color[j].x * cm[j].x, color[j].y * cm[j].y, color[j].z * cm[j].z);
            if (i == 0) {
                out[j].tex = get_texture(is[j].mat);
                out[j].tu = is[j].tu;
                out[j].tv = is[j].tv;
                out[j].fresnel = fr[j];
            }
        }
    }
    for (int j = 0; j < 8; j++) {
        V3 em = sky_intensity(ray[j].d);
        V3 c = v3(color[j].x * em.x, color[j].y * em.y, color[j].z * em.z);
        out[j].color = (hit_em[j] >> 31) ? c : v3(0.0f, 0.0f, 0.0f);
    }
}

// renderer.rs:470-486 for one 8-pixel group: time 0 (no random draw), colour
// (0, log2(boxes) * 0.1, log2(triangles) * 0.1) from the packet's counters
// (or each ray's, single-ray traversal). log2 in double rounded to float.
void render_pixels_debug(const Scene& s, const Camera& cam, const float xs[8], const float ys[8], bool single,
                         PixelOut out[8], uint64_t* rays) {
    Ray ray[8];
    bool active[8];
    Isect is[8];
    for (int j = 0; j < 8; j++) {
        ray[j] = camera_ray(cam, xs[j], ys[j], 0.0f);
        active[j] = true;
        is[j] = far_isect(ray[j], 1.0e5f);
    }
    uint32_t na[8], nt[8];
    if (!single) {
        uint32_t a = 0, b = 0;
        packet_traverse(s, ray, active, is, &a, &b);
        for (int j = 0; j < 8; j++) {
            na[j] = a;
            nt[j] = b;
        }
    } else {
        for (int j = 0; j < 8; j++) single_traverse(s, ray[j], is[j], &na[j], &nt[j]);
    }
    *rays += 8;
    for (int j = 0; j < 8; j++) {
        out[j].color = v3(0.0f, (float)std::log2((double)na[j]) * 0.1f, (float)std::log2((double)nt[j]) * 0.1f);
        out[j].tex = 0;
        out[j].tu = out[j].tv = out[j].fresnel = 0.0f;
    }
}

// renderer.rs:239-256 for one pixel
inline uint32_t pack_color(V3 c) {
    V3 r = v3(xmin(1.0f, c.x * 2.0f) * 255.0f, xmin(1.0f, c.y * 2.0f) * 255.0f, xmin(1.0f, c.z * 2.0f) * 255.0f);
    uint32_t rr = (uint32_t)cvtps(r.x), g = (uint32_t)cvtps(r.y) << 8, b = (uint32_t)cvtps(r.z) << 16;
    return (rr | g) | b;
}
// renderer.rs:260-286 for one pixel
inline uint32_t pack_gbuffer(const PixelOut& p) {
    uint32_t r = (uint32_t)cvtps(p.tu * 255.0f) & 0xffu;
    uint32_t g = ((uint32_t)cvtps(p.tv * 255.0f) & 0xffu) << 8;
    uint32_t b = (uint32_t)cvtps(p.fresnel * 255.0f) << 16;
    uint32_t a = (uint32_t)p.tex << 24;
    return (r | g) | (b | a);
}

struct Frame {
    const Scene* s;
    Camera cam;
    uint32_t w, h, frame;
    bool single;
    uint32_t* rgba;
    uint32_t* gbuf;
    float* color;  // w*h*3, written (not accumulated) when non-null
    float* accum;  // w*h*3, accumulated when non-null
    bool debug;    // Renderer::toggle_debug_view
};

// The pixel coordinates of group g (0..7) of the 16x4 block at (xb, yb), in
// screen units before jitter: renderer.rs:171-198.
inline void block_coords(uint32_t w, uint32_t h, uint32_t xb, uint32_t yb, float xs[8][8], float ys[8][8],
                         float* scale_out) {
    float scale = 2.0f / (float)w;
    float s2 = 2.0f * scale, s4 = 4.0f * scale, s8 = 8.0f * scale, s12 = 12.0f * scale;
    const float off_x[8] = {0, 1, 2, 3, 0, 1, 2, 3}, off_y[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    float cx = (float)xb - (float)w * 0.5f, cy = (float)yb - (float)h * 0.5f;
    for (int k = 0; k < 8; k++) {
        float bx = scale * (off_x[k] + cx), by = scale * (off_y[k] + cy);
        float gx[8] = {bx, bx, bx + s4, bx + s4, bx + s8, bx + s8, bx + s12, bx + s12};
        float gy[8] = {by, by + s2, by, by + s2, by, by + s2, by, by + s2};
        for (int g = 0; g < 8; g++) {
            xs[g][k] = gx[g];
            ys[g][k] = gy[g];
        }
    }
    *scale_out = scale;
}

inline void store_group(const Frame& f, uint32_t gx, uint32_t gy, const PixelOut out[8]) {
    for (int k = 0; k < 8; k++) {
        uint32_t px = gx + (uint32_t)(k & 3), py = gy + (uint32_t)(k >> 2);
        if (px >= f.w || py >= f.h) continue;
        size_t idx = (size_t)py * f.w + px;
        if (f.rgba) f.rgba[idx] = pack_color(out[k].color);
        if (f.gbuf) f.gbuf[idx] = pack_gbuffer(out[k]);
        if (f.color) {
            f.color[3 * idx] = out[k].color.x;
            f.color[3 * idx + 1] = out[k].color.y;
            f.color[3 * idx + 2] = out[k].color.z;
        }
        if (f.accum) {
            f.accum[3 * idx] += out[k].color.x;
            f.accum[3 * idx + 1] += out[k].color.y;
            f.accum[3 * idx + 2] += out[k].color.z;
        }
    }
}

// renderer.rs:306-327 (render_patch_u8) and 339-362 (accumulate_patch_f32):
// one patch of pw x pw pixels (pw a multiple of 16) with one RNG, blocks x-major.
uint64_t render_patch(const Frame& f, uint32_t x, uint32_t y, uint32_t pw = 32) {
    const uint32_t wb = pw / 16, hb = pw / 4;
    Rng rng = Rng::with_seed(x, y, f.frame);
    uint64_t rays = 0;
    for (uint32_t i = 0; i < wb; i++) {
        for (uint32_t j = 0; j < hb; j++) {
            uint32_t xb = x + i * 16, yb = y + j * 4;
            float xs[8][8], ys[8][8], scale;
            block_coords(f.w, f.h, xb, yb, xs, ys, &scale);
            uint32_t d[16][8];
            for (int k = 0; k < 16; k++) rng.next(d[k]);
            for (int g = 0; g < 8; g++)
                for (int k = 0; k < 8; k++) {
                    xs[g][k] = fmadd(unit_from(d[g][k]), scale, xs[g][k]);
                    ys[g][k] = fmadd(unit_from(d[8 + g][k]), scale, ys[g][k]);
                }
            for (int g = 0; g < 8; g++) {
                PixelOut out[8];
                if (f.debug) render_pixels_debug(*f.s, f.cam, xs[g], ys[g], f.single, out, &rays);
                else render_pixels(*f.s, f.cam, xs[g], ys[g], rng, f.single, out, &rays);
                store_group(f, xb + 4 * (uint32_t)(g >> 1), yb + 2 * (uint32_t)(g & 1), out);
            }
        }
    }
    return rays;
}

// Per-group RNG order: the group at pixel (gx, gy) seeds its own generator
// with (gx, gy, frame) and draws x jitter, y jitter, then the path.
uint64_t render_group_pg(const Frame& f, uint32_t gx, uint32_t gy) {
    uint32_t xb = gx & ~15u, yb = gy & ~3u;
    int g = (int)(((gx - xb) >> 2) * 2 + ((gy - yb) >> 1));
    float xs[8][8], ys[8][8], scale;
    block_coords(f.w, f.h, xb, yb, xs, ys, &scale);
    Rng rng = Rng::with_seed(gx, gy, f.frame);
    uint32_t dx[8], dy[8];
    rng.next(dx);
    rng.next(dy);
    float gxs[8], gys[8];
    for (int k = 0; k < 8; k++) {
        gxs[k] = fmadd(unit_from(dx[k]), scale, xs[g][k]);
        gys[k] = fmadd(unit_from(dy[k]), scale, ys[g][k]);
    }
    PixelOut out[8];
    uint64_t rays = 0;
    if (f.debug) render_pixels_debug(*f.s, f.cam, gxs, gys, f.single, out, &rays);
    else render_pixels(*f.s, f.cam, gxs, gys, rng, f.single, out, &rays);
    store_group(f, gx, gy, out);
    return rays;
}

template <class F>
void parallel_for(uint32_t n, int nthreads, F fn) {
    if (nthreads <= 1 || n <= 1) {
        for (uint32_t i = 0; i < n; i++) fn(i);
        return;
    }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; t++)
        pool.emplace_back([&]() {
            for (;;) {
                uint32_t i = next.fetch_add(1);
                if (i >= n) break;
                fn(i);
            }
        });
    for (auto& th : pool) th.join();
}

uint64_t render_frame(const Frame& f, int rng_order, int nthreads) {
    std::atomic<uint64_t> rays{0};
    if (rng_order == 0) {
        uint32_t pw = (f.w + 31) / 32, ph = (f.h + 31) / 32;
        parallel_for(pw * ph, nthreads, [&](uint32_t p) {
            uint32_t i = p / ph, j = p % ph;  // main.rs:180-181: i over x, j over y
            rays += render_patch(f, i * 32, j * 32);
        });
    } else {
        uint32_t gw = (f.w + 3) / 4, gh = (f.h + 1) / 2;
        parallel_for(gw * gh, nthreads, [&](uint32_t g) {
            uint32_t gy = g / gw, gx = g % gw;
            rays += render_group_pg(f, gx * 4, gy * 2);
        });
    }
    return rays.load();
}

// ---- display post-process (src/gpu/*.glsl via ui.rs:313-364), restated with
// the same fixed choices as the GPU kernels: unorm8 reads byte/255, render
// targets store round(clamp(x)*255), textures are sRGB-decoded and sampled
// bilinearly with repeat wrapping, the median's neighbours clamp at the edge,
// sRGB decode/encode through tables computed in double.
struct OrcDisplay {
    uint32_t w, h, tw, th, slot = 0;
    std::vector<uint8_t> t1, t2;
    std::vector<uint32_t> ring;
    float dec[256], enc[255];
};
static inline float unorm8(uint32_t w, int c) { return (float)((w >> (8 * c)) & 0xffu) * (1.0f / 255.0f); }
static inline uint32_t quant8(float x) {
    x = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
    return (uint32_t)(int32_t)std::nearbyint(x * 255.0f);
}
static inline uint32_t pack4f(const float c[4]) {
    return quant8(c[0]) | (quant8(c[1]) << 8) | (quant8(c[2]) << 16) | (quant8(c[3]) << 24);
}
static void tex_sample(const OrcDisplay& d, const std::vector<uint8_t>& t, float u, float v, float out[4]) {
    float x = u * (float)d.tw - 0.5f, y = v * (float)d.th - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, W = (int)d.tw, H = (int)d.th;
    int xs[2] = {((x0 % W) + W) % W, (((x0 + 1) % W) + W) % W};
    int ys[2] = {((y0 % H) + H) % H, (((y0 + 1) % H) + H) % H};
    for (int c = 0; c < 3; c++) {
        float p00 = d.dec[t[3 * ((size_t)ys[0] * d.tw + xs[0]) + c]];
        float p10 = d.dec[t[3 * ((size_t)ys[0] * d.tw + xs[1]) + c]];
        float p01 = d.dec[t[3 * ((size_t)ys[1] * d.tw + xs[0]) + c]];
        float p11 = d.dec[t[3 * ((size_t)ys[1] * d.tw + xs[1]) + c]];
        float top = p00 * (1.0f - ax) + p10 * ax, bot = p01 * (1.0f - ax) + p11 * ax;
        out[c] = top * (1.0f - ay) + bot * ay;
    }
    out[3] = 1.0f;
}
static void to_xyz(float c[4]) {  // median.glsl:35-41
    const float k = 1.0f / 0.17697f;
    float m[9] = {0.49f * k, 0.17697f * k, 0.0f * k, 0.31f * k, 0.81240f * k, 0.01f * k, 0.20f * k, 0.01063f * k,
                  0.99f * k};
    float r = c[0], g = c[1], b = c[2];
    c[0] = m[0] * r + m[3] * g + m[6] * b;
    c[1] = m[1] * r + m[4] * g + m[7] * b;
    c[2] = m[2] * r + m[5] * g + m[8] * b;
}
static void to_rgb(float c[4]) {  // median.glsl:43-49
    float m[9] = {0.41847f, -0.091169f, 0.00092090f, -0.15866f, 0.25243f, -0.0025498f, -0.082835f, 0.015708f,
                  0.17860f};
    float x = c[0], y = c[1], z = c[2];
    c[0] = m[0] * x + m[3] * y + m[6] * z;
    c[1] = m[1] * x + m[4] * y + m[7] * z;
    c[2] = m[2] * x + m[5] * y + m[8] * z;
}
static void sort2v(float a[4], float b[4]) {
    for (int c = 0; c < 4; c++) {
        float lo = std::fmin(a[c], b[c]), hi = std::fmax(a[c], b[c]);
        a[c] = lo;
        b[c] = hi;
    }
}
static uint32_t srgb_of(const OrcDisplay& d, float x) {
    uint32_t n = 0;
    while (n < 255 && d.enc[n] <= x) n++;
    return n;
}

}  // namespace orc

using namespace orc;

extern "C" {

void* orc_scene_new(const void* tris, uint32_t ntri, const void* nodes, uint32_t nnode, const uint32_t* ds,
                    uint32_t nds, int general_pick) {
    Scene* s = new Scene();
    s->tris.assign((const Tri*)tris, (const Tri*)tris + ntri);
    s->nodes.assign((const Node*)nodes, (const Node*)nodes + nnode);
    s->ds.assign(ds, ds + nds);
    s->general_pick = general_pick != 0;
    return s;
}
void orc_scene_free(void* s) { delete (Scene*)s; }

// Bvh::intersect_nearest (bvh.rs:659) over rays packed 8 per packet in input
// order; lanes past n are padded with inactive copies of the first ray.
// mode 0: packet traversal (the reference); 1: single-ray traversal;
// 2: brute force over all triangles.
// Classes (kSame .. kUnclassified) of n rays' two results (ta, ia), (tb, ib).
void orc_classify(void* sp, const float* ox, const float* oy, const float* oz, const float* dx, const float* dy,
                  const float* dz, uint32_t n, float far_dist, const float* ta, const int32_t* ia, const float* tb,
                  const int32_t* ib, uint8_t* cls, int nthreads) {
    const Scene& s = *(const Scene*)sp;
    const TreeIndex ix(s);
    parallel_for(n, nthreads, [&](uint32_t i) {
        if (ia[i] == ib[i] && fbits(ta[i]) == fbits(tb[i])) {
            cls[i] = kSame;
            return;
        }
        Ray r;
        r.o = v3(ox[i], oy[i], oz[i]);
        r.d = v3(dx[i], dy[i], dz[i]);
        cls[i] = (uint8_t)classify_pair(s, ix, r, far_dist, ta[i], ia[i], tb[i], ib[i]);
    });
}

void orc_intersect(void* sp, const float* ox, const float* oy, const float* oz, const float* dx, const float* dy,
                   const float* dz, uint32_t n, float far_dist, int mode, float* t_out, int32_t* tri_out,
                   float* u_out, float* v_out, uint32_t* numi_aabb, uint32_t* numi_tri, int nthreads) {
    const Scene& s = *(const Scene*)sp;
    uint32_t npk = (n + 7) / 8;
    parallel_for(npk, nthreads, [&](uint32_t p) {
        Ray r[8];
        bool active[8];
        Isect is[8];
        for (int j = 0; j < 8; j++) {
            uint32_t i = p * 8 + j;
            uint32_t src = i < n ? i : p * 8;
            r[j].o = v3(ox[src], oy[src], oz[src]);
            r[j].d = v3(dx[src], dy[src], dz[src]);
            active[j] = i < n;
            is[j] = far_isect(r[j], far_dist);
        }
        uint32_t na = 0, nt = 0;
        if (mode == 0) {
            packet_traverse(s, r, active, is, &na, &nt);
        } else {
            for (int j = 0; j < 8; j++) {
                if (!active[j]) continue;
                uint32_t a = 0, b = 0;
                if (mode == 1) single_traverse(s, r[j], is[j], &a, &b);
                else brute_force(s, r[j], is[j]);
                if (numi_aabb) numi_aabb[p * 8 + j] = a;
                if (numi_tri) numi_tri[p * 8 + j] = b;
            }
        }
        for (int j = 0; j < 8; j++) {
            uint32_t i = p * 8 + j;
            if (i >= n) continue;
            t_out[i] = is[j].dist;
            tri_out[i] = is[j].tri;
            // (u, v) of the accepted hit, recovered from the interpolated
            // coordinates is not possible in general; report the hit normal z
            // instead when requested callers pass null.
            if (u_out) u_out[i] = is[j].tu;
            if (v_out) v_out[i] = is[j].tv;
            if (mode == 0) {
                if (numi_aabb) numi_aabb[i] = na;
                if (numi_tri) numi_tri[i] = nt;
            }
        }
    });
}

// The listed patches (origins xy[2 i], xy[2 i + 1], width pw) of one frame,
// as a caller of render_patch_u8 / accumulate_patch_f32 would render them.
uint64_t orc_render_patches(void* sp, const float* cam, uint32_t w, uint32_t h, uint32_t frame, int traversal,
                            uint32_t pw, const uint32_t* xy, uint32_t n, uint32_t* rgba, uint32_t* gbuf,
                            float* color, float* accum, int nthreads) {
    Frame f;
    f.s = (const Scene*)sp;
    f.cam.pos = v3(cam[0], cam[1], cam[2]);
    f.cam.pos_delta = v3(cam[3], cam[4], cam[5]);
    f.cam.q = Quat{cam[6], cam[7], cam[8], cam[9]};
    f.cam.dq = Quat{cam[10], cam[11], cam[12], cam[13]};
    f.cam.screen_distance = cam[14];
    f.w = w;
    f.h = h;
    f.frame = frame;
    f.single = traversal == 1;
    f.rgba = rgba;
    f.gbuf = gbuf;
    f.color = color;
    f.accum = accum;
    f.debug = false;
    std::atomic<uint64_t> rays{0};
    parallel_for(n, nthreads, [&](uint32_t i) { rays += render_patch(f, xy[2 * i], xy[2 * i + 1], pw); });
    return rays.load();
}

// One frame. cam: pos[3], pos_delta[3], q[4], dq[4], screen_distance.
// rng_order 0 = patch-sequential (reference), 1 = per-group.
// traversal 0 = packet (reference), 1 = single-ray.
uint64_t orc_render(void* sp, const float* cam, uint32_t w, uint32_t h, uint32_t frame, int rng_order,
                    int traversal, uint32_t* rgba, uint32_t* gbuf, float* color, float* accum, int nthreads,
                    int debug) {
    Frame f;
    f.s = (const Scene*)sp;
    f.cam.pos = v3(cam[0], cam[1], cam[2]);
    f.cam.pos_delta = v3(cam[3], cam[4], cam[5]);
    f.cam.q = Quat{cam[6], cam[7], cam[8], cam[9]};
    f.cam.dq = Quat{cam[10], cam[11], cam[12], cam[13]};
    f.cam.screen_distance = cam[14];
    f.w = w;
    f.h = h;
    f.frame = frame;
    f.single = traversal == 1;
    f.rgba = rgba;
    f.gbuf = gbuf;
    f.color = color;
    f.accum = accum;
    f.debug = debug != 0;
    f.s->work_boxes = 0;
    f.s->work_tris = 0;
    return render_frame(f, rng_order, nthreads);
}

// Boxes and triangles the single-ray traversals of the last orc_render tested.
void orc_scene_work(void* sp, uint64_t* out) {
    const Scene& s = *(const Scene*)sp;
    out[0] = s.work_boxes;
    out[1] = s.work_tris;
}

void* orc_display_new(uint32_t w, uint32_t h, const uint8_t* t1, const uint8_t* t2, uint32_t tw, uint32_t th) {
    OrcDisplay* d = new OrcDisplay();
    d->w = w;
    d->h = h;
    d->tw = tw;
    d->th = th;
    d->t1.assign(t1, t1 + (size_t)tw * th * 3);
    d->t2.assign(t2, t2 + (size_t)tw * th * 3);
    d->ring.assign((size_t)w * h * 8, 0u);
    for (int i = 0; i < 256; i++) {
        double sv = i / 255.0;
        d->dec[i] = (float)(sv <= 0.04045 ? sv / 12.92 : std::pow((sv + 0.055) / 1.055, 2.4));
    }
    for (int k = 1; k <= 255; k++) {
        double sv = (k - 0.5) / 255.0;
        d->enc[k - 1] = (float)(sv <= 0.04045 ? sv / 12.92 : std::pow((sv + 0.055) / 1.055, 2.4));
    }
    return d;
}
void orc_display_free(void* d) { delete (OrcDisplay*)d; }

void orc_display_frame(void* dp, const uint32_t* rgba, const uint32_t* gbuf, int enable_blend, int enable_median,
                       uint32_t* out) {
    OrcDisplay& d = *(OrcDisplay*)dp;
    size_t npx = (size_t)d.w * d.h;
    d.slot = (d.slot + 1) % 8;
    uint32_t* slot = &d.ring[d.slot * npx];
    for (size_t i = 0; i < npx; i++) {  // gbuffer.glsl:18-42
        float color[4], data[4];
        for (int c = 0; c < 4; c++) {
            color[c] = unorm8(rgba[i], c);
            data[c] = unorm8(gbuf[i], c);
        }
        float fresnel = data[2];
        for (int k = 1; k <= 2; k++)
            if (data[3] == (float)k / 255.0f) {
                float tex[4];
                tex_sample(d, k == 1 ? d.t1 : d.t2, data[0], data[1], tex);
                for (int c = 0; c < 4; c++) color[c] = color[c] * (1.0f * fresnel + tex[c] * (1.0f - fresnel));
            }
        slot[i] = pack4f(color);
    }
    std::vector<uint32_t> scratch(npx);
    for (size_t i = 0; i < npx; i++) {  // blend.glsl:22-34
        float sum[4] = {0, 0, 0, 0};
        for (int f = 0; f < 8; f++) {
            uint32_t w = d.ring[(size_t)(enable_blend ? f : (int)d.slot) * npx + i];
            for (int c = 0; c < 4; c++) sum[c] = f == 0 ? unorm8(w, c) : sum[c] + unorm8(w, c);
        }
        float o[4] = {sum[0] * 0.125f, sum[1] * 0.125f, sum[2] * 0.125f, 1.0f};
        scratch[i] = pack4f(o);
    }
    for (size_t i = 0; i < npx; i++) {  // median.glsl:51-75 / id.glsl, then the sRGB framebuffer
        int x = (int)(i % d.w), y = (int)(i / d.w);
        float res[4];
        if (!enable_median) {
            for (int c = 0; c < 4; c++) res[c] = unorm8(scratch[i], c);
        } else {
            const int dx[5] = {0, 1, 0, -1, 0}, dy[5] = {0, 0, 1, 0, -1};
            float c5[5][4];
            for (int t = 0; t < 5; t++) {
                int xx = std::min(std::max(x + dx[t], 0), (int)d.w - 1);
                int yy = std::min(std::max(y + dy[t], 0), (int)d.h - 1);
                for (int c = 0; c < 4; c++) c5[t][c] = unorm8(scratch[(size_t)yy * d.w + xx], c);
                to_xyz(c5[t]);
            }
            sort2v(c5[0], c5[1]);
            sort2v(c5[3], c5[4]);
            sort2v(c5[0], c5[2]);
            sort2v(c5[1], c5[2]);
            sort2v(c5[0], c5[3]);
            sort2v(c5[2], c5[3]);
            sort2v(c5[1], c5[4]);
            sort2v(c5[1], c5[2]);
            sort2v(c5[3], c5[4]);
            for (int c = 0; c < 4; c++) res[c] = c5[2][c] * 0.667f + c5[1][c] * 0.1666f + c5[3][c] * 0.1666f;
            to_rgb(res);
        }
        out[i] = srgb_of(d, res[0]) | (srgb_of(d, res[1]) << 8) | (srgb_of(d, res[2]) << 16) | (quant8(res[3]) << 24);
    }
}

// renderer.rs:378-410 on a row-major w*h*3 accumulation buffer.
void orc_resolve(const float* accum, uint32_t w, uint32_t h, uint32_t n, uint32_t* rgba) {
    float factor = 1.0f / (float)n;
    for (size_t i = 0; i < (size_t)w * h; i++)
        rgba[i] = pack_color(v3(accum[3 * i] * factor, accum[3 * i + 1] * factor, accum[3 * i + 2] * factor));
}

// ---- element functions for the ported unit tests ----
float orc_rcp(float x) { return rcp(x); }
float orc_rsqrt(float x) { return rsqrt(x); }
float orc_recip_precise(float x) { return recip_precise(x); }
float orc_sin(float x) { return poly_sin(x); }
float orc_cos(float x) { return poly_cos(x); }
float orc_acos(float x) { return poly_acos(x); }
float orc_acos_fast(float x) { return poly_acos_fast(x); }
int32_t orc_cvtps(float x) { return cvtps(x); }
// Mf32::mul_add / mul_sub / neg_mul_add (simd.rs:82-95) for kind 0 / 1 / 2.
float orc_fma3(int kind, float a, float b, float c) {
    return kind == 0 ? fmadd(a, b, c) : kind == 1 ? fmsub(a, b, c) : fnmadd(a, b, c);
}
// Mf32::abs (simd.rs:291-299): the sign bit cleared.
float orc_abs(float x) { return fabs_bits(x); }
// Mf32::any_sign_bit_positive_masked (simd.rs:355-371): not testc(a, mask),
// on raw sign bits: some lane whose mask sign bit is set has its own clear.
int orc_any_sign_bit_positive_masked(const float* a, const float* mask) {
    for (int k = 0; k < 8; k++)
        if ((fbits(mask[k]) >> 31) != 0u && (fbits(a[k]) >> 31) == 0u) return 1;
    return 0;
}

void orc_rng_draws(uint32_t x, uint32_t y, uint32_t i, uint32_t n, uint32_t* out) {
    Rng r = Rng::with_seed(x, y, i);
    for (uint32_t k = 0; k < n; k++) r.next(out + 8 * k);
}
// kind 0 unit, 1 biunit, 2 angle, 3 hemisphere (3 floats per lane, two draws each)
void orc_rng_samples(uint32_t x, uint32_t y, uint32_t i, int kind, uint32_t n, float* out) {
    Rng r = Rng::with_seed(x, y, i);
    for (uint32_t k = 0; k < n; k++) {
        uint32_t a[8], b[8];
        r.next(a);
        if (kind == 3) {
            r.next(b);
            for (int j = 0; j < 8; j++) {
                V3 v = hemisphere_from(a[j], b[j]);
                out[24 * k + 3 * j] = v.x;
                out[24 * k + 3 * j + 1] = v.y;
                out[24 * k + 3 * j + 2] = v.z;
            }
            continue;
        }
        for (int j = 0; j < 8; j++)
            out[8 * k + j] = kind == 0 ? unit_from(a[j]) : kind == 1 ? biunit_from(a[j]) : angle_from(a[j]);
    }
}
void orc_rotate_hemisphere(const float* v, const float* n, float* out) {
    V3 r = rotate_hemisphere(ld(v), ld(n));
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}
void orc_quat_rotate(const float* v, const float* q, float* out) {
    V3 r = rotate(ld(v), Quat{q[0], q[1], q[2], q[3]});
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}
void orc_quat_interpolate(const float* q, const float* dq, float t, float* out) {
    Quat r = interpolate(Quat{q[0], q[1], q[2], q[3]}, Quat{dq[0], dq[1], dq[2], dq[3]}, t);
    out[0] = r.a;
    out[1] = r.b;
    out[2] = r.c;
    out[3] = r.d;
}
// Returns tmin, tmax and the hit predicate `any()` (aabb.rs:146-151).
int orc_aabb_intersect(const float* box, const float* o, const float* d, float* tmin, float* tmax) {
    Node n;
    std::memcpy(n.origin, box, 12);
    std::memcpy(n.far_, box + 3, 12);
    V3 inv = v3(rcp(d[0]), rcp(d[1]), rcp(d[2]));
    BoxHit b = box_hit(n, ld(o), inv);
    *tmin = b.tmin;
    *tmax = b.tmax;
    return b.mask && !sneg(b.tmax);
}
// triangle.rs:59-148 for one ray from a far intersection at `far_dist`.
// out: dist, pos[3], normal[3], tu, tv; returns 1 on a hit.
int orc_triangle_intersect(const float* tri, const float* o, const float* d, float far_dist, float* out) {
    Tri t;
    std::memset(&t, 0, sizeof t);
    std::memcpy(t.v0, tri, 36);
    t.material = 0x00ffffffu;
    Ray r{ld(o), ld(d)};
    Isect is = far_isect(r, far_dist);
    tri_intersect(t, 0, r, true, is);
    out[0] = is.dist;
    out[1] = is.pos.x;
    out[2] = is.pos.y;
    out[3] = is.pos.z;
    out[4] = is.normal.x;
    out[5] = is.normal.y;
    out[6] = is.normal.z;
    out[7] = is.tu;
    out[8] = is.tv;
    return is.tri == 0;
}
// triangle.rs:152-185. out: dist, area, normal[3]; returns 1 when not masked out.
int orc_intersect_direct(const float* tri, const float* o, const float* d, float* out) {
    Tri t;
    std::memset(&t, 0, sizeof t);
    std::memcpy(t.v0, tri, 36);
    DirectHit h = intersect_direct(t, Ray{ld(o), ld(d)});
    out[0] = h.dist;
    out[1] = h.area;
    out[2] = h.normal.x;
    out[3] = h.normal.y;
    out[4] = h.normal.z;
    return !h.miss;
}
void orc_camera_ray(const float* cam, float x, float y, float t, float* out) {
    Camera c;
    c.pos = v3(cam[0], cam[1], cam[2]);
    c.pos_delta = v3(cam[3], cam[4], cam[5]);
    c.q = Quat{cam[6], cam[7], cam[8], cam[9]};
    c.dq = Quat{cam[10], cam[11], cam[12], cam[13]};
    c.screen_distance = cam[14];
    Ray r = camera_ray(c, x, y, t);
    out[0] = r.o.x;
    out[1] = r.o.y;
    out[2] = r.o.z;
    out[3] = r.d.x;
    out[4] = r.d.y;
    out[5] = r.d.z;
}
void orc_sky_intensity(const float* d, float* out) {
    V3 s = sky_intensity(ld(d));
    out[0] = s.x;
    out[1] = s.y;
    out[2] = s.z;
}

}  // extern "C"
