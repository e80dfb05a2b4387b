// ORACLE / TEST INFRASTRUCTURE. Only tests/ and the CPU legs of bench.py load
// liboracle; the product path never does.
//
// Bvh::build of ruuda/convector (bvh.rs:44-545), restated on its own from the
// reference's Rust, in the reference's shape: interim nodes that own their
// triangle references, 64 bins per axis, a recursive split with the tree
// surface area heuristic, and a recursive crystallize into node pairs. It is
// the independent check of the product's host and device builds (node array,
// triangle order, source indices, statistics), which are written for speed
// (parallel, iterative) and share no code with this file.
//
// Where the 2017 reference leaves a case undefined or aborts, this file takes
// the same documented choice as the product:
//  * f32::min / f32::max (vector3.rs:127-142, through aabb.rs:56-89) keep the
//    first operand when the two compare equal (+0 against -0), as LLVM's x86
//    lowering of minnum/maxnum does; a NaN operand yields the other one;
//  * the float-to-usize cast of the bin index (bvh.rs:155) saturates, NaN to 0
//    (the 2017 compiler left it undefined; Rust defines it so since 1.45);
//  * a node whose triangles no axis can split (every barycentre in one bin,
//    which needs 33..64 triangles sharing a barycentre) becomes a leaf; the
//    reference asserts (bvh.rs:302);
//  * a root that does not split is refused (status 1); the reference asserts
//    (bvh.rs:512).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

namespace orc_bvh {

struct Tri {  // triangle.rs:24-32, 64 bytes
    float v0[3], v1[3], v2[3];
    float uv0[2], uv1[2], uv2[2];
    uint32_t material;
};
struct Node {  // bvh.rs:21-30, 32 bytes
    float origin[3], far_[3];
    uint32_t index, len;
};
static_assert(sizeof(Tri) == 64 && sizeof(Node) == 32, "reference layouts");

inline float fmin_ref(float a, float b) {  // f32::min, first operand on ties
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    return b < a ? b : a;
}
inline float fmax_ref(float a, float b) {  // f32::max, first operand on ties
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    return b > a ? b : a;
}

struct V {
    float c[3];
};
struct Aabb {  // aabb.rs:22-30
    V origin, far_;
};

inline V vmin(const V& a, const V& b) {
    return V{{fmin_ref(a.c[0], b.c[0]), fmin_ref(a.c[1], b.c[1]), fmin_ref(a.c[2], b.c[2])}};
}
inline V vmax(const V& a, const V& b) {
    return V{{fmax_ref(a.c[0], b.c[0]), fmax_ref(a.c[1], b.c[1]), fmax_ref(a.c[2], b.c[2])}};
}
// aabb.rs:74-89: the running bound is the first operand.
inline void enclose(Aabb& acc, const Aabb& b) {
    acc.origin = vmin(acc.origin, b.origin);
    acc.far_ = vmax(acc.far_, b.far_);
}
// aabb.rs:97-103
inline float area(const Aabb& b) {
    float sx = b.far_.c[0] - b.origin.c[0], sy = b.far_.c[1] - b.origin.c[1], sz = b.far_.c[2] - b.origin.c[2];
    float x = sy * sz, y = sz * sx, z = sx * sy;
    return 2.0f * ((x + y) + z);
}

struct TriRef {  // bvh.rs:45-50, 89-97
    Aabb aabb;
    V barycenter;
    size_t index;
};

inline TriRef make_ref(size_t i, const Tri& t) {
    TriRef r;
    V a{{t.v0[0], t.v0[1], t.v0[2]}}, b{{t.v1[0], t.v1[1], t.v1[2]}}, c{{t.v2[0], t.v2[1], t.v2[2]}};
    // aabb.rs:56-71 enclose_points([v0, v1, v2])
    r.aabb.origin = vmin(vmin(a, b), c);
    r.aabb.far_ = vmax(vmax(a, b), c);
    // triangle.rs:55-57: (v0 + v1 + v2) * 3.0f32.recip()
    const float third = 1.0f / 3.0f;
    for (int k = 0; k < 3; k++) r.barycenter.c[k] = ((a.c[k] + b.c[k]) + c.c[k]) * third;
    r.index = i;
    return r;
}

struct Bin {  // bvh.rs:64-67, 99-121
    std::vector<const TriRef*> tris;
    Aabb aabb{};
    void push(const TriRef* t) {
        if (tris.empty()) aabb = t->aabb;
        else enclose(aabb, t->aabb);
        tris.push_back(t);
    }
    void clear() { tris.clear(); }
};

// TreeSurfaceAreaHeuristic (bvh.rs:452-477) with the costs of bvh.rs:495-499.
struct Tsah {
    float aabb_cost_k = 40.0f, tri_cost_k = 120.0f, p = 0.8f;
    float aabb_cost(const Aabb& parent, const Aabb& box, size_t num_tris) const {
        float ac_ap = area(box) / area(parent);
        float n = (float)num_tris;
        float m = std::log2(n);
        float aabb_term = 1.0f + ac_ap * (2.0f * p - n * std::pow(p, m)) / (p - 2.0f * p * p);
        float tri_term = n * std::pow(p, m - 1.0f) * ac_ap;
        return aabb_term * aabb_cost_k + tri_term * tri_cost_k;
    }
    float tris_cost(size_t num_tris) const { return (float)num_tris * tri_cost_k; }
};

struct Interim {  // bvh.rs:52-62
    Aabb outer, inner;
    std::vector<std::unique_ptr<Interim>> children;
    std::vector<TriRef> tris;

    // bvh.rs:124-132
    explicit Interim(std::vector<TriRef> refs) : tris(std::move(refs)) {
        outer = tris[0].aabb;
        inner.origin = inner.far_ = tris[0].barycenter;
        for (size_t i = 1; i < tris.size(); i++) {
            enclose(outer, tris[i].aabb);
            inner.origin = vmin(inner.origin, tris[i].barycenter);
            inner.far_ = vmax(inner.far_, tris[i].barycenter);
        }
    }

    // bvh.rs:174-200: sorted by the coordinate (a stable sort), chunks of
    // ceil(n / bins) in bin order.
    void bin_uniform(std::vector<Bin>& bins, int axis) const {
        std::vector<const TriRef*> ptrs;
        ptrs.reserve(tris.size());
        for (const TriRef& t : tris) ptrs.push_back(&t);
        std::stable_sort(ptrs.begin(), ptrs.end(), [axis](const TriRef* a, const TriRef* b) {
            return a->barycenter.c[axis] < b->barycenter.c[axis];
        });
        size_t per_bin = (ptrs.size() + bins.size() - 1) / bins.size();
        if (per_bin == 0) per_bin = 1;
        for (size_t i = 0; i < ptrs.size(); i++) bins[i / per_bin].push(ptrs[i]);
    }

    // bvh.rs:140-170
    void bin(std::vector<Bin>& bins, int axis) const {
        if (tris.size() <= bins.size() / 2) return bin_uniform(bins, axis);
        const float min = inner.origin.c[axis];
        const float size = inner.far_.c[axis] - min;
        const size_t nb = bins.size(), n = tris.size();
        for (const TriRef& t : tris) {
            float f = std::floor(((float)nb * (t.barycenter.c[axis] - min)) / size);
            size_t index;
            if (std::isnan(f) || f <= 0.0f) index = 0;
            else if (f >= 18446744073709551616.0f) index = SIZE_MAX;
            else index = (size_t)f;
            if (index >= nb) index = nb - 1;
            bins[index].push(&t);
            if (bins[index].tris.size() > n / 8 && n > nb) {
                for (Bin& b : bins) b.clear();
                return bin_uniform(bins, axis);
            }
        }
    }

    // bvh.rs:212-259: the first of the cheapest split positions between the
    // first and the last non-empty bin.
    float cheapest_split(const Tsah& h, const std::vector<Bin>& bins, size_t* split_at) const {
        size_t first = 0, last = 0;
        while (bins[first].tris.empty()) first++;
        for (size_t i = 0; i < bins.size(); i++)
            if (!bins[i].tris.empty()) last = i;
        first += 1;
        last += 1;
        float best = 0.0f;
        bool is_first = true;
        for (size_t i = first; i < last; i++) {
            Aabb l{}, r{};
            bool lset = false, rset = false;
            size_t lc = 0, rc = 0;
            for (size_t b = 0; b < bins.size(); b++) {
                if (bins[b].tris.empty()) continue;
                Aabb& acc = b < i ? l : r;
                bool& set = b < i ? lset : rset;
                (b < i ? lc : rc) += bins[b].tris.size();
                if (!set) acc = bins[b].aabb;
                else enclose(acc, bins[b].aabb);
                set = true;
            }
            float cost = h.aabb_cost(outer, l, lc) + h.aabb_cost(outer, r, rc);
            if (cost < best || is_first) {
                best = cost;
                *split_at = i;
                is_first = false;
            }
        }
        return best;
    }

    // bvh.rs:263-320
    void split(const Tsah& h) {
        if (tris.size() <= 1) return;
        std::vector<Bin> bins(64);
        std::vector<TriRef> best_left, best_right;
        float best_cost = 0.0f;
        bool is_first = true;
        for (int axis = 0; axis < 3; axis++) {
            bin(bins, axis);
            size_t nonempty = 0;
            for (const Bin& b : bins) nonempty += b.tris.empty() ? 0 : 1;
            if (nonempty > 1) {  // bvh.rs:207-210 are_bins_valid
                size_t at = 0;
                float cost = cheapest_split(h, bins, &at);
                if (cost < best_cost || is_first) {
                    best_left.clear();
                    best_right.clear();
                    for (size_t b = 0; b < bins.size(); b++)
                        for (const TriRef* t : bins[b].tris) (b < at ? best_left : best_right).push_back(*t);
                    best_cost = cost;
                    is_first = false;
                }
            }
            for (Bin& b : bins) b.clear();
        }
        if (is_first) return;  // no axis splits: a leaf (the reference asserts)
        if (h.tris_cost(tris.size()) < best_cost) return;
        children.emplace_back(new Interim(std::move(best_left)));
        children.emplace_back(new Interim(std::move(best_right)));
        tris.clear();
    }

    // bvh.rs:324-354: the child of smaller area first.
    void split_recursive(const Tsah& h) {
        split(h);
        if (children.empty()) return;
        if (area(children[0]->outer) > area(children[1]->outer)) std::swap(children[0], children[1]);
        children[0]->split_recursive(h);
        children[1]->split_recursive(h);
    }

    size_t count_nodes() const {  // bvh.rs:364-368
        size_t c = 1;
        for (const auto& ch : children) c += ch->count_nodes();
        return c;
    }
    size_t count_leaves() const {  // bvh.rs:371-375
        if (children.empty()) return 1;
        size_t c = 0;
        for (const auto& ch : children) c += ch->count_leaves();
        return c;
    }
    float summed_area_ratio() const {  // bvh.rs:379-384
        float contribution = 0.0f, child_sum = 0.0f;
        for (const auto& ch : children) contribution = contribution + ch->summed_area_ratio();
        const float self_area = area(outer);
        for (const auto& ch : children) child_sum = child_sum + area(ch->outer) / self_area;
        return child_sum + contribution;
    }
    uint32_t depth() const {
        uint32_t d = 0;
        for (const auto& ch : children) d = std::max(d, ch->depth());
        return d + 1;
    }

    // bvh.rs:389-428
    void crystallize(const Tri* src, std::vector<Node>& nodes, std::vector<Tri>& sorted,
                     std::vector<uint32_t>& source, size_t into) const {
        Node& self = nodes[into];
        std::memcpy(self.origin, outer.origin.c, 12);
        std::memcpy(self.far_, outer.far_.c, 12);
        if (tris.empty()) {
            const size_t child = nodes.size();
            nodes.push_back(Node{});
            nodes.push_back(Node{});
            children[0]->crystallize(src, nodes, sorted, source, child);
            children[1]->crystallize(src, nodes, sorted, source, child + 1);
            nodes[into].index = (uint32_t)child;
            nodes[into].len = 0;
        } else {
            nodes[into].index = (uint32_t)sorted.size();
            nodes[into].len = (uint32_t)tris.size();
            for (const TriRef& t : tris) {
                sorted.push_back(src[t.index]);
                source.push_back((uint32_t)t.index);
            }
        }
    }
};

struct Bvh {
    std::vector<Node> nodes;
    std::vector<Tri> tris;
    std::vector<uint32_t> source;
    float avg_area_ratio = 0.0f, avg_tris_per_leaf = 0.0f;
    uint32_t depth = 0;
};

// Bvh::build (bvh.rs:488-545). Returns null when the root does not split.
Bvh* build(const Tri* src, size_t n) {
    std::vector<TriRef> refs;
    refs.reserve(n);
    for (size_t i = 0; i < n; i++) refs.push_back(make_ref(i, src[i]));
    Interim root(std::move(refs));
    Tsah h;
    root.split_recursive(h);
    if (root.children.size() != 2) return nullptr;
    std::unique_ptr<Bvh> b(new Bvh());
    const size_t num_nodes = root.count_nodes();
    b->nodes.reserve(num_nodes);
    b->nodes.push_back(Node{});
    b->nodes.push_back(Node{});
    root.children[0]->crystallize(src, b->nodes, b->tris, b->source, 0);
    root.children[1]->crystallize(src, b->nodes, b->tris, b->source, 1);
    b->avg_area_ratio = root.summed_area_ratio() / (float)num_nodes;
    b->avg_tris_per_leaf = (float)b->tris.size() / (float)root.count_leaves();
    b->depth = root.depth() - 1;  // the roots (nodes 0 and 1) at depth 1
    return b.release();
}

}  // namespace orc_bvh

extern "C" {

void* orc_bvh_build(const void* tris, uint32_t n) {
    if (n < 2) return nullptr;
    return orc_bvh::build(static_cast<const orc_bvh::Tri*>(tris), n);
}
uint32_t orc_bvh_num_nodes(const void* b) { return (uint32_t)static_cast<const orc_bvh::Bvh*>(b)->nodes.size(); }
uint32_t orc_bvh_num_triangles(const void* b) { return (uint32_t)static_cast<const orc_bvh::Bvh*>(b)->tris.size(); }
void orc_bvh_copy(const void* bp, void* nodes, void* tris, uint32_t* source) {
    const orc_bvh::Bvh& b = *static_cast<const orc_bvh::Bvh*>(bp);
    std::memcpy(nodes, b.nodes.data(), b.nodes.size() * sizeof(orc_bvh::Node));
    std::memcpy(tris, b.tris.data(), b.tris.size() * sizeof(orc_bvh::Tri));
    std::memcpy(source, b.source.data(), b.source.size() * 4);
}
void orc_bvh_stats(const void* bp, float* avg_tris_per_leaf, float* avg_area_ratio, uint32_t* depth) {
    const orc_bvh::Bvh& b = *static_cast<const orc_bvh::Bvh*>(bp);
    *avg_tris_per_leaf = b.avg_tris_per_leaf;
    *avg_area_ratio = b.avg_area_ratio;
    *depth = b.depth;
}
void orc_bvh_free(void* b) { delete static_cast<orc_bvh::Bvh*>(b); }

}  // extern "C"
