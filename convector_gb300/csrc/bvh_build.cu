// Device BVH build: the binned TSAH build of bvh.rs:44-545 on the GPU, with
// the host build's node order, triangle order and statistics.
//
// Exactness. Every decision of the host build is reproduced:
//  * split costs are computed with the same float operations in the same
//    order (the n-dependent TSAH factors come from a host-made table, so the
//    libm powf/log2f results are the host's own);
//  * bin boxes only feed costs, whose values do not depend on the sign of a
//    zero bound, so they are plain min/max reductions;
//  * node boxes are written out and must be bit-identical: from_refs folds
//    the triangle boxes in node order with f32::min / f32::max, which keep
//    the first of equal operands (+0 / -0), so a node bound is the bound of
//    the first triangle in node order that attains the extreme value. The
//    reduction key is (value with -0 as +0, position).
//  * triangle order inside a child is the host's: bins concatenated in bin
//    order, each bin in insertion order (node order for coordinate binning,
//    sorted order for the uniform split of bvh.rs:176-201).
// Inputs with NaN or infinite coordinates are refused (the host build takes
// them; its min/max folds then depend on NaN placement).
//
// Structure. Nodes of more than 32 triangles are split level by level by the
// whole device (coordinate binning with shared-memory histograms, a segmented
// sort for the uniform fallback, a stable counting-sort partition); every
// node of 2..32 triangles is then built completely by one warp (per = 1 in
// the uniform split, so bins are single triangles in sorted order). The host
// crystallizes the interim tree into the reference's node array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "internal.h"

namespace cvx {
namespace {

constexpr int kBins = 64;
constexpr uint32_t kSmall = 32;      // nodes up to this size are built by one warp
constexpr int kTile = 256;           // positions per tile (one per thread)
constexpr uint32_t kBlockSort = 4096;  // uniform sorts up to this size run in one block
constexpr uint32_t kMaxTris = 1u << 26;

struct Refs {
    float* lo[3];
    float* hi[3];
    float* bc[3];
};

struct Tile {
    uint32_t slot, axis, start, len;
};

// Per-slot state of the level being split.
struct Slot {
    uint32_t id, beg, cnt;
};

struct Decision {
    uint32_t axis, at, nl, leaf;  // axis 3: no axis had two non-empty bins
};

// Orderable key of a float with -0 and +0 equal (no NaN reaches here).
__device__ __forceinline__ uint32_t okey(float x) {
    uint32_t u = __float_as_uint(x);
    if ((u << 1) == 0u) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_okey(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
// f32::min / f32::max of the host build (first operand on equal values).
__device__ __forceinline__ float fmin_rs(float a, float b) { return a != a ? b : (b < a ? b : a); }
__device__ __forceinline__ float fmax_rs(float a, float b) { return a != a ? b : (b > a ? b : a); }

struct Box {
    float lo[3], hi[3];
};
// aabb.rs:97-103
__device__ __forceinline__ float area(const Box& b) {
    float sx = b.hi[0] - b.lo[0], sy = b.hi[1] - b.lo[1], sz = b.hi[2] - b.lo[2];
    float x = sy * sz, y = sz * sx, z = sx * sy;
    return 2.0f * (x + y + z);
}

struct Tsah {
    const float* x;  // 2p - n p^log2(n)
    const float* t;  // n p^(log2(n) - 1)
    float y;         // p - 2p^2
};
// TreeSurfaceAreaHeuristic::aabb_cost (bvh.rs:452-474), the host's operation order.
__device__ __forceinline__ float tsah_cost(const Tsah& ts, float parent_area, const Box& b, uint32_t n) {
    float ac_ap = area(b) / parent_area;
    float aabb_term = 1.0f + ac_ap * ts.x[n] / ts.y;
    float tri_term = ts.t[n] * ac_ap;
    return aabb_term * 40.0f + tri_term * 120.0f;
}

// ---------------------------------------------------------------------------
// Triangle boxes and barycentres (bvh.rs:495-499).

__global__ void k_prep(const cvx_triangle* __restrict__ tris, uint32_t n, float third, Refs r,
                       uint32_t* __restrict__ order, uint32_t* __restrict__ bad) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cvx_triangle& t = tris[i];
    bool ok = true;
    for (int c = 0; c < 3; c++) {
        float a = t.v0[c], b = t.v1[c], d = t.v2[c];
        ok = ok && isfinite(a) && isfinite(b) && isfinite(d);
        r.lo[c][i] = fmin_rs(fmin_rs(a, b), d);
        r.hi[c][i] = fmax_rs(fmax_rs(a, b), d);
        r.bc[c][i] = ((a + b) + d) * third;
    }
    order[i] = i;
    if (!ok) atomicOr(bad, 1u);
}

// ---------------------------------------------------------------------------
// Exact node boxes of a list of ranges (from_refs, bvh.rs:125-132): outer
// bounds as (key, position) extremes, the barycentre box (inner) by value.

struct BoxAcc {
    unsigned long long omin[3], omax[3];
    uint32_t imin[3], imax[3];
};

__global__ void k_box_init(BoxAcc* acc, uint32_t m) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    for (int c = 0; c < 3; c++) {
        acc[j].omin[c] = ~0ull;
        acc[j].omax[c] = 0ull;
        acc[j].imin[c] = ~0u;
        acc[j].imax[c] = 0u;
    }
}

__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int o) {
    uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
    lo = __shfl_xor_sync(0xffffffffu, lo, o);
    hi = __shfl_xor_sync(0xffffffffu, hi, o);
    return ((unsigned long long)hi << 32) | lo;
}

// One block per tile; the tile's slot indexes `acc`.
__global__ void __launch_bounds__(kTile) k_box(const Tile* __restrict__ tiles, uint32_t n_tiles, Refs r,
                                               const uint32_t* __restrict__ order, uint32_t n, BoxAcc* acc,
                                               uint32_t n_acc, uint32_t* err) {
    if (blockIdx.x >= n_tiles) return;
    Tile tl = tiles[blockIdx.x];
    if (tl.slot >= n_acc || tl.start > n || tl.len > (uint32_t)kTile || tl.start + tl.len > n) {
        if (threadIdx.x == 0) atomicOr(err, 2u);
        return;
    }
    BoxAcc a;
    for (int c = 0; c < 3; c++) {
        a.omin[c] = ~0ull;
        a.omax[c] = 0ull;
        a.imin[c] = ~0u;
        a.imax[c] = 0u;
    }
    if (threadIdx.x < tl.len) {
        uint32_t p = tl.start + threadIdx.x;
        uint32_t t = order[p];
        for (int c = 0; c < 3; c++) {
            a.omin[c] = ((unsigned long long)okey(r.lo[c][t]) << 32) | p;
            a.omax[c] = ((unsigned long long)okey(r.hi[c][t]) << 32) | (0xffffffffu - p);
            uint32_t kb = okey(r.bc[c][t]);
            a.imin[c] = kb;
            a.imax[c] = kb;
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int c = 0; c < 3; c++) {
            a.omin[c] = min(a.omin[c], shfl64(a.omin[c], o));
            a.omax[c] = max(a.omax[c], shfl64(a.omax[c], o));
            a.imin[c] = min(a.imin[c], __shfl_xor_sync(0xffffffffu, a.imin[c], o));
            a.imax[c] = max(a.imax[c], __shfl_xor_sync(0xffffffffu, a.imax[c], o));
        }
    __shared__ BoxAcc sm;
    if (threadIdx.x == 0) sm = a;
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && threadIdx.x) {
        for (int c = 0; c < 3; c++) {
            atomicMin(&sm.omin[c], a.omin[c]);
            atomicMax(&sm.omax[c], a.omax[c]);
            atomicMin(&sm.imin[c], a.imin[c]);
            atomicMax(&sm.imax[c], a.imax[c]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        BoxAcc* g = acc + tl.slot;
        for (int c = 0; c < 3; c++) {
            atomicMin(&g->omin[c], sm.omin[c]);
            atomicMax(&g->omax[c], sm.omax[c]);
            atomicMin(&g->imin[c], sm.imin[c]);
            atomicMax(&g->imax[c], sm.imax[c]);
        }
    }
}

// Writes the decoded boxes into the interim nodes of list `ids`.
__global__ void k_box_store(const uint32_t* __restrict__ ids, uint32_t m, const BoxAcc* __restrict__ acc, Refs r,
                            const uint32_t* __restrict__ order, uint32_t n, InterimNode* nodes, uint32_t n_nodes,
                            float* inner, uint32_t* err) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    uint32_t id = ids[j];
    if (id >= n_nodes) {
        atomicOr(err, 2u);
        return;
    }
    for (int c = 0; c < 3; c++) {
        uint32_t pmin = (uint32_t)acc[j].omin[c], pmax = 0xffffffffu - (uint32_t)acc[j].omax[c];
        if (pmin >= n || pmax >= n) {
            atomicOr(err, 2u);
            return;
        }
        nodes[id].lo[c] = r.lo[c][order[pmin]];
        nodes[id].hi[c] = r.hi[c][order[pmax]];
        inner[6 * (size_t)id + c] = from_okey(acc[j].imin[c]);
        inner[6 * (size_t)id + 3 + c] = from_okey(acc[j].imax[c]);
    }
}

// ---------------------------------------------------------------------------
// Level split of nodes above kSmall triangles.

// Bin statistics per (slot, axis, bin): count and the bin box as value keys.
struct BinStats {
    uint32_t* count;  // [K][3][64]
    uint32_t* key;    // [K][3][64][6]: lo x y z (min), hi x y z (max)
};

__global__ void k_stats_init(BinStats st, uint32_t entries) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= entries) return;
    st.count[i] = 0u;
    for (int c = 0; c < 3; c++) {
        st.key[6 * (size_t)i + c] = ~0u;
        st.key[6 * (size_t)i + 3 + c] = 0u;
    }
}

// Adds triangle t to the shared-memory histogram of (axis, bin).
__device__ __forceinline__ void sm_add(uint32_t* cnt, uint32_t* key, int a, int b, const Refs& r, uint32_t t) {
    int e = a * kBins + b;
    atomicAdd(&cnt[e], 1u);
    for (int c = 0; c < 3; c++) {
        atomicMin(&key[6 * e + c], okey(r.lo[c][t]));
        atomicMax(&key[6 * e + 3 + c], okey(r.hi[c][t]));
    }
}

__device__ __forceinline__ void sm_flush(const uint32_t* cnt, const uint32_t* key, BinStats st, uint32_t slot,
                                         int axis_lo, int axis_hi) {
    for (int e = threadIdx.x; e < 3 * kBins; e += blockDim.x) {
        int a = e / kBins;
        if (a < axis_lo || a > axis_hi || cnt[e] == 0u) continue;
        size_t g = (size_t)slot * 3 * kBins + e;
        atomicAdd(&st.count[g], cnt[e]);
        for (int c = 0; c < 3; c++) {
            atomicMin(&st.key[6 * g + c], key[6 * e + c]);
            atomicMax(&st.key[6 * g + 3 + c], key[6 * e + 3 + c]);
        }
    }
}

__device__ __forceinline__ void sm_init(uint32_t* cnt, uint32_t* key) {
    for (int e = threadIdx.x; e < 3 * kBins; e += blockDim.x) {
        cnt[e] = 0u;
        for (int c = 0; c < 3; c++) {
            key[6 * e + c] = ~0u;
            key[6 * e + 3 + c] = 0u;
        }
    }
}

// Coordinate binning of bvh.rs:142-171 on all three axes.
__global__ void __launch_bounds__(kTile) k_bin_float(const Tile* __restrict__ tiles, uint32_t n_tiles,
                                                     const Slot* __restrict__ slots, uint32_t n_slots, Refs r,
                                                     const uint32_t* __restrict__ order, uint32_t n,
                                                     const float* __restrict__ inner, uint8_t* __restrict__ binf,
                                                     BinStats st, uint32_t* err) {
    __shared__ uint32_t cnt[3 * kBins];
    __shared__ uint32_t key[3 * kBins * 6];
    if (blockIdx.x >= n_tiles) return;
    Tile tl = tiles[blockIdx.x];
    if (tl.slot >= n_slots || tl.len > (uint32_t)kTile || tl.start + tl.len > n) {
        if (threadIdx.x == 0) atomicOr(err, 2u);
        return;
    }
    sm_init(cnt, key);
    __syncthreads();
    Slot s = slots[tl.slot];
    if (threadIdx.x < tl.len) {
        uint32_t p = tl.start + threadIdx.x;
        uint32_t t = order[p];
        for (int a = 0; a < 3; a++) {
            float mn = inner[6 * (size_t)s.id + a];
            float size = inner[6 * (size_t)s.id + 3 + a] - mn;
            float f = floorf((float)kBins * (r.bc[a][t] - mn) / size);
            // `as usize` saturates NaN and negatives to 0; clamp to the last bin.
            int b = (f != f || f <= 0.0f) ? 0 : (f >= (float)(kBins - 1) ? kBins - 1 : (int)f);
            binf[(size_t)a * n + p] = (uint8_t)b;
            sm_add(cnt, key, a, b, r, t);
        }
    }
    __syncthreads();
    sm_flush(cnt, key, st, tl.slot, 0, 2);
}

// bvh.rs:160-166: a bin above n/8 triangles (n > 64) sends the axis to the
// uniform split. mode[slot][axis]: 0 coordinate bins, 1 uniform.
__global__ void k_fallback(const Slot* __restrict__ slots, uint32_t n_slots, BinStats st, uint32_t* mode) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_slots) return;
    uint32_t n = slots[k].cnt;
    for (int a = 0; a < 3; a++) {
        uint32_t mx = 0;
        for (int b = 0; b < kBins; b++) mx = max(mx, st.count[((size_t)k * 3 + a) * kBins + b]);
        mode[3 * k + a] = (mx > n / 8u && n > (uint32_t)kBins) ? 1u : 0u;
    }
}

// Uniform split keys: (barycentre coordinate key, position); ascending order
// is std::stable_sort by the coordinate (-0 and +0 compare equal).
__device__ __forceinline__ unsigned long long ukey(const Refs& r, const uint32_t* order, int a, uint32_t p) {
    return ((unsigned long long)okey(r.bc[a][order[p]]) << 32) | p;
}

// One block sorts the positions of one (slot, axis) of at most kBlockSort
// triangles; srt[axis][beg + rank] = position.
__global__ void __launch_bounds__(1024) k_sort_block(const Tile* __restrict__ pairs, uint32_t n_pairs, Refs r,
                                                     const uint32_t* __restrict__ order, uint32_t n,
                                                     uint32_t* __restrict__ srt, uint32_t* err) {
    __shared__ unsigned long long k[kBlockSort];
    if (blockIdx.x >= n_pairs) return;
    Tile pr = pairs[blockIdx.x];  // slot, axis, start = beg, len = cnt
    if (pr.len > kBlockSort || pr.start + pr.len > n || pr.axis > 2) {
        if (threadIdx.x == 0) atomicOr(err, 2u);
        return;
    }
    uint32_t m = 1;
    while (m < pr.len) m <<= 1;
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x)
        k[i] = i < pr.len ? ukey(r, order, pr.axis, pr.start + i) : ~0ull;
    __syncthreads();
    for (uint32_t size = 2; size <= m; size <<= 1)
        for (uint32_t j = size >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
                uint32_t l = i ^ j;
                if (l > i) {
                    bool up = (i & size) == 0u;
                    unsigned long long x = k[i], y = k[l];
                    if ((x > y) == up) {
                        k[i] = y;
                        k[l] = x;
                    }
                }
            }
            __syncthreads();
        }
    for (uint32_t i = threadIdx.x; i < pr.len; i += blockDim.x)
        srt[(size_t)pr.axis * n + pr.start + i] = (uint32_t)k[i];
}

// Device-wide bitonic sort of one large (slot, axis) in `buf` (m a power of two).
__global__ void k_sort_fill(Tile pr, uint32_t m, Refs r, const uint32_t* __restrict__ order,
                            unsigned long long* __restrict__ buf) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    buf[i] = i < pr.len ? ukey(r, order, pr.axis, pr.start + i) : ~0ull;
}
__global__ void k_sort_step(unsigned long long* __restrict__ buf, uint32_t m, uint32_t size, uint32_t j) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    uint32_t l = i ^ j;
    if (l <= i) return;
    bool up = (i & size) == 0u;
    unsigned long long x = buf[i], y = buf[l];
    if ((x > y) == up) {
        buf[i] = y;
        buf[l] = x;
    }
}
// All steps j < 2048 of stage `size` (from j0 down), on 4096-element chunks.
__global__ void __launch_bounds__(1024) k_sort_chunk(unsigned long long* __restrict__ buf, uint32_t m,
                                                     uint32_t size_lo, uint32_t size_hi, uint32_t j0) {
    __shared__ unsigned long long k[4096];
    uint32_t base = blockIdx.x * 4096u;
    if (base >= m) return;
    for (uint32_t i = threadIdx.x; i < 4096u; i += blockDim.x) k[i] = buf[base + i];
    __syncthreads();
    for (uint32_t size = size_lo; size <= size_hi; size <<= 1)
        for (uint32_t j = (size == size_lo ? j0 : (size >> 1)); j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < 4096u; i += blockDim.x) {
                uint32_t l = i ^ j;
                if (l > i) {
                    bool up = ((base + i) & size) == 0u;
                    unsigned long long x = k[i], y = k[l];
                    if ((x > y) == up) {
                        k[i] = y;
                        k[l] = x;
                    }
                }
            }
            __syncthreads();
        }
    for (uint32_t i = threadIdx.x; i < 4096u; i += blockDim.x) buf[base + i] = k[i];
}
__global__ void k_sort_extract(Tile pr, const unsigned long long* __restrict__ buf, uint32_t n,
                               uint32_t* __restrict__ srt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pr.len) return;
    srt[(size_t)pr.axis * n + pr.start + i] = (uint32_t)buf[i];
}

// Statistics of the uniform bins (bin = rank / per) of the (slot, axis) tiles;
// tile.start is a rank offset inside the slot.
__global__ void k_axis_reset(const Tile* __restrict__ pairs, uint32_t n_pairs, BinStats st) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pairs * kBins) return;
    Tile pr = pairs[i / kBins];
    size_t g = ((size_t)pr.slot * 3 + pr.axis) * kBins + (i % kBins);
    st.count[g] = 0u;
    for (int c = 0; c < 3; c++) {
        st.key[6 * g + c] = ~0u;
        st.key[6 * g + 3 + c] = 0u;
    }
}
__global__ void __launch_bounds__(kTile) k_uniform_stats(const Tile* __restrict__ tiles, uint32_t n_tiles,
                                                         const Slot* __restrict__ slots, uint32_t n_slots, Refs r,
                                                         const uint32_t* __restrict__ order, uint32_t n,
                                                         const uint32_t* __restrict__ srt, BinStats st,
                                                         uint32_t* err) {
    __shared__ uint32_t cnt[3 * kBins];
    __shared__ uint32_t key[3 * kBins * 6];
    if (blockIdx.x >= n_tiles) return;
    Tile tl = tiles[blockIdx.x];
    if (tl.slot >= n_slots || tl.axis > 2 || tl.len > (uint32_t)kTile) {
        if (threadIdx.x == 0) atomicOr(err, 2u);
        return;
    }
    Slot s = slots[tl.slot];
    if (tl.start + tl.len > s.cnt || s.beg + s.cnt > n) {
        if (threadIdx.x == 0) atomicOr(err, 2u);
        return;
    }
    sm_init(cnt, key);
    __syncthreads();
    uint32_t per = (s.cnt + kBins - 1) / kBins;  // bvh.rs:186-188
    if (threadIdx.x < tl.len) {
        uint32_t rank = tl.start + threadIdx.x;
        uint32_t p = srt[(size_t)tl.axis * n + s.beg + rank];
        if (p < n) sm_add(cnt, key, tl.axis, (int)(rank / per), r, order[p]);
    }
    __syncthreads();
    sm_flush(cnt, key, st, tl.slot, tl.axis, tl.axis);
}

// bvh.rs:218-322: the cheapest split over the three axes, or a leaf. One
// warp per slot (lane l owns bins l and l + 32):
// prefix and suffix boxes and counts by warp scans, the candidate costs in
// parallel, and lane 0 applying the host's first-minimum rule in bin order.
__device__ __forceinline__ void box_scan_empty(Box& b) {
    for (int c = 0; c < 3; c++) {
        b.lo[c] = __int_as_float(0x7f800000);   // +inf
        b.hi[c] = __int_as_float((int)0xff800000u);  // -inf
    }
}
__device__ __forceinline__ void box_join(Box& a, const Box& b) {
    for (int c = 0; c < 3; c++) {
        a.lo[c] = fminf(a.lo[c], b.lo[c]);
        a.hi[c] = fmaxf(a.hi[c], b.hi[c]);
    }
}
__device__ __forceinline__ Box box_shfl_up(const Box& b, int o) {
    Box r;
    for (int c = 0; c < 3; c++) {
        r.lo[c] = __shfl_up_sync(0xffffffffu, b.lo[c], o);
        r.hi[c] = __shfl_up_sync(0xffffffffu, b.hi[c], o);
    }
    return r;
}
__device__ __forceinline__ Box box_shfl_down(const Box& b, int o) {
    Box r;
    for (int c = 0; c < 3; c++) {
        r.lo[c] = __shfl_down_sync(0xffffffffu, b.lo[c], o);
        r.hi[c] = __shfl_down_sync(0xffffffffu, b.hi[c], o);
    }
    return r;
}
__device__ __forceinline__ Box box_shfl(const Box& b, int src) {
    Box r;
    for (int c = 0; c < 3; c++) {
        r.lo[c] = __shfl_sync(0xffffffffu, b.lo[c], src);
        r.hi[c] = __shfl_sync(0xffffffffu, b.hi[c], src);
    }
    return r;
}

__global__ void __launch_bounds__(128) k_choose_warp(const Slot* __restrict__ slots, uint32_t n_slots,
                                                     const InterimNode* __restrict__ nodes, BinStats st, Tsah ts,
                                                     Decision* __restrict__ dec) {
    const int lane = threadIdx.x & 31;
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (k >= n_slots) return;  // warp-uniform
    Slot s = slots[k];
    Box outer;
    for (int c = 0; c < 3; c++) {
        outer.lo[c] = nodes[s.id].lo[c];
        outer.hi[c] = nodes[s.id].hi[c];
    }
    const float parent_area = area(outer);
    float best_cost = 0.0f;
    bool is_first = true;
    Decision d{3u, 0u, 0u, 1u};
    for (int a = 0; a < 3; a++) {
        const uint32_t* cn = st.count + ((size_t)k * 3 + a) * kBins;
        const uint32_t* ky = st.key + ((size_t)k * 3 + a) * kBins * 6;
        uint32_t c0 = cn[lane], c1 = cn[lane + 32];
        unsigned m0 = __ballot_sync(0xffffffffu, c0 != 0u), m1 = __ballot_sync(0xffffffffu, c1 != 0u);
        int nonempty = __popc(m0) + __popc(m1);
        if (nonempty <= 1) continue;  // warp-uniform
        int first = (m0 ? __ffs(m0) - 1 : 32 + __ffs(m1) - 1) + 1;
        int last = (m1 ? 32 + 31 - __clz(m1) : 31 - __clz(m0)) + 1;
        Box b0, b1;
        box_scan_empty(b0);
        box_scan_empty(b1);
        if (c0)
            for (int c = 0; c < 3; c++) {
                b0.lo[c] = from_okey(ky[6 * lane + c]);
                b0.hi[c] = from_okey(ky[6 * lane + 3 + c]);
            }
        if (c1)
            for (int c = 0; c < 3; c++) {
                b1.lo[c] = from_okey(ky[6 * (lane + 32) + c]);
                b1.hi[c] = from_okey(ky[6 * (lane + 32) + 3 + c]);
            }
        // Inclusive prefix (bins 0..b) and suffix (bins b..63) of boxes and counts.
        Box p0 = b0, p1 = b1, q0 = b0, q1 = b1;
        uint32_t pc0 = c0, pc1 = c1, qc0 = c0, qc1 = c1;
        for (int o = 1; o < 32; o <<= 1) {
            Box u0 = box_shfl_up(p0, o), u1 = box_shfl_up(p1, o);
            uint32_t uc0 = __shfl_up_sync(0xffffffffu, pc0, o), uc1 = __shfl_up_sync(0xffffffffu, pc1, o);
            Box v0 = box_shfl_down(q0, o), v1 = box_shfl_down(q1, o);
            uint32_t vc0 = __shfl_down_sync(0xffffffffu, qc0, o), vc1 = __shfl_down_sync(0xffffffffu, qc1, o);
            if (lane >= o) {
                box_join(p0, u0);
                box_join(p1, u1);
                pc0 += uc0;
                pc1 += uc1;
            }
            if (lane + o < 32) {
                box_join(q0, v0);
                box_join(q1, v1);
                qc0 += vc0;
                qc1 += vc1;
            }
        }
        Box lowtot = box_shfl(p0, 31), hightot = box_shfl(q1, 0);
        uint32_t lowcnt = __shfl_sync(0xffffffffu, pc0, 31), highcnt = __shfl_sync(0xffffffffu, qc1, 0);
        box_join(p1, lowtot);  // prefix of bins 32 + lane includes all of 0..31
        pc1 += lowcnt;
        box_join(q0, hightot);  // suffix of bins lane includes all of 32..63
        qc0 += highcnt;
        // Split i = b + 1 puts bins 0..b left and i..63 right: left = prefix(b),
        // right = suffix(b + 1). Lane l evaluates i = l + 1 and i = l + 33.
        Box r0 = box_shfl_down(q0, 1), r1 = box_shfl_down(q1, 1);
        uint32_t rc0 = __shfl_down_sync(0xffffffffu, qc0, 1), rc1 = __shfl_down_sync(0xffffffffu, qc1, 1);
        Box q1_first = box_shfl(q1, 0);  // suffix(32) for i = 32
        uint32_t qc1_first = __shfl_sync(0xffffffffu, qc1, 0);
        if (lane == 31) {
            r0 = q1_first;
            rc0 = qc1_first;
        }
        int i0 = lane + 1, i1 = lane + 33;
        float cost0 = 0.0f, cost1 = 0.0f;
        if (i0 >= first && i0 < last) cost0 = tsah_cost(ts, parent_area, p0, pc0) + tsah_cost(ts, parent_area, r0, rc0);
        if (i1 >= first && i1 < last) cost1 = tsah_cost(ts, parent_area, p1, pc1) + tsah_cost(ts, parent_area, r1, rc1);
        // bvh.rs:241-258: the first candidate, then strictly cheaper ones, in bin order.
        float best = 0.0f;
        int at = 0;
        bool first_i = true;
        for (int i = first; i < last; i++) {
            float c = i <= 32 ? __shfl_sync(0xffffffffu, cost0, i - 1) : __shfl_sync(0xffffffffu, cost1, i - 33);
            if (c < best || first_i) {
                best = c;
                at = i;
                first_i = false;
            }
        }
        if (best < best_cost || is_first) {
            best_cost = best;
            is_first = false;
            // left count: prefix count of bin at - 1
            uint32_t nl = at <= 32 ? __shfl_sync(0xffffffffu, pc0, at - 1) : __shfl_sync(0xffffffffu, pc1, at - 33);
            d = Decision{(uint32_t)a, (uint32_t)at, nl, 0u};
        }
    }
    if (is_first || (float)s.cnt * 120.0f < best_cost) d.leaf = 1u;
    if (lane == 0) dec[k] = d;
}

// Partition of the split slots. Coordinate-binned axis: a stable counting
// sort by bin (bins in order, node order inside a bin); uniform axis: the
// sorted order. tile_off[t][b]: first new index (relative to beg) of tile t's
// triangles in bin b.
__global__ void __launch_bounds__(kTile) k_tile_hist(const Tile* __restrict__ tiles, uint32_t n_tiles,
                                                     const uint8_t* __restrict__ binf, uint32_t n,
                                                     uint32_t* __restrict__ tile_hist) {
    __shared__ uint32_t h[kBins];
    if (blockIdx.x >= n_tiles) return;
    Tile tl = tiles[blockIdx.x];
    if (threadIdx.x < kBins) h[threadIdx.x] = 0u;
    __syncthreads();
    if (threadIdx.x < tl.len && tl.start + threadIdx.x < n && tl.axis < 3)
        atomicAdd(&h[binf[(size_t)tl.axis * n + tl.start + threadIdx.x]], 1u);
    __syncthreads();
    if (threadIdx.x < kBins) tile_hist[(size_t)blockIdx.x * kBins + threadIdx.x] = h[threadIdx.x];
}

// One block per split slot with coordinate bins; its tiles are t0..t1-1.
__global__ void __launch_bounds__(1024) k_tile_offsets(const uint32_t* __restrict__ slot_tiles, uint32_t n_split,
                                                       const uint32_t* __restrict__ tile_hist,
                                                       uint32_t* __restrict__ tile_off) {
    __shared__ uint32_t part[16][kBins];
    __shared__ uint32_t bin_start[kBins];
    if (blockIdx.x >= n_split) return;
    uint32_t t0 = slot_tiles[2 * blockIdx.x], t1 = slot_tiles[2 * blockIdx.x + 1];
    uint32_t nt = t1 - t0;
    int b = threadIdx.x % kBins, ch = threadIdx.x / kBins;
    uint32_t per = (nt + 15) / 16;
    uint32_t c0 = t0 + min(nt, ch * per), c1 = t0 + min(nt, (ch + 1) * per);
    uint32_t sum = 0;
    for (uint32_t t = c0; t < c1; t++) sum += tile_hist[(size_t)t * kBins + b];
    part[ch][b] = sum;
    __syncthreads();
    if (threadIdx.x < kBins) {
        uint32_t tot = 0;
        for (int c = 0; c < 16; c++) tot += part[c][threadIdx.x];
        bin_start[threadIdx.x] = tot;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int k = 0; k < kBins; k++) {
            uint32_t v = bin_start[k];
            bin_start[k] = run;
            run += v;
        }
    }
    __syncthreads();
    uint32_t off = bin_start[b];
    for (int c = 0; c < ch; c++) off += part[c][b];
    for (uint32_t t = c0; t < c1; t++) {
        tile_off[(size_t)t * kBins + b] = off;
        off += tile_hist[(size_t)t * kBins + b];
    }
}

// tiles: the split slots' tiles; axis = 3 + axis for a uniform axis.
__global__ void __launch_bounds__(kTile) k_scatter(const Tile* __restrict__ tiles, uint32_t n_tiles,
                                                   const Slot* __restrict__ slots, uint32_t n_slots,
                                                   const uint8_t* __restrict__ binf, const uint32_t* __restrict__ srt,
                                                   const uint32_t* __restrict__ tile_off,
                                                   const uint32_t* __restrict__ order, uint32_t n,
                                                   uint32_t* __restrict__ order_tmp, uint32_t* err) {
    __shared__ uint32_t wcount[kTile / 32][kBins];
    if (blockIdx.x >= n_tiles) return;
    Tile tl = tiles[blockIdx.x];
    if (tl.slot >= n_slots || tl.len > (uint32_t)kTile || tl.start + tl.len > n || tl.axis > 5) {
        if (threadIdx.x == 0) atomicOr(err, 2u);
        return;
    }
    Slot s = slots[tl.slot];
    uint32_t p = tl.start + threadIdx.x;
    bool live = threadIdx.x < tl.len;
    if (tl.axis >= 3) {  // uniform: new index = rank
        if (live) {
            uint32_t rank = p - s.beg;
            uint32_t src = srt[(size_t)(tl.axis - 3) * n + p];
            if (src < n && rank < s.cnt) order_tmp[p] = order[src];
            else atomicOr(err, 2u);
        }
        return;
    }
    int w = threadIdx.x / 32, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < (kTile / 32) * kBins; i += blockDim.x) (&wcount[0][0])[i] = 0u;
    __syncthreads();
    int b = live ? binf[(size_t)tl.axis * n + p] : kBins;  // kBins: no bin
    unsigned same = __match_any_sync(0xffffffffu, b);
    uint32_t rank = __popc(same & ((1u << lane) - 1u));
    if (live && rank == 0u) wcount[w][b] = __popc(same);
    __syncthreads();
    if (live) {
        uint32_t before = 0;
        for (int k = 0; k < w; k++) before += wcount[k][b];
        uint32_t dst = s.beg + tile_off[(size_t)blockIdx.x * kBins + b] + before + rank;
        if (dst < s.beg + s.cnt) order_tmp[dst] = order[p];
        else atomicOr(err, 2u);
    }
}

__global__ void k_copy_back(const Tile* __restrict__ tiles, uint32_t n_tiles, const uint32_t* __restrict__ src,
                            uint32_t* __restrict__ dst, uint32_t n) {
    if (blockIdx.x >= n_tiles) return;
    Tile tl = tiles[blockIdx.x];
    uint32_t p = tl.start + threadIdx.x;
    if (threadIdx.x < tl.len && p < n) dst[p] = src[p];
}

// Links split parents to their children, smaller box first (bvh.rs:333-335).
__global__ void k_link(const uint32_t* __restrict__ triples, uint32_t m, InterimNode* nodes, uint32_t n_nodes,
                       uint32_t* err) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    uint32_t parent = triples[3 * j], l = triples[3 * j + 1], r = triples[3 * j + 2];
    if (parent >= n_nodes || l >= n_nodes || r >= n_nodes) {
        atomicOr(err, 2u);
        return;
    }
    Box bl, br;
    for (int c = 0; c < 3; c++) {
        bl.lo[c] = nodes[l].lo[c];
        bl.hi[c] = nodes[l].hi[c];
        br.lo[c] = nodes[r].lo[c];
        br.hi[c] = nodes[r].hi[c];
    }
    bool swap = area(bl) > area(br);
    nodes[parent].c0 = swap ? r : l;
    nodes[parent].c1 = swap ? l : r;
}

// ---------------------------------------------------------------------------
// Warp build of a node of 2..32 triangles and its whole subtree. Every split
// is the uniform split with one triangle per bin, so the split candidates
// are the prefixes of the triangles sorted by barycentre coordinate. The
// node's range of `order` is rewritten in depth-first leaf order.

constexpr int kSmallWarps = 4;

__device__ __forceinline__ float shf(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }

__global__ void __launch_bounds__(32 * kSmallWarps) k_small(const uint32_t* __restrict__ ids, uint32_t m,
                                                            InterimNode* nodes, uint32_t n_nodes,
                                                            uint32_t* next_id, uint32_t* order, uint32_t n, Refs r,
                                                            Tsah ts, uint32_t* err) {
    __shared__ uint8_t lists[kSmallWarps][kSmall + 1][kSmall];
    __shared__ uint32_t st_id[kSmallWarps][kSmall + 1];
    __shared__ uint32_t st_cnt[kSmallWarps][kSmall + 1];
    __shared__ uint8_t perm[kSmallWarps][3][kSmall];
    const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
    uint32_t job = blockIdx.x * kSmallWarps + w;
    if (job >= m) return;
    uint32_t root = ids[job];
    if (root >= n_nodes) {
        if (lane == 0) atomicOr(err, 2u);
        return;
    }
    uint32_t beg = nodes[root].beg, cnt = nodes[root].cnt;
    if (cnt < 2u || cnt > kSmall || beg + cnt > n) {
        if (lane == 0) atomicOr(err, 2u);
        return;
    }
    // Element e (0..cnt-1) = the triangle at beg + e; its data sits in lane e.
    uint32_t tri = lane < (int)cnt ? order[beg + lane] : 0u;
    float lo[3], hi[3], bc[3];
    for (int c = 0; c < 3; c++) {
        lo[c] = lane < (int)cnt ? r.lo[c][tri] : 0.0f;
        hi[c] = lane < (int)cnt ? r.hi[c][tri] : 0.0f;
        bc[c] = lane < (int)cnt ? r.bc[c][tri] : 0.0f;
    }
    __syncwarp();
    int sp = 0;
    if (lane < (int)cnt) lists[w][0][lane] = (uint8_t)lane;
    if (lane == 0) {
        st_id[w][0] = root;
        st_cnt[w][0] = cnt;
    }
    sp = 1;
    uint32_t out_pos = 0;
    __syncwarp();
    while (sp > 0) {
        sp--;
        uint32_t u = st_id[w][sp], mm = st_cnt[w][sp];
        int me = lane < (int)mm ? lists[w][sp][lane] : 0;  // element at node position `lane`
        __syncwarp();
        bool leaf = mm <= 1u;
        int best_axis = 0, best_at = 0;
        if (!leaf) {
            Box outer;
            for (int c = 0; c < 3; c++) {
                outer.lo[c] = nodes[u].lo[c];
                outer.hi[c] = nodes[u].hi[c];
            }
            float parent_area = area(outer);
            float best_cost = 0.0f;
            bool is_first = true;
            for (int a = 0; a < 3; a++) {
                uint32_t mykey = okey(shf(bc[a], me));
                int rank = 0;
                for (int j = 0; j < (int)mm; j++) {
                    uint32_t kj = __shfl_sync(0xffffffffu, mykey, j);
                    rank += (kj < mykey || (kj == mykey && j < lane)) ? 1 : 0;
                }
                if (lane < (int)mm) perm[w][a][rank] = (uint8_t)lane;
                __syncwarp();
                // Lane q holds the element of rank q.
                int eq = lane < (int)mm ? lists[w][sp][perm[w][a][lane]] : 0;
                Box pb, sb;
                for (int c = 0; c < 3; c++) {
                    float l = shf(lo[c], eq), h = shf(hi[c], eq);
                    pb.lo[c] = l;
                    pb.hi[c] = h;
                    sb.lo[c] = l;
                    sb.hi[c] = h;
                }
                for (int o = 1; o < 32; o <<= 1)
                    for (int c = 0; c < 3; c++) {
                        float pl = __shfl_up_sync(0xffffffffu, pb.lo[c], o);
                        float ph = __shfl_up_sync(0xffffffffu, pb.hi[c], o);
                        float sl = __shfl_down_sync(0xffffffffu, sb.lo[c], o);
                        float sh = __shfl_down_sync(0xffffffffu, sb.hi[c], o);
                        if (lane >= o) {
                            pb.lo[c] = fminf(pb.lo[c], pl);
                            pb.hi[c] = fmaxf(pb.hi[c], ph);
                        }
                        if (lane + o < (int)mm) {
                            sb.lo[c] = fminf(sb.lo[c], sl);
                            sb.hi[c] = fmaxf(sb.hi[c], sh);
                        }
                    }
                // Split i (1 <= i < mm): left = ranks 0..i-1, right = ranks i..mm-1.
                Box la;
                for (int c = 0; c < 3; c++) {
                    la.lo[c] = __shfl_up_sync(0xffffffffu, pb.lo[c], 1);
                    la.hi[c] = __shfl_up_sync(0xffffffffu, pb.hi[c], 1);
                }
                float cost = 0.0f;
                if (lane >= 1 && lane < (int)mm)
                    cost = tsah_cost(ts, parent_area, la, (uint32_t)lane) +
                           tsah_cost(ts, parent_area, sb, mm - (uint32_t)lane);
                float best = shf(cost, 1);
                int at = 1;
                for (int i = 2; i < (int)mm; i++) {
                    float ci = shf(cost, i);
                    if (ci < best) {
                        best = ci;
                        at = i;
                    }
                }
                if (best < best_cost || is_first) {
                    best_cost = best;
                    best_axis = a;
                    best_at = at;
                    is_first = false;
                }
            }
            leaf = (float)mm * 120.0f < best_cost;
        }
        if (leaf) {
            uint32_t tv = __shfl_sync(0xffffffffu, tri, me);
            if (lane < (int)mm) order[beg + out_pos + lane] = tv;
            if (lane == 0) {
                nodes[u].beg = beg + out_pos;
                nodes[u].cnt = mm;
                nodes[u].c0 = 0u;
                nodes[u].c1 = 0u;
            }
            out_pos += mm;
            __syncwarp();
            continue;
        }
        // Children in sorted order of the chosen axis; exact boxes with the
        // first of equal bounds in child order.
        uint32_t at = (uint32_t)best_at;
        int eq = lane < (int)mm ? lists[w][sp][perm[w][best_axis][lane]] : 0;
        bool in_left = lane < (int)at, in_right = lane >= (int)at && lane < (int)mm;
        Box cb[2];
        for (int side = 0; side < 2; side++) {
            bool mine = side == 0 ? in_left : in_right;
            for (int c = 0; c < 3; c++) {
                float vl = shf(lo[c], eq), vh = shf(hi[c], eq);
                unsigned long long kmin = mine ? (((unsigned long long)okey(vl) << 32) | (uint32_t)lane) : ~0ull;
                unsigned long long kmax =
                    mine ? (((unsigned long long)okey(vh) << 32) | (0xffffffffu - (uint32_t)lane)) : 0ull;
                for (int o = 16; o > 0; o >>= 1) {
                    kmin = min(kmin, shfl64(kmin, o));
                    kmax = max(kmax, shfl64(kmax, o));
                }
                int qmin = (int)((uint32_t)kmin & 31u), qmax = (int)((0xffffffffu - (uint32_t)kmax) & 31u);
                int emin = __shfl_sync(0xffffffffu, eq, qmin), emax = __shfl_sync(0xffffffffu, eq, qmax);
                float bl = shf(lo[c], emin), bh = shf(hi[c], emax);
                cb[side].lo[c] = bl;
                cb[side].hi[c] = bh;
            }
        }
        bool swap = area(cb[0]) > area(cb[1]);
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(next_id, 2u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base + 2u > n_nodes || sp + 2 > (int)kSmall + 1) {
            if (lane == 0) atomicOr(err, 4u);
            return;
        }
        uint32_t id_l = base, id_r = base + 1u;
        if (lane == 0) {
            for (int c = 0; c < 3; c++) {
                nodes[id_l].lo[c] = cb[0].lo[c];
                nodes[id_l].hi[c] = cb[0].hi[c];
                nodes[id_r].lo[c] = cb[1].lo[c];
                nodes[id_r].hi[c] = cb[1].hi[c];
            }
            nodes[id_l].cnt = at;
            nodes[id_r].cnt = mm - at;
            nodes[u].c0 = swap ? id_r : id_l;
            nodes[u].c1 = swap ? id_l : id_r;
        }
        // Element lists of the children (ranks in order); the second child
        // goes below the first on the stack so that the first is built first.
        uint32_t first = swap ? id_r : id_l, second = swap ? id_l : id_r;
        uint32_t first_cnt = swap ? mm - at : at, second_cnt = swap ? at : mm - at;
        uint32_t first_off = swap ? at : 0u, second_off = swap ? 0u : at;
        int v1 = __shfl_sync(0xffffffffu, eq, (int)((first_off + (uint32_t)lane) & 31u));
        int v2 = __shfl_sync(0xffffffffu, eq, (int)((second_off + (uint32_t)lane) & 31u));
        __syncwarp();  // every read of the popped list is done
        if (lane < (int)second_cnt) lists[w][sp][lane] = (uint8_t)v2;
        if (lane < (int)first_cnt) lists[w][sp + 1][lane] = (uint8_t)v1;
        if (lane == 0) {
            st_id[w][sp] = second;
            st_cnt[w][sp] = second_cnt;
            st_id[w][sp + 1] = first;
            st_cnt[w][sp + 1] = first_cnt;
        }
        sp += 2;
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

#define BK(call, what)                                                                             \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return set_error(CVX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
static int32_t dalloc(DevBuf& b, size_t count, const char* what) {
    cudaError_t e = cudaMalloc(&b.p, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return set_error(CVX_ERR_DEVICE, std::string("device BVH build: ") + what + ": " +
                                                                  cudaGetErrorString(e));
    return CVX_OK;
}

static void tiles_of(std::vector<Tile>& out, uint32_t slot, uint32_t axis, uint32_t beg, uint32_t cnt) {
    for (uint32_t s = 0; s < cnt; s += kTile) out.push_back(Tile{slot, axis, beg + s, std::min<uint32_t>(kTile, cnt - s)});
}

static unsigned blocks(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

int32_t bvh_build_device(const cvx_triangle* tris, uint32_t n, cvx_bvh** out) {
    if (n == 0) return set_error(CVX_ERR_INVALID, "cannot build a BVH of zero triangles");
    if (n > kMaxTris) return set_error(CVX_ERR_CAPACITY, "device BVH build: more than 2^26 triangles");
    cudaStream_t st = nullptr;
    BK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{st};

    std::vector<float> tx, tt;
    float ty;
    tsah_tables(n, tx, tt, &ty);
    const uint32_t max_nodes = 2 * n;
    const uint32_t max_slots = n / (kSmall + 1) + 1;

    DevBuf d_tris, d_refs, d_order, d_tmp, d_srt, d_binf, d_nodes, d_inner, d_tx, d_tt, d_misc, d_cnt, d_key,
        d_mode, d_dec, d_slots, d_tiles, d_tiles2, d_hist, d_off, d_ids, d_acc, d_sortbuf, d_pairs;
    int32_t s = 0;
    if ((s = dalloc<cvx_triangle>(d_tris, n, "triangles")) || (s = dalloc<float>(d_refs, (size_t)9 * n, "refs")) ||
        (s = dalloc<uint32_t>(d_order, n, "order")) || (s = dalloc<uint32_t>(d_tmp, n, "order")) ||
        (s = dalloc<uint32_t>(d_srt, (size_t)3 * n, "sort")) || (s = dalloc<uint8_t>(d_binf, (size_t)3 * n, "bins")) ||
        (s = dalloc<InterimNode>(d_nodes, max_nodes, "nodes")) ||
        (s = dalloc<float>(d_inner, (size_t)6 * max_nodes, "inner boxes")) ||
        (s = dalloc<float>(d_tx, (size_t)n + 1, "tsah")) || (s = dalloc<float>(d_tt, (size_t)n + 1, "tsah")) ||
        (s = dalloc<uint32_t>(d_misc, 4, "flags")) ||
        (s = dalloc<uint32_t>(d_cnt, (size_t)max_slots * 3 * kBins, "bin counts")) ||
        (s = dalloc<uint32_t>(d_key, (size_t)max_slots * 3 * kBins * 6, "bin boxes")) ||
        (s = dalloc<uint32_t>(d_mode, (size_t)max_slots * 3, "modes")) ||
        (s = dalloc<Decision>(d_dec, max_slots, "decisions")) || (s = dalloc<Slot>(d_slots, max_slots, "slots")))
        return s;
    cvx_triangle* tri_d = (cvx_triangle*)d_tris.p;
    float* refs = (float*)d_refs.p;
    Refs R;
    for (int c = 0; c < 3; c++) {
        R.lo[c] = refs + (size_t)c * n;
        R.hi[c] = refs + (size_t)(3 + c) * n;
        R.bc[c] = refs + (size_t)(6 + c) * n;
    }
    uint32_t* order = (uint32_t*)d_order.p;
    uint32_t* order_tmp = (uint32_t*)d_tmp.p;
    uint32_t* srt = (uint32_t*)d_srt.p;
    uint8_t* binf = (uint8_t*)d_binf.p;
    InterimNode* nodes = (InterimNode*)d_nodes.p;
    float* inner = (float*)d_inner.p;
    uint32_t* misc = (uint32_t*)d_misc.p;  // [0] bad input, [1] error bits, [2] next node id
    BinStats bs{(uint32_t*)d_cnt.p, (uint32_t*)d_key.p};
    Tsah ts{(const float*)d_tx.p, (const float*)d_tt.p, ty};

    BK(cudaMemcpyAsync(tri_d, tris, (size_t)n * sizeof(cvx_triangle), cudaMemcpyHostToDevice, st), "upload");
    BK(cudaMemcpyAsync(d_tx.p, tx.data(), tx.size() * 4, cudaMemcpyHostToDevice, st), "upload");
    BK(cudaMemcpyAsync(d_tt.p, tt.data(), tt.size() * 4, cudaMemcpyHostToDevice, st), "upload");
    BK(cudaMemsetAsync(misc, 0, 16, st), "memset");
    BK(cudaMemsetAsync(nodes, 0, (size_t)max_nodes * sizeof(InterimNode), st), "memset");
    const float third = 1.0f / 3.0f;
    k_prep<<<blocks(n, 256), 256, 0, st>>>(tri_d, n, third, R, order, misc);

    // Host-side copies of every interim node's range.
    std::vector<uint32_t> h_beg(max_nodes, 0), h_cnt(max_nodes, 0);
    uint32_t next_id = 1;
    h_beg[0] = 0;
    h_cnt[0] = n;

    // Scratch that grows with the largest list of a level.
    size_t cap_tiles = 0, cap_tiles2 = 0, cap_ids = 0, cap_pairs = 0, cap_sort = 0;
    auto ensure = [&](DevBuf& b, size_t& cap, size_t bytes, const char* what) -> int32_t {
        if (bytes <= cap) return CVX_OK;
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        cap = std::max(bytes, (size_t)4096);
        cudaError_t e = cudaMalloc(&b.p, cap);
        if (e != cudaSuccess)
            return set_error(CVX_ERR_DEVICE, std::string("device BVH build: ") + what + ": " + cudaGetErrorString(e));
        return CVX_OK;
    };
    size_t cap_hist = 0, cap_off = 0, cap_acc = 0;

    // Exact boxes of a list of interim nodes (their ranges are current).
    auto node_boxes = [&](const std::vector<uint32_t>& ids) -> int32_t {
        if (ids.empty()) return CVX_OK;
        std::vector<Tile> tl;
        for (size_t j = 0; j < ids.size(); j++) tiles_of(tl, (uint32_t)j, 0, h_beg[ids[j]], h_cnt[ids[j]]);
        int32_t e;
        if ((e = ensure(d_tiles2, cap_tiles2, tl.size() * sizeof(Tile), "tiles")) ||
            (e = ensure(d_ids, cap_ids, ids.size() * 4, "ids")) ||
            (e = ensure(d_acc, cap_acc, ids.size() * sizeof(BoxAcc), "boxes")))
            return e;
        BK(cudaMemcpyAsync(d_tiles2.p, tl.data(), tl.size() * sizeof(Tile), cudaMemcpyHostToDevice, st), "upload");
        BK(cudaMemcpyAsync(d_ids.p, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice, st), "upload");
        k_box_init<<<blocks(ids.size(), 128), 128, 0, st>>>((BoxAcc*)d_acc.p, (uint32_t)ids.size());
        k_box<<<(unsigned)tl.size(), kTile, 0, st>>>((const Tile*)d_tiles2.p, (uint32_t)tl.size(), R, order, n,
                                                     (BoxAcc*)d_acc.p, (uint32_t)ids.size(), misc + 1);
        k_box_store<<<blocks(ids.size(), 128), 128, 0, st>>>((const uint32_t*)d_ids.p, (uint32_t)ids.size(),
                                                              (const BoxAcc*)d_acc.p, R, order, n, nodes, max_nodes,
                                                              inner, misc + 1);
        // the tile and id buffers are reused by the next call: finish this one
        BK(cudaStreamSynchronize(st), "node boxes");
        return CVX_OK;
    };

    // Root: range [0, n) in input order.
    std::vector<uint32_t> root_ids{0};
    {
        InterimNode r0{};
        r0.beg = 0;
        r0.cnt = n;
        BK(cudaMemcpyAsync(nodes, &r0, sizeof r0, cudaMemcpyHostToDevice, st), "upload");
    }
    if ((s = node_boxes(root_ids))) return s;
    uint32_t bad = 0;
    BK(cudaMemcpy(&bad, misc, 4, cudaMemcpyDeviceToHost), "flags");
    if (bad)
        return set_error(CVX_ERR_INVALID,
                         "device BVH build: NaN or infinite vertex coordinates (the host build takes them)");

    std::vector<uint32_t> active, small;
    if (n > kSmall) active.push_back(0);
    else if (n >= 2) small.push_back(0);

    while (!active.empty()) {
        const uint32_t K = (uint32_t)active.size();
        std::vector<Slot> slots(K);
        std::vector<Tile> tl;
        for (uint32_t k = 0; k < K; k++) {
            uint32_t id = active[k];
            slots[k] = Slot{id, h_beg[id], h_cnt[id]};
            tiles_of(tl, k, 0, h_beg[id], h_cnt[id]);
        }
        if ((s = ensure(d_tiles, cap_tiles, tl.size() * sizeof(Tile), "tiles"))) return s;
        BK(cudaMemcpyAsync(d_slots.p, slots.data(), K * sizeof(Slot), cudaMemcpyHostToDevice, st), "upload");
        BK(cudaMemcpyAsync(d_tiles.p, tl.data(), tl.size() * sizeof(Tile), cudaMemcpyHostToDevice, st), "upload");
        const Slot* ds = (const Slot*)d_slots.p;
        k_stats_init<<<blocks((size_t)K * 3 * kBins, 256), 256, 0, st>>>(bs, K * 3 * kBins);
        k_bin_float<<<(unsigned)tl.size(), kTile, 0, st>>>((const Tile*)d_tiles.p, (uint32_t)tl.size(), ds, K, R,
                                                          order, n, inner, binf, bs, misc + 1);
        k_fallback<<<blocks(K, 128), 128, 0, st>>>(ds, K, bs, (uint32_t*)d_mode.p);
        std::vector<uint32_t> mode((size_t)K * 3);
        BK(cudaMemcpyAsync(mode.data(), d_mode.p, mode.size() * 4, cudaMemcpyDeviceToHost, st), "download");
        BK(cudaStreamSynchronize(st), "binning");

        // Uniform split (bvh.rs:176-201) where coordinate binning fell back.
        std::vector<Tile> small_pairs, uni_tiles;
        std::vector<Tile> big_pairs;
        for (uint32_t k = 0; k < K; k++)
            for (uint32_t a = 0; a < 3; a++)
                if (mode[3 * k + a]) {
                    Tile pr{k, a, slots[k].beg, slots[k].cnt};
                    (pr.len <= kBlockSort ? small_pairs : big_pairs).push_back(pr);
                    for (uint32_t r0 = 0; r0 < pr.len; r0 += kTile)
                        uni_tiles.push_back(Tile{k, a, r0, std::min<uint32_t>(kTile, pr.len - r0)});
                }
        if (!uni_tiles.empty()) {
            std::vector<Tile> pairs = small_pairs;
            pairs.insert(pairs.end(), big_pairs.begin(), big_pairs.end());
            if ((s = ensure(d_pairs, cap_pairs, pairs.size() * sizeof(Tile), "pairs")) ||
                (s = ensure(d_tiles2, cap_tiles2, uni_tiles.size() * sizeof(Tile), "tiles")))
                return s;
            BK(cudaMemcpyAsync(d_pairs.p, pairs.data(), pairs.size() * sizeof(Tile), cudaMemcpyHostToDevice, st),
               "upload");
            BK(cudaMemcpyAsync(d_tiles2.p, uni_tiles.data(), uni_tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice,
                               st),
               "upload");
            if (!small_pairs.empty())
                k_sort_block<<<(unsigned)small_pairs.size(), 1024, 0, st>>>((const Tile*)d_pairs.p,
                                                                           (uint32_t)small_pairs.size(), R, order, n,
                                                                           srt, misc + 1);
            for (const Tile& pr : big_pairs) {
                uint32_t m2 = 4096;
                while (m2 < pr.len) m2 <<= 1;
                if ((s = ensure(d_sortbuf, cap_sort, (size_t)m2 * 8, "sort buffer"))) return s;
                unsigned long long* buf = (unsigned long long*)d_sortbuf.p;
                k_sort_fill<<<blocks(m2, 256), 256, 0, st>>>(pr, m2, R, order, buf);
                // stages 2..4096 inside chunks, then the larger ones
                k_sort_chunk<<<m2 / 4096, 1024, 0, st>>>(buf, m2, 2, 4096, 1);
                for (uint32_t size = 8192; size <= m2; size <<= 1) {
                    uint32_t j = size >> 1;
                    for (; j >= 4096; j >>= 1) k_sort_step<<<blocks(m2, 256), 256, 0, st>>>(buf, m2, size, j);
                    k_sort_chunk<<<m2 / 4096, 1024, 0, st>>>(buf, m2, size, size, j);
                }
                k_sort_extract<<<blocks(pr.len, 256), 256, 0, st>>>(pr, buf, n, srt);
            }
            k_axis_reset<<<blocks(pairs.size() * kBins, 256), 256, 0, st>>>((const Tile*)d_pairs.p,
                                                                             (uint32_t)pairs.size(), bs);
            k_uniform_stats<<<(unsigned)uni_tiles.size(), kTile, 0, st>>>(
                (const Tile*)d_tiles2.p, (uint32_t)uni_tiles.size(), ds, K, R, order, n, srt, bs, misc + 1);
        }
        k_choose_warp<<<blocks((size_t)K * 32, 128), 128, 0, st>>>(ds, K, nodes, bs, ts, (Decision*)d_dec.p);
        std::vector<Decision> dec(K);
        BK(cudaMemcpyAsync(dec.data(), d_dec.p, K * sizeof(Decision), cudaMemcpyDeviceToHost, st), "download");
        BK(cudaStreamSynchronize(st), "split choice");

        // Partition the split slots.
        std::vector<Tile> part;            // axis: 0..2 coordinate bins, 3..5 uniform
        std::vector<uint32_t> slot_tiles;  // per coordinate-binned split slot: [t0, t1) in `fl`
        std::vector<Tile> fl;              // coordinate-binned tiles (for the histograms)
        std::vector<uint32_t> triples, children, next_active;
        for (uint32_t k = 0; k < K; k++) {
            const Decision& d = dec[k];
            if (d.leaf) continue;
            if (d.axis > 2 || d.nl == 0 || d.nl >= slots[k].cnt) return set_error(CVX_ERR_DEVICE, "device BVH build: bad split");
            bool uni = mode[3 * k + d.axis] != 0;
            if (uni) {
                tiles_of(part, k, 3 + d.axis, slots[k].beg, slots[k].cnt);
            } else {
                uint32_t t0 = (uint32_t)fl.size();
                tiles_of(fl, k, d.axis, slots[k].beg, slots[k].cnt);
                slot_tiles.push_back(t0);
                slot_tiles.push_back((uint32_t)fl.size());
            }
            uint32_t l = next_id, r = next_id + 1;
            next_id += 2;
            if (next_id > max_nodes) return set_error(CVX_ERR_DEVICE, "device BVH build: node overflow");
            h_beg[l] = slots[k].beg;
            h_cnt[l] = d.nl;
            h_beg[r] = slots[k].beg + d.nl;
            h_cnt[r] = slots[k].cnt - d.nl;
            triples.insert(triples.end(), {slots[k].id, l, r});
            children.push_back(l);
            children.push_back(r);
        }
        if (!children.empty()) {
            // coordinate-binned tiles first (their block index is the tile_off row), then uniform
            size_t n_fl = fl.size();
            std::vector<Tile> all = fl;
            all.insert(all.end(), part.begin(), part.end());
            if ((s = ensure(d_tiles, cap_tiles, all.size() * sizeof(Tile), "tiles")) ||
                (s = ensure(d_hist, cap_hist, std::max<size_t>(n_fl, 1) * kBins * 4, "histograms")) ||
                (s = ensure(d_off, cap_off, std::max<size_t>(n_fl, 1) * kBins * 4, "offsets")) ||
                (s = ensure(d_ids, cap_ids, std::max(slot_tiles.size(), triples.size()) * 4, "ids")))
                return s;
            BK(cudaMemcpyAsync(d_tiles.p, all.data(), all.size() * sizeof(Tile), cudaMemcpyHostToDevice, st), "upload");
            if (n_fl) {
                BK(cudaMemcpyAsync(d_ids.p, slot_tiles.data(), slot_tiles.size() * 4, cudaMemcpyHostToDevice, st),
                   "upload");
                k_tile_hist<<<(unsigned)n_fl, kTile, 0, st>>>((const Tile*)d_tiles.p, (uint32_t)n_fl, binf, n,
                                                              (uint32_t*)d_hist.p);
                k_tile_offsets<<<(unsigned)(slot_tiles.size() / 2), 1024, 0, st>>>(
                    (const uint32_t*)d_ids.p, (uint32_t)(slot_tiles.size() / 2), (const uint32_t*)d_hist.p,
                    (uint32_t*)d_off.p);
            }
            k_scatter<<<(unsigned)all.size(), kTile, 0, st>>>((const Tile*)d_tiles.p, (uint32_t)all.size(), ds, K,
                                                              binf, srt, (const uint32_t*)d_off.p, order, n, order_tmp,
                                                              misc + 1);
            k_copy_back<<<(unsigned)all.size(), kTile, 0, st>>>((const Tile*)d_tiles.p, (uint32_t)all.size(),
                                                                order_tmp, order, n);
            BK(cudaStreamSynchronize(st), "partition");
            // Children: ranges, exact boxes, then the parents' links.
            {
                std::vector<InterimNode> ch(children.size());
                for (size_t j = 0; j < children.size(); j++) {
                    ch[j] = InterimNode{};
                    ch[j].beg = h_beg[children[j]];
                    ch[j].cnt = h_cnt[children[j]];
                }
                // children ids are consecutive
                BK(cudaMemcpyAsync(nodes + children[0], ch.data(), ch.size() * sizeof(InterimNode),
                                   cudaMemcpyHostToDevice, st),
                   "upload");
            }
            if ((s = node_boxes(children))) return s;
            if ((s = ensure(d_ids, cap_ids, triples.size() * 4, "ids"))) return s;
            BK(cudaMemcpyAsync(d_ids.p, triples.data(), triples.size() * 4, cudaMemcpyHostToDevice, st), "upload");
            k_link<<<blocks(triples.size() / 3, 128), 128, 0, st>>>((const uint32_t*)d_ids.p,
                                                                     (uint32_t)(triples.size() / 3), nodes, max_nodes,
                                                                     misc + 1);
            BK(cudaStreamSynchronize(st), "children");
            for (uint32_t c : children) {
                if (h_cnt[c] > kSmall) next_active.push_back(c);
                else if (h_cnt[c] >= 2) small.push_back(c);
            }
        }
        active.swap(next_active);
        uint32_t errbits = 0;
        BK(cudaMemcpy(&errbits, misc + 1, 4, cudaMemcpyDeviceToHost), "flags");
        if (errbits) return set_error(CVX_ERR_DEVICE, "device BVH build: internal range check failed");
    }

    if (!small.empty()) {
        if ((s = ensure(d_ids, cap_ids, small.size() * 4, "ids"))) return s;
        BK(cudaMemcpyAsync(d_ids.p, small.data(), small.size() * 4, cudaMemcpyHostToDevice, st), "upload");
        BK(cudaMemcpyAsync(misc + 2, &next_id, 4, cudaMemcpyHostToDevice, st), "upload");
        k_small<<<blocks(small.size(), kSmallWarps), 32 * kSmallWarps, 0, st>>>(
            (const uint32_t*)d_ids.p, (uint32_t)small.size(), nodes, max_nodes, misc + 2, order, n, R, ts, misc + 1);
        BK(cudaMemcpyAsync(&next_id, misc + 2, 4, cudaMemcpyDeviceToHost, st), "download");
    }
    uint32_t errbits = 0;
    BK(cudaMemcpyAsync(&errbits, misc + 1, 4, cudaMemcpyDeviceToHost, st), "download");
    BK(cudaStreamSynchronize(st), "small builds");
    if (errbits) return set_error(CVX_ERR_DEVICE, "device BVH build: internal range check failed");
    if (next_id > max_nodes) return set_error(CVX_ERR_DEVICE, "device BVH build: node overflow");

    std::vector<InterimNode> tree(next_id);
    std::vector<uint32_t> h_order(n);
    BK(cudaMemcpyAsync(tree.data(), nodes, (size_t)next_id * sizeof(InterimNode), cudaMemcpyDeviceToHost, st),
       "download");
    BK(cudaMemcpyAsync(h_order.data(), order, (size_t)n * 4, cudaMemcpyDeviceToHost, st), "download");
    BK(cudaStreamSynchronize(st), "download");
    return bvh_from_interim(tree, h_order, tris, n, out);
}

}  // namespace cvx

extern "C" int32_t cvx_bvh_build_device(const cvx_triangle* triangles, uint32_t n, cvx_bvh** out) {
    if (!out || (!triangles && n)) return cvx::set_error(CVX_ERR_INVALID, "null argument");
    return cvx::bvh_build_device(triangles, n, out);
}
