// Device layout of a scene. Everything is kept in the reference's BVH order
// (bvh.rs:389-428 `crystallize`): triangle i of the device arrays is
// `Bvh::triangles[i]`, node pair p holds `Bvh::nodes[2p]` and `[2p+1]`.
//
//  * NodePair, 64 B (4 x 16 B): the two sibling nodes the traversal always
//    fetches together (bvh.rs:635-636), one cache-line-sized record:
//      q0 = lo0.x lo0.y lo0.z hi0.x     q1 = hi0.y hi0.z lo1.x lo1.y
//      q2 = lo1.z hi1.x hi1.y hi1.z     q3 = index0 len0 index1 len1 (u32)
//  * TriGeom, 48 B (3 x 16 B): what the triangle test reads
//    (triangle.rs:65-80): v0, e1 = v0 - v2, e2 = v1 - v0 and the unnormalized
//    normal n = cross_fma(e1, e2), precomputed with the same operations:
//      q0 = v0.x v0.y v0.z n.x   q1 = e1.x e1.y e1.z n.y   q2 = e2.x e2.y e2.z n.z
//  * TriShade, 32 B: what only the hit triangle needs: uv0..uv2, material.
//  * LightRec, 64 B: direct-sample triangles (scene.rs:117-122) with the
//    per-triangle factors of intersect_direct / get_direct_sample
//    (triangle.rs:158-161, scene.rs:169-174) precomputed:
//      q0 = v0, area   q1 = e1, rnorm   q2 = e2, -   q3 = normal (n * rnorm), -
#pragma once
#include <cstdint>

namespace cvx {

struct TriShade {
    float uv[6];
    uint32_t material;
    uint32_t pad;
};

struct DeviceScene {
    const float4* nodes;  // NodePair[n_nodes / 2], 4 float4 each
    const float4* geom;   // TriGeom[n_tris], 3 float4 each
    const TriShade* shade;
    const float4* lights;  // LightRec[n_lights], 4 float4 each
    uint32_t n_nodes, n_tris, n_lights;
    uint32_t general_pick;  // 1: (bits * n) >> 32; 0: bits >> 29 (needs n == 8)
    uint32_t depth;         // BVH depth (launch choices only)
    // Every node bound is finite, lo <= hi on each axis and none is -0: the
    // ray-cast kernel may take the select-form slab test (box_test_sel).
    uint32_t slab_sel;
};

struct DeviceCamera {
    float pos[3], pos_delta[3], q[4], dq[4], screen_distance;
};

constexpr uint32_t kSkyMaterial = 0xC0000000u;  // material.rs:85-90
constexpr int kStackDepth = 128;  // >= BVH depth + 2 (checked at scene creation)

// Error bits a kernel reports through its status word instead of trapping.
constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrIterationCap = 2u;

}  // namespace cvx
