// Shared host-side helpers of libconvector_gpu (not part of the C-ABI).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/convector_gpu.h"

namespace cvx {

int32_t set_error(int32_t status, const std::string& msg);

// Allocation-failure injection (cvx_inject_allocation_failure): called by the
// library's device-allocation helpers before each cudaMalloc; true when this
// allocation is to fail as if the device were out of memory.
bool injected_allocation_failure();

// A node of the interim tree of the device BVH build (bvh.rs:52-62): its
// exact bounding box, its triangles order[beg .. beg + cnt) and its children
// (c0 == 0: a leaf; node 0 is the root and never a child).
struct InterimNode {
    float lo[3], hi[3];
    uint32_t beg, cnt;
    uint32_t c0, c1;
};

// TSAH factors for triangle counts 0..n (index 0 unused) and the constant
// denominator, as the host build computes them.
void tsah_tables(uint32_t n, std::vector<float>& x, std::vector<float>& t, float* y);
// crystallize and statistics over an interim tree (same results as the host build).
int32_t bvh_from_interim(const std::vector<InterimNode>& t, const std::vector<uint32_t>& order,
                         const cvx_triangle* src, uint32_t n, cvx_bvh** out);

struct MeshTri {
    uint32_t v[3];
    int64_t t[3];  // -1: the face has no texture coordinates
    uint32_t material;
};

}  // namespace cvx

struct cvx_mesh {
    std::vector<float> vertices;    // 3 per vertex
    std::vector<float> tex_coords;  // 2 per coordinate
    std::vector<cvx::MeshTri> triangles;
};

struct cvx_bvh {
    std::vector<cvx_bvh_node> nodes;
    std::vector<cvx_triangle> triangles;  // BVH (leaf) order
    std::vector<uint32_t> source_index;   // input index of each BVH-order triangle
    float avg_area_ratio = 0.0f;
    float avg_tris_per_leaf = 0.0f;
    uint32_t depth = 0;
};
