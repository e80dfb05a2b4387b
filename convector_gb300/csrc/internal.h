// Shared host-side helpers of libconvector_gpu (not part of the C-ABI).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/convector_gpu.h"

namespace cvx {

int32_t set_error(int32_t status, const std::string& msg);

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
