// The host kd-tree object shared by the builder (kdtree_build.cpp) and the
// tree-file reader/writer (tree_file.cpp).
#pragma once

#include <cstdint>
#include <vector>

#include "turner_gpu.h"

struct turner_kdtree {
    std::vector<uint64_t> nodes;
    std::vector<turner_triangle> tris;
    float box[6];
    uint32_t height = 0;
};

namespace turner {
namespace host {
// Triangle records as the Triangle constructor precomputes them
// (lib/triangle.h:22-39) and the scene box as KDTree::KDTree takes it (the
// union of the triangle boxes, lib/kdtree.cpp:474-490): min xyz, max xyz.
void make_records(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris,
                  std::vector<turner_triangle>& tris, float box[6]);
} // namespace host
} // namespace turner
