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
