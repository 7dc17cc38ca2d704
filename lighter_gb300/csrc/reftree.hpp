// Per-instance triangle trees with the reference's leaf structure, used only
// by the sample-offset pass.
//
// TriTree::OffsetSample (lighter_math.cpp:991-1044) moves a sample while it
// walks one instance's AABBTree, and it tests every triangle stored in a leaf
// the query box reaches, whether or not the triangle's own box meets the
// query. Its result therefore depends on the tree's leaves and their order,
// so this pass rebuilds that tree with the same split rules
// (AABBTree::SetAABBs/_MakeNode, lighter_math.cpp:653-781): leaf at <= 4
// items or depth 16; items with volume * 3 >= node volume stay in the node;
// the rest are sorted (std::sort) by box centre along the longest axis of
// their union and halved. Every other query of the bake uses the flat GPU BVH.
#pragma once

#include <cstdint>
#include <vector>

#include "common.cuh"

namespace lg {

// Node in the reference layout: box, right child `ch` (left = node + 1, -1 for
// none) and `ido`, the offset of <count, ids...> in the item list (-1: none).
struct RefNode {
    float mn[3], mx[3];
    int32_t ch, ido;
};

struct RefTree {
    std::vector<RefNode> nodes;
    std::vector<int32_t> items;
};

// Builds the tree over `n` triangles given as 9 floats each (P1, P2, P3); with
// `threads`, the halves of the top levels are built on two threads each (the
// layout is the same either way).
void build_ref_tree(const float* tri_xyz, size_t n, RefTree& out, bool threads = true);

}  // namespace lg
