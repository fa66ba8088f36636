// Eight-wide BVH with quantized child boxes, collapsed from the binary SAH tree.
//
// Node record, 96 bytes = 6 x uint4 (24 words), 16-byte aligned:
//   w[0..2]  origin p of the node's quantization grid (float bits)
//   w[3]     exponent bytes ex | ey << 8 | ez << 16 (grid step 2^(e-127) per axis) | imask << 24
//            (imask bit s: slot s holds an interior child)
//   w[4]     child_base: node index of the first interior child; interior children are stored
//            contiguously in slot order, so slot s's node is child_base + popc(imask & ((1<<s)-1))
//   w[5]     tri_base: first triangle record of this node's leaves
//   w[6..7]  meta bytes, one per slot: a leaf slot's first triangle, relative to tri_base
//   w[8..19] quantized boxes: lo_x[8], lo_y[8], lo_z[8], hi_x[8], hi_y[8], hi_z[8] (bytes);
//            a child box is p + q * step, rounded outwards by at least one step
//   w[20]    leaf triangle counts, 4 bits per slot (0: interior or empty slot)
//   w[21]    leaf mask (bit s: slot s is a leaf with at least one triangle)
//   w[22..23] unused
// Child slots are assigned per node so that, for a ray whose direction has sign octant o
// (bit a set when d[a] < 0), visiting slots in the order k ^ o for k = 0..7 goes roughly front
// to back (the ordering of Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs
// Through Compressed Wide BVHs", HPG 2017, whose node compression this layout follows in spirit).
#pragma once

#include "bvh.h"

#include <cstdint>
#include <vector>

namespace e8g {

constexpr uint32_t kWideWords = 24;     // 32-bit words per node
constexpr uint32_t kWideMaxLeaf = 15;   // triangles per leaf slot (4-bit count)
constexpr uint32_t kWideMaxDepth = 16;  // traversal stack entries; deeper trees are rejected

struct wide_bvh {
    std::vector<uint32_t> nodes;     // kWideWords per node, node 0 is the root
    std::vector<uint32_t> tri_order; // triangle record position -> global triangle index
    uint32_t num_nodes = 0;
    uint32_t num_leaves = 0;         // leaf slots
    uint32_t max_depth = 0;          // levels of wide nodes
    std::vector<uint32_t> level_start; // first node of every level (breadth-first), then num_nodes
    bool ok = false;                 // false: deeper than kWideMaxDepth (use the binary tree)
};

// Collapses the binary SAH tree `b` (inflated boxes, child pairs) into an eight-wide tree.
// pos / tris give the triangles' boxes for leaves that must be split (more than kWideMaxLeaf
// triangles); max_abs is the largest absolute coordinate the rays and the scene reach, which
// sets the smallest grid step (the quantized boxes stay conservative under float rounding).
wide_bvh collapse_wide(flat_bvh const &b, float const *pos, uint32_t const *tris, float max_abs);

} // namespace e8g
