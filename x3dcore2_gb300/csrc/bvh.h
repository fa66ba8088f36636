// Host BVH builder: binned SAH over triangles, flattened to 32-byte nodes in two
// structure-of-arrays halves (lo: min xyz + link, hi: max xyz + count), children stored as
// adjacent pairs so one interior visit reads 64 contiguous bytes per half-array pair.
#pragma once

#include <cstdint>
#include <vector>

namespace e8g {

// Traversal stacks live in shared memory with this many entries per thread; the builder never
// makes the tree deeper than this, so a push can never overflow.
constexpr uint32_t kMaxTreeDepth = 32;

struct bvh_build_opts {
    // Tuned for the GPU traversal (measured on a 1.3M-triangle scene: 4% more paths/s than the
    // reference's constants BVH_MAX_PRIMS 4, BVH_BUCKET_COUNT 20, triangle cost 8, box cost 1 of
    // pathspace.cpp:121-124, which the reference layout keeps).
    uint32_t max_leaf_prims = 8;
    uint32_t num_bins = 32;
    float tri_cost = 0.0f; // <= 0: the layout's tuned value (effective_tri_cost)
    float node_cost = 1.0f;
    uint32_t num_threads = 0;
    uint32_t layout = 0; // 0: SAH child pairs, 1: the reference's tree, 2: eight-wide
    uint32_t builder = 0; // 0: host, 1: device (gpu_build.cu)
};

// The SAH triangle cost a build uses: the given one, or, when it is <= 0, the value measured
// best for the layout's traversal (1 for SAH pairs in the megakernel; 3 for the eight-wide tree
// in the wavefront, whose lanes then wait less on leaves of uneven size: 1.92 vs 1.85 G paths/s).
inline float effective_tri_cost(bvh_build_opts const &o) {
    return o.tri_cost > 0.0f ? o.tri_cost : (o.layout == 2 ? 3.0f : 1.0f);
}

struct flat_bvh {
    // node i: lo[i] = (min.x, min.y, min.z, link), hi[i] = (max.x, max.y, max.z, count)
    // count == 0: interior, children at link and link + 1; count > 0: leaf of `count`
    // triangles starting at position `link` of tri_order.
    std::vector<float> lo;      // 4 per node
    std::vector<float> hi;      // 4 per node
    std::vector<uint32_t> tri_order; // BVH position -> global triangle index
    uint32_t num_nodes = 0;
    uint32_t num_leaves = 0;
    uint32_t max_depth = 0;
    double avg_leaf_depth = 0;
    float eps = 0; // boxes are the exact unions pushed out by |v| * 1e-6 + eps (bvh_boxes.h)
};

// tris: 3 global vertex indices per triangle; pos: 3 floats per vertex.
flat_bvh build_bvh(float const *pos, uint32_t const *tris, uint32_t num_tris, bvh_build_opts const &o);

// The reference's tree (bvh_path_space_layout::commit) in depth-first order: node n's left child
// is n + 1, its right child `link`; boxes are the reference's, uninflated.
flat_bvh build_bvh_reference(float const *pos, uint32_t const *tris, uint32_t num_tris);

// Deepest reference tree the 64-entry traversal stack can walk (the stack never holds more than
// depth + 1 entries).
constexpr uint32_t kMaxRefTreeDepth = 63;

} // namespace e8g
