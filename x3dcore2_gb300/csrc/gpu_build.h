// BVH build on the device (gpu_build.cu): the SAH-pair layout of bvh.h from the scene's device
// vertices, without a host round trip.
#pragma once

#include "device.cuh"

namespace e8g {

struct GpuBuildIn {
    uint4 const *tidx;   // per triangle: global vertex indices
    float4 const *vpos;  // per vertex
    uint32_t num_tris;
    uint32_t max_leaf;   // largest leaf (at most 15)
    float tri_cost, node_cost;
    uint32_t max_depth;  // levels the traversal stack allows
    int num_sms;
    void *scratch;       // gpu_build_scratch_bytes(num_tris) bytes of device memory
    void *host_pinned;   // 32 bytes of pinned host memory
    float4 *nlo, *nhi;   // 2 * num_tris nodes each
    float4 *tri;         // 3 * num_tris triangle records
};

struct GpuBuildOut {
    uint32_t num_nodes = 0, num_leaves = 0, max_depth = 0, ploc_rounds = 0;
    double avg_leaf_depth = 0;
    float scene_lo[3] = {0, 0, 0}, scene_hi[3] = {0, 0, 0}; // exact box of all triangles
    bool ok = false; // false: deeper than max_depth (the caller builds on the host instead)
};

size_t gpu_build_scratch_bytes(uint32_t num_tris);
// Synchronises `st` once per clustering round and per level. cudaErrorUnknown: no progress
// (non-finite boxes); the caller builds on the host instead.
cudaError_t gpu_build_sah_pairs(GpuBuildIn const &in, GpuBuildOut &out, cudaStream_t st);

// The eight-wide collapse of a device-built SAH-pair tree (leaves of at most 15 triangles), on the
// device: the same nodes, byte for byte, as the host collapse (bvh_wide.cpp) of that tree. The
// triangle records are reordered in place. Uses the scratch of the build that made the tree.
struct GpuWideIn {
    float4 const *nlo, *nhi; // the binary tree
    float4 *tri;             // its triangle records; the wide order on success
    uint32_t num_tris;
    float max_abs;           // largest |coordinate| of the vertices and the camera
    uint32_t max_depth;      // levels the eight-wide stack allows
    void *scratch;           // gpu_build_scratch_bytes(num_tris) bytes
    void *host_pinned;       // 8 bytes of pinned host memory
    uint4 *wide;             // room for num_tris nodes of 96 bytes
};
struct GpuWideOut {
    uint32_t num_nodes = 0, max_depth = 0;
    uint32_t level_start[32] = {0}; // first node of every level (breadth first), then num_nodes
    bool ok = false; // false: deeper than max_depth (the binary tree stays)
};
cudaError_t gpu_collapse_wide(GpuWideIn const &in, GpuWideOut &out, cudaStream_t st);

} // namespace e8g
