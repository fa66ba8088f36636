// Device-side scene updates: mesh transform and tree refit (refit.cu).
#pragma once

#include "device.cuh"

namespace e8g {

// Reduction words of a refit: [0..2] / [3..5] min / max over the triangles' vertices (order-
// preserving integer keys), [6..8] / [9..11] the same over all vertices, [12] largest |coordinate|.
constexpr int kRefitRedWords = 16;

struct RefitScratch {
    uint32_t *red;
    float4 *ex_lo, *ex_hi; // exact (not pushed-out) box of every node
    uint32_t *parent;      // parent node, 0xFFFFFFFF for the root
    uint32_t *counter;     // children finished, per node
    float4 *tlo, *thi;     // exact box of every triangle record
};

// trimesh::transform of the vertices [v_begin, v_end): m the matrix, n the normal matrix (both
// row-major); directions: normals as (n, 0) without the w divide.
struct XformArgs {
    float m[16], n[16];
    uint32_t v_begin, v_end, directions;
};

size_t refit_scratch_bytes(uint32_t num_nodes, uint32_t num_tris);
RefitScratch refit_carve(void *base, uint32_t num_nodes, uint32_t num_tris);
// Parent links of the current tree (once per build).
void launch_refit_parents(DevScene const &S, RefitScratch const &R, cudaStream_t st);
// Triangle records, scene and vertex boxes, then every node bottom-up. cam_abs: the camera
// origin's largest |coordinate| (the eight-wide grid's smallest step covers it).
// wide_levels: the eight-wide layout's level boundaries (num_levels + 1 entries, host memory).
void launch_refit(DevScene const &S, RefitScratch const &R, uint32_t nv, float cam_abs, int grid_cap,
                  uint32_t const *wide_levels, uint32_t num_levels, cudaStream_t st);
void launch_transform(float4 const *vpos0, float4 const *vnrm0, float4 *vpos, float4 *vnrm, XformArgs const &X,
                      cudaStream_t st);
// The interleaved shading copy of the vertices (DevScene::vtx, 2 float4 per vertex).
void launch_interleave(float4 const *vpos, float4 const *vnrm, uint32_t nv, float4 *vtx, cudaStream_t st);
// The vertex box and largest |coordinate| alone into red[6..12] (kRefitRedWords words).
void launch_vertex_bounds(float4 const *vpos, uint32_t nv, uint32_t *red, int grid_cap, cudaStream_t st);
// The vertex box of a finished refit from its reduction words (copied to the host).
void refit_read_bounds(uint32_t const *red_host, float bmin[3], float bmax[3]);

} // namespace e8g
