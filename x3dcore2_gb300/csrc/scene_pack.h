// Host-side packing of an e8g_scene_desc into the GPU layout (arrays uploaded as-is).
#pragma once

#include "../../include/e8g.h"
#include "bvh.h"
#include "bvh_wide.h"
#include "layout.h"

#include <cstdint>
#include <vector>

namespace e8g {

struct packed_scene {
    uint32_t nm = 0, nv = 0, nt = 0, nmat = 0, nl = 0;
    std::vector<float> vpos, vnrm;  // 4 floats per vertex
    std::vector<float> vtx;         // 8 floats per vertex: position, normal (the shading copy, DevScene::vtx)
    std::vector<uint32_t> tidx;     // 4 per triangle: global vertex indices, mesh
    std::vector<int32_t> mesh_mat;  // fail-safe remapped to nmat
    std::vector<int32_t> mesh_light;
    std::vector<uint32_t> mesh_toff;
    std::vector<uint32_t> mesh_voff; // num_meshes + 1 prefix offsets into the vertices
    std::vector<float> mesh_area;   // trimesh::update_face_cdf (geometry.cpp:105-118)
    std::vector<float> tri_cum;
    std::vector<DevMaterial> mats;  // nmat + 1
    std::vector<uint32_t> light_mesh;
    std::vector<float> light_rad;   // 4 per light
    std::vector<float> light_cum, light_pnorm;
    float total_power = 0;
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    DevCamera cam{};
    // BVH (after build). Layout 2 keeps the eight-wide nodes in `wide` and only the triangle
    // order and counts in `bvh`.
    flat_bvh bvh;
    std::vector<uint32_t> wide;
    std::vector<uint32_t> wide_levels; // first node of every level of `wide`, then its node count
    std::vector<float> tri;         // 12 floats per BVH position
    double build_ms = 0;
    uint32_t layout = 0;
};

// Fills everything but the BVH. Float arithmetic follows the reference (built with
// -ffp-contract=off) so light areas, powers and the light CDF are bit-identical to corelib's.
void pack_scene(e8g_scene_desc const &d, packed_scene &out);
// Area prefix sums of mesh m's triangles from s.vpos (trimesh::update_face_cdf, geometry.cpp:105-118).
void mesh_areas(packed_scene &s, uint32_t m);
// Light powers |pi * area * L| and their CDF in light order (basic_light_sources::commit,
// lightsources.cpp:45-52) from mesh_area and light_rad.
void light_table(packed_scene &s);
void pack_materials(e8g_material const *m, uint32_t n, std::vector<DevMaterial> &out);
void build_scene_bvh(packed_scene &s, bvh_build_opts const &o);
// The eight-wide layout from a binary SAH tree built elsewhere (the device builder), with the
// triangle records in its order; keeps the binary tree when the wide one would be too deep.
void collapse_scene_bvh(packed_scene &s, flat_bvh &&bin);
// ~(m ^ -1) of a row-major 4x4 matrix in the reference's float arithmetic (xform.cpp); false when
// |det m| <= 1e-5, the reference's "matrix not invertible".
bool reference_normal_matrix(float const m[16], float n_out[16]);

} // namespace e8g
