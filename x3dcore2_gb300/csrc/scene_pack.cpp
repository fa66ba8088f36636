#include "scene_pack.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

namespace e8g {
namespace {

inline float dot3(float const *a, float const *b) {
    float v = 0;
    v += a[0] * b[0];
    v += a[1] * b[1];
    v += a[2] * b[2];
    return v;
}

} // namespace

void pack_materials(e8g_material const *m, uint32_t n, std::vector<DevMaterial> &out) {
    out.assign(n + 1, DevMaterial{});
    for (uint32_t i = 0; i < n; i++) {
        DevMaterial &d = out[i];
        d.type = m[i].type;
        for (int k = 0; k < 3; k++)
            d.albedo[k] = m[i].albedo[k];
        if (m[i].type == E8G_MAT_OREN_NAYAR) { // oren_nayar ctor, material.cpp:108-116
            float sigma = m[i].roughness;
            float sigma2 = sigma * sigma;
            d.a = 1 - 0.5f * sigma2 / (sigma2 + 0.33f);
            d.b = 0.45f * sigma2 / (sigma2 + 0.09f);
        } else if (m[i].type == E8G_MAT_COOK_TORR) { // cook_torr ctor, material.cpp:171-176
            d.alpha2 = 2 * m[i].roughness * m[i].roughness;
            d.rough = m[i].roughness;
            d.ior_re = m[i].ior_re;
            d.ior_im = m[i].ior_im;
        } else if (m[i].type == E8G_MAT_MIXTURE) {
            d.mix0 = m[i].mix0;
            d.mix1 = m[i].mix1;
            d.ratio = m[i].ratio;
        } else { // mat_fail_safe, material.cpp:54-55
            d.type = E8G_MAT_FAIL_SAFE;
            d.albedo[0] = d.albedo[1] = d.albedo[2] = 0.8f;
        }
    }
    DevMaterial &fs = out[n];
    fs.type = E8G_MAT_FAIL_SAFE;
    fs.albedo[0] = fs.albedo[1] = fs.albedo[2] = 0.8f;
}

void mesh_areas(packed_scene &s, uint32_t m) {
    float cum = 0;
    for (uint32_t t = s.mesh_toff[m]; t < s.mesh_toff[m + 1]; t++) {
        float const *p0 = &s.vpos[4 * static_cast<size_t>(s.tidx[4 * static_cast<size_t>(t)])];
        float const *p1 = &s.vpos[4 * static_cast<size_t>(s.tidx[4 * static_cast<size_t>(t) + 1])];
        float const *p2 = &s.vpos[4 * static_cast<size_t>(s.tidx[4 * static_cast<size_t>(t) + 2])];
        float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
        float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        float a = 0.5f * std::sqrt(dot3(c, c));
        cum += a;
        s.tri_cum[t] = cum;
    }
    s.mesh_area[m] = cum;
}

void light_table(packed_scene &s) {
    s.total_power = 0;
    const float pi = static_cast<float>(M_PI);
    for (uint32_t l = 0; l < s.nl; l++) {
        float k = pi * s.mesh_area[s.light_mesh[l]]; // m_power = pi * area * rad (light.cpp:20)
        float pw[3];
        for (int c = 0; c < 3; c++)
            pw[c] = k * s.light_rad[4 * static_cast<size_t>(l) + c];
        s.light_pnorm[l] = std::sqrt(dot3(pw, pw));
        s.total_power += s.light_pnorm[l];
        s.light_cum[l] = s.total_power;
    }
}

void pack_scene(e8g_scene_desc const &d, packed_scene &s) {
    s.nm = d.num_meshes;
    s.nv = d.mesh_vert_offset[d.num_meshes];
    s.nt = d.mesh_tri_offset[d.num_meshes];
    s.nmat = d.num_materials;
    s.nl = d.num_lights;
    s.vpos.assign(4 * static_cast<size_t>(s.nv), 0.0f);
    s.vnrm.assign(4 * static_cast<size_t>(s.nv), 0.0f);
    for (uint32_t v = 0; v < s.nv; v++)
        for (int k = 0; k < 3; k++) {
            s.vpos[4 * static_cast<size_t>(v) + k] = d.positions[3 * static_cast<size_t>(v) + k];
            s.vnrm[4 * static_cast<size_t>(v) + k] = d.normals[3 * static_cast<size_t>(v) + k];
        }
    s.vtx.assign(8 * static_cast<size_t>(s.nv), 0.0f);
    for (uint32_t v = 0; v < s.nv; v++)
        for (int k = 0; k < 3; k++) {
            s.vtx[8 * static_cast<size_t>(v) + k] = d.positions[3 * static_cast<size_t>(v) + k];
            s.vtx[8 * static_cast<size_t>(v) + 3 + k] = d.normals[3 * static_cast<size_t>(v) + k];
        }
    s.tidx.assign(4 * static_cast<size_t>(s.nt), 0u);
    s.mesh_mat.resize(s.nm);
    s.mesh_light.assign(s.nm, -1);
    s.mesh_toff.assign(d.mesh_tri_offset, d.mesh_tri_offset + s.nm + 1);
    s.mesh_area.assign(s.nm, 0.0f);
    s.tri_cum.assign(s.nt, 0.0f);
    bool have_bound = false;
    s.mesh_voff.assign(d.mesh_vert_offset, d.mesh_vert_offset + s.nm + 1);
    for (uint32_t m = 0; m < s.nm; m++) {
        int32_t mi = d.mesh_material ? d.mesh_material[m] : -1;
        s.mesh_mat[m] = (mi < 0 || static_cast<uint32_t>(mi) >= s.nmat) ? static_cast<int32_t>(s.nmat) : mi;
        uint32_t vb = d.mesh_vert_offset[m];
        for (uint32_t t = d.mesh_tri_offset[m]; t < d.mesh_tri_offset[m + 1]; t++) {
            for (int k = 0; k < 3; k++)
                s.tidx[4 * static_cast<size_t>(t) + k] = vb + d.triangles[3 * static_cast<size_t>(t) + k];
            s.tidx[4 * static_cast<size_t>(t) + 3] = m;
        }
        mesh_areas(s, m);
        // trimesh::update_aabb + if_path_space::load (geometry.cpp:97-103, pathspace.cpp:17)
        for (uint32_t v = vb; v < d.mesh_vert_offset[m + 1]; v++) {
            for (int k = 0; k < 3; k++) {
                float x = d.positions[3 * static_cast<size_t>(v) + k];
                if (!have_bound) {
                    s.bmin[k] = s.bmax[k] = x;
                } else {
                    s.bmin[k] = x < s.bmin[k] ? x : s.bmin[k];
                    s.bmax[k] = s.bmax[k] < x ? x : s.bmax[k];
                }
            }
            have_bound = true;
        }
    }
    pack_materials(d.materials, s.nmat, s.mats);
    // lights: load() order decides the mesh lookup (first wins), commit() the CDF
    s.light_mesh.resize(s.nl);
    s.light_rad.assign(4 * static_cast<size_t>(s.nl), 0.0f);
    s.light_cum.resize(s.nl);
    s.light_pnorm.resize(s.nl);
    for (uint32_t l = 0; l < s.nl; l++) {
        uint32_t m = d.lights[l].mesh;
        s.light_mesh[l] = m;
        if (s.mesh_light[m] < 0)
            s.mesh_light[m] = static_cast<int32_t>(l);
        for (int c = 0; c < 3; c++)
            s.light_rad[4 * static_cast<size_t>(l) + c] = d.lights[l].radiance[c];
    }
    light_table(s);
    std::memcpy(s.cam.origin, d.camera.origin, sizeof(s.cam.origin));
    std::memcpy(s.cam.rot, d.camera.rot, sizeof(s.cam.rot));
    s.cam.sensor = d.camera.sensor_size;
    s.cam.focal = d.camera.focal_len;
    s.cam.aspect = d.camera.aspect;
}

namespace {

void scene_arrays(packed_scene const &s, std::vector<float> &p3, std::vector<uint32_t> &t3) {
    p3.resize(3 * static_cast<size_t>(s.nv));
    for (uint32_t v = 0; v < s.nv; v++)
        for (int k = 0; k < 3; k++)
            p3[3 * static_cast<size_t>(v) + k] = s.vpos[4 * static_cast<size_t>(v) + k];
    t3.resize(3 * static_cast<size_t>(s.nt));
    for (uint32_t t = 0; t < s.nt; t++)
        for (int k = 0; k < 3; k++)
            t3[3 * static_cast<size_t>(t) + k] = s.tidx[4 * static_cast<size_t>(t) + k];
}

// Keeps the binary SAH tree (layout 0) or collapses it to eight-wide nodes (layout 2, falling
// back to the binary tree when too deep), then writes the triangle records in tree order.
void finish_tree(packed_scene &s, flat_bvh &&bin, uint32_t layout, std::vector<float> const &p3,
                 std::vector<uint32_t> const &t3) {
    s.wide.clear();
    s.layout = 0;
    if (layout == 2) {
        // the grid of the quantized boxes is sized for coordinates up to the scene's and the
        // camera's largest magnitude
        float max_abs = 0.0f;
        for (float v : p3)
            max_abs = std::max(max_abs, std::fabs(v));
        for (int k = 0; k < 3; k++)
            max_abs = std::max(max_abs, std::fabs(s.cam.origin[k]));
        wide_bvh w = collapse_wide(bin, p3.data(), t3.data(), max_abs);
        if (w.ok) {
            s.bvh = flat_bvh{};
            s.bvh.num_nodes = w.num_nodes;
            s.bvh.num_leaves = w.num_leaves;
            s.bvh.max_depth = w.max_depth;
            s.bvh.eps = bin.eps;
            s.bvh.tri_order = std::move(w.tri_order);
            s.wide = std::move(w.nodes);
            s.wide_levels = std::move(w.level_start);
            s.layout = 2;
        } else { // deeper than the traversal stack: keep the binary tree
            s.bvh = std::move(bin);
        }
    } else {
        s.bvh = std::move(bin);
    }
}

void write_tri_records(packed_scene &s, std::vector<float> const &p3, std::vector<uint32_t> const &t3) {
    s.tri.assign(12 * static_cast<size_t>(s.nt), 0.0f);
    for (uint32_t k = 0; k < s.nt; k++) {
        uint32_t t = s.bvh.tri_order[k];
        float const *v0 = &p3[3 * static_cast<size_t>(t3[3 * static_cast<size_t>(t)])];
        float const *v1 = &p3[3 * static_cast<size_t>(t3[3 * static_cast<size_t>(t) + 1])];
        float const *v2 = &p3[3 * static_cast<size_t>(t3[3 * static_cast<size_t>(t) + 2])];
        float *dst = &s.tri[12 * static_cast<size_t>(k)];
        for (int c = 0; c < 3; c++) {
            dst[c] = v0[c];
            dst[4 + c] = v1[c] - v0[c]; // the reference's va = v1 - v0 (tensor.h:694)
            dst[8 + c] = v2[c] - v0[c]; // vb = v2 - v0 (tensor.h:695)
        }
        std::memcpy(&dst[3], &t, 4);
    }
}

} // namespace

void build_scene_bvh(packed_scene &s, bvh_build_opts const &o) {
    auto t0 = std::chrono::steady_clock::now();
    std::vector<float> p3;
    std::vector<uint32_t> t3;
    scene_arrays(s, p3, t3);
    if (o.layout == 1) {
        s.wide.clear();
        s.bvh = build_bvh_reference(p3.data(), t3.data(), s.nt);
        s.layout = 1;
    } else if (o.layout == 3) { // no tree: the records in global triangle order
        s.wide.clear();
        s.bvh = flat_bvh{};
        s.bvh.tri_order.resize(s.nt);
        for (uint32_t t = 0; t < s.nt; t++)
            s.bvh.tri_order[t] = t;
        s.layout = 3;
    } else {
        bvh_build_opts ob = o;
        ob.tri_cost = effective_tri_cost(o);
        finish_tree(s, build_bvh(p3.data(), t3.data(), s.nt, ob), o.layout, p3, t3);
    }
    write_tri_records(s, p3, t3);
    s.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void collapse_scene_bvh(packed_scene &s, flat_bvh &&bin) {
    std::vector<float> p3;
    std::vector<uint32_t> t3;
    scene_arrays(s, p3, t3);
    finish_tree(s, std::move(bin), 2, p3, t3);
    write_tri_records(s, p3, t3);
}

} // namespace e8g
