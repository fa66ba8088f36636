// Host-side scene container shared by the generators, the C ABI and the BVH builder.
#pragma once

#include "../../include/e8g.h"

#include <cstdint>
#include <vector>

struct e8g_host_scene {
    std::vector<uint32_t> voff{0};
    std::vector<uint32_t> toff{0};
    std::vector<int32_t> mesh_mat;
    std::vector<float> pos;
    std::vector<float> nrm;
    std::vector<uint32_t> tris;
    std::vector<e8g_material> mats;
    std::vector<e8g_light> lights;
    e8g_camera cam{};

    // Appends a mesh; returns its index. Vertex indices in `t` are mesh-local.
    uint32_t add_mesh(std::vector<float> const &p, std::vector<float> const &n,
                      std::vector<uint32_t> const &t, int32_t material) {
        pos.insert(pos.end(), p.begin(), p.end());
        nrm.insert(nrm.end(), n.begin(), n.end());
        tris.insert(tris.end(), t.begin(), t.end());
        voff.push_back(static_cast<uint32_t>(pos.size() / 3));
        toff.push_back(static_cast<uint32_t>(tris.size() / 3));
        mesh_mat.push_back(material);
        return static_cast<uint32_t>(mesh_mat.size() - 1);
    }

    e8g_scene_desc desc() const {
        e8g_scene_desc d{};
        d.num_meshes = static_cast<uint32_t>(mesh_mat.size());
        d.mesh_vert_offset = voff.data();
        d.mesh_tri_offset = toff.data();
        d.mesh_material = mesh_mat.data();
        d.positions = pos.data();
        d.normals = nrm.data();
        d.triangles = tris.data();
        d.num_materials = static_cast<uint32_t>(mats.size());
        d.materials = mats.data();
        d.num_lights = static_cast<uint32_t>(lights.size());
        d.lights = lights.data();
        d.camera = cam;
        return d;
    }
};

// Deterministic generators (SplitMix64-seeded), used by tests and benchmarks.
namespace e8g_gen {
e8g_host_scene *cornell(e8g_gen_opts const &o);
e8g_host_scene *displaced_icosphere(e8g_gen_opts const &o);
e8g_host_scene *soup(e8g_gen_opts const &o);
e8g_host_scene *furnace(e8g_gen_opts const &o);
} // namespace e8g_gen

// Validates a scene description (sizes, indices); returns a message or nullptr.
char const *e8g_validate_desc(e8g_scene_desc const *d);
