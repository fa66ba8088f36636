// A Cornell-style room built from corelib objects through the e8g adapters (e8g_corelib.h):
// Lambert and GGX materials, a uv_sphere, a wall without a material (fail-safe), one area light
// and a transformed pinhole camera. Shared by the adapter checks.
#pragma once

#include "e8g_corelib.h"

#include <memory>

namespace adapter_scene {

using e8util::vec3;

inline std::shared_ptr<e8::trimesh> quad(char const *name, vec3 a, vec3 b, vec3 c, vec3 d, vec3 n) {
    auto m = std::make_shared<e8::trimesh>(name);
    m->vertices({a, b, c, d});
    m->normals({n, n, n, n});
    m->triangles({e8::triangle{0, 1, 2}, e8::triangle{0, 2, 3}});
    m->update();
    return m;
}

struct room {
    std::shared_ptr<e8g_corelib::gpu_oren_nayar> white, red, black;
    std::shared_ptr<e8g_corelib::gpu_cook_torr> metal;
    std::shared_ptr<e8::trimesh> floor, ceil, back, left, right, lamp;
    std::shared_ptr<e8::uv_sphere> sphere;
    std::shared_ptr<e8::area_light> light;
    e8g_corelib::gpu_material_container mc;
    e8g_corelib::gpu_path_space_layout ps;
    e8g_corelib::gpu_light_sources ls;
    std::unique_ptr<e8::if_camera> cam;

    room() {
        e8util::mat44 I = e8util::mat44_scale(1.0f);
        white = std::make_shared<e8g_corelib::gpu_oren_nayar>("white", vec3{0.73f, 0.73f, 0.73f}, 0.0f);
        red = std::make_shared<e8g_corelib::gpu_oren_nayar>("red", vec3{0.63f, 0.065f, 0.05f}, 0.0f);
        metal = std::make_shared<e8g_corelib::gpu_cook_torr>("metal", vec3{0.9f, 0.8f, 0.6f}, 0.3f,
                                                             std::complex<float>(2.5f, 0.5f));
        black = std::make_shared<e8g_corelib::gpu_oren_nayar>("black", vec3{0.0f, 0.0f, 0.0f}, 0.0f);
        mc.load(*white, I);
        mc.load(*red, I);
        mc.load(*metal, I);
        mc.load(*black, I);
        mc.commit();
        floor = quad("floor", {0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0});
        ceil = quad("ceiling", {0, 1, 0}, {0, 1, 1}, {1, 1, 1}, {1, 1, 0}, {0, -1, 0});
        back = quad("back", {0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 1});
        left = quad("left", {0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 0, 0});
        right = quad("right", {1, 0, 0}, {1, 1, 0}, {1, 1, 1}, {1, 0, 1}, {-1, 0, 0});
        sphere = std::make_shared<e8::uv_sphere>("ball", vec3{0.5f, 0.25f, 0.5f}, 0.2f, 12);
        sphere->update();
        lamp = quad("lamp", {0.4f, 0.999f, 0.4f}, {0.4f, 0.999f, 0.6f}, {0.6f, 0.999f, 0.6f}, {0.6f, 0.999f, 0.4f},
                    {0, -1, 0});
        floor->attach_material(white->id());
        ceil->attach_material(white->id());
        back->attach_material(metal->id());
        left->attach_material(red->id());
        sphere->attach_material(metal->id());
        lamp->attach_material(black->id());
        // the right wall has no material: the fail-safe one
        for (auto const &g : {floor, ceil, back, left, right, std::static_pointer_cast<e8::trimesh>(sphere), lamp})
            ps.load(*g, I);
        ps.commit();
        light = std::make_shared<e8::area_light>("light", lamp, vec3{17.0f, 12.0f, 4.0f});
        ls.load(*light, I);
        ls.commit();
        e8g_corelib::gpu_pinhole_camera cam0("cam", 0.7279404f, 1.0f, 1.25f);
        e8util::mat44 trans = e8util::mat44_translate({0.5f, 0.5f, 2.0f}) * e8util::mat44_rotate(0.1f, {0, 1, 0});
        cam = cam0.transform(trans);
    }

    e8g_corelib::gpu_pinhole_camera const &gpu_cam() const {
        return dynamic_cast<e8g_corelib::gpu_pinhole_camera const &>(*cam);
    }
};

} // namespace adapter_scene
