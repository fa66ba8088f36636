// Builds a Cornell-style scene from corelib objects through the e8g adapters (e8g_corelib.h),
// packs it into an e8g_scene_desc, and checks that the oracle fed the packed description
// reproduces, bit for bit, the reference's own unidirect_lt1 and bidirect_mis radiance on the
// reference objects for the same per-path draw streams. Prints "OK <paths>" or "FAIL ...".
#include "e8g_corelib.h"

extern "C" {
#include "e8_oracle.h"
}

#include <cstdio>
#include <cstring>

using e8util::vec3;

static std::shared_ptr<e8::trimesh> quad(char const *name, vec3 a, vec3 b, vec3 c, vec3 d, vec3 n) {
    auto m = std::make_shared<e8::trimesh>(name);
    m->vertices({a, b, c, d});
    m->normals({n, n, n, n});
    m->triangles({e8::triangle{0, 1, 2}, e8::triangle{0, 2, 3}});
    m->update();
    return m;
}

int main() {
    using namespace e8g_corelib;
    e8util::mat44 I = e8util::mat44_scale(1.0f);
    auto white = std::make_shared<gpu_oren_nayar>("white", vec3{0.73f, 0.73f, 0.73f}, 0.0f);
    auto red = std::make_shared<gpu_oren_nayar>("red", vec3{0.63f, 0.065f, 0.05f}, 0.0f);
    auto metal = std::make_shared<gpu_cook_torr>("metal", vec3{0.9f, 0.8f, 0.6f}, 0.3f, std::complex<float>(2.5f, 0.5f));
    auto black = std::make_shared<gpu_oren_nayar>("black", vec3{0.0f, 0.0f, 0.0f}, 0.0f);
    gpu_material_container mc;
    for (auto const &m : {std::static_pointer_cast<e8::if_material>(white), std::static_pointer_cast<e8::if_material>(red),
                          std::static_pointer_cast<e8::if_material>(metal), std::static_pointer_cast<e8::if_material>(black)})
        mc.load(*m, I);
    mc.commit();
    auto floor = quad("floor", {0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0});
    auto ceil = quad("ceiling", {0, 1, 0}, {0, 1, 1}, {1, 1, 1}, {1, 1, 0}, {0, -1, 0});
    auto back = quad("back", {0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 1});
    auto left = quad("left", {0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 0, 0});
    auto right = quad("right", {1, 0, 0}, {1, 1, 0}, {1, 1, 1}, {1, 0, 1}, {-1, 0, 0});
    auto sphere = std::make_shared<e8::uv_sphere>("ball", vec3{0.5f, 0.25f, 0.5f}, 0.2f, 12);
    sphere->update();
    auto lamp = quad("lamp", {0.4f, 0.999f, 0.4f}, {0.4f, 0.999f, 0.6f}, {0.6f, 0.999f, 0.6f}, {0.6f, 0.999f, 0.4f}, {0, -1, 0});
    floor->attach_material(white->id());
    ceil->attach_material(white->id());
    back->attach_material(metal->id());
    left->attach_material(red->id());
    sphere->attach_material(metal->id());
    lamp->attach_material(black->id());
    // right wall: no material -> fail-safe
    gpu_path_space_layout ps;
    for (auto const &g : {floor, ceil, back, left, right, std::static_pointer_cast<e8::trimesh>(sphere), lamp})
        ps.load(*g, I);
    ps.commit();
    auto light = std::make_shared<e8::area_light>("light", lamp, vec3{17.0f, 12.0f, 4.0f});
    gpu_light_sources ls;
    ls.load(*light, I);
    ls.commit();
    gpu_pinhole_camera cam0("cam", 0.7279404f, 1.0f, 1.25f);
    e8util::mat44 trans = e8util::mat44_translate({0.5f, 0.5f, 2.0f}) * e8util::mat44_rotate(0.1f, {0, 1, 0});
    std::unique_ptr<e8::if_camera> cam = cam0.transform(trans);

    scene_storage st;
    pack_scene(ps, mc, ls, dynamic_cast<gpu_pinhole_camera const &>(*cam), st);
    if (st.desc.num_meshes != 7 || st.desc.num_lights != 1 || st.desc.lights[0].mesh != 6 || st.mesh_mat[4] != -1) {
        std::printf("FAIL packing\n");
        return 1;
    }
    o_scene *os = o_scene_create(&st.desc);
    o_policy pol{0, 2, 0.5f, 8};
    unsigned const w = 40, h = 32;
    e8::unidirect_lt1_path_tracer lt1;
    e8::bidirect_mis_path_tracer bd;
    int fails = 0, n = 0;
    for (uint32_t k = 0; k < 400; k++) {
        uint32_t px = (k * 97u) % (w * h), seed = o_path_seed(21, px, k);
        e8util::rng cr(1);
        float pdf;
        std::vector<e8util::ray> rays{cam->sample(cr, px % w, px / w, w, h, pdf)};
        auto hits = e8::if_path_tracer::compute_first_hit(rays, ps, ls);
        for (int which = 0; which < 2; which++) {
            e8util::rng rng(seed);
            e8::if_path_tracer const &tr = which ? static_cast<e8::if_path_tracer const &>(bd) : lt1;
            e8util::vec3 ref = tr.sample(rng, rays, hits, ps, mc, ls)[0];
            float got[3];
            o_render_paths(os, which ? E8G_MODE_REF_BDPT : E8G_MODE_REF_LT1, E8G_RNG_MINSTD, 0, &pol, w, h, &px, &seed, 1,
                           got, 1);
            n++;
            for (int i = 0; i < 3; i++)
                if (std::memcmp(&got[i], &ref(i), 4) != 0) {
                    fails++;
                    break;
                }
        }
    }
    o_scene_free(os);
    if (fails) {
        std::printf("FAIL %d of %d paths differ\n", fails, n);
        return 1;
    }
    std::printf("OK %d\n", n);
    return 0;
}
