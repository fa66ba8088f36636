// Builds a Cornell-style scene from corelib objects through the e8g adapters (e8g_corelib.h),
// packs it into an e8g_scene_desc, and checks that the oracle fed the packed description
// reproduces, bit for bit, the reference's own unidirect_lt1 and bidirect_mis radiance on the
// reference objects for the same per-path draw streams. Prints "OK <paths>" or "FAIL ...".
#include "adapter_scene.h"

extern "C" {
#include "e8_oracle.h"
}

#include <cstdio>
#include <cstring>

int main() {
    using namespace e8g_corelib;
    adapter_scene::room R;
    auto const &ps = R.ps;
    auto const &mc = R.mc;
    auto const &ls = R.ls;
    auto const &cam = R.cam;
    scene_storage st;
    pack_scene(ps, mc, ls, R.gpu_cam(), st);
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
