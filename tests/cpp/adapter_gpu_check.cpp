// Runs the reference-side adapters' GPU paths on a scene built from corelib objects
// (adapter_scene.h):
//  1. gpu_image_renderer::render (the stand-in for pt_image_renderer::render, renderer.h:57-59)
//     with unidirect_lt1 and bidirect_mis into a corelib compositor: equal to e8g_render of the
//     packed scene with the same parameters, and to the oracle's image of the same streams;
//  2. a second frame after the sphere moved (the adapter uploads the changed mesh and refits):
//     equal to the oracle's image of the moved scene;
//  3. gpu_path_tracer::sample (if_path_tracer::sample, pathtracer.h:59-63) on a batch of camera
//     rays: each path equal to the oracle's path fed the same stream, and, where the reference was
//     compiled for x86-64, to the reference's own tracer fed that stream. The reference's paths
//     depend on the machine it was compiled for: its AArch64 build agrees with neither the oracle
//     nor the GPU on most paths while its x86-64 build agrees with both bit for bit (it passes two
//     draws to one call in several places, e.g. vec3_cos_hemisphere_sample(n, rng.draw(),
//     rng.draw()), an evaluation order C++ leaves to the compiler — the likely cause). The GPU and
//     the oracle follow the x86-64 build, to which the oracle is pinned.
// Prints "OK ..." or "FAIL ..." and returns nonzero on failure.
#include "adapter_scene.h"

extern "C" {
#include "e8_oracle.h"
}

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

struct mem_compositor : public e8::if_compositor {
    mem_compositor(unsigned w, unsigned h) : e8::if_compositor(w, h) {}
    void commit(e8::if_frame *) const override {}
};

bool close(float a, float b, float rtol) { return std::fabs(a - b) <= std::fmax(rtol * std::fabs(b), 1e-6f); }

// Fraction of pixels whose three channels agree.
double agree(mem_compositor const &c, std::vector<float> const &ref, float rtol) {
    unsigned w = c.width(), h = c.height(), ok = 0;
    for (unsigned j = 0; j < h; j++)
        for (unsigned i = 0; i < w; i++) {
            e8::rgba_color px = c(i, j);
            float const *r = &ref[4 * (j * w + i)];
            ok += close(px(0), r[0], rtol) && close(px(1), r[1], rtol) && close(px(2), r[2], rtol);
        }
    return static_cast<double>(ok) / (w * h);
}

} // namespace

int main() {
    using namespace e8g_corelib;
    adapter_scene::room R;
    unsigned const w = 48, h = 40, spp = 8;
    int failures = 0;
    struct tracer_case {
        e8::pathtracer_factory::pt_type type;
        uint32_t mode;
        char const *name;
    } cases[] = {{e8::pathtracer_factory::unidirect_lt1, E8G_MODE_REF_LT1, "unidirect_lt1"},
                 {e8::pathtracer_factory::bidirect_mis, E8G_MODE_REF_BDPT, "bidirect_mis"}};
    for (auto const &tc : cases) {
        gpu_image_renderer renderer(tc.type, 0);
        mem_compositor comp(w, h);
        auto st = renderer.render(&comp, R.ps, R.mc, R.ls, *R.cam, spp, false);
        if (st.num_samples != spp) {
            std::printf("FAIL %s: num_samples %u\n", tc.name, st.num_samples);
            return 1;
        }
        // the same render through the C ABI on another context, and the oracle
        scene_storage ss;
        pack_scene(R.ps, R.mc, R.ls, R.gpu_cam(), ss);
        e8g_ctx *ctx = nullptr;
        e8g_device_opts o{0, 0};
        e8g_bvh_opts bo;
        e8g_default_bvh_opts(&bo);
        if (e8g_create(&ctx, &o) != E8G_OK || e8g_scene_upload(ctx, &ss.desc) != E8G_OK ||
            e8g_scene_build_bvh(ctx, &bo) != E8G_OK) {
            std::printf("FAIL %s: context\n", tc.name);
            return 1;
        }
        e8g_render_params p;
        e8g_default_params(&p, tc.mode, w, h, spp);
        p.seed = 1361; // the adapter's first frame
        std::vector<float> direct(4 * w * h);
        if (e8g_render(ctx, &p, direct.data()) != E8G_OK) {
            std::printf("FAIL %s: e8g_render %s\n", tc.name, e8g_last_error(ctx));
            return 1;
        }
        o_scene *os = o_scene_create(&ss.desc);
        o_policy pol{0, 2, 0.5f, 8};
        std::vector<float> oracle(4 * w * h);
        o_render(os, tc.mode, E8G_RNG_MINSTD, 1361, &pol, w, h, spp, 0, 0, 0, w, h, oracle.data(), 4);
        double same_abi = agree(comp, direct, 1e-5f), same_oracle = agree(comp, oracle, 1e-4f);
        std::printf("%s frame 1: adapter = C ABI on %.4f of pixels, = oracle on %.4f\n", tc.name, same_abi,
                    same_oracle);
        if (same_abi < 0.999 || same_oracle < 0.995)
            failures++;

        // frame 2: the sphere moves (new vertices, same topology): the adapter uploads that mesh and
        // refits; its seed is the next frame's
        std::vector<e8util::vec3> moved = R.sphere->vertices();
        for (auto &v : moved)
            v = v + e8util::vec3{0.07f, 0.02f, -0.05f};
        std::vector<e8util::vec3> keep = R.sphere->vertices();
        R.sphere->vertices(moved);
        R.sphere->update();
        R.ps.unload(*R.sphere);
        R.ps.load(*R.sphere, e8util::mat44_scale(1.0f));
        R.ps.commit();
        mem_compositor comp2(w, h);
        renderer.render(&comp2, R.ps, R.mc, R.ls, *R.cam, spp, false);
        scene_storage ss2;
        pack_scene(R.ps, R.mc, R.ls, R.gpu_cam(), ss2);
        o_scene *os2 = o_scene_create(&ss2.desc);
        o_render(os2, tc.mode, E8G_RNG_MINSTD, 1362, &pol, w, h, spp, 0, 0, 0, w, h, oracle.data(), 4);
        double same2 = agree(comp2, oracle, 1e-4f);
        std::printf("%s frame 2 (sphere moved): adapter = oracle on %.4f of pixels\n", tc.name, same2);
        if (same2 < 0.995)
            failures++;
        o_scene_free(os2);
        R.sphere->vertices(keep);
        R.sphere->update();
        R.ps.unload(*R.sphere);
        R.ps.load(*R.sphere, e8util::mat44_scale(1.0f));
        R.ps.commit();

        // gpu_path_tracer::sample on camera rays of every fifth pixel, against the reference's own
        // tracer fed each path's stream (e8g_path_seed of the seed the adapter draws, the ray, 0)
        gpu_path_tracer gt(ctx, tc.type);
        e8util::rng cam_rng(1);
        std::vector<e8util::ray> rays;
        for (unsigned k = 0; k < w * h; k += 5) {
            float pdf;
            rays.push_back(R.cam->sample(cam_rng, k % w, k / w, w, h, pdf));
        }
        e8::if_path_tracer::first_hits none(0);
        e8util::rng rng(77), shadow(77);
        std::vector<e8util::vec3> got = gt.sample(rng, rays, none, R.ps, R.mc, R.ls);
        uint64_t seed = static_cast<uint64_t>(shadow.draw() * 4294967296.0);
        std::unique_ptr<e8::if_path_tracer> ref_tracer(e8::pathtracer_factory(tc.type, e8::pathtracer_factory::options()).create());
        unsigned ok_ref = 0, ok_oracle = 0, shown = 0;
        for (size_t i = 0; i < rays.size(); i++) {
            std::vector<e8util::ray> one{rays[i]};
            auto hits = e8::if_path_tracer::compute_first_hit(one, R.ps, R.ls);
            uint32_t ps = e8g_path_seed(seed, static_cast<uint32_t>(i), 0);
            e8util::rng pr(ps);
            e8util::vec3 r = ref_tracer->sample(pr, one, hits, R.ps, R.mc, R.ls)[0];
            // the oracle's path of the same stream starts at the camera ray of pixel 5 i, which the
            // oracle's camera reproduces within a few ulp of the reference's ray
            uint32_t px = static_cast<uint32_t>(5 * i);
            float orc[3];
            o_render_paths(os, tc.mode, E8G_RNG_MINSTD, 0, &pol, w, h, &px, &ps, 1, orc, 1);
            bool same_ref = close(got[i](0), r(0), 1e-4f) && close(got[i](1), r(1), 1e-4f) &&
                            close(got[i](2), r(2), 1e-4f);
            bool same_oracle = close(got[i](0), orc[0], 1e-4f) && close(got[i](1), orc[1], 1e-4f) &&
                               close(got[i](2), orc[2], 1e-4f);
            ok_ref += same_ref;
            ok_oracle += same_oracle;
            if (!same_oracle && shown++ < 4)
                std::printf("  path %zu (pixel %u, seed %u): reference %g %g %g, gpu %g %g %g, oracle %g %g %g\n", i, px,
                            ps, r(0), r(1), r(2), got[i](0), got[i](1), got[i](2), orc[0], orc[1], orc[2]);
        }
        double frac_ref = static_cast<double>(ok_ref) / rays.size();
        double frac_oracle = static_cast<double>(ok_oracle) / rays.size();
        std::printf("%s gpu_path_tracer::sample = oracle on %.4f of %zu paths, = this machine's compiled reference "
                    "sample() on %.4f\n",
                    tc.name, frac_oracle, rays.size(), frac_ref);
        if (frac_oracle < 0.995)
            failures++;
#if defined(__x86_64__)
        if (frac_ref < 0.995)
            failures++;
#endif
        o_scene_free(os);
        e8g_destroy(ctx);
    }
    if (failures) {
        std::printf("FAIL %d checks\n", failures);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
