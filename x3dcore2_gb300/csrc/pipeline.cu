// The render pipeline's frame and its flex_config-style settings (include/e8g.h, "pipeline"):
// pt_render_pipeline::render_frame (corelib/src/pipeline.cpp:73-101) and update_pipeline
// (:123-185) on one device: commit the scene's changes, render, composite, return 8-bit pixels.
#include "../../include/e8g.h"
#include "api_internal.h"

#include <cstdlib>
#include <cstring>
#include <string>

using namespace e8g;

namespace {

bool parse_bool(char const *v, uint32_t *out) {
    std::string s(v);
    if (s == "true" || s == "1") {
        *out = 1;
        return true;
    }
    if (s == "false" || s == "0") {
        *out = 0;
        return true;
    }
    return false;
}

bool parse_uint(char const *v, uint64_t *out) {
    if (!*v || *v == '-')
        return false;
    char *end = nullptr;
    unsigned long long x = std::strtoull(v, &end, 10);
    if (*end)
        return false;
    *out = x;
    return true;
}

bool same_config(e8g_pipeline_config const &a, e8g_pipeline_config const &b) {
    return a.mode == b.mode && a.layout == b.layout && a.samples_per_frame == b.samples_per_frame &&
           a.firefly_filter == b.firefly_filter && a.progressive == b.progressive && a.integrator == b.integrator &&
           a.seed == b.seed;
}

} // namespace

extern "C" {

void e8g_pipeline_config_default(e8g_pipeline_config *c) {
    if (!c)
        return;
    std::memset(c, 0, sizeof(*c));
    c->mode = E8G_MODE_REF_UNI; // "unidirectional"
    c->layout = E8G_BVH_SAH;    // "static_bvh"
    c->samples_per_frame = 64;
    c->firefly_filter = 0;
    c->auto_exposure = 0;
    c->exposure = 1.0f;
    c->num_threads = 0;
    c->progressive = 0;
    c->integrator = E8G_INTEGRATOR_MEGAKERNEL;
    c->seed = 1;
}

e8g_status e8g_pipeline_config_set(e8g_pipeline_config *c, char const *key, char const *value) {
    if (!c || !key || !value)
        return E8G_ERR_INVALID_ARG;
    std::string k(key), v(value);
    if (k == "path_tracer") {
        static const struct {
            char const *name;
            uint32_t mode;
        } names[] = {{"normal", E8G_MODE_NORMAL},
                     {"position", E8G_MODE_POSITION},
                     {"direct", E8G_MODE_REF_DIRECT},
                     {"unidirectional", E8G_MODE_REF_UNI},
                     {"unidirectional_lt1", E8G_MODE_REF_LT1},
                     {"bidirectional_lt2", E8G_MODE_REF_LT2},
                     {"bidirectional_mis", E8G_MODE_REF_BDPT},
                     {"mis", E8G_MODE_MIS},
                     {"bidirectional_power", E8G_MODE_BDPT_POWER}};
        for (auto const &n : names)
            if (v == n.name) {
                c->mode = n.mode;
                return E8G_OK;
            }
        return E8G_ERR_INVALID_ARG;
    }
    if (k == "path_space") {
        if (v == "static_bvh")
            c->layout = E8G_BVH_SAH;
        else if (v == "reference_bvh")
            c->layout = E8G_BVH_REFERENCE;
        else if (v == "wide_bvh")
            c->layout = E8G_BVH_WIDE;
        else if (v == "linear")
            c->layout = E8G_BVH_LINEAR;
        else
            return E8G_ERR_INVALID_ARG;
        return E8G_OK;
    }
    if (k == "light_sources")
        return v == "basic" ? E8G_OK : E8G_ERR_INVALID_ARG;
    if (k == "auto_exposure")
        return parse_bool(value, &c->auto_exposure) ? E8G_OK : E8G_ERR_INVALID_ARG;
    if (k == "firefly_filter")
        return parse_bool(value, &c->firefly_filter) ? E8G_OK : E8G_ERR_INVALID_ARG;
    if (k == "progressive")
        return parse_bool(value, &c->progressive) ? E8G_OK : E8G_ERR_INVALID_ARG;
    if (k == "exposure") {
        char *end = nullptr;
        float x = std::strtof(value, &end);
        if (end == value || *end)
            return E8G_ERR_INVALID_ARG;
        c->exposure = x;
        return E8G_OK;
    }
    uint64_t x = 0;
    if (k == "samples_per_frame") {
        if (!parse_uint(value, &x) || x == 0 || x > 0xFFFFFFFFull)
            return E8G_ERR_INVALID_ARG;
        c->samples_per_frame = static_cast<uint32_t>(x);
        return E8G_OK;
    }
    if (k == "num_threads") {
        if (!parse_uint(value, &x) || x > 4096)
            return E8G_ERR_INVALID_ARG;
        c->num_threads = static_cast<uint32_t>(x);
        return E8G_OK;
    }
    if (k == "super_samples")
        return parse_uint(value, &x) ? E8G_OK : E8G_ERR_INVALID_ARG;
    if (k == "seed") {
        if (!parse_uint(value, &x))
            return E8G_ERR_INVALID_ARG;
        c->seed = x;
        return E8G_OK;
    }
    if (k == "integrator") {
        if (v == "megakernel")
            c->integrator = E8G_INTEGRATOR_MEGAKERNEL;
        else if (v == "wavefront")
            c->integrator = E8G_INTEGRATOR_WAVEFRONT;
        else if (v == "plain")
            c->integrator = E8G_INTEGRATOR_PLAIN;
        else
            return E8G_ERR_INVALID_ARG;
        return E8G_OK;
    }
    return E8G_ERR_INVALID_ARG;
}

e8g_status e8g_pipeline_frame(e8g_ctx *c, e8g_pipeline_config const *cfg, uint32_t w, uint32_t h, uint8_t *pixels,
                              float *rgba_out) {
    if (!c || !cfg || !pixels || w == 0 || h == 0)
        return fail(c, E8G_ERR_INVALID_ARG, "bad pipeline arguments");
    if (!c->uploaded)
        return fail(c, E8G_ERR_NO_SCENE, "no scene uploaded");
    if (cfg->layout > E8G_BVH_LINEAR)
        return fail(c, E8G_ERR_INVALID_ARG, "unknown BVH layout");
    if (cfg->progressive && cfg->firefly_filter)
        return fail(c, E8G_ERR_UNSUPPORTED, "progressive frames do not run the firefly clamp");
    cudaSetDevice(c->device);
    e8g_status s = E8G_OK;
    // push_updates: a build when there is no tree or another layout was asked for, else a refit of
    // whatever changed
    if (!c->built || c->bvh_opts.layout != cfg->layout) {
        e8g_bvh_opts bo;
        e8g_default_bvh_opts(&bo);
        bo.layout = cfg->layout;
        bo.num_threads = cfg->num_threads;
        bo.builder = c->bvh_opts.builder;
        s = e8g_scene_build_bvh(c, &bo);
    } else if (c->dirty) {
        s = e8g_scene_commit(c, E8G_COMMIT_REFIT, nullptr);
    }
    if (s != E8G_OK)
        return s;
    e8g_render_params p;
    e8g_default_params(&p, cfg->mode, w, h, cfg->samples_per_frame);
    p.seed = cfg->seed;
    p.integrator = cfg->integrator;
    p.firefly = cfg->firefly_filter;
    s = validate_params(c, &p);
    if (s != E8G_OK)
        return s;
    size_t npix = static_cast<size_t>(w) * h;
    cudaError_t e = c->b_pipe.reserve(npix * 16);
    if (e == cudaSuccess)
        e = c->b_io1.reserve(npix * 4);
    if (e == cudaSuccess)
        e = c->b_counts.reserve(64);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "pipeline buffers");
    float *d_rgba = static_cast<float *>(c->b_pipe.ptr);
    if (cfg->progressive) {
        bool reset = !c->pipe_valid || !same_config(c->pipe_cfg, *cfg) || c->prog_spp == 0;
        s = e8g_render_progressive(c, &p, reset ? 1 : 0, d_rgba, nullptr);
    } else {
        s = render_image(c, &p, d_rgba, nullptr);
    }
    if (s != E8G_OK)
        return s;
    c->pipe_cfg = *cfg;
    c->pipe_valid = true;
    e8g_composite_params cp{E8G_TONEMAP_ACES, cfg->auto_exposure, cfg->exposure};
    e = launch_composite(d_rgba, w, h, cp, static_cast<uint8_t *>(c->b_io1.ptr), static_cast<double *>(c->b_counts.ptr),
                         c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(pixels, c->b_io1.ptr, npix * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && rgba_out)
        e = cudaMemcpyAsync(rgba_out, d_rgba, npix * 16, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "pipeline frame");
}

} // extern "C"
