// Render orchestration: first hits, integrator dispatch, resolve, timing.
#include "api_internal.h"

#include <algorithm>

namespace e8g {

namespace {

e8g_status run_integrator(e8g_ctx *c, RenderArgs const &A, float4 *accum, float *path_rgb,
                          unsigned long long *d_counts) {
    cudaError_t e = cudaMemsetAsync(c->b_work.ptr, 0, 64, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "work counter");
    auto *work = static_cast<unsigned long long *>(c->b_work.ptr);
    auto const *fh = static_cast<FirstHit const *>(c->b_fh.ptr);
    if (A.mode == E8G_MODE_REF_BDPT) {
        launch_bdpt(c->dev, A, fh, accum, path_rgb, work, persistent_grid(c, bdpt_blocks_per_sm()), c->stream);
    } else {
        int grid = persistent_grid(c, megakernel_blocks_per_sm());
        launch_megakernel(c->dev, A, fh, accum, path_rgb, work, d_counts, grid, c->stream);
    }
    c->launches++;
    return E8G_OK;
}

} // namespace

e8g_status render_image(e8g_ctx *c, e8g_render_params const *p, float *d_rgba, unsigned long long *counts) {
    if (p->mode == E8G_MODE_BDPT_POWER)
        return fail(c, E8G_ERR_UNSUPPORTED, "power-heuristic BDPT is not available yet");
    if (counts && p->mode == E8G_MODE_REF_BDPT)
        return fail(c, E8G_ERR_UNSUPPORTED, "traversal counters cover the unidirectional integrators");
    c->launches = 0;
    size_t npix = static_cast<size_t>(p->width) * p->height;
    cudaError_t e = c->b_accum.reserve(npix * sizeof(float4));
    if (e == cudaSuccess && counts)
        e = c->b_counts.reserve(64);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "render buffers");
    unsigned long long *d_counts = counts ? static_cast<unsigned long long *>(c->b_counts.ptr) : nullptr;
    cudaEventRecord(c->ev0, c->stream);
    e8g_status s = first_hits(c, p->width, p->height);
    if (s != E8G_OK)
        return s;
    e = cudaMemsetAsync(c->b_accum.ptr, 0, npix * sizeof(float4), c->stream);
    if (e == cudaSuccess && d_counts)
        e = cudaMemsetAsync(d_counts, 0, 64, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "render clear");
    RenderArgs A = make_args(p);
    cudaEventRecord(c->ev2, c->stream);
    s = run_integrator(c, A, static_cast<float4 *>(c->b_accum.ptr), nullptr, d_counts);
    if (s != E8G_OK)
        return s;
    cudaEventRecord(c->ev3, c->stream);
    launch_resolve(static_cast<float4 const *>(c->b_accum.ptr), static_cast<uint32_t>(npix),
                   p->spp ? 1.0f / static_cast<float>(p->spp) : 0.0f, d_rgba, c->stream);
    c->launches++;
    cudaEventRecord(c->ev1, c->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(c, e, "render launch");
    if (counts) {
        e = cudaMemcpyAsync(counts, d_counts, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "counter readback");
    }
    e = cudaEventSynchronize(c->ev1);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "render");
    float ms = 0, kms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    cudaEventElapsedTime(&kms, c->ev2, c->ev3);
    c->stats.ms = ms;
    c->stats.kernel_ms = kms;
    c->stats.paths = npix * p->spp;
    c->stats.launches = c->launches;
    c->stats.counted = 0;
    return E8G_OK;
}

e8g_status render_list(e8g_ctx *c, e8g_render_params const *p, uint32_t const *d_pixel, uint32_t const *d_sample,
                       uint32_t n, float *d_rgb) {
    if (p->mode == E8G_MODE_BDPT_POWER)
        return fail(c, E8G_ERR_UNSUPPORTED, "power-heuristic BDPT is not available yet");
    c->launches = 0;
    e8g_status s = first_hits(c, p->width, p->height);
    if (s != E8G_OK)
        return s;
    RenderArgs A = make_args(p);
    A.list_pixel = d_pixel;
    A.list_sample = d_sample;
    A.total_paths = n;
    s = run_integrator(c, A, nullptr, d_rgb, nullptr);
    if (s != E8G_OK)
        return s;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "render_paths launch");
}

} // namespace e8g

extern "C" {

e8g_status e8g_forward(e8g_ctx *c, e8g_render_params const *, float *) {
    return e8g::fail(c, E8G_ERR_UNSUPPORTED, "adjoint not available yet");
}
e8g_status e8g_backward(e8g_ctx *c, float const *, float *, float *) {
    return e8g::fail(c, E8G_ERR_UNSUPPORTED, "adjoint not available yet");
}
e8g_status e8g_set_materials(e8g_ctx *c, e8g_material const *, uint32_t) {
    return e8g::fail(c, E8G_ERR_UNSUPPORTED, "not available yet");
}
e8g_status e8g_batch_render(e8g_ctx *c, e8g_batch_item const *, uint32_t, e8g_render_stats *) {
    return e8g::fail(c, E8G_ERR_UNSUPPORTED, "batched rendering not available yet");
}

} // extern "C"
