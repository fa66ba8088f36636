// Context and helpers shared by the C ABI translation units.
#pragma once

#include "../../include/e8g.h"
#include "host_scene.h"
#include "launch.h"
#include "refit.h"
#include "scene_pack.h"

#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <string>
#include <vector>

namespace e8g {

// Device memory a context may hold (e8g_set_memory_limit): cap 0 = no limit.
struct mem_budget {
    size_t cap = 0;
    size_t used = 0;
};

struct dev_buffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    mem_budget *budget = nullptr;
    // Grows the buffer to n bytes (contents not kept). A request beyond the context's memory
    // limit fails with cudaErrorMemoryAllocation before anything is freed; a failed cudaMalloc
    // leaves the buffer empty.
    cudaError_t reserve(size_t n);
    void release();
};

// An NVTX range for the lifetime of the object (named phases in Nsight timelines; no cost
// without a tool attached).
struct nvtx_range {
    explicit nvtx_range(char const *name) { nvtxRangePushA(name); }
    ~nvtx_range() { nvtxRangePop(); }
    nvtx_range(nvtx_range const &) = delete;
    nvtx_range &operator=(nvtx_range const &) = delete;
};

} // namespace e8g

struct e8g_ctx {
    int device = 0;
    int num_sms = 1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    std::string err;
    bool uploaded = false, built = false;
    e8g::packed_scene pack;
    std::vector<e8g_material> materials;
    e8g::DevScene dev{};
    e8g_bvh_stats bvh_stats{};
    e8g_render_stats stats{};
    uint32_t launches = 0;
    // scene
    e8g::dev_buffer b_nlo, b_nhi, b_wide, b_tri, b_tidx, b_vpos, b_vnrm, b_vtx, b_mesh_mat, b_mesh_light, b_mesh_toff, b_mesh_area,
        b_tri_cum, b_mats, b_light_mesh, b_light_rad, b_light_cum, b_light_pnorm;
    // render scratch
    e8g::dev_buffer b_fh, b_accum, b_work, b_img, b_io0, b_io1, b_counts;
    // wavefront queues and adjoint state
    e8g::dev_buffer b_wf, b_grad, b_ff, b_batch; // b_ff: firefly per-sample images; b_batch: staged batch scenes
    e8g::dev_buffer b_bdw; // subpaths and connection lists of the split bidirectional form
    e8g_render_params fwd_params{};
    bool have_forward = false;
    // wavefront configuration (autotuned per context) and a pinned word for its termination test
    uint32_t wf_capacity = 1u << 21, wf_bounces = 4, wf_threshold = 16, wf_shade_variant = 0;
    // concurrent wavefront: two slot pools on two streams, one shading while the other traces
    bool wf_concurrent = false;
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    // per-kernel timing of the wavefront (e8g_set_kernel_timing): three events per bounce of the
    // graph (bounce start, shading done, trace done) and the sums over the current render
    bool kernel_timing = false;
    std::vector<cudaEvent_t> kt_events;
    double kt_trace_ms = 0, kt_shade_ms = 0;
    uint32_t kt_trace_launches = 0;
    // device memory limit of the context's buffers, and the cancellation request (e8g_cancel)
    e8g::mem_budget budget;
    std::atomic<bool> cancel{false};
    void *host_pinned = nullptr;
    // progressive rendering: samples in the accumulator, and the image they belong to
    uint64_t prog_spp = 0;
    uint32_t prog_w = 0, prog_h = 0;
    // incremental updates: the build options of the last build, meshes changed since the last
    // commit (dirty), host vertex copies behind the device's (host_stale: after device transforms),
    // parent links of the current tree computed (refit_ready), the blueprint vertices transforms
    // start from (b_vpos0 / b_vnrm0, made at the first transform), and the largest |coordinate|
    // the eight-wide grid was sized for
    e8g::bvh_build_opts bvh_opts{};
    bool dirty = false, host_stale = false, refit_ready = false;
    float tree_max_abs = 0;
    e8g::dev_buffer b_refit, b_vpos0, b_vnrm0, b_gbuild; // b_gbuild: device builder scratch
    // the render pipeline: its float frame and the settings of its last frame
    e8g::dev_buffer b_pipe;
    // the check word of the bounds-checked debug build (E8G_CHECKS; empty otherwise)
    e8g::dev_buffer b_check;
    e8g_pipeline_config pipe_cfg{};
    bool pipe_valid = false;

    std::vector<e8g::dev_buffer *> all_buffers() {
        return {&b_nlo, &b_nhi, &b_wide, &b_tri, &b_tidx, &b_vpos, &b_vnrm, &b_vtx, &b_mesh_mat, &b_mesh_light, &b_mesh_toff,
                &b_mesh_area, &b_tri_cum, &b_mats, &b_light_mesh, &b_light_rad, &b_light_cum, &b_light_pnorm,
                &b_fh, &b_accum, &b_work, &b_img, &b_io0, &b_io1, &b_counts, &b_wf, &b_grad, &b_ff, &b_batch,
                &b_refit, &b_vpos0, &b_vnrm0, &b_gbuild, &b_pipe, &b_check, &b_bdw};
    }
};

namespace e8g {

e8g_status fail(e8g_ctx *ctx, e8g_status st, std::string const &msg);
e8g_status cuda_fail(e8g_ctx *ctx, cudaError_t e, char const *what);
e8g_status check_ready(e8g_ctx *c);
// A pending e8g_cancel: waits for the context's stream, clears the request and returns true.
bool take_cancel(e8g_ctx *c);
// The bounds-checked debug build (E8G_CHECKS): waits for the stream, and when a device check
// failed since the last call returns E8G_ERR_INTERNAL naming it (and clears it). E8G_OK in every
// other build, without waiting.
e8g_status read_checks(e8g_ctx *c);
e8g_status validate_params(e8g_ctx *c, e8g_render_params const *p);
RenderArgs make_args(e8g_render_params const *p);
e8g_status first_hits(e8g_ctx *c, uint32_t w, uint32_t h);
int persistent_grid(e8g_ctx *c, int blocks_per_sm);
void fill_dev_scene(e8g_ctx *c);
// Builds the tree on the host with c->bvh_opts and uploads it (e8g_scene_build_bvh, commit rebuild).
e8g_status build_tree(e8g_ctx *c);
// Copies the device's vertices back into the host pack when device transforms left it behind.
e8g_status sync_host_vertices(e8g_ctx *c);

// Renders an image into d_rgba (device). counts (host, 3 values) requests the instrumented run.
e8g_status render_image(e8g_ctx *c, e8g_render_params const *p, float *d_rgba, unsigned long long *counts,
                        uint64_t prior_spp = 0);
// Wavefront integrator over the image or a path list (E8G_MODE_MIS).
e8g_status run_wavefront(e8g_ctx *c, RenderArgs const &A, float4 *accum, float *path_rgb, uint32_t capacity,
                         uint32_t bounces, uint32_t threshold, BatchDev const *B = nullptr,
                         FirstHit const *fh_all = nullptr);

// The same with two slot pools interleaving on two streams (e8g_wavefront_set_concurrent).
e8g_status run_wavefront_concurrent(e8g_ctx *c, RenderArgs const &A, float4 *accum, float *path_rgb, uint32_t capacity,
                                    uint32_t bounces, uint32_t threshold);

// Per-path radiance for device lists of pixels and samples into d_rgb (3 floats per path).
// first_hits_ready: the first-hit cache already holds path i's first hit at index list_pixel[i].
e8g_status render_list(e8g_ctx *c, e8g_render_params const *p, uint32_t const *d_pixel, uint32_t const *d_sample,
                       uint32_t n, float *d_rgb, bool first_hits_ready = false);

} // namespace e8g

extern "C" e8g_status e8g_count_traversal(e8g_ctx *c, e8g_render_params const *p, e8g_render_stats *out);
