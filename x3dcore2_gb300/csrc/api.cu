// C ABI of the path-tracing core (include/e8g.h). Host orchestration only: scene packing and
// the BVH build run on the host (scene_pack.cpp, bvh.cpp), everything per-ray runs in the CUDA
// kernels of trace.cu, mega.cu, bdpt.cu and wavefront.cu. No entry point throws.
#include "../../include/e8g.h"
#include "api_internal.h"
#include "bvh_boxes.h"
#include "gpu_build.h"

#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

using namespace e8g;

namespace e8g {

e8g_status fail(e8g_ctx *ctx, e8g_status st, std::string const &msg) {
    if (ctx)
        ctx->err = msg;
    return st;
}

e8g_status cuda_fail(e8g_ctx *ctx, cudaError_t e, char const *what) {
    if (e == cudaErrorMemoryAllocation) {
        size_t cap = ctx ? ctx->budget.cap : 0;
        return fail(ctx, E8G_ERR_OUT_OF_MEMORY,
                    std::string(what) + ": out of device memory" +
                        (cap ? " (context limit " + std::to_string(cap) + " bytes)" : std::string()));
    }
    return fail(ctx, E8G_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

e8g_status read_checks(e8g_ctx *c) {
#if defined(E8G_CHECKS)
    if (!c->b_check.ptr)
        return E8G_OK;
    unsigned long long w = 0;
    cudaError_t e = cudaMemcpyAsync(&w, c->b_check.ptr, 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "check word");
    if (w == 0)
        return E8G_OK;
    cudaMemsetAsync(c->b_check.ptr, 0, 8, c->stream);
    static char const *const names[] = {"?",          "node index",     "triangle index", "traversal stack",
                                        "vertex index", "mesh index",   "material index", "light index",
                                        "queue entry", "slot index"};
    uint32_t code = static_cast<uint32_t>(w >> 32), idx = static_cast<uint32_t>(w);
    return fail(c, E8G_ERR_INTERNAL,
                std::string("device bounds check failed: ") + (code < 10 ? names[code] : "?") + " " +
                    std::to_string(idx));
#else
    (void)c;
    return E8G_OK;
#endif
}

bool take_cancel(e8g_ctx *c) {
    if (!c->cancel.load(std::memory_order_acquire))
        return false;
    cudaStreamSynchronize(c->stream);
    c->cancel.store(false, std::memory_order_release);
    return true;
}

void dev_buffer::release() {
    if (ptr)
        cudaFree(ptr);
    if (budget)
        budget->used -= bytes;
    ptr = nullptr;
    bytes = 0;
}

cudaError_t dev_buffer::reserve(size_t n) {
    if (n <= bytes)
        return cudaSuccess;
    if (budget && budget->cap && budget->used - bytes + n > budget->cap)
        return cudaErrorMemoryAllocation;
    release();
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
        cudaGetLastError(); // not sticky: keep it out of later launch checks
        ptr = nullptr;
        return e;
    }
    bytes = n;
    if (budget)
        budget->used += n;
    return cudaSuccess;
}

template <class T> static cudaError_t upload(dev_buffer &b, std::vector<T> const &v, cudaStream_t st) {
    size_t n = std::max<size_t>(v.size() * sizeof(T), 16);
    cudaError_t e = b.reserve(n);
    if (e != cudaSuccess)
        return e;
    if (!v.empty())
        e = cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
    return e;
}

void fill_dev_scene(e8g_ctx *c) {
    DevScene &S = c->dev;
    packed_scene &p = c->pack;
    S.nlo = static_cast<float4 const *>(c->b_nlo.ptr);
    S.nhi = static_cast<float4 const *>(c->b_nhi.ptr);
    S.wnodes = static_cast<uint4 const *>(c->b_wide.ptr);
    S.tri = static_cast<float4 const *>(c->b_tri.ptr);
    S.tidx = static_cast<uint4 const *>(c->b_tidx.ptr);
    S.vpos = static_cast<float4 const *>(c->b_vpos.ptr);
    S.vnrm = static_cast<float4 const *>(c->b_vnrm.ptr);
    S.vtx = static_cast<float4 const *>(c->b_vtx.ptr);
    S.mesh_mat = static_cast<int32_t const *>(c->b_mesh_mat.ptr);
    S.mesh_light = static_cast<int32_t const *>(c->b_mesh_light.ptr);
    S.mesh_toff = static_cast<uint32_t const *>(c->b_mesh_toff.ptr);
    S.mesh_area = static_cast<float const *>(c->b_mesh_area.ptr);
    S.tri_cum = static_cast<float const *>(c->b_tri_cum.ptr);
    S.mats = static_cast<DevMaterial const *>(c->b_mats.ptr);
    S.light_mesh = static_cast<uint32_t const *>(c->b_light_mesh.ptr);
    S.light_rad = static_cast<float4 const *>(c->b_light_rad.ptr);
    S.light_cum = static_cast<float const *>(c->b_light_cum.ptr);
    S.light_pnorm = static_cast<float const *>(c->b_light_pnorm.ptr);
    S.nmat = p.nmat;
    S.nl = p.nl;
    S.nm = p.nm;
    S.nnodes = p.bvh.num_nodes;
    S.ntris = p.nt;
    S.nverts = p.nv;
    S.check = static_cast<unsigned long long *>(c->b_check.ptr);
    S.layout = p.layout;
    S.total_power = p.total_power;
    for (int k = 0; k < 3; k++) {
        S.bmin[k] = p.bmin[k];
        S.bmax[k] = p.bmax[k];
    }
    S.cam = p.cam;
}

e8g_status check_ready(e8g_ctx *c) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    if (!c->uploaded)
        return fail(c, E8G_ERR_NO_SCENE, "no scene uploaded");
    if (!c->built)
        return fail(c, E8G_ERR_NOT_BUILT, "BVH not built (call e8g_scene_build_bvh)");
    if (c->dirty)
        return fail(c, E8G_ERR_NOT_BUILT, "the scene changed since the last commit (call e8g_scene_commit)");
    return E8G_OK;
}

e8g_status validate_params(e8g_ctx *c, e8g_render_params const *p) {
    if (!p)
        return fail(c, E8G_ERR_INVALID_ARG, "params is NULL");
    if (p->width < 2 || p->height < 2)
        return fail(c, E8G_ERR_INVALID_ARG, "image must be at least 2x2 (pinhole_camera divides by w-1, h-1)");
    if (static_cast<uint64_t>(p->width) * p->height > (1ull << 28))
        return fail(c, E8G_ERR_INVALID_ARG, "image too large");
    if (p->mode > E8G_MODE_REF_LT2)
        return fail(c, E8G_ERR_INVALID_ARG, "unknown mode");
    if (p->rng > E8G_RNG_PHILOX)
        return fail(c, E8G_ERR_INVALID_ARG, "unknown rng");
    if (p->integrator > E8G_INTEGRATOR_PLAIN)
        return fail(c, E8G_ERR_INVALID_ARG, "unknown integrator");
    if (!(p->rr_prob > 0.0f) || p->rr_prob > 1.0f)
        return fail(c, E8G_ERR_INVALID_ARG, "rr_prob must be in (0, 1]");
    if (p->bdpt_max_len > 16)
        return fail(c, E8G_ERR_INVALID_ARG, "bdpt_max_len must be <= 16");
    if (p->max_depth > 256)
        return fail(c, E8G_ERR_INVALID_ARG, "max_depth must be <= 256");
    // Without a depth cap only Russian roulette ends a path in a closed scene: keep it effective.
    if (p->max_depth == 0 && (p->rr_prob > 0.95f || p->rr_start > 64))
        return fail(c, E8G_ERR_INVALID_ARG, "unbounded paths: set max_depth, or rr_prob <= 0.95 and rr_start <= 64");
    return E8G_OK;
}

RenderArgs make_args(e8g_render_params const *p) {
    RenderArgs A{};
    A.mode = p->mode;
    A.rng = p->rng;
    A.width = p->width;
    A.height = p->height;
    A.spp = p->spp;
    A.sample_offset = p->sample_offset;
    A.seed = p->seed;
    A.max_depth = p->max_depth;
    A.rr_start = p->rr_start;
    A.rr_prob = p->rr_prob;
    A.bdpt_max_len = p->bdpt_max_len;
    A.tiles_x = (p->width + 7) / 8;
    A.tiles_y = (p->height + 3) / 4;
    A.paths_per_sample = A.tiles_x * A.tiles_y * 32;
    A.total_paths = static_cast<uint64_t>(A.paths_per_sample) * p->spp;
    return A;
}

// First hits for the whole image (cached per render, like pt_image_renderer::render:121-122).
e8g_status first_hits(e8g_ctx *c, uint32_t w, uint32_t h) {
    size_t n = static_cast<size_t>(w) * h;
    cudaError_t e = c->b_fh.reserve(n * sizeof(FirstHit));
    if (e != cudaSuccess)
        return cuda_fail(c, e, "first-hit buffer");
    launch_first_hits(c->dev, w, h, static_cast<FirstHit *>(c->b_fh.ptr), c->stream);
    c->launches++;
    return E8G_OK;
}

int persistent_grid(e8g_ctx *c, int blocks_per_sm) { return c->num_sms * std::max(1, blocks_per_sm); }

} // namespace e8g

namespace e8g {

e8g_status sync_host_vertices(e8g_ctx *c) {
    if (!c->host_stale)
        return E8G_OK;
    packed_scene &p = c->pack;
    cudaError_t e = cudaMemcpyAsync(p.vpos.data(), c->b_vpos.ptr, p.vpos.size() * sizeof(float),
                                    cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p.vnrm.data(), c->b_vnrm.ptr, p.vnrm.size() * sizeof(float), cudaMemcpyDeviceToHost,
                            c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "vertex read-back");
    c->host_stale = false;
    return E8G_OK;
}

namespace {

// The device builder: the SAH-pair tree straight into the device buffers; the eight-wide layout
// collapses it on the host. *built is false when the tree came out too deep (or clustering made no
// progress): the caller then builds on the host.
e8g_status build_on_device(e8g_ctx *c, bool *built) {
    *built = false;
    packed_scene &p = c->pack;
    uint32_t nt = p.nt;
    bvh_build_opts const &o = c->bvh_opts;
    fill_dev_scene(c);
    cudaError_t e = c->b_nlo.reserve(32 * static_cast<size_t>(nt));
    if (e == cudaSuccess)
        e = c->b_nhi.reserve(32 * static_cast<size_t>(nt));
    if (e == cudaSuccess)
        e = c->b_tri.reserve(48 * static_cast<size_t>(nt));
    if (e == cudaSuccess)
        e = c->b_gbuild.reserve(gpu_build_scratch_bytes(nt));
    if (e != cudaSuccess)
        return cuda_fail(c, e, "device build buffers");
    GpuBuildIn in{};
    in.tidx = c->dev.tidx;
    in.vpos = c->dev.vpos;
    in.num_tris = nt;
    in.max_leaf = std::min<uint32_t>(o.max_leaf_prims, 15);
    in.tri_cost = effective_tri_cost(o);
    in.node_cost = o.node_cost;
    in.max_depth = kMaxTreeDepth;
    in.num_sms = c->num_sms;
    in.scratch = c->b_gbuild.ptr;
    in.host_pinned = c->host_pinned;
    in.nlo = static_cast<float4 *>(c->b_nlo.ptr);
    in.nhi = static_cast<float4 *>(c->b_nhi.ptr);
    in.tri = static_cast<float4 *>(c->b_tri.ptr);
    GpuBuildOut out;
    auto t0 = std::chrono::steady_clock::now();
    e = gpu_build_sah_pairs(in, out, c->stream);
    if (e == cudaErrorUnknown || (e == cudaSuccess && !out.ok))
        return E8G_OK; // too deep or no progress: the host builds
    if (e != cudaSuccess)
        return cuda_fail(c, e, "device build");
    flat_bvh bin;
    bin.num_nodes = out.num_nodes;
    bin.num_leaves = out.num_leaves;
    bin.max_depth = out.max_depth;
    bin.avg_leaf_depth = out.avg_leaf_depth;
    bin.eps = scene_eps(out.scene_lo, out.scene_hi);
    if (o.layout == E8G_BVH_WIDE) {
        // the eight-wide collapse on the device; its grid covers the vertices and the camera
        e = c->b_refit.reserve(std::max<size_t>(c->b_refit.bytes, 4 * kRefitRedWords));
        if (e == cudaSuccess)
            e = c->b_wide.reserve(96 * static_cast<size_t>(nt));
        if (e != cudaSuccess)
            return cuda_fail(c, e, "wide collapse buffers");
        uint32_t *red = static_cast<uint32_t *>(c->b_refit.ptr);
        launch_vertex_bounds(c->dev.vpos, p.nv, red, 8 * c->num_sms, c->stream);
        uint32_t words[kRefitRedWords];
        e = cudaMemcpyAsync(words, red, sizeof(words), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "vertex bounds");
        float max_abs;
        std::memcpy(&max_abs, &words[12], 4);
        for (int k = 0; k < 3; k++)
            max_abs = std::max(max_abs, std::fabs(p.cam.origin[k]));
        GpuWideIn wi{};
        wi.nlo = in.nlo;
        wi.nhi = in.nhi;
        wi.tri = in.tri;
        wi.num_tris = nt;
        wi.max_abs = max_abs;
        wi.max_depth = kWideMaxDepth;
        wi.scratch = in.scratch;
        wi.host_pinned = c->host_pinned;
        wi.wide = static_cast<uint4 *>(c->b_wide.ptr);
        GpuWideOut wo;
        e = gpu_collapse_wide(wi, wo, c->stream);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "device wide collapse");
        p.wide.clear();
        p.tri.clear();
        if (wo.ok) {
            p.wide_levels.assign(wo.level_start, wo.level_start + wo.max_depth + 1);
            p.bvh = flat_bvh{};
            p.bvh.num_nodes = wo.num_nodes;
            p.bvh.num_leaves = bin.num_leaves;
            p.bvh.max_depth = wo.max_depth;
            p.bvh.eps = bin.eps;
            p.layout = E8G_BVH_WIDE;
        } else { // too deep for the eight-wide stack: the binary tree stays
            p.bvh = std::move(bin);
            p.layout = E8G_BVH_SAH;
        }
    } else {
        p.wide.clear();
        p.tri.clear();
        p.bvh = std::move(bin);
        p.layout = E8G_BVH_SAH;
    }
    p.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    *built = true;
    return E8G_OK;
}

} // namespace

e8g_status build_tree(e8g_ctx *c) {
    nvtx_range range("e8g build tree");
    cudaSetDevice(c->device);
    c->built = false; // buffers are replaced below: no render until the build completes
    packed_scene &p = c->pack;
    bool on_device = false;
    if (c->bvh_opts.builder == E8G_BUILDER_DEVICE && c->bvh_opts.layout != E8G_BVH_REFERENCE &&
        c->bvh_opts.layout != E8G_BVH_LINEAR && p.nt > 0) {
        e8g_status st = build_on_device(c, &on_device);
        if (st != E8G_OK)
            return st;
    }
    if (!on_device) {
        e8g_status st = sync_host_vertices(c);
        if (st != E8G_OK)
            return st;
        try {
            build_scene_bvh(p, c->bvh_opts);
        } catch (std::bad_alloc const &) {
            return fail(c, E8G_ERR_OUT_OF_MEMORY, "host allocation failed while building the BVH");
        }
        if (p.layout == E8G_BVH_REFERENCE && p.bvh.max_depth > kMaxRefTreeDepth) {
            c->built = false;
            return fail(c, E8G_ERR_UNSUPPORTED, "reference BVH deeper than the traversal stack (63 levels)");
        }
        cudaError_t e = upload(c->b_nlo, p.bvh.lo, c->stream);
        if (e == cudaSuccess)
            e = upload(c->b_nhi, p.bvh.hi, c->stream);
        if (e == cudaSuccess)
            e = upload(c->b_wide, p.wide, c->stream);
        if (e == cudaSuccess)
            e = upload(c->b_tri, p.tri, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "BVH upload");
    }
    // the vertex box (if_path_space::aabb) and the largest coordinate follow the device's vertices
    cudaError_t e = c->b_refit.reserve(std::max<size_t>(c->b_refit.bytes, 4 * kRefitRedWords));
    if (e != cudaSuccess)
        return cuda_fail(c, e, "bounds scratch");
    e = c->b_vtx.reserve(std::max<size_t>(32 * static_cast<size_t>(p.nv), 32));
    if (e != cudaSuccess)
        return cuda_fail(c, e, "shading vertices");
    launch_interleave(static_cast<float4 const *>(c->b_vpos.ptr), static_cast<float4 const *>(c->b_vnrm.ptr), p.nv,
                      static_cast<float4 *>(c->b_vtx.ptr), c->stream);
    uint32_t *red = static_cast<uint32_t *>(c->b_refit.ptr);
    launch_vertex_bounds(static_cast<float4 const *>(c->b_vpos.ptr), p.nv, red, 8 * c->num_sms, c->stream);
    uint32_t words[kRefitRedWords];
    e = cudaMemcpyAsync(words, red, sizeof(words), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "vertex bounds");
    if (p.nv) {
        refit_read_bounds(words, p.bmin, p.bmax);
    }
    float max_abs;
    std::memcpy(&max_abs, &words[12], 4);
    for (int k = 0; k < 3; k++)
        max_abs = std::max(max_abs, std::fabs(p.cam.origin[k]));
    c->tree_max_abs = max_abs;
    c->bvh_stats.num_nodes = p.bvh.num_nodes;
    c->bvh_stats.num_leaves = p.bvh.num_leaves;
    c->bvh_stats.max_depth = p.bvh.max_depth;
    c->bvh_stats.num_tris = p.nt;
    c->bvh_stats.avg_leaf_depth = p.bvh.avg_leaf_depth;
    c->bvh_stats.build_ms = p.build_ms;
    c->bvh_stats.node_bytes = static_cast<uint64_t>(p.bvh.num_nodes) * (p.layout == 2 ? 4 * kWideWords : 32);
    c->bvh_stats.layout = p.layout;
    c->bvh_stats.tri_bytes = static_cast<uint64_t>(p.nt) * 48;
    c->built = true;
    c->dirty = false;
    c->refit_ready = false;
    c->prog_spp = 0;
    fill_dev_scene(c);
    return E8G_OK;
}

} // namespace e8g

extern "C" {

char const *e8g_version(void) { return "e8g 0.1 (sm_103a)"; }

char const *e8g_last_error(e8g_ctx const *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void e8g_default_bvh_opts(e8g_bvh_opts *o) {
    if (!o)
        return;
    o->max_leaf_prims = 8;
    o->num_bins = 32;
    o->tri_cost = 0.0f; // the layout's tuned value
    o->node_cost = 1.0f;
    o->num_threads = 0;
    o->layout = E8G_BVH_SAH;
    o->builder = E8G_BUILDER_HOST;
}

void e8g_default_params(e8g_render_params *p, uint32_t mode, uint32_t width, uint32_t height, uint32_t spp) {
    if (!p)
        return;
    std::memset(p, 0, sizeof(*p));
    p->mode = mode;
    p->integrator = E8G_INTEGRATOR_MEGAKERNEL;
    p->rng = (mode == E8G_MODE_MIS || mode == E8G_MODE_BDPT_POWER) ? E8G_RNG_PHILOX : E8G_RNG_MINSTD;
    p->width = width;
    p->height = height;
    p->spp = spp;
    p->seed = 1;
    p->max_depth = 0;
    p->rr_start = mode == E8G_MODE_REF_LT2 ? 1 : 2; // bidirect_lt2's mutate_depth (pathtracer.cpp:705)
    p->rr_prob = 0.5f;
    p->bdpt_max_len = 8;
}

uint32_t e8g_path_seed(uint64_t seed, uint32_t pixel, uint32_t sample) {
    return path_seed(splitmix64(seed), pixel, sample);
}

e8g_status e8g_create(e8g_ctx **out, e8g_device_opts const *opts) {
    if (!out)
        return E8G_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return E8G_ERR_NO_DEVICE;
    }
    int dev = opts ? opts->device : 0;
    if (dev < 0 || dev >= count)
        return E8G_ERR_INVALID_ARG;
    e8g_ctx *c = new (std::nothrow) e8g_ctx();
    if (!c)
        return E8G_ERR_OUT_OF_MEMORY;
    c->device = dev;
    for (dev_buffer *b : c->all_buffers())
        b->budget = &c->budget;
    cudaError_t e = cudaSetDevice(dev);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess)
        e = cudaEventCreate(&c->ev2);
    if (e == cudaSuccess)
        e = cudaEventCreate(&c->ev3);
    if (e == cudaSuccess)
        e = c->b_work.reserve(64);
    if (e == cudaSuccess)
        e = cudaMallocHost(&c->host_pinned, 64);
#if defined(E8G_CHECKS)
    if (e == cudaSuccess)
        e = c->b_check.reserve(8);
    if (e == cudaSuccess)
        e = cudaMemset(c->b_check.ptr, 0, 8);
#endif
    if (e != cudaSuccess) {
        delete c;
        return E8G_ERR_CUDA;
    }
    *out = c;
    return E8G_OK;
}

e8g_status e8g_destroy(e8g_ctx *c) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (dev_buffer *b : c->all_buffers())
        b->release();
    if (c->ev0)
        cudaEventDestroy(c->ev0);
    if (c->ev1)
        cudaEventDestroy(c->ev1);
    if (c->ev2)
        cudaEventDestroy(c->ev2);
    if (c->ev3)
        cudaEventDestroy(c->ev3);
    for (cudaEvent_t ev : c->kt_events)
        cudaEventDestroy(ev);
    if (c->ev_a)
        cudaEventDestroy(c->ev_a);
    if (c->ev_b)
        cudaEventDestroy(c->ev_b);
    if (c->stream2)
        cudaStreamDestroy(c->stream2);
    if (c->stream)
        cudaStreamDestroy(c->stream);
    if (c->host_pinned)
        cudaFreeHost(c->host_pinned);
    delete c;
    return E8G_OK;
}

e8g_status e8g_scene_upload(e8g_ctx *c, e8g_scene_desc const *d) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    char const *bad = e8g_validate_desc(d);
    if (bad)
        return fail(c, E8G_ERR_INVALID_ARG, bad);
    nvtx_range range("e8g_scene_upload");
    cudaSetDevice(c->device);
    // the previous scene is gone from here on: a failure below leaves no scene
    c->uploaded = c->built = false;
    try {
        c->pack = packed_scene();
        pack_scene(*d, c->pack);
        c->materials.assign(d->materials, d->materials + d->num_materials);
    } catch (std::bad_alloc const &) {
        return fail(c, E8G_ERR_OUT_OF_MEMORY, "host allocation failed while packing the scene");
    }
    packed_scene &p = c->pack;
    cudaError_t e = cudaSuccess;
#define UP(buf, vec)                                                                                                   \
    if (e == cudaSuccess)                                                                                              \
        e = upload(c->buf, p.vec, c->stream);
    UP(b_vpos, vpos)
    UP(b_vnrm, vnrm)
    UP(b_tidx, tidx)
    UP(b_mesh_mat, mesh_mat)
    UP(b_mesh_light, mesh_light)
    UP(b_mesh_toff, mesh_toff)
    UP(b_mesh_area, mesh_area)
    UP(b_tri_cum, tri_cum)
    UP(b_mats, mats)
    UP(b_light_mesh, light_mesh)
    UP(b_light_rad, light_rad)
    UP(b_light_cum, light_cum)
    UP(b_light_pnorm, light_pnorm)
#undef UP
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "scene upload");
    c->uploaded = true;
    c->built = false;
    c->dirty = false;
    c->host_stale = false;
    c->refit_ready = false;
    c->b_vpos0.release();
    c->b_vnrm0.release();
    c->prog_spp = 0;
    fill_dev_scene(c);
    return E8G_OK;
}

e8g_status e8g_scene_build_bvh(e8g_ctx *c, e8g_bvh_opts const *o) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    if (!c->uploaded)
        return fail(c, E8G_ERR_NO_SCENE, "no scene uploaded");
    bvh_build_opts bo;
    if (o) {
        if (o->max_leaf_prims == 0 || o->num_bins < 2 || o->num_bins > 64)
            return fail(c, E8G_ERR_INVALID_ARG, "bvh options out of range");
        bo.max_leaf_prims = o->max_leaf_prims;
        bo.num_bins = o->num_bins;
        bo.tri_cost = o->tri_cost;
        bo.node_cost = o->node_cost;
        bo.num_threads = o->num_threads;
        if (o->layout > E8G_BVH_LINEAR)
            return fail(c, E8G_ERR_INVALID_ARG, "unknown BVH layout");
        if (o->builder > E8G_BUILDER_DEVICE)
            return fail(c, E8G_ERR_INVALID_ARG, "unknown BVH builder");
        bo.layout = o->layout;
        bo.builder = o->builder;
    }
    c->bvh_opts = bo;
    return build_tree(c);
}

e8g_status e8g_bvh_read(e8g_ctx *c, void *nodes_out, void *tris_out) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    if (!c->built)
        return fail(c, E8G_ERR_NOT_BUILT, "BVH not built");
    cudaSetDevice(c->device);
    packed_scene const &p = c->pack;
    size_t nn = p.bvh.num_nodes;
    cudaError_t e = cudaSuccess;
    if (nodes_out && p.layout == E8G_BVH_WIDE) {
        e = cudaMemcpyAsync(nodes_out, c->b_wide.ptr, nn * 4 * kWideWords, cudaMemcpyDeviceToHost, c->stream);
    } else if (nodes_out && nn) {
        e = cudaMemcpyAsync(nodes_out, c->b_nlo.ptr, nn * 16, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<char *>(nodes_out) + nn * 16, c->b_nhi.ptr, nn * 16,
                                cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess && tris_out && p.nt)
        e = cudaMemcpyAsync(tris_out, c->b_tri.ptr, static_cast<size_t>(p.nt) * 48, cudaMemcpyDeviceToHost,
                            c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "tree read-back");
}

e8g_status e8g_bvh_get_stats(e8g_ctx const *c, e8g_bvh_stats *s) {
    if (!c || !s)
        return E8G_ERR_INVALID_ARG;
    if (!c->built)
        return E8G_ERR_NOT_BUILT;
    *s = c->bvh_stats;
    return E8G_OK;
}

e8g_status e8g_camera_rays(e8g_ctx *c, uint32_t w, uint32_t h, e8g_ray *rays_out) {
    if (!c || !rays_out || w < 2 || h < 2)
        return fail(c, E8G_ERR_INVALID_ARG, "bad arguments");
    if (!c->uploaded)
        return fail(c, E8G_ERR_NO_SCENE, "no scene uploaded");
    cudaSetDevice(c->device);
    size_t bytes = static_cast<size_t>(w) * h * sizeof(e8g_ray);
    cudaError_t e = c->b_io0.reserve(bytes);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "ray buffer");
    launch_camera_rays(c->dev, w, h, static_cast<float *>(c->b_io0.ptr), c->stream);
    e = cudaMemcpyAsync(rays_out, c->b_io0.ptr, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "camera rays");
}

e8g_status e8g_trace_closest_dev(e8g_ctx *c, e8g_ray const *d_rays, uint32_t n, e8g_hit *d_hits, void *stream) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    if (n && (!d_rays || !d_hits))
        return fail(c, E8G_ERR_INVALID_ARG, "NULL buffers");
    cudaSetDevice(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    launch_trace_closest(c->dev, reinterpret_cast<float const *>(d_rays), n, reinterpret_cast<float *>(d_hits), st);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "trace_closest launch");
}

e8g_status e8g_trace_closest(e8g_ctx *c, e8g_ray const *rays, uint32_t n, e8g_hit *hits) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    if (n == 0)
        return E8G_OK;
    if (!rays || !hits)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL buffers");
    cudaSetDevice(c->device);
    size_t rb = static_cast<size_t>(n) * sizeof(e8g_ray), hb = static_cast<size_t>(n) * sizeof(e8g_hit);
    cudaError_t e = c->b_io0.reserve(rb);
    if (e == cudaSuccess)
        e = c->b_io1.reserve(hb);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->b_io0.ptr, rays, rb, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "trace_closest upload");
    launch_trace_closest(c->dev, static_cast<float const *>(c->b_io0.ptr), n, static_cast<float *>(c->b_io1.ptr),
                         c->stream);
    e = cudaMemcpyAsync(hits, c->b_io1.ptr, hb, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? read_checks(c) : cuda_fail(c, e, "trace_closest");
}

e8g_status e8g_trace_any(e8g_ctx *c, e8g_ray const *rays, float const *t_min, float const *t_max, uint32_t n,
                         uint8_t *occluded) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    if (n == 0)
        return E8G_OK;
    if (!rays || !t_min || !t_max || !occluded)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL buffers");
    cudaSetDevice(c->device);
    size_t rb = static_cast<size_t>(n) * sizeof(e8g_ray), tb = static_cast<size_t>(n) * sizeof(float);
    cudaError_t e = c->b_io0.reserve(rb + 2 * tb + n);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "trace_any buffers");
    char *base = static_cast<char *>(c->b_io0.ptr);
    float *dtmin = reinterpret_cast<float *>(base + rb), *dtmax = reinterpret_cast<float *>(base + rb + tb);
    uint8_t *docc = reinterpret_cast<uint8_t *>(base + rb + 2 * tb);
    e = cudaMemcpyAsync(base, rays, rb, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dtmin, t_min, tb, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dtmax, t_max, tb, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "trace_any upload");
    launch_trace_any(c->dev, reinterpret_cast<float const *>(base), dtmin, dtmax, n, docc, c->stream);
    e = cudaMemcpyAsync(occluded, docc, n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? read_checks(c) : cuda_fail(c, e, "trace_any");
}

e8g_status e8g_render_dev(e8g_ctx *c, e8g_render_params const *p, float *d_rgba, void *stream) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, p);
    if (s != E8G_OK)
        return s;
    if (!d_rgba)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL output");
    cudaSetDevice(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    cudaStream_t saved = c->stream;
    c->stream = st;
    s = render_image(c, p, d_rgba, nullptr);
    c->stream = saved;
    return s;
}

e8g_status e8g_render_progressive(e8g_ctx *c, e8g_render_params const *p, int reset, float *d_rgba, void *stream) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, p);
    if (s != E8G_OK)
        return s;
    if (!d_rgba)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL output");
    if (p->firefly)
        return fail(c, E8G_ERR_UNSUPPORTED, "progressive rendering does not run the firefly clamp");
    cudaSetDevice(c->device);
    if (reset || c->prog_w != p->width || c->prog_h != p->height)
        c->prog_spp = 0;
    e8g_render_params q = *p;
    q.sample_offset = static_cast<uint32_t>(p->sample_offset + c->prog_spp); // continue the sample sequence
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    cudaStream_t saved = c->stream;
    c->stream = st;
    s = render_image(c, &q, d_rgba, nullptr, c->prog_spp);
    c->stream = saved;
    if (s != E8G_OK) {
        c->prog_spp = 0;
        return s;
    }
    c->prog_w = p->width;
    c->prog_h = p->height;
    c->prog_spp += p->spp;
    c->stats.paths = static_cast<uint64_t>(p->width) * p->height * p->spp;
    return E8G_OK;
}

e8g_status e8g_render(e8g_ctx *c, e8g_render_params const *p, float *rgba_out) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, p);
    if (s != E8G_OK)
        return s;
    if (!rgba_out)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL output");
    cudaSetDevice(c->device);
    size_t bytes = static_cast<size_t>(p->width) * p->height * 4 * sizeof(float);
    cudaError_t e = c->b_img.reserve(bytes);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "image buffer");
    s = render_image(c, p, static_cast<float *>(c->b_img.ptr), nullptr);
    if (s != E8G_OK)
        return s;
    e = cudaMemcpyAsync(rgba_out, c->b_img.ptr, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "render readback");
}

e8g_status e8g_count_traversal(e8g_ctx *c, e8g_render_params const *p, e8g_render_stats *out) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, p);
    if (s != E8G_OK)
        return s;
    cudaSetDevice(c->device);
    size_t bytes = static_cast<size_t>(p->width) * p->height * 4 * sizeof(float);
    cudaError_t e = c->b_img.reserve(bytes);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "image buffer");
    unsigned long long counts[3] = {0, 0, 0};
    s = render_image(c, p, static_cast<float *>(c->b_img.ptr), counts);
    if (s != E8G_OK)
        return s;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "count traversal");
    c->stats.rays = counts[0];
    c->stats.nodes = counts[1];
    c->stats.tris = counts[2];
    c->stats.counted = 1;
    if (out)
        *out = c->stats;
    return E8G_OK;
}

e8g_status e8g_set_memory_limit(e8g_ctx *c, uint64_t bytes) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    c->budget.cap = static_cast<size_t>(bytes);
    return E8G_OK;
}

e8g_status e8g_memory_used(e8g_ctx const *c, uint64_t *bytes) {
    if (!c || !bytes)
        return E8G_ERR_INVALID_ARG;
    *bytes = c->budget.used;
    return E8G_OK;
}

e8g_status e8g_cancel(e8g_ctx *c) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    c->cancel.store(true, std::memory_order_release);
    return E8G_OK;
}

e8g_status e8g_progressive_save(e8g_ctx *c, float *accum, uint32_t *width, uint32_t *height, uint64_t *spp) {
    if (!c || !width || !height || !spp)
        return E8G_ERR_INVALID_ARG;
    *width = c->prog_spp ? c->prog_w : 0;
    *height = c->prog_spp ? c->prog_h : 0;
    *spp = c->prog_spp;
    if (!accum || c->prog_spp == 0)
        return E8G_OK;
    cudaSetDevice(c->device);
    size_t bytes = static_cast<size_t>(c->prog_w) * c->prog_h * sizeof(float4);
    cudaError_t e = cudaMemcpyAsync(accum, c->b_accum.ptr, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "progressive save");
}

e8g_status e8g_progressive_load(e8g_ctx *c, float const *accum, uint32_t width, uint32_t height, uint64_t spp) {
    if (!c || !accum || width == 0 || height == 0 || spp == 0)
        return fail(c, E8G_ERR_INVALID_ARG, "progressive load: empty state");
    if (static_cast<uint64_t>(width) * height > (1ull << 28) || spp > 0xFFFFFFFFull)
        return fail(c, E8G_ERR_INVALID_ARG, "progressive load: state out of range");
    cudaSetDevice(c->device);
    size_t bytes = static_cast<size_t>(width) * height * sizeof(float4);
    cudaError_t e = c->b_accum.reserve(bytes);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->b_accum.ptr, accum, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        c->prog_spp = 0;
        return cuda_fail(c, e, "progressive load");
    }
    c->prog_w = width;
    c->prog_h = height;
    c->prog_spp = spp;
    return E8G_OK;
}

e8g_status e8g_set_kernel_timing(e8g_ctx *c, int on) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    c->kernel_timing = on != 0;
    return E8G_OK;
}

e8g_status e8g_get_render_stats(e8g_ctx const *c, e8g_render_stats *out) {
    if (!c || !out)
        return E8G_ERR_INVALID_ARG;
    *out = c->stats;
    return E8G_OK;
}

e8g_status e8g_render_paths(e8g_ctx *c, e8g_render_params const *p, uint32_t const *pixel, uint32_t const *sample,
                            uint32_t n, float *rgb_out) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, p);
    if (s != E8G_OK)
        return s;
    if (n == 0)
        return E8G_OK;
    if (!pixel || !sample || !rgb_out)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL buffers");
    uint32_t npix = p->width * p->height;
    for (uint32_t k = 0; k < n; k++)
        if (pixel[k] >= npix)
            return fail(c, E8G_ERR_INVALID_ARG, "pixel index out of range");
    cudaSetDevice(c->device);
    size_t lb = static_cast<size_t>(n) * sizeof(uint32_t), ob = static_cast<size_t>(n) * 3 * sizeof(float);
    cudaError_t e = c->b_io0.reserve(2 * lb);
    if (e == cudaSuccess)
        e = c->b_io1.reserve(ob);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "path buffers");
    uint32_t *dpx = static_cast<uint32_t *>(c->b_io0.ptr), *dsm = dpx + n;
    e = cudaMemcpyAsync(dpx, pixel, lb, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dsm, sample, lb, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "path upload");
    s = render_list(c, p, dpx, dsm, n, static_cast<float *>(c->b_io1.ptr));
    if (s != E8G_OK)
        return s;
    e = cudaMemcpyAsync(rgb_out, c->b_io1.ptr, ob, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? read_checks(c) : cuda_fail(c, e, "render_paths");
}

e8g_status e8g_render_rays(e8g_ctx *c, e8g_render_params const *params, e8g_ray const *rays, uint32_t n,
                           float *rgb_out) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    if (!params)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL params");
    if (n == 0)
        return E8G_OK;
    if (!rays || !rgb_out)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL buffers");
    e8g_render_params p = *params; // one path per ray (list mode: the image size only has to be valid)
    p.width = n < 2 ? 2 : n;
    p.height = 2;
    p.spp = 1;
    p.firefly = 0;
    s = validate_params(c, &p);
    if (s != E8G_OK)
        return s;
    cudaSetDevice(c->device);
    size_t rb = static_cast<size_t>(n) * sizeof(e8g_ray), lb = static_cast<size_t>(n) * sizeof(uint32_t),
           ob = static_cast<size_t>(n) * 3 * sizeof(float);
    cudaError_t e = c->b_io0.reserve(rb + 2 * lb);
    if (e == cudaSuccess)
        e = c->b_io1.reserve(ob);
    if (e == cudaSuccess)
        e = c->b_fh.reserve(static_cast<size_t>(n) * sizeof(FirstHit));
    if (e != cudaSuccess)
        return cuda_fail(c, e, "ray buffers");
    char *base = static_cast<char *>(c->b_io0.ptr);
    float *drays = reinterpret_cast<float *>(base);
    uint32_t *dpx = reinterpret_cast<uint32_t *>(base + rb), *dsm = dpx + n;
    e = cudaMemcpyAsync(drays, rays, rb, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "ray upload");
    launch_first_hits_rays(c->dev, drays, n, static_cast<FirstHit *>(c->b_fh.ptr), p.sample_offset, dpx, dsm,
                           c->stream);
    s = render_list(c, &p, dpx, dsm, n, static_cast<float *>(c->b_io1.ptr), true);
    if (s != E8G_OK)
        return s;
    e = cudaMemcpyAsync(rgb_out, c->b_io1.ptr, ob, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? read_checks(c) : cuda_fail(c, e, "render_rays");
}

} // extern "C"
