// e8g_batch_render: many independent scenes rendered together.
//
// Every scene is packed and its tree built on the host (scene by scene), then all scenes go to
// the device in one allocation: per-scene arrays at 256-byte aligned offsets, one DevScene record
// and one RenderArgs record per scene. One batched first-hit kernel, the integrator over the
// concatenated path ranges and one batched resolve render the whole batch. The integrator is the
// many-scene wavefront on eight-wide trees (slots shared by all scenes, the bounce loop one CUDA
// graph) when every item asks for E8G_INTEGRATOR_WAVEFRONT with E8G_MODE_MIS and one stream kind,
// else the persistent megakernel on SAH-pair trees (k_mega_batch).
#include "api_internal.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace e8g {
namespace {

struct staged {
    std::vector<unsigned char> bytes;
    size_t put(void const *src, size_t n) {
        size_t off = (bytes.size() + 255) & ~static_cast<size_t>(255);
        bytes.resize(off + std::max<size_t>(n, 16));
        if (n)
            std::memcpy(bytes.data() + off, src, n);
        return off;
    }
    template <class T> size_t put(std::vector<T> const &v) { return put(v.data(), v.size() * sizeof(T)); }
};

} // namespace
} // namespace e8g

extern "C" e8g_status e8g_batch_render(e8g_ctx *c, e8g_batch_item const *items, uint32_t n, e8g_render_stats *stats) {
    using namespace e8g;
    if (!c || (!items && n))
        return E8G_ERR_INVALID_ARG;
    if (n == 0)
        return E8G_OK;
    for (uint32_t k = 0; k < n; k++) {
        char const *bad = e8g_validate_desc(items[k].scene);
        if (bad)
            return fail(c, E8G_ERR_INVALID_ARG, std::string("batch scene: ") + bad);
        e8g_status s = validate_params(c, &items[k].params);
        if (s != E8G_OK)
            return s;
        if (!items[k].rgba_out)
            return fail(c, E8G_ERR_INVALID_ARG, "batch item has no output");
        uint32_t m = items[k].params.mode;
        if (m == E8G_MODE_REF_BDPT || m == E8G_MODE_BDPT_POWER || m == E8G_MODE_REF_LT2)
            return fail(c, E8G_ERR_UNSUPPORTED, "batches run the unidirectional integrators");
        if (items[k].params.firefly)
            return fail(c, E8G_ERR_UNSUPPORTED, "batches do not run the firefly clamp");
    }
    bool use_wf = true;
    for (uint32_t k = 0; k < n; k++)
        use_wf = use_wf && items[k].params.integrator == E8G_INTEGRATOR_WAVEFRONT &&
                 items[k].params.mode == E8G_MODE_MIS && items[k].params.rng == items[0].params.rng;
    nvtx_range range("e8g_batch_render");
    if (take_cancel(c))
        return fail(c, E8G_ERR_CANCELLED, "batch cancelled");
    cudaSetDevice(c->device);
    c->prog_spp = 0; // the batch reuses the accumulator
    // host: pack, build, stage
    staged st;
    struct offs {
        size_t nlo, nhi, wide, tri, tidx, vpos, vnrm, vtx, mesh_mat, mesh_light, mesh_toff, mesh_area, tri_cum, mats, light_mesh,
            light_rad, light_cum, light_pnorm;
    };
    std::vector<offs> off(n);
    std::vector<packed_scene> packs(n);
    std::vector<RenderArgs> args(n);
    std::vector<uint64_t> path_prefix(n + 1, 0), pix_prefix(n + 1, 0);
    uint32_t rng_kinds = 0;
    for (uint32_t k = 0; k < n; k++)
        rng_kinds |= 1u << items[k].params.rng;
    try {
        for (uint32_t k = 0; k < n; k++)
            pack_scene(*items[k].scene, packs[k]);
        bvh_build_opts bo;
        bo.layout = use_wf ? 2u : 0u;
        for (uint32_t k = 0; k < n; k++)
            build_scene_bvh(packs[k], bo);
        for (uint32_t k = 0; k < n && use_wf; k++)
            if (packs[k].layout != 2) { // a tree too deep for the wide stack: SAH pairs for all
                use_wf = false;
                bo.layout = 0;
                for (uint32_t j = 0; j < n; j++)
                    build_scene_bvh(packs[j], bo);
            }
        for (uint32_t k = 0; k < n; k++) {
            packed_scene &p = packs[k];
            offs &o = off[k];
            o.nlo = st.put(p.bvh.lo);
            o.nhi = st.put(p.bvh.hi);
            o.wide = st.put(p.wide);
            o.tri = st.put(p.tri);
            o.tidx = st.put(p.tidx);
            o.vpos = st.put(p.vpos);
            o.vnrm = st.put(p.vnrm);
            o.vtx = st.put(p.vtx);
            o.mesh_mat = st.put(p.mesh_mat);
            o.mesh_light = st.put(p.mesh_light);
            o.mesh_toff = st.put(p.mesh_toff);
            o.mesh_area = st.put(p.mesh_area);
            o.tri_cum = st.put(p.tri_cum);
            o.mats = st.put(p.mats);
            o.light_mesh = st.put(p.light_mesh);
            o.light_rad = st.put(p.light_rad);
            o.light_cum = st.put(p.light_cum);
            o.light_pnorm = st.put(p.light_pnorm);
            args[k] = make_args(&items[k].params);
            path_prefix[k + 1] = path_prefix[k] + args[k].total_paths;
            pix_prefix[k + 1] = pix_prefix[k] + static_cast<uint64_t>(items[k].params.width) * items[k].params.height;
        }
    } catch (std::bad_alloc const &) {
        return fail(c, E8G_ERR_OUT_OF_MEMORY, "host allocation failed while packing the batch");
    }
    size_t recs = st.put(args);
    size_t pp = st.put(path_prefix);
    size_t px = st.put(pix_prefix);
    size_t scene_rec = (st.bytes.size() + 255) & ~static_cast<size_t>(255);
    st.bytes.resize(scene_rec + n * sizeof(DevScene));
    uint64_t total_pix = pix_prefix[n];
    cudaError_t e = c->b_batch.reserve(st.bytes.size());
    if (e == cudaSuccess)
        e = c->b_fh.reserve(total_pix * sizeof(FirstHit));
    if (e == cudaSuccess)
        e = c->b_accum.reserve(total_pix * sizeof(float4));
    if (e == cudaSuccess)
        e = c->b_img.reserve(total_pix * 4 * sizeof(float));
    if (e != cudaSuccess)
        return cuda_fail(c, e, "batch buffers");
    unsigned char *base = static_cast<unsigned char *>(c->b_batch.ptr);
    for (uint32_t k = 0; k < n; k++) { // device records point into the one allocation
        packed_scene &p = packs[k];
        offs &o = off[k];
        DevScene S{};
        S.nlo = reinterpret_cast<float4 const *>(base + o.nlo);
        S.nhi = reinterpret_cast<float4 const *>(base + o.nhi);
        S.wnodes = reinterpret_cast<uint4 const *>(base + o.wide);
        S.tri = reinterpret_cast<float4 const *>(base + o.tri);
        S.tidx = reinterpret_cast<uint4 const *>(base + o.tidx);
        S.vpos = reinterpret_cast<float4 const *>(base + o.vpos);
        S.vnrm = reinterpret_cast<float4 const *>(base + o.vnrm);
        S.vtx = reinterpret_cast<float4 const *>(base + o.vtx);
        S.mesh_mat = reinterpret_cast<int32_t const *>(base + o.mesh_mat);
        S.mesh_light = reinterpret_cast<int32_t const *>(base + o.mesh_light);
        S.mesh_toff = reinterpret_cast<uint32_t const *>(base + o.mesh_toff);
        S.mesh_area = reinterpret_cast<float const *>(base + o.mesh_area);
        S.tri_cum = reinterpret_cast<float const *>(base + o.tri_cum);
        S.mats = reinterpret_cast<DevMaterial const *>(base + o.mats);
        S.light_mesh = reinterpret_cast<uint32_t const *>(base + o.light_mesh);
        S.light_rad = reinterpret_cast<float4 const *>(base + o.light_rad);
        S.light_cum = reinterpret_cast<float const *>(base + o.light_cum);
        S.light_pnorm = reinterpret_cast<float const *>(base + o.light_pnorm);
        S.nmat = p.nmat;
        S.nl = p.nl;
        S.nm = p.nm;
        S.nnodes = p.bvh.num_nodes;
        S.ntris = p.nt;
        S.nverts = p.nv;
        S.check = static_cast<unsigned long long *>(c->b_check.ptr);
        S.layout = p.layout;
        S.total_power = p.total_power;
        for (int i = 0; i < 3; i++) {
            S.bmin[i] = p.bmin[i];
            S.bmax[i] = p.bmax[i];
        }
        S.cam = p.cam;
        std::memcpy(st.bytes.data() + scene_rec + k * sizeof(DevScene), &S, sizeof(DevScene));
    }
    BatchDev B{};
    B.scenes = reinterpret_cast<DevScene const *>(base + scene_rec);
    B.args = reinterpret_cast<RenderArgs const *>(base + recs);
    B.path_prefix = reinterpret_cast<uint64_t const *>(base + pp);
    B.pix_prefix = reinterpret_cast<uint64_t const *>(base + px);
    B.n = n;
    B.total_paths = path_prefix[n];
    e = cudaMemcpyAsync(base, st.bytes.data(), st.bytes.size(), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "batch upload");
    // device: one first-hit launch, one persistent integrator launch, one resolve
    cudaEventRecord(c->ev0, c->stream);
    launch_first_hits_batch(B, nullptr, nullptr, pix_prefix.data(), static_cast<FirstHit *>(c->b_fh.ptr), c->stream);
    e = cudaMemsetAsync(c->b_accum.ptr, 0, total_pix * sizeof(float4), c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(c->b_work.ptr, 0, 64, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "batch clear");
    cudaEventRecord(c->ev2, c->stream);
    c->launches = 0;
    if (use_wf) {
        e8g_status s = run_wavefront(c, args[0], static_cast<float4 *>(c->b_accum.ptr), nullptr, c->wf_capacity,
                                     c->wf_bounces, c->wf_threshold, &B, static_cast<FirstHit const *>(c->b_fh.ptr));
        if (s != E8G_OK)
            return s;
    } else {
        launch_megakernel_batch(B, static_cast<FirstHit const *>(c->b_fh.ptr), static_cast<float4 *>(c->b_accum.ptr),
                                static_cast<unsigned long long *>(c->b_work.ptr), rng_kinds,
                                persistent_grid(c, megakernel_batch_blocks_per_sm(rng_kinds)), c->stream);
        c->launches = 1;
    }
    cudaEventRecord(c->ev3, c->stream);
    launch_resolve_batch(B, total_pix, static_cast<float4 const *>(c->b_accum.ptr), static_cast<float *>(c->b_img.ptr),
                         c->stream);
    cudaEventRecord(c->ev1, c->stream);
    e = cudaGetLastError();
    for (uint32_t k = 0; k < n && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(items[k].rgba_out, static_cast<float *>(c->b_img.ptr) + 4 * pix_prefix[k],
                            (pix_prefix[k + 1] - pix_prefix[k]) * 4 * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "batch render");
    float ms = 0, kms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    cudaEventElapsedTime(&kms, c->ev2, c->ev3);
    c->stats = e8g_render_stats{};
    c->stats.ms = ms;
    c->stats.kernel_ms = kms;
    uint64_t paths = 0;
    for (uint32_t k = 0; k < n; k++)
        paths += static_cast<uint64_t>(items[k].params.width) * items[k].params.height * items[k].params.spp;
    c->stats.paths = paths;
    c->stats.launches = c->launches + 2; // first hits, integrator, resolve
    if (stats)
        *stats = c->stats;
    return read_checks(c);
}
