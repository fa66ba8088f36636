// C ABI of incremental scene updates (include/e8g.h, "incremental updates"): dirty-only vertex
// uploads, device-side mesh transforms and the commit that refits or rebuilds the tree.
//
// Reference flow replaced: objdb::push_updates (corelib/src/objdb.cpp:59-87) unloads and reloads
// every dirty object through its actuator (if_path_space::load copies the transformed geometry,
// trimesh::transform, geometry.cpp:76-87) and then commits each actuator, and the path space's
// commit rebuilds the whole BVH on the host (bvh_path_space_layout::commit, pathspace.cpp:292-328).
#include "../../include/e8g.h"
#include "api_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cmath>
#include <cstring>

using namespace e8g;

namespace {

e8g_status check_mesh(e8g_ctx *c, uint32_t mesh) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    if (!c->uploaded)
        return fail(c, E8G_ERR_NO_SCENE, "no scene uploaded");
    if (mesh >= c->pack.nm)
        return fail(c, E8G_ERR_INVALID_ARG, "mesh index out of range");
    return E8G_OK;
}

// Copies vertices [v0, v1) of the host pack's 4-float arrays to the device array(s).
cudaError_t upload_vertex_range(e8g_ctx *c, std::vector<float> const &src, dev_buffer &dst, uint32_t v0,
                                uint32_t v1) {
    if (v1 <= v0 || !dst.ptr)
        return cudaSuccess;
    size_t off = 16 * static_cast<size_t>(v0), n = 16 * static_cast<size_t>(v1 - v0);
    return cudaMemcpyAsync(static_cast<char *>(dst.ptr) + off, reinterpret_cast<char const *>(src.data()) + off, n,
                           cudaMemcpyHostToDevice, c->stream);
}

template <class T>
cudaError_t upload_all(e8g_ctx *c, std::vector<T> const &src, dev_buffer &dst) {
    if (src.empty())
        return cudaSuccess;
    return cudaMemcpyAsync(dst.ptr, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream);
}

float camera_abs(packed_scene const &p) {
    float a = 0.0f;
    for (int k = 0; k < 3; k++)
        a = std::max(a, std::fabs(p.cam.origin[k]));
    return a;
}

} // namespace

e8g_status e8g_scene_update_mesh(e8g_ctx *c, uint32_t mesh, float const *positions, float const *normals) {
    e8g_status st = check_mesh(c, mesh);
    if (st != E8G_OK)
        return st;
    if (!positions)
        return fail(c, E8G_ERR_INVALID_ARG, "positions is NULL");
    cudaSetDevice(c->device);
    packed_scene &p = c->pack;
    uint32_t v0 = p.mesh_voff[mesh], v1 = p.mesh_voff[mesh + 1];
    for (size_t i = 0; i < 3 * static_cast<size_t>(v1 - v0); i++)
        if (!std::isfinite(positions[i]) || (normals && !std::isfinite(normals[i])))
            return fail(c, E8G_ERR_INVALID_ARG, "vertex positions and normals must be finite");
    for (uint32_t v = v0; v < v1; v++)
        for (int k = 0; k < 3; k++) {
            p.vpos[4 * static_cast<size_t>(v) + k] = positions[3 * static_cast<size_t>(v - v0) + k];
            if (normals)
                p.vnrm[4 * static_cast<size_t>(v) + k] = normals[3 * static_cast<size_t>(v - v0) + k];
        }
    // the new blueprint's area (trimesh::update) and the light table built on it
    mesh_areas(p, mesh);
    light_table(p);
    cudaError_t e = upload_vertex_range(c, p.vpos, c->b_vpos, v0, v1);
    if (e == cudaSuccess)
        e = upload_vertex_range(c, p.vpos, c->b_vpos0, v0, v1);
    if (e == cudaSuccess && normals)
        e = upload_vertex_range(c, p.vnrm, c->b_vnrm, v0, v1);
    if (e == cudaSuccess && normals)
        e = upload_vertex_range(c, p.vnrm, c->b_vnrm0, v0, v1);
    if (e == cudaSuccess)
        e = upload_all(c, p.mesh_area, c->b_mesh_area);
    if (e == cudaSuccess && p.mesh_toff[mesh + 1] > p.mesh_toff[mesh])
        e = cudaMemcpyAsync(static_cast<float *>(c->b_tri_cum.ptr) + p.mesh_toff[mesh], p.tri_cum.data() + p.mesh_toff[mesh],
                            sizeof(float) * (p.mesh_toff[mesh + 1] - p.mesh_toff[mesh]), cudaMemcpyHostToDevice,
                            c->stream);
    if (e == cudaSuccess)
        e = upload_all(c, p.light_cum, c->b_light_cum);
    if (e == cudaSuccess)
        e = upload_all(c, p.light_pnorm, c->b_light_pnorm);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream); // the host arrays may change again on return
    if (e != cudaSuccess)
        return cuda_fail(c, e, "mesh update");
    c->dirty = true;
    c->prog_spp = 0;
    fill_dev_scene(c);
    return E8G_OK;
}

e8g_status e8g_scene_transform_mesh(e8g_ctx *c, uint32_t mesh, float const m[16], uint32_t flags) {
    e8g_status st = check_mesh(c, mesh);
    if (st != E8G_OK)
        return st;
    if (!m || flags > E8G_XFORM_NORMALS_AS_DIRECTIONS)
        return fail(c, E8G_ERR_INVALID_ARG, "bad transform arguments");
    for (int k = 0; k < 16; k++)
        if (!std::isfinite(m[k]))
            return fail(c, E8G_ERR_INVALID_ARG, "transform must be finite");
    XformArgs X{};
    std::memcpy(X.m, m, sizeof(X.m));
    if (!reference_normal_matrix(m, X.n))
        return fail(c, E8G_ERR_INVALID_ARG, "matrix not invertible");
    cudaSetDevice(c->device);
    packed_scene &p = c->pack;
    size_t bytes = 16 * static_cast<size_t>(p.nv);
    cudaError_t e = cudaSuccess;
    if (!c->b_vpos0.ptr) { // the first transform keeps the blueprint vertices
        e = c->b_vpos0.reserve(std::max<size_t>(bytes, 16));
        if (e == cudaSuccess)
            e = c->b_vnrm0.reserve(std::max<size_t>(bytes, 16));
        if (e == cudaSuccess && bytes)
            e = cudaMemcpyAsync(c->b_vpos0.ptr, c->b_vpos.ptr, bytes, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess && bytes)
            e = cudaMemcpyAsync(c->b_vnrm0.ptr, c->b_vnrm.ptr, bytes, cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) {
            c->b_vpos0.release();
            c->b_vnrm0.release();
            return cuda_fail(c, e, "blueprint copy");
        }
    }
    X.v_begin = p.mesh_voff[mesh];
    X.v_end = p.mesh_voff[mesh + 1];
    X.directions = flags == E8G_XFORM_NORMALS_AS_DIRECTIONS;
    launch_transform(static_cast<float4 const *>(c->b_vpos0.ptr), static_cast<float4 const *>(c->b_vnrm0.ptr),
                     static_cast<float4 *>(c->b_vpos.ptr), static_cast<float4 *>(c->b_vnrm.ptr), X, c->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(c, e, "transform launch");
    c->host_stale = true;
    c->dirty = true;
    c->prog_spp = 0;
    return E8G_OK;
}

e8g_status e8g_scene_set_camera(e8g_ctx *c, e8g_camera const *cam) {
    if (!c || !cam)
        return E8G_ERR_INVALID_ARG;
    if (!c->uploaded)
        return fail(c, E8G_ERR_NO_SCENE, "no scene uploaded");
    packed_scene &p = c->pack;
    std::memcpy(p.cam.origin, cam->origin, sizeof(p.cam.origin));
    std::memcpy(p.cam.rot, cam->rot, sizeof(p.cam.rot));
    p.cam.sensor = cam->sensor_size;
    p.cam.focal = cam->focal_len;
    p.cam.aspect = cam->aspect;
    // the eight-wide grid's smallest step was sized for the coordinates the rays start from
    if (c->built && p.layout == E8G_BVH_WIDE && camera_abs(p) > c->tree_max_abs)
        c->dirty = true;
    c->prog_spp = 0;
    fill_dev_scene(c);
    return E8G_OK;
}

e8g_status e8g_scene_get_mesh(e8g_ctx *c, uint32_t mesh, float *positions, float *normals) {
    e8g_status st = check_mesh(c, mesh);
    if (st != E8G_OK)
        return st;
    cudaSetDevice(c->device);
    st = sync_host_vertices(c);
    if (st != E8G_OK)
        return st;
    packed_scene const &p = c->pack;
    for (uint32_t v = p.mesh_voff[mesh]; v < p.mesh_voff[mesh + 1]; v++)
        for (int k = 0; k < 3; k++) {
            size_t o = 3 * static_cast<size_t>(v - p.mesh_voff[mesh]) + k;
            if (positions)
                positions[o] = p.vpos[4 * static_cast<size_t>(v) + k];
            if (normals)
                normals[o] = p.vnrm[4 * static_cast<size_t>(v) + k];
        }
    return E8G_OK;
}

e8g_status e8g_scene_commit(e8g_ctx *c, uint32_t mode, e8g_bvh_stats *stats) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    if (!c->uploaded)
        return fail(c, E8G_ERR_NO_SCENE, "no scene uploaded");
    if (mode > E8G_COMMIT_REBUILD)
        return fail(c, E8G_ERR_INVALID_ARG, "unknown commit mode");
    cudaSetDevice(c->device);
    packed_scene &p = c->pack;
    bool refit = mode == E8G_COMMIT_REFIT && c->built && p.layout != E8G_BVH_REFERENCE &&
                 p.layout != E8G_BVH_LINEAR && p.nt > 0;
    if (!refit) {
        auto t0 = std::chrono::steady_clock::now();
        e8g_status st = build_tree(c);
        if (st != E8G_OK)
            return st;
        c->bvh_stats.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    } else {
        cudaError_t e = c->b_refit.reserve(refit_scratch_bytes(p.bvh.num_nodes, p.nt));
        if (e != cudaSuccess)
            return cuda_fail(c, e, "refit scratch");
        RefitScratch R = refit_carve(c->b_refit.ptr, p.bvh.num_nodes, p.nt);
        fill_dev_scene(c);
        cudaEventRecord(c->ev0, c->stream);
        if (!c->refit_ready)
            launch_refit_parents(c->dev, R, c->stream);
        float cam_abs = camera_abs(p);
        uint32_t nlev = p.wide_levels.empty() ? 0u : static_cast<uint32_t>(p.wide_levels.size() - 1);
        if (p.layout == E8G_BVH_WIDE && (nlev == 0 || p.wide_levels.back() != p.bvh.num_nodes))
            return fail(c, E8G_ERR_INTERNAL, "eight-wide tree without level boundaries");
        launch_refit(c->dev, R, p.nv, cam_abs, 8 * c->num_sms, p.wide_levels.data(), nlev, c->stream);
        launch_interleave(c->dev.vpos, c->dev.vnrm, p.nv, static_cast<float4 *>(c->b_vtx.ptr), c->stream);
        cudaEventRecord(c->ev1, c->stream);
        uint32_t red[kRefitRedWords];
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(red, R.red, sizeof(red), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "refit");
        c->refit_ready = true;
        refit_read_bounds(red, p.bmin, p.bmax);
        float vmax;
        std::memcpy(&vmax, &red[12], 4);
        c->tree_max_abs = std::max(vmax, cam_abs);
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        c->bvh_stats.build_ms = ms;
        c->dirty = false;
        c->prog_spp = 0;
        fill_dev_scene(c);
    }
    if (stats)
        *stats = c->bvh_stats;
    return E8G_OK;
}
