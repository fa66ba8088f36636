#include "e8g_corelib.h"

#include <cstring>

#include <stdexcept>

namespace e8g_corelib {

gpu_oren_nayar::gpu_oren_nayar(std::string const &name, e8util::vec3 const &albedo, float sigma)
    : e8::oren_nayar(name, albedo, sigma), m_albedo_copy(albedo), m_sigma_copy(sigma) {}

std::unique_ptr<e8::if_material> gpu_oren_nayar::copy() const { return std::make_unique<gpu_oren_nayar>(*this); }

e8g_material gpu_oren_nayar::pack() const {
    e8g_material m{};
    m.type = E8G_MAT_OREN_NAYAR;
    for (int i = 0; i < 3; i++)
        m.albedo[i] = m_albedo_copy(i);
    m.roughness = m_sigma_copy;
    m.mix0 = m.mix1 = -1;
    return m;
}

gpu_cook_torr::gpu_cook_torr(std::string const &name, e8util::vec3 const &albedo, float roughness,
                             std::complex<float> const &ior)
    : e8::cook_torr(name, albedo, roughness, ior), m_albedo_copy(albedo), m_roughness_copy(roughness),
      m_ior_copy(ior) {}

std::unique_ptr<e8::if_material> gpu_cook_torr::copy() const { return std::make_unique<gpu_cook_torr>(*this); }

e8g_material gpu_cook_torr::pack() const {
    e8g_material m{};
    m.type = E8G_MAT_COOK_TORR;
    for (int i = 0; i < 3; i++)
        m.albedo[i] = m_albedo_copy(i);
    m.roughness = m_roughness_copy;
    m.ior_re = m_ior_copy.real();
    m.ior_im = m_ior_copy.imag();
    m.mix0 = m.mix1 = -1;
    return m;
}

std::vector<e8g_material> gpu_material_container::pack(std::vector<e8::obj_id_t> const &ids) const {
    std::vector<e8g_material> out;
    for (e8::obj_id_t id : ids) {
        auto it = m_mats.find(id);
        auto const *pm = it == m_mats.end() ? nullptr : dynamic_cast<packable_material const *>(it->second.get());
        if (pm) {
            out.push_back(pm->pack());
        } else {
            e8g_material fs{};
            fs.type = E8G_MAT_FAIL_SAFE;
            fs.mix0 = fs.mix1 = -1;
            out.push_back(fs);
        }
    }
    return out;
}

gpu_path_space_layout::packed gpu_path_space_layout::pack() const {
    packed p;
    for (auto const &kv : m_geometries) {
        e8::if_geometry const &g = *kv.second;
        for (auto const &v : g.vertices())
            for (int i = 0; i < 3; i++)
                p.pos.push_back(v(i));
        for (auto const &n : g.normals())
            for (int i = 0; i < 3; i++)
                p.nrm.push_back(n(i));
        for (auto const &t : g.triangles())
            for (int i = 0; i < 3; i++)
                p.tris.push_back(t(i));
        p.voff.push_back(static_cast<uint32_t>(p.pos.size() / 3));
        p.toff.push_back(static_cast<uint32_t>(p.tris.size() / 3));
        p.geo_ids.push_back(kv.first);
        p.mat_ids.push_back(g.material_id());
    }
    return p;
}

std::vector<e8g_light> gpu_light_sources::pack(std::vector<e8::obj_id_t> const &geo_ids) const {
    std::vector<e8g_light> out;
    for (auto const &kv : m_lights) {
        auto const *al = dynamic_cast<e8::area_light const *>(kv.second.get());
        if (!al)
            throw std::runtime_error("e8g: only area lights run on the GPU");
        std::vector<e8::if_geometry const *> gs = al->geometries();
        uint32_t mesh = UINT32_MAX;
        for (uint32_t m = 0; m < geo_ids.size(); m++)
            if (!gs.empty() && geo_ids[m] == gs[0]->id())
                mesh = m;
        if (mesh == UINT32_MAX)
            throw std::runtime_error("e8g: light geometry is not in the path space");
        e8util::vec3 n{0.0f, 0.0f, 1.0f};
        e8util::vec3 rad = al->radiance(n, n);
        e8g_light l{};
        l.mesh = mesh;
        for (int i = 0; i < 3; i++)
            l.radiance[i] = rad(i);
        out.push_back(l);
    }
    return out;
}

gpu_pinhole_camera::gpu_pinhole_camera(std::string const &name, float sensor_size, float f, float aspect)
    : e8::pinhole_camera(name, sensor_size, f, aspect), m_sensor(sensor_size), m_f(f), m_aspect(aspect) {}

std::unique_ptr<e8::if_camera> gpu_pinhole_camera::copy() const { return std::make_unique<gpu_pinhole_camera>(*this); }

std::unique_ptr<e8::if_camera> gpu_pinhole_camera::transform(e8util::mat44 const &trans) const {
    // pinhole_camera::transform keeps the translation column and the rotation block
    // (camera.cpp:63-71); the GPU camera records the matrix it was given.
    auto c = std::make_unique<gpu_pinhole_camera>(name(), m_sensor, m_f, m_aspect);
    auto base = e8::pinhole_camera::transform(trans);
    static_cast<e8::pinhole_camera &>(*c) = static_cast<e8::pinhole_camera const &>(*base);
    c->m_trans = trans;
    return c;
}

e8g_camera gpu_pinhole_camera::pack() const {
    e8g_camera c{};
    for (int i = 0; i < 3; i++) {
        c.origin[i] = m_trans(i, 3);
        for (int j = 0; j < 3; j++)
            c.rot[3 * i + j] = m_trans(i, j);
    }
    c.sensor_size = m_sensor;
    c.focal_len = m_f;
    c.aspect = m_aspect;
    return c;
}

void pack_scene(gpu_path_space_layout const &ps, gpu_material_container const &mats, gpu_light_sources const &lights,
                gpu_pinhole_camera const &cam, scene_storage &out) {
    out.geo = ps.pack();
    std::vector<e8::obj_id_t> mat_ids;
    std::map<e8::obj_id_t, int32_t> index;
    out.mesh_mat.clear();
    for (auto const &m : out.geo.mat_ids) {
        if (!m.has_value()) {
            out.mesh_mat.push_back(-1);
            continue;
        }
        auto it = index.find(*m);
        if (it == index.end()) {
            it = index.emplace(*m, static_cast<int32_t>(mat_ids.size())).first;
            mat_ids.push_back(*m);
        }
        out.mesh_mat.push_back(it->second);
    }
    out.mats = mats.pack(mat_ids);
    out.lights = lights.pack(out.geo.geo_ids);
    e8g_scene_desc &d = out.desc;
    d.num_meshes = static_cast<uint32_t>(out.mesh_mat.size());
    d.mesh_vert_offset = out.geo.voff.data();
    d.mesh_tri_offset = out.geo.toff.data();
    d.mesh_material = out.mesh_mat.data();
    d.positions = out.geo.pos.data();
    d.normals = out.geo.nrm.data();
    d.triangles = out.geo.tris.data();
    d.num_materials = static_cast<uint32_t>(out.mats.size());
    d.materials = out.mats.data();
    d.num_lights = static_cast<uint32_t>(out.lights.size());
    d.lights = out.lights.data();
    d.camera = cam.pack();
}

gpu_image_renderer::gpu_image_renderer(e8::pathtracer_factory::pt_type type, int device) : m_type(type) {
    e8g_device_opts o{device, 0};
    if (e8g_create(&m_ctx, &o) != E8G_OK)
        throw std::runtime_error("e8g: no CUDA device");
}

gpu_image_renderer::~gpu_image_renderer() {
    if (m_ctx)
        e8g_destroy(m_ctx);
}

namespace {

template <class T> bool same_bytes(std::vector<T> const &a, std::vector<T> const &b) {
    return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}

bool same_structure(scene_storage const &a, scene_storage const &b) {
    return same_bytes(a.geo.voff, b.geo.voff) && same_bytes(a.geo.toff, b.geo.toff) &&
           same_bytes(a.geo.tris, b.geo.tris) && same_bytes(a.mesh_mat, b.mesh_mat) &&
           a.geo.geo_ids == b.geo.geo_ids && same_bytes(a.lights, b.lights) && a.mats.size() == b.mats.size();
}

} // namespace

void gpu_image_renderer::commit_scene(scene_storage &next) {
    auto check = [this](e8g_status st) {
        if (st != E8G_OK)
            throw std::runtime_error(std::string("e8g: ") + e8g_last_error(m_ctx));
    };
    if (!m_have_scene || !same_structure(m_scene, next)) {
        e8g_bvh_opts bo;
        e8g_default_bvh_opts(&bo);
        check(e8g_scene_upload(m_ctx, &next.desc));
        check(e8g_scene_build_bvh(m_ctx, &bo));
    } else {
        bool moved = false;
        for (uint32_t m = 0; m + 1 < next.geo.voff.size(); m++) {
            size_t b = 3 * static_cast<size_t>(next.geo.voff[m]), n = 3 * static_cast<size_t>(next.geo.voff[m + 1]) - b;
            bool pos_same = std::memcmp(&next.geo.pos[b], &m_scene.geo.pos[b], n * sizeof(float)) == 0;
            bool nrm_same = std::memcmp(&next.geo.nrm[b], &m_scene.geo.nrm[b], n * sizeof(float)) == 0;
            if (n && (!pos_same || !nrm_same)) {
                check(e8g_scene_update_mesh(m_ctx, m, &next.geo.pos[b], &next.geo.nrm[b]));
                moved = true;
            }
        }
        if (std::memcmp(&next.desc.camera, &m_scene.desc.camera, sizeof(e8g_camera)) != 0)
            check(e8g_scene_set_camera(m_ctx, &next.desc.camera));
        if (!same_bytes(next.mats, m_scene.mats))
            check(e8g_set_materials(m_ctx, next.mats.data(), static_cast<uint32_t>(next.mats.size())));
        if (moved)
            check(e8g_scene_commit(m_ctx, E8G_COMMIT_REFIT, nullptr));
    }
    m_scene = std::move(next);
    // the description points into the storage's own vectors
    scene_storage &s = m_scene;
    s.desc.mesh_vert_offset = s.geo.voff.data();
    s.desc.mesh_tri_offset = s.geo.toff.data();
    s.desc.mesh_material = s.mesh_mat.data();
    s.desc.positions = s.geo.pos.data();
    s.desc.normals = s.geo.nrm.data();
    s.desc.triangles = s.geo.tris.data();
    s.desc.materials = s.mats.data();
    s.desc.lights = s.lights.data();
    m_have_scene = true;
}

uint32_t mode_of(e8::pathtracer_factory::pt_type type) {
    switch (type) {
    case e8::pathtracer_factory::unidirect:
        return E8G_MODE_REF_UNI;
    case e8::pathtracer_factory::bidirect_mis:
        return E8G_MODE_REF_BDPT;
    case e8::pathtracer_factory::bidirect_lt2:
        return E8G_MODE_REF_LT2;
    case e8::pathtracer_factory::direct:
        return E8G_MODE_REF_DIRECT;
    case e8::pathtracer_factory::normal:
        return E8G_MODE_NORMAL;
    case e8::pathtracer_factory::position:
        return E8G_MODE_POSITION;
    default:
        return E8G_MODE_REF_LT1;
    }
}

gpu_path_tracer::gpu_path_tracer(e8g_ctx *ctx, e8::pathtracer_factory::pt_type type)
    : m_ctx(ctx), m_mode(mode_of(type)) {}

std::vector<e8util::vec3> gpu_path_tracer::sample(e8util::rng &rng, std::vector<e8util::ray> const &rays,
                                                  first_hits const &, e8::if_path_space const &,
                                                  e8::if_material_container const &,
                                                  e8::if_light_sources const &) const {
    std::vector<e8g_ray> in(rays.size());
    for (size_t i = 0; i < rays.size(); i++)
        for (int k = 0; k < 3; k++) {
            in[i].o[k] = rays[i].o()(k);
            in[i].d[k] = rays[i].v()(k);
        }
    e8g_render_params p;
    e8g_default_params(&p, m_mode, 1, 1, 1);
    p.seed = static_cast<uint64_t>(rng.draw() * 4294967296.0);
    std::vector<float> rgb(3 * rays.size());
    if (e8g_render_rays(m_ctx, &p, in.data(), static_cast<uint32_t>(rays.size()), rgb.data()) != E8G_OK)
        throw std::runtime_error(std::string("e8g: ") + e8g_last_error(m_ctx));
    std::vector<e8util::vec3> out(rays.size());
    for (size_t i = 0; i < rays.size(); i++)
        out[i] = e8util::vec3{rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]};
    return out;
}

e8::pt_image_renderer::numerical_stats
gpu_image_renderer::render(e8::if_compositor *compositor, e8::if_path_space const &path_space,
                           e8::if_material_container const &mats, e8::if_light_sources const &light_sources,
                           e8::if_camera const &cam, unsigned num_samps, bool firefly_filter) {
    auto const &ps = dynamic_cast<gpu_path_space_layout const &>(path_space);
    auto const &mc = dynamic_cast<gpu_material_container const &>(mats);
    auto const &ls = dynamic_cast<gpu_light_sources const &>(light_sources);
    auto const &pc = dynamic_cast<gpu_pinhole_camera const &>(cam);
    scene_storage next;
    pack_scene(ps, mc, ls, pc, next);
    commit_scene(next);
    uint32_t mode = mode_of(m_type);
    unsigned w = compositor->width(), h = compositor->height();
    e8g_render_params p;
    e8g_default_params(&p, mode, w, h, num_samps);
    p.seed = 1361 + m_frame++;
    p.firefly = firefly_filter ? 1u : 0u;
    std::vector<float> rgba(static_cast<size_t>(w) * h * 4);
    if (e8g_render(m_ctx, &p, rgba.data()) != E8G_OK)
        throw std::runtime_error(std::string("e8g: ") + e8g_last_error(m_ctx));
    for (unsigned j = 0; j < h; j++)
        for (unsigned i = 0; i < w; i++) {
            float const *px = &rgba[4 * (static_cast<size_t>(j) * w + i)];
            (*compositor)(i, j) = e8::rgba_color({px[0], px[1], px[2], px[3]});
        }
    e8::pt_image_renderer::numerical_stats st{};
    st.num_samples = num_samps;
    return st;
}

} // namespace e8g_corelib
