// ref_driver.cpp — drives the UNMODIFIED reference corelib (compiled from its own sources by
// oracle/Makefile into oracle/_ref/) through its public C++ API, for parity pinning.
//
// TEST INFRASTRUCTURE ONLY. It builds reference objects (trimesh, oren_nayar, cook_torr,
// mat_mixture, area_light, pinhole_camera, bvh_path_space_layout, basic_light_sources,
// default_material_container) from an e8g_scene_desc and exposes the reference's own calls:
//   if_path_space::intersect / has_intersect    corelib/src/pathspace.cpp:36-114, :330-456
//   pinhole_camera::sample                      corelib/src/camera.cpp:38-48
//   if_path_tracer::compute_first_hit + sample  corelib/src/pathtracer.cpp:456-803
//   pt_image_renderer::render                   corelib/src/renderer.cpp:106-166
//   if_material::eval / sample                  corelib/src/material.cpp:54-252
// Per-path draw streams are fresh e8util::rng(seed) objects — the reference's own rng class,
// constructed with a per-path seed — so no reference source is patched.
#include "../include/e8g.h"

#include "camera.h"
#include "compositor.h"
#include "geometry.h"
#include "light.h"
#include "lightsources.h"
#include "material.h"
#include "materialcontainer.h"
#include "pathspace.h"
#include "pathtracer.h"
#include "pathtracerfact.h"
#include "renderer.h"
#include "resource.h"

#include <chrono>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

namespace {

// Exposes the protected geometry map so a hit's geometry pointer maps back to a mesh index.
template <class Base> struct open_space : public Base {
    std::map<e8::obj_id_t, std::unique_ptr<e8::if_geometry const>> const &geos() const {
        return this->m_geometries;
    }
};

struct mem_frame : public e8::if_frame {
    mem_frame(unsigned w, unsigned h) { back().resize(w, h); }
    void commit() override {}
};

struct mem_compositor : public e8::if_compositor {
    mem_compositor(unsigned w, unsigned h) : e8::if_compositor(w, h) {}
    void commit(e8::if_frame *) const override {}
};

std::unique_ptr<e8::if_material> make_leaf(e8g_material const &d, std::string const &name) {
    e8util::vec3 albedo{d.albedo[0], d.albedo[1], d.albedo[2]};
    switch (d.type) {
    case E8G_MAT_OREN_NAYAR:
        return std::make_unique<e8::oren_nayar>(name, albedo, d.roughness);
    case E8G_MAT_COOK_TORR:
        return std::make_unique<e8::cook_torr>(name, albedo, d.roughness,
                                               std::complex<float>(d.ior_re, d.ior_im));
    default:
        return std::make_unique<e8::mat_fail_safe>(name);
    }
}

e8::pathtracer_factory::pt_type tracer_type(uint32_t mode) {
    switch (mode) {
    case E8G_MODE_REF_UNI:
        return e8::pathtracer_factory::unidirect;
    case E8G_MODE_REF_LT1:
        return e8::pathtracer_factory::unidirect_lt1;
    case E8G_MODE_REF_BDPT:
        return e8::pathtracer_factory::bidirect_mis;
    case E8G_MODE_REF_DIRECT:
        return e8::pathtracer_factory::direct;
    case E8G_MODE_NORMAL:
        return e8::pathtracer_factory::normal;
    case E8G_MODE_POSITION:
        return e8::pathtracer_factory::position;
    case E8G_MODE_REF_LT2:
        return e8::pathtracer_factory::bidirect_lt2;
    default:
        return e8::pathtracer_factory::unidirect_lt1;
    }
}

} // namespace

struct r_scene {
    std::vector<std::shared_ptr<e8::trimesh>> meshes;
    std::vector<std::shared_ptr<e8::if_material>> mats;
    std::vector<std::shared_ptr<e8::if_light>> lights;
    std::unique_ptr<open_space<e8::bvh_path_space_layout>> bvh;
    std::unique_ptr<open_space<e8::linear_path_space_layout>> linear;
    std::unique_ptr<e8::default_material_container> mc;
    std::unique_ptr<e8::basic_light_sources> ls;
    std::unique_ptr<e8::if_camera> cam;
    std::map<e8::if_geometry const *, int> geo_index;
    std::vector<uint32_t> tri_off;
};

extern "C" {

r_scene *r_scene_create(e8g_scene_desc const *d) {
    auto s = new r_scene();
    // Materials first (ids ascend in creation order; the container is keyed by id).
    s->mc = std::make_unique<e8::default_material_container>();
    for (uint32_t i = 0; i < d->num_materials; i++) {
        e8g_material const &m = d->materials[i];
        std::string name = "mat" + std::to_string(i);
        std::shared_ptr<e8::if_material> mat;
        if (m.type == E8G_MAT_MIXTURE) {
            mat = std::make_shared<e8::mat_mixture>(name, make_leaf(d->materials[m.mix0], name + "a"),
                                                    make_leaf(d->materials[m.mix1], name + "b"),
                                                    m.ratio);
        } else {
            mat = make_leaf(m, name);
        }
        s->mats.push_back(mat);
        s->mc->load(*mat, e8util::mat44_scale(1.0f));
    }
    s->mc->commit();

    s->bvh = std::make_unique<open_space<e8::bvh_path_space_layout>>();
    s->linear = std::make_unique<open_space<e8::linear_path_space_layout>>();
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        auto mesh = std::make_shared<e8::trimesh>("mesh" + std::to_string(m));
        uint32_t v0 = d->mesh_vert_offset[m], v1 = d->mesh_vert_offset[m + 1];
        std::vector<e8util::vec3> verts, norms;
        for (uint32_t v = v0; v < v1; v++) {
            verts.push_back(e8util::vec3{d->positions[3 * v], d->positions[3 * v + 1], d->positions[3 * v + 2]});
            norms.push_back(e8util::vec3{d->normals[3 * v], d->normals[3 * v + 1], d->normals[3 * v + 2]});
        }
        std::vector<e8::triangle> tris;
        for (uint32_t t = d->mesh_tri_offset[m]; t < d->mesh_tri_offset[m + 1]; t++) {
            tris.push_back(e8::triangle{d->triangles[3 * t], d->triangles[3 * t + 1], d->triangles[3 * t + 2]});
        }
        mesh->vertices(verts);
        mesh->normals(norms);
        mesh->triangles(tris);
        mesh->update();
        if (d->mesh_material && d->mesh_material[m] >= 0) {
            mesh->attach_material(s->mats[d->mesh_material[m]]->id());
        }
        s->meshes.push_back(mesh);
        s->bvh->load(*mesh, e8util::mat44_scale(1.0f));
        s->linear->load(*mesh, e8util::mat44_scale(1.0f));
    }
    s->bvh->commit();
    s->linear->commit();
    for (auto const &kv : s->bvh->geos()) {
        for (uint32_t m = 0; m < s->meshes.size(); m++)
            if (s->meshes[m]->id() == kv.first)
                s->geo_index[kv.second.get()] = static_cast<int>(m);
    }
    for (auto const &kv : s->linear->geos()) {
        for (uint32_t m = 0; m < s->meshes.size(); m++)
            if (s->meshes[m]->id() == kv.first)
                s->geo_index[kv.second.get()] = static_cast<int>(m);
    }
    s->tri_off.assign(d->mesh_tri_offset, d->mesh_tri_offset + d->num_meshes + 1);

    s->ls = std::make_unique<e8::basic_light_sources>();
    for (uint32_t l = 0; l < d->num_lights; l++) {
        e8g_light const &L = d->lights[l];
        auto light = std::make_shared<e8::area_light>(
            "light" + std::to_string(l), s->meshes[L.mesh],
            e8util::vec3{L.radiance[0], L.radiance[1], L.radiance[2]});
        s->lights.push_back(light);
        s->ls->load(*light, e8util::mat44_scale(1.0f));
    }
    s->ls->commit();

    e8g_camera const &c = d->camera;
    e8::pinhole_camera cam("cam", c.sensor_size, c.focal_len, c.aspect);
    // mat44 initialiser lists are column-major (tensor.h:345-353).
    e8util::mat44 trans({c.rot[0], c.rot[3], c.rot[6], 0.0f, c.rot[1], c.rot[4], c.rot[7], 0.0f,
                         c.rot[2], c.rot[5], c.rot[8], 0.0f, c.origin[0], c.origin[1], c.origin[2],
                         1.0f});
    s->cam = cam.transform(trans);
    return s;
}

void r_scene_free(r_scene *s) { delete s; }

// Closest hit through the reference path space. The reference returns the hit geometry, t, the
// interpolated vertex and normal; the triangle index is recovered as the triangle of that mesh
// whose ray::intersect reproduces the returned t bit for bit (first such in index order).
void r_trace_closest(r_scene const *s, e8g_ray const *rays, uint32_t n, int use_bvh, float *t_out,
                     int32_t *mesh_out, int32_t *tri_out, float *vertex_out, float *normal_out) {
    e8::if_path_space const &ps =
        use_bvh ? static_cast<e8::if_path_space const &>(*s->bvh) : *s->linear;
    for (uint32_t k = 0; k < n; k++) {
        e8util::ray r(e8util::vec3{rays[k].o[0], rays[k].o[1], rays[k].o[2]},
                      e8util::vec3{rays[k].d[0], rays[k].d[1], rays[k].d[2]});
        e8::intersect_info h = ps.intersect(r);
        if (!h.valid()) {
            t_out[k] = 0;
            mesh_out[k] = -1;
            tri_out[k] = -1;
            continue;
        }
        int m = s->geo_index.at(h.geo);
        t_out[k] = h.t;
        mesh_out[k] = m;
        for (int i = 0; i < 3; i++) {
            vertex_out[3 * k + i] = h.vertex(i);
            normal_out[3 * k + i] = h.normal(i);
        }
        tri_out[k] = -1;
        auto const &verts = h.geo->vertices();
        auto const &tris = h.geo->triangles();
        for (uint32_t t = 0; t < tris.size(); t++) {
            e8util::vec3 b;
            float t0;
            if (r.intersect(verts[tris[t](0)], verts[tris[t](1)], verts[tris[t](2)], 1e-4f, 1000.0f, b,
                            t0) &&
                t0 == h.t) {
                tri_out[k] = static_cast<int32_t>(t);
                break;
            }
        }
    }
}

void r_trace_any(r_scene const *s, e8g_ray const *rays, float const *t_min, float const *t_max,
                 uint32_t n, int use_bvh, uint8_t *occluded) {
    e8::if_path_space const &ps =
        use_bvh ? static_cast<e8::if_path_space const &>(*s->bvh) : *s->linear;
    for (uint32_t k = 0; k < n; k++) {
        e8util::ray r(e8util::vec3{rays[k].o[0], rays[k].o[1], rays[k].o[2]},
                      e8util::vec3{rays[k].d[0], rays[k].d[1], rays[k].d[2]});
        float t;
        occluded[k] = ps.has_intersect(r, t_min[k], t_max[k], t) ? 1 : 0;
    }
}

void r_camera_rays(r_scene const *s, uint32_t w, uint32_t h, e8g_ray *rays) {
    e8util::rng rng(1361);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) {
            float pdf;
            e8util::ray r = s->cam->sample(rng, x, y, w, h, pdf);
            for (int i = 0; i < 3; i++) {
                rays[y * w + x].o[i] = r.o()(i);
                rays[y * w + x].d[i] = r.v()(i);
            }
        }
}

// One path per (pixel, seed): a fresh e8util::rng(seed) and a single-ray call to sample(), the
// way tst_pathtracer.cpp:67-73 drives the integrators.
void r_render_paths(r_scene const *s, uint32_t mode, uint32_t w, uint32_t h, uint32_t const *pixel,
                    uint32_t const *seeds, uint32_t n, float *rgb_out) {
    e8::pathtracer_factory fact(tracer_type(mode), e8::pathtracer_factory::options());
    std::unique_ptr<e8::if_path_tracer> tracer(fact.create());
    e8util::rng cam_rng(1361);
    for (uint32_t k = 0; k < n; k++) {
        float pdf;
        std::vector<e8util::ray> rays{s->cam->sample(cam_rng, pixel[k] % w, pixel[k] / w, w, h, pdf)};
        e8::if_path_tracer::first_hits hits =
            e8::if_path_tracer::compute_first_hit(rays, *s->bvh, *s->ls);
        e8util::rng rng(seeds[k]);
        std::vector<e8util::vec3> est = tracer->sample(rng, rays, hits, *s->bvh, *s->mc, *s->ls);
        for (int i = 0; i < 3; i++)
            rgb_out[3 * k + i] = est[0](i);
    }
}

// pt_image_renderer::render with num_threads threads; returns wall seconds and the number of
// samples per pixel actually taken (spp rounded up to a multiple of the thread count).
double r_render(r_scene const *s, uint32_t mode, uint32_t w, uint32_t h, uint32_t spp,
                uint32_t num_threads, float *rgba_out, uint32_t *samples_taken, int firefly) {
    e8::pt_image_renderer renderer(
        std::make_unique<e8::pathtracer_factory>(tracer_type(mode), e8::pathtracer_factory::options()),
        num_threads);
    mem_compositor comp(w, h);
    auto t0 = std::chrono::steady_clock::now();
    e8::pt_image_renderer::numerical_stats st =
        renderer.render(&comp, *s->bvh, *s->mc, *s->ls, *s->cam, spp, firefly != 0);
    auto t1 = std::chrono::steady_clock::now();
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++)
            for (int i = 0; i < 4; i++)
                rgba_out[4 * (y * w + x) + i] = comp(x, y)(i);
    *samples_taken = st.num_samples;
    return std::chrono::duration<double>(t1 - t0).count();
}

void r_bsdf_eval(r_scene const *s, int32_t m, float const n[3], float const o[3], float const i[3],
                 float f_out[3]) {
    e8::if_material const &mat =
        m < 0 ? s->mc->find(std::optional<e8::obj_id_t>()) : s->mc->find(s->mats[m]->id());
    e8util::vec3 f = mat.eval(e8util::vec2(), e8util::vec3{n[0], n[1], n[2]},
                              e8util::vec3{o[0], o[1], o[2]}, e8util::vec3{i[0], i[1], i[2]});
    for (int k = 0; k < 3; k++)
        f_out[k] = f(k);
}

void r_bsdf_sample(r_scene const *s, int32_t m, uint32_t seed, float const n[3], float const o[3],
                   uint32_t count, float *dirs_out, float *pdf_out) {
    e8::if_material const &mat =
        m < 0 ? s->mc->find(std::optional<e8::obj_id_t>()) : s->mc->find(s->mats[m]->id());
    e8util::rng rng(seed);
    for (uint32_t k = 0; k < count; k++) {
        float dens = -1;
        e8util::vec3 i = mat.sample(&rng, &dens, e8util::vec2(), e8util::vec3{n[0], n[1], n[2]},
                                    e8util::vec3{o[0], o[1], o[2]});
        for (int c = 0; c < 3; c++)
            dirs_out[3 * k + c] = i(c);
        pdf_out[k] = dens;
    }
}

void r_minstd_draws(uint32_t seed, uint32_t n, float *out) {
    e8util::rng rng(seed);
    for (uint32_t i = 0; i < n; i++)
        out[i] = rng.draw();
}

// The reference's uv_sphere generator (geometry.cpp:162-241): vertex, normal and index arrays.
uint32_t r_uv_sphere(float r, uint32_t res, int flip, float *pos_out, float *nrm_out, uint32_t *tris_out) {
    e8::uv_sphere sp("sphere", e8util::vec3{0.0f, 0.0f, 0.0f}, r, res, flip != 0);
    auto const &v = sp.vertices();
    auto const &n = sp.normals();
    auto const &t = sp.triangles();
    if (pos_out) {
        for (size_t i = 0; i < v.size(); i++)
            for (int k = 0; k < 3; k++) {
                pos_out[3 * i + k] = v[i](k);
                nrm_out[3 * i + k] = n[i](k);
            }
        for (size_t i = 0; i < t.size(); i++)
            for (int k = 0; k < 3; k++)
                tris_out[3 * i + k] = t[i](k);
    }
    return static_cast<uint32_t>(t.size());
}

// trimesh::transform (geometry.cpp:76-87) of a mesh given as vertex and normal arrays; returns 0
// when the reference throws (a singular matrix).
int r_transform_mesh(float const m[16], float const *pos, float const *nrm, uint32_t n, float *pos_out,
                     float *nrm_out) {
    e8::trimesh mesh("xform");
    std::vector<e8util::vec3> verts, norms;
    for (uint32_t v = 0; v < n; v++) {
        verts.push_back(e8util::vec3{pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]});
        norms.push_back(e8util::vec3{nrm[3 * v], nrm[3 * v + 1], nrm[3 * v + 2]});
    }
    mesh.vertices(verts);
    mesh.normals(norms);
    e8util::mat44 t;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            t(i, j) = m[4 * i + j];
    std::unique_ptr<e8::if_geometry> out;
    try {
        out = mesh.transform(t);
    } catch (std::string const &) {
        return 0;
    }
    auto const &tv = out->vertices();
    auto const &tn = out->normals();
    for (uint32_t v = 0; v < n; v++)
        for (int k = 0; k < 3; k++) {
            pos_out[3 * v + k] = tv[v](k);
            nrm_out[3 * v + k] = tn[v](k);
        }
    return 1;
}

// wavefront_obj::load_geometry (resource.cpp:137-255) of the file at `path`. Returns 1 and fills
// the counts (and the arrays when pos is not NULL: 3 floats per vertex for positions and normals,
// 2 for texcoords, 3 indices per triangle), or 0 when the reference throws (err receives the
// message).
int r_obj_load(char const *path, uint32_t *nv, uint32_t *nt, float *pos, float *nrm, float *uv, uint32_t *tris,
               char *err, uint32_t err_len) {
    std::string msg;
    try {
        std::shared_ptr<e8::if_geometry> g = e8util::wavefront_obj(path).load_geometry();
        if (!g) {
            msg = "cannot open";
        } else {
            auto const &v = g->vertices();
            auto const &n = g->normals();
            auto const &t = g->texcoords();
            auto const &f = g->triangles();
            *nv = static_cast<uint32_t>(v.size());
            *nt = static_cast<uint32_t>(f.size());
            if (pos) {
                for (size_t i = 0; i < v.size(); i++) {
                    for (int k = 0; k < 3; k++) {
                        pos[3 * i + k] = v[i](k);
                        nrm[3 * i + k] = n[i](k);
                    }
                    uv[2 * i] = t[i](0);
                    uv[2 * i + 1] = t[i](1);
                }
                for (size_t i = 0; i < f.size(); i++)
                    for (int k = 0; k < 3; k++)
                        tris[3 * i + k] = f[i](k);
            }
            return 1;
        }
    } catch (std::string const &e) {
        msg = e;
    } catch (std::exception const &e) {
        msg = e.what();
    }
    if (err && err_len)
        std::snprintf(err, err_len, "%s", msg.c_str());
    return 0;
}

uint32_t r_bvh_num_nodes(r_scene const *s) { return s->bvh->num_nodes(); }
uint32_t r_bvh_max_depth(r_scene const *s) { return s->bvh->max_depth(); }

// aces_compositor / clamp_compositor::commit (compositor.cpp:49-69) into a memory frame.
void r_composite(float const *rgba, uint32_t w, uint32_t h, uint32_t tonemap, int auto_exposure, float exposure,
                 uint8_t *out) {
    std::unique_ptr<e8::if_compositor> comp;
    if (tonemap == E8G_TONEMAP_ACES) {
        auto a = std::make_unique<e8::aces_compositor>(w, h);
        a->enable_auto_exposure(auto_exposure != 0);
        a->exposure(exposure);
        comp = std::move(a);
    } else {
        comp = std::make_unique<e8::clamp_compositor>(w, h);
    }
    for (uint32_t j = 0; j < h; j++)
        for (uint32_t i = 0; i < w; i++) {
            float const *c = &rgba[4 * (static_cast<size_t>(j) * w + i)];
            (*comp)(i, j) = e8::rgba_color({c[0], c[1], c[2], c[3]});
        }
    mem_frame frame(w, h);
    comp->commit(&frame);
    for (uint32_t j = 0; j < h; j++)
        for (uint32_t i = 0; i < w; i++)
            for (int k = 0; k < 4; k++)
                out[4 * (static_cast<size_t>(j) * w + i) + k] = frame(i, j)(k);
}

} // extern "C"
