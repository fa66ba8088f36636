// e8g_corelib.h — reference-side adapters: corelib's own interfaces implemented on top of the
// e8g C ABI, so that an e8yescg build renders on the GPU by swapping containers and the renderer.
//
// Compiled inside (or against) corelib: it includes corelib's headers. Replaces, one for one:
//   bvh_path_space_layout      -> gpu_path_space_layout   (pathspace.h:71-186)
//   default_material_container -> gpu_material_container  (materialcontainer.h:44-56)
//   basic_light_sources        -> gpu_light_sources       (lightsources.h:42-63)
//   pinhole_camera             -> gpu_pinhole_camera      (camera.h:28-52)
//   oren_nayar / cook_torr     -> gpu_oren_nayar / gpu_cook_torr (material.h:139-199)
//   pt_image_renderer::render  -> gpu_image_renderer::render     (renderer.h:57-59)
// The reference keeps material and camera parameters private, so the GPU-side classes remember
// their constructor arguments and pack them; everything else is read through public or
// protected members the subclasses can see.
#pragma once

#include "e8g.h"

#include "camera.h"
#include "compositor.h"
#include "lightsources.h"
#include "material.h"
#include "materialcontainer.h"
#include "pathspace.h"
#include "pathtracerfact.h"
#include "renderer.h"

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace e8g_corelib {

// Implemented by materials whose parameters can be handed to the GPU.
class packable_material {
  public:
    virtual ~packable_material() = default;
    virtual e8g_material pack() const = 0;
};

class gpu_oren_nayar : public e8::oren_nayar, public packable_material {
  public:
    gpu_oren_nayar(std::string const &name, e8util::vec3 const &albedo, float sigma);
    std::unique_ptr<e8::if_material> copy() const override;
    e8g_material pack() const override;

  private:
    e8util::vec3 m_albedo_copy;
    float m_sigma_copy;
};

class gpu_cook_torr : public e8::cook_torr, public packable_material {
  public:
    gpu_cook_torr(std::string const &name, e8util::vec3 const &albedo, float roughness,
                  std::complex<float> const &ior);
    std::unique_ptr<e8::if_material> copy() const override;
    e8g_material pack() const override;

  private:
    e8util::vec3 m_albedo_copy;
    float m_roughness_copy;
    std::complex<float> m_ior_copy;
};

class gpu_material_container : public e8::default_material_container {
  public:
    // Material table in the order of `ids`; unknown ids and non-packable materials become the
    // fail-safe material, as if_material_container::find would return it.
    std::vector<e8g_material> pack(std::vector<e8::obj_id_t> const &ids) const;
};

class gpu_path_space_layout : public e8::bvh_path_space_layout {
  public:
    // Flat geometry in the order of the path space's map (ascending object id).
    struct packed {
        std::vector<uint32_t> voff{0}, toff{0};
        std::vector<float> pos, nrm;
        std::vector<uint32_t> tris;
        std::vector<e8::obj_id_t> geo_ids;
        std::vector<std::optional<e8::obj_id_t>> mat_ids;
    };
    packed pack() const;
};

class gpu_light_sources : public e8::basic_light_sources {
  public:
    // Area lights in id order (the order basic_light_sources::commit walks), each bound to the
    // index of its geometry in `geo_ids`; radiance recovered as radiance(n, n).
    std::vector<e8g_light> pack(std::vector<e8::obj_id_t> const &geo_ids) const;
};

class gpu_pinhole_camera : public e8::pinhole_camera {
  public:
    gpu_pinhole_camera(std::string const &name, float sensor_size, float f, float aspect);
    std::unique_ptr<e8::if_camera> copy() const override;
    std::unique_ptr<e8::if_camera> transform(e8util::mat44 const &trans) const override;
    e8g_camera pack() const;

  private:
    float m_sensor, m_f, m_aspect;
    e8util::mat44 m_trans = e8util::mat44_scale(1.0f);
};

// Builds the e8g scene description the containers describe (host arrays owned by `storage`).
struct scene_storage {
    gpu_path_space_layout::packed geo;
    std::vector<e8g_material> mats;
    std::vector<int32_t> mesh_mat;
    std::vector<e8g_light> lights;
    e8g_scene_desc desc{};
};
void pack_scene(gpu_path_space_layout const &ps, gpu_material_container const &mats,
                gpu_light_sources const &lights, gpu_pinhole_camera const &cam, scene_storage &out);

// The e8g mode of a tracer type (pathtracerfact.h:12): unidirect -> E8G_MODE_REF_UNI,
// unidirect_lt1 -> E8G_MODE_REF_LT1, bidirect_mis -> E8G_MODE_REF_BDPT, bidirect_lt2 ->
// E8G_MODE_REF_LT2, direct, normal, position.
uint32_t mode_of(e8::pathtracer_factory::pt_type type);

// if_path_tracer on the GPU (pathtracer.h:59-63), for code that drives tracers one batch of rays
// at a time (the reference's own tests do): sample() traces every ray's path on the context,
// whose scene the caller uploaded from the same containers (pack_scene + e8g_scene_upload +
// e8g_scene_build_bvh). Path i's first hit is computed on the device from ray i, as
// compute_first_hit computes the cached ones; its stream is keyed by one draw of `rng` and i.
class gpu_path_tracer : public e8::if_path_tracer {
  public:
    gpu_path_tracer(e8g_ctx *ctx, e8::pathtracer_factory::pt_type type);
    std::vector<e8util::vec3> sample(e8util::rng &rng, std::vector<e8util::ray> const &rays,
                                     first_hits const &first_hits, e8::if_path_space const &path_space,
                                     e8::if_material_container const &mats,
                                     e8::if_light_sources const &light_sources) const override;

  private:
    e8g_ctx *m_ctx;
    uint32_t m_mode;
};

// pt_image_renderer on the GPU: same render() signature and meaning; the tracer type selects
// the integrator (unidirect -> E8G_MODE_REF_UNI, unidirect_lt1 -> E8G_MODE_REF_LT1,
// bidirect_mis -> E8G_MODE_REF_BDPT, direct, normal, position).
class gpu_image_renderer {
  public:
    gpu_image_renderer(e8::pathtracer_factory::pt_type type, int device = 0);
    ~gpu_image_renderer();

    e8::pt_image_renderer::numerical_stats render(e8::if_compositor *compositor, e8::if_path_space const &path_space,
                                                   e8::if_material_container const &mats,
                                                   e8::if_light_sources const &light_sources, e8::if_camera const &cam,
                                                   unsigned num_samps, bool firefly_filter);

  private:
    // Brings the context's scene up to date with `next`: a full upload and build when the scene's
    // structure changed (meshes, triangles, lights), otherwise only the meshes whose vertices
    // changed are uploaded and the tree is refitted (objdb::push_updates, objdb.cpp:59-87, followed
    // by the path space's commit), and camera and materials are replaced when they changed.
    void commit_scene(scene_storage &next);

    e8::pathtracer_factory::pt_type m_type;
    e8g_ctx *m_ctx = nullptr;
    scene_storage m_scene;
    bool m_have_scene = false;
    uint64_t m_frame = 0;
};

} // namespace e8g_corelib
