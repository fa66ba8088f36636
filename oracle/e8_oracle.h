/*
 * e8_oracle.h — CPU restatement of e8yescg corelib's per-pixel path integral.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker that the CUDA path is compared against, and the
 * CPU stand-in for the reference when the reference itself cannot be built (on the GPU host).
 * The product never links, loads or calls it.
 *
 * Every function restates the reference's arithmetic in the same operation order (no FMA
 * contraction: built with -ffp-contract=off), so that, built the same way, it reproduces the
 * compiled reference bit for bit on the same inputs and the same draw sequence. Each function
 * cites the reference file:line it follows (paths relative to the reference project).
 */
#ifndef E8_ORACLE_H
#define E8_ORACLE_H

#include "../include/e8g.h"
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct o_scene o_scene;

/* Policy knobs: defaults reproduce the reference exactly (unlimited depth, Russian roulette from
 * depth 2 with survival 0.5, BDPT subpaths of at most 8 vertices). */
typedef struct o_policy {
    uint32_t max_depth;
    uint32_t rr_start;
    float rr_prob;
    uint32_t bdpt_max_len;
} o_policy;

typedef struct o_hit {
    float t;
    int32_t mesh;
    int32_t tri;
    float b1, b2;
    float vertex[3];
    float normal[3];
} o_hit;

o_scene *o_scene_create(const e8g_scene_desc *desc);
void o_scene_free(o_scene *s);
/* BVH statistics of the reference-style build: nodes, max depth. */
void o_bvh_stats(const o_scene *s, uint32_t *num_nodes, uint32_t *max_depth, uint32_t *num_leaves);

/* Closest hit, pathspace.cpp:330-413 (use_bvh=1) or :36-92 (use_bvh=0). */
void o_trace_closest(const o_scene *s, const e8g_ray *rays, uint32_t n, int use_bvh, o_hit *hits);
/* Any hit in [t_min, t_max], pathspace.cpp:415-456 / :94-114. */
void o_trace_any(const o_scene *s, const e8g_ray *rays, const float *t_min, const float *t_max,
                 uint32_t n, int use_bvh, uint8_t *occluded);
/* Traversal work counters for closest-hit (nodes whose box was tested, triangles tested). */
void o_trace_closest_counts(const o_scene *s, const e8g_ray *rays, uint32_t n, uint64_t *nodes,
                            uint64_t *tris);

/* pinhole_camera::sample for every pixel, camera.cpp:38-48. rays: width*height. */
void o_camera_rays(const o_scene *s, uint32_t width, uint32_t height, e8g_ray *rays);

/* Per-path radiance. Each path (pixel, stream seed) runs the integrator `mode` (E8G_MODE_*) on
 * the pixel's camera ray with its first hit, drawing from a fresh std::minstd_rand0-equivalent
 * stream seeded with seeds[k] (rng kind E8G_RNG_MINSTD) or from Philox keyed by (seed, pixel,
 * sample) (E8G_RNG_PHILOX, then seeds[] holds sample indices and `seed` the key). */
void o_render_paths(const o_scene *s, uint32_t mode, uint32_t rng_kind, uint64_t seed,
                    const o_policy *pol, uint32_t width, uint32_t height, const uint32_t *pixel,
                    const uint32_t *seeds, uint32_t n, float *rgb_out, int num_threads);

/* Image: for each pixel p and sample k < spp, path seed e8g-compatible (seed, p, k + offset);
 * rgba_out = mean radiance, alpha 1. Rows are spread over num_threads threads. */
void o_render(const o_scene *s, uint32_t mode, uint32_t rng_kind, uint64_t seed,
              const o_policy *pol, uint32_t width, uint32_t height, uint32_t spp,
              uint32_t sample_offset, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
              float *rgba_out, int num_threads);

/* The firefly clamp of pt_image_renderer (renderer.cpp:46-83) on one sample image est (w*h
 * rgb), added to acc (w*h rgb). */
void o_firefly_add(const float *est, uint32_t w, uint32_t h, float *acc);
/* pt_image_renderer::render with one sampling task whose sequential minstd stream is seeded
 * task_seed (renderer.cpp:35-166): rgba_out as the reference's compositor holds it. */
void o_render_task(const o_scene *s, uint32_t mode, const o_policy *pol, uint32_t w, uint32_t h, uint32_t spp,
                   int firefly, uint32_t task_seed, float *rgba_out);

/* The reference's compositors (compositor.cpp:29-98) on a float RGBA image: tonemap
 * E8G_TONEMAP_CLAMP or E8G_TONEMAP_ACES (auto exposure or the given one); 8-bit RGBA out. */
void o_composite(const float *rgba, uint32_t w, uint32_t h, uint32_t tonemap, int auto_exposure, float exposure,
                 unsigned char *out);

/* Seed of the per-path minstd stream; the same function as e8g_path_seed. */
/* trimesh::transform (geometry.cpp:76-87) of n vertices by the row-major 4x4 matrix m:
 * positions (m * (p, 1)).cart(), normals (~(m ^ -1) * (n, 1)).cart() with mat::operator^(-1)'s
 * cofactor inverse (tensor.h:451-540). Returns 0 when |det m| <= 1e-5 (the reference throws
 * "matrix not invertible"), 1 otherwise. */
int o_transform_mesh(const float m[16], const float *pos, const float *nrm, uint32_t n, float *pos_out,
                     float *nrm_out);

uint32_t o_path_seed(uint64_t seed, uint32_t pixel, uint32_t sample);
/* First n draws of the minstd stream with this seed (tensor.h:987-1001 + libstdc++
 * generate_canonical<float>). */
void o_minstd_draws(uint32_t seed, uint32_t n, float *out);
void o_philox_draws(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t n, float *out);

/* BSDF of material index m (-1 = fail-safe): eval f(o, i) and a sample with its density,
 * material.cpp:54-252. */
void o_bsdf_eval(const o_scene *s, int32_t m, const float n[3], const float o[3], const float i[3],
                 float f_out[3]);
void o_bsdf_sample(const o_scene *s, int32_t m, uint32_t seed, const float n[3], const float o[3],
                   uint32_t count, float *dirs_out, float *pdf_out);

/* Double-precision path-replay gradient of one path's radiance (mode E8G_MODE_MIS, Philox
 * stream), dL/dalbedo (3 per material) and dL/droughness (1 per material), weighted by the
 * upstream gradient w[3] of the path's pixel and accumulated into the outputs. */
void o_path_gradient_f64(const o_scene *s, uint64_t seed, const o_policy *pol, uint32_t width,
                         uint32_t height, uint32_t pixel, uint32_t sample, const float w[3],
                         double *d_albedo, double *d_roughness, double rgb_out[3]);
/* The sum of o_path_gradient_f64 over every pixel of a width x height image and samples
 * 0 .. spp - 1, each path weighted by dl[3 * pixel ..] / spp; d_albedo (3 per material) and
 * d_roughness are overwritten. num_threads threads. */
void o_image_gradient_f64(const o_scene *s, uint64_t seed, const o_policy *pol, uint32_t width,
                          uint32_t height, uint32_t spp, const float *dl, double *d_albedo,
                          double *d_roughness, int num_threads);

#ifdef __cplusplus
}
#endif

#endif
