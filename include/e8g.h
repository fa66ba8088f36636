/*
 * e8g.h — C ABI of the GB300 path-tracing core.
 *
 * Every entry point returns an e8g_status and never throws. Pointers are plain host pointers
 * unless the function name ends in `_dev`, in which case they are CUDA device pointers and the
 * call is asynchronous on the stream passed in (NULL = the context's own stream).
 *
 * The entry points replace, one for one, the reference interfaces of e8yescg's corelib
 * (paths relative to the reference project):
 *
 *   e8g_scene_upload + e8g_scene_build_bvh
 *       if_path_space::load / bvh_path_space_layout::commit   corelib/src/pathspace.cpp:15-19, :292-328
 *       if_material_container::load                           corelib/src/materialcontainer.cpp:19-23
 *       if_light_sources::load / basic_light_sources::commit  corelib/src/lightsources.cpp:11-18, :45-52
 *       camera_container / pinhole_camera::transform          corelib/src/camera.cpp:63-71
 *   e8g_trace_closest   bvh_path_space_layout::intersect      corelib/src/pathspace.cpp:330-413
 *   e8g_trace_any       bvh_path_space_layout::has_intersect  corelib/src/pathspace.cpp:415-456
 *   e8g_camera_rays     pinhole_camera::sample                corelib/src/camera.cpp:38-48
 *   e8g_render          pt_image_renderer::render             corelib/src/renderer.cpp:106-166
 *   e8g_render_paths    if_path_tracer::sample (one ray per call, as the reference's own
 *                       furnace test drives it)              corelib/src/pathtracer.h:59-63,
 *                                                            corelib/test/tst_pathtracer/tst_pathtracer.cpp:58-86
 *   e8g_scene_update_mesh / e8g_scene_transform_mesh / e8g_scene_commit
 *                       objdb::push_updates + actuator commit  corelib/src/objdb.cpp:59-87,
 *                       trimesh::transform                     corelib/src/geometry.cpp:76-87
 *   e8g_composite       aces_compositor / clamp_compositor     corelib/src/compositor.cpp:29-98
 *   e8g_obj_load        wavefront_obj::load_geometry           corelib/src/resource.cpp:137-255
 *   e8g_pipeline_*      pt_render_pipeline                     corelib/src/pipeline.cpp:73-185
 *   e8g_forward / e8g_backward, e8g_batch_render: no counterpart in the reference (new).
 */
#ifndef E8G_H
#define E8G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum e8g_status {
    E8G_OK = 0,
    E8G_ERR_INVALID_ARG = 1,
    E8G_ERR_CUDA = 2,
    E8G_ERR_OUT_OF_MEMORY = 3,
    E8G_ERR_NO_SCENE = 4,
    E8G_ERR_NOT_BUILT = 5,
    E8G_ERR_UNSUPPORTED = 6,
    E8G_ERR_TIMEOUT = 7,
    E8G_ERR_INTERNAL = 8,
    E8G_ERR_NO_DEVICE = 9,
    E8G_ERR_CANCELLED = 10 /* e8g_cancel stopped the call; its outputs are unspecified */
} e8g_status;

typedef struct e8g_ctx e8g_ctx;

typedef struct e8g_device_opts {
    int device;     /* CUDA ordinal */
    uint32_t flags; /* reserved, 0 */
} e8g_device_opts;

/* ---------------------------------------------------------------- scene ---- */

/* Material types: corelib/src/material.h:96-199. */
enum {
    E8G_MAT_FAIL_SAFE = 0,  /* mat_fail_safe: Lambert rho=0.8, no cosine cut   material.cpp:54-76 */
    E8G_MAT_OREN_NAYAR = 1, /* oren_nayar(albedo, sigma)                       material.cpp:108-169 */
    E8G_MAT_COOK_TORR = 2,  /* cook_torr(albedo, roughness, complex ior)       material.cpp:171-252 */
    E8G_MAT_MIXTURE = 3     /* mat_mixture(mix0, mix1, ratio)                   material.cpp:78-106 */
};

typedef struct e8g_material {
    uint32_t type;
    float albedo[3];
    float roughness; /* oren_nayar: sigma; cook_torr: r, alpha^2 = 2 r^2 (material.cpp:176) */
    float ior_re;    /* cook_torr complex index of refraction */
    float ior_im;
    int32_t mix0; /* mixture: indices of two non-mixture materials */
    int32_t mix1;
    float ratio; /* mixture: probability of mix0 */
} e8g_material;

/* area_light on a mesh of the scene: light.cpp:17-71. */
typedef struct e8g_light {
    uint32_t mesh;
    float radiance[3];
} e8g_light;

/* pinhole_camera after transform(): camera.cpp:23-30, :63-71.
 * rot is the 3x3 upper-left block of the camera transform, row-major. */
typedef struct e8g_camera {
    float origin[3];
    float rot[9];
    float sensor_size;
    float focal_len;
    float aspect;
} e8g_camera;

/*
 * A scene is a list of triangle meshes (corelib trimesh), given in the order of the reference
 * path space's std::map, i.e. ascending object id. Meshes are already in world space.
 * Lights are given in ascending object id order (the order basic_light_sources::commit walks).
 * All arrays are caller-owned host memory and are copied by e8g_scene_upload.
 */
typedef struct e8g_scene_desc {
    uint32_t num_meshes;
    const uint32_t *mesh_vert_offset; /* num_meshes + 1 prefix offsets into positions/normals */
    const uint32_t *mesh_tri_offset;  /* num_meshes + 1 prefix offsets into triangles */
    const int32_t *mesh_material;     /* per mesh: index into materials, -1 = fail-safe */
    const float *positions;           /* 3 * V */
    const float *normals;             /* 3 * V */
    const uint32_t *triangles;        /* 3 * T, mesh-local vertex indices */
    uint32_t num_materials;
    const e8g_material *materials;
    uint32_t num_lights;
    const e8g_light *lights;
    e8g_camera camera;
} e8g_scene_desc;

/* Build options of the SAH layouts. e8g_default_bvh_opts gives values tuned for the GPU traversal
 * (8, 32, 0, 1: a triangle cost <= 0 takes the layout's tuned value, 1 for SAH pairs and 3 for the
 * eight-wide tree); the reference's own constants are 4, 20, 8, 1 (pathspace.cpp:121-124). The
 * reference layout ignores them: it always builds the reference's tree. */
typedef struct e8g_bvh_opts {
    uint32_t max_leaf_prims; /* largest leaf (reference BVH_MAX_PRIMS = 4) */
    uint32_t num_bins;       /* SAH bins per axis, 2..64 (reference BVH_BUCKET_COUNT = 20) */
    float tri_cost;          /* SAH triangle-test cost (reference BVH_RAY_TRIANGLE_COST = 8); <= 0: tuned */
    float node_cost;         /* SAH box-test cost (reference BVH_RAY_BOX_COST = 1) */
    uint32_t num_threads;    /* host build threads, 0 = all */
    uint32_t layout;         /* E8G_BVH_SAH, E8G_BVH_REFERENCE, E8G_BVH_WIDE or E8G_BVH_LINEAR */
    uint32_t builder;        /* E8G_BUILDER_HOST or E8G_BUILDER_DEVICE (SAH pairs and eight-wide) */
} e8g_bvh_opts;

enum {
    E8G_BUILDER_HOST = 0,  /* binned SAH on the host threads */
    E8G_BUILDER_DEVICE = 1 /* on the GPU from the device's vertices: Morton order, PLOC clustering
                              (radius 24), SAH leaf collapse (leaves of at most min(max_leaf_prims,
                              15) triangles); no host round trip for SAH pairs, the eight-wide
                              collapse then runs on the host. Falls back to the host builder when
                              the tree would be deeper than the traversal stack */
};

enum {
    E8G_BVH_SAH = 0,       /* binned SAH over 3 axes, child pairs, ordered traversal */
    E8G_BVH_REFERENCE = 1, /* the reference's own tree and visiting order (pathspace.cpp:121-456):
                              hit identities match the reference bit for bit, ties included */
    E8G_BVH_WIDE = 2,      /* the SAH tree collapsed to eight-wide nodes with quantized child
                              boxes (96 bytes per node), octant-ordered traversal: the fastest */
    E8G_BVH_LINEAR = 3     /* no tree: every triangle in mesh order, the first of equal distances
                              kept (linear_path_space_layout, pathspace.cpp:36-114); for tiny
                              scenes and as the reference's brute-force ground truth */
};

typedef struct e8g_bvh_stats {
    uint32_t num_nodes;
    uint32_t num_leaves;
    uint32_t max_depth;
    uint32_t num_tris;
    double avg_leaf_depth;
    double build_ms;
    uint64_t node_bytes;  /* bytes of the node array (32 per binary node, 96 per wide node) */
    uint64_t tri_bytes;
    uint32_t layout;      /* the layout built (E8G_BVH_WIDE falls back to E8G_BVH_SAH when its
                             tree would be deeper than the traversal stack) */
} e8g_bvh_stats;

/* ----------------------------------------------------------- traversal ---- */

typedef struct e8g_ray {
    float o[3];
    float d[3];
} e8g_ray;

/* Closest hit. mesh = -1 on a miss. b1, b2 are the barycentrics of ray::intersect
 * (corelib/src/tensor.h:688-725); b0 = 1 - b1 - b2. */
typedef struct e8g_hit {
    float t;
    int32_t mesh;
    int32_t tri; /* mesh-local triangle index */
    float b1;
    float b2;
} e8g_hit;

/* ------------------------------------------------------------- render ---- */

enum {
    E8G_MODE_REF_UNI = 0,     /* unidirect_path_tracer        pathtracer.cpp:528-585 */
    E8G_MODE_REF_LT1 = 1,     /* unidirect_lt1_path_tracer    pathtracer.cpp:587-653 */
    E8G_MODE_MIS = 2,         /* NEE + BSDF sampling, power-heuristic MIS (new) */
    E8G_MODE_REF_BDPT = 3,    /* bidirect_mis_path_tracer     pathtracer.cpp:754-803 */
    E8G_MODE_BDPT_POWER = 4,  /* bidirectional, power-heuristic MIS (new) */
    E8G_MODE_REF_DIRECT = 5,  /* direct_path_tracer           pathtracer.cpp:508-526 */
    E8G_MODE_NORMAL = 6,      /* normal_tracer                pathtracer.cpp:492-506 */
    E8G_MODE_POSITION = 7,    /* position_tracer              pathtracer.cpp:474-490 */
    E8G_MODE_REF_LT2 = 8      /* bidirect_lt2_path_tracer     pathtracer.cpp:655-752 */
};

enum {
    E8G_INTEGRATOR_MEGAKERNEL = 0, /* persistent threads; a lane whose path ends takes the next one */
    E8G_INTEGRATOR_WAVEFRONT = 1,  /* E8G_MODE_MIS: queues of path slots, bounce loop as a CUDA graph;
                                      E8G_MODE_BDPT_POWER: the split form, subpaths sampled by one
                                      kernel and every (t, s) connection evaluated by one thread of
                                      another; other modes: the megakernel */
    E8G_INTEGRATOR_PLAIN = 2       /* one thread per path for its whole length: the baseline kernel */
};

enum {
    E8G_RNG_MINSTD = 0, /* the reference's std::minstd_rand0 stream, one stream per path */
    E8G_RNG_PHILOX = 1  /* Philox4x32-10 counter-based stream */
};

typedef struct e8g_render_params {
    uint32_t mode;
    uint32_t integrator;
    uint32_t rng;
    uint32_t width;
    uint32_t height;
    uint32_t spp;
    uint64_t seed;
    uint32_t max_depth;     /* 0 = unlimited (the reference) */
    uint32_t rr_start;      /* first depth with Russian roulette (reference: 2) */
    float rr_prob;          /* survival probability (reference: 0.5) */
    uint32_t bdpt_max_len;  /* subpath vertex cap (reference: 8, pathtracer.h:201) */
    uint32_t firefly;       /* nonzero: pt_image_renderer's 8-neighbour firefly clamp on every
                               sample image (renderer.cpp:46-83); not taken by
                               e8g_render_dev_noalloc or e8g_batch_render */
    uint32_t sample_offset; /* first sample index (progressive rendering) */
} e8g_render_params;

/* Fill p with the reference's defaults for a mode: rr_start 2 (1 for E8G_MODE_REF_LT2, the
 * reference's mutate_depth of that tracer), rr_prob 0.5, unlimited depth, bdpt_max_len 8, minstd
 * stream for reference modes and Philox otherwise. */
void e8g_default_params(e8g_render_params *p, uint32_t mode, uint32_t width, uint32_t height,
                        uint32_t spp);

/* Per-path seed of the minstd stream for (seed, pixel, sample): the value an oracle feeds to
 * e8util::rng(unsigned) so both sides draw the same sequence. */
uint32_t e8g_path_seed(uint64_t seed, uint32_t pixel, uint32_t sample);

typedef struct e8g_render_stats {
    double ms;          /* device time of the render, CUDA events */
    double kernel_ms;   /* device time of the dominant kernel */
    uint64_t paths;
    uint64_t rays;      /* extension + shadow rays traced (when counted) */
    uint64_t nodes;     /* BVH nodes whose box was fetched (when counted) */
    uint64_t tris;      /* triangles tested (when counted) */
    uint32_t launches;  /* kernels launched by the call */
    uint32_t counted;   /* 1 when rays/nodes/tris are filled */
    double trace_ms;    /* wavefront only, with e8g_set_kernel_timing on: device time of its trace
                           kernels over the render (CUDA events around each launch); else 0 */
    double shade_ms;    /* the same for its shading kernels (queue reset included) */
    uint32_t trace_launches; /* trace kernels the wavefront launched (when timed) */
    uint32_t pad_;
} e8g_render_stats;

/* ------------------------------------------------------------ batch ---- */

typedef struct e8g_batch_item {
    const e8g_scene_desc *scene;
    e8g_render_params params;
    float *rgba_out; /* host, width*height*4 */
} e8g_batch_item;

/* ------------------------------------------------------- compositing ---- */

/* Tone mapping of a float RGBA image to 8-bit pixels (if_compositor::commit,
 * compositor.cpp:29-98): clamp_compositor clamps every channel to [0, 1]; aces_compositor
 * multiplies RGB by the exposure and applies the ACES filmic curve, alpha unchanged. Both then
 * write pow(clamp(c, 0, 1), 1 / 2.2) * 255 truncated (alpha: a * 255 truncated). */
enum { E8G_TONEMAP_CLAMP = 0, E8G_TONEMAP_ACES = 1 };
typedef struct e8g_composite_params {
    uint32_t tonemap;       /* E8G_TONEMAP_* */
    uint32_t auto_exposure; /* ACES: exposure = exp(mean log(luminance + 1e-3)) over the pixels not
                               all-zero (aces_compositor::exposure, compositor.cpp:87-98) */
    float exposure;         /* ACES without auto exposure */
} e8g_composite_params;

/* ----------------------------------------------------------- functions ---- */

e8g_status e8g_create(e8g_ctx **ctx, const e8g_device_opts *opts);
e8g_status e8g_destroy(e8g_ctx *ctx);
const char *e8g_last_error(const e8g_ctx *ctx);
const char *e8g_version(void);

e8g_status e8g_scene_upload(e8g_ctx *ctx, const e8g_scene_desc *desc);
e8g_status e8g_scene_build_bvh(e8g_ctx *ctx, const e8g_bvh_opts *opts);
e8g_status e8g_bvh_get_stats(const e8g_ctx *ctx, e8g_bvh_stats *stats);
/* Copies the device tree to host memory: nodes_out receives stats.node_bytes (SAH pairs and the
 * reference layout: num_nodes float4 (min xyz | link) followed by num_nodes float4
 * (max xyz | count); eight-wide: num_nodes records of 96 bytes), tris_out stats.tri_bytes (per
 * triangle position: v0 | triangle id, v1 - v0, v2 - v0 as three float4). Either may be NULL. */
e8g_status e8g_bvh_read(e8g_ctx *ctx, void *nodes_out, void *tris_out);
void e8g_default_bvh_opts(e8g_bvh_opts *opts);

e8g_status e8g_camera_rays(e8g_ctx *ctx, uint32_t width, uint32_t height, e8g_ray *rays_out);

e8g_status e8g_trace_closest(e8g_ctx *ctx, const e8g_ray *rays, uint32_t n, e8g_hit *hits);
e8g_status e8g_trace_any(e8g_ctx *ctx, const e8g_ray *rays, const float *t_min, const float *t_max,
                         uint32_t n, uint8_t *occluded);
e8g_status e8g_trace_closest_dev(e8g_ctx *ctx, const e8g_ray *d_rays, uint32_t n, e8g_hit *d_hits,
                                 void *stream);

/* Image render: rgba_out is host memory of width*height*4 floats (alpha = 1). */
e8g_status e8g_render(e8g_ctx *ctx, const e8g_render_params *params, float *rgba_out);
/* Same, writing a device buffer; the caller synchronises. */
e8g_status e8g_render_dev(e8g_ctx *ctx, const e8g_render_params *params, float *d_rgba_out,
                          void *stream);
/* Progressive rendering on the device: adds params->spp samples per call to the context's
 * accumulator, continuing the sample sequence (sample indices params->sample_offset + samples
 * already accumulated), and writes the running mean to d_rgba_out. The accumulator restarts
 * when reset is nonzero, when the image size changes, and after any other render of the
 * context or a scene or material change (those reuse or invalidate it). Four calls of 16 spp
 * give the image of one 64-spp render. No firefly clamp. */
e8g_status e8g_render_progressive(e8g_ctx *ctx, const e8g_render_params *params, int reset, float *d_rgba_out,
                                  void *stream);
e8g_status e8g_get_render_stats(const e8g_ctx *ctx, e8g_render_stats *stats);
/* Nonzero: the wavefront integrator records CUDA events around its shading and trace kernels of
 * every bounce (event-record nodes in its bounce graph) and fills trace_ms / shade_ms of the
 * render stats. A measurement aid with no counterpart in the reference; off by default. */
e8g_status e8g_set_kernel_timing(e8g_ctx *ctx, int on);
/* Measurement aid: the GPU's L2 read bandwidth in GB/s (*gbs), from `reps` passes of a streaming
 * kernel over a buffer of `bytes` (>= 1 MiB, allocated and freed by the call) that fits in L2 —
 * the second denominator of the traversal roofline. No counterpart in the reference. */
e8g_status e8g_l2_read_bandwidth(e8g_ctx *ctx, uint64_t bytes, uint32_t reps, double *gbs);

/* ------------------------------------------------- robustness and control ---- *
 * None of these has a counterpart in the reference, whose errors are C++ exceptions. */

/* Checks a scene description the way e8g_scene_upload does, without a GPU: sizes, indices,
 * material and light references, finite positions, normals, camera, material and light values,
 * and a positive total light power. Returns E8G_OK, or E8G_ERR_INVALID_ARG with the reason in msg
 * (msg_cap bytes, may be NULL). */
e8g_status e8g_scene_validate(const e8g_scene_desc *desc, char *msg, size_t msg_cap);

/* Caps the device memory the context's buffers may hold (0 = no limit, the default). An upload,
 * build or render that would need more fails with E8G_ERR_OUT_OF_MEMORY, as a failed cudaMalloc
 * does, and the context stays usable: a failed upload or build leaves no scene or no tree (the
 * next render reports E8G_ERR_NO_SCENE or E8G_ERR_NOT_BUILT) until one succeeds. For callers
 * with a memory budget, and for testing the out-of-memory paths. */
e8g_status e8g_set_memory_limit(e8g_ctx *ctx, uint64_t bytes);
/* Device memory the context's buffers hold now. */
e8g_status e8g_memory_used(const e8g_ctx *ctx, uint64_t *bytes);

/* Asks the call running on the context (from another host thread), or the next one, to stop:
 * it returns E8G_ERR_CANCELLED after its kernels in flight have finished, at its next host-side
 * step (between wavefront graph replays, firefly sample chunks, tuner renders, batch scenes) or
 * at its start. A single kernel is never interrupted. The request is consumed by the call that
 * honours it. */
e8g_status e8g_cancel(e8g_ctx *ctx);

/* Checkpoint of progressive rendering (e8g_render_progressive): the running sums of the
 * accumulator (width * height float4, rgb sums and sample weight), its image size and the samples
 * taken. e8g_progressive_save with accum = NULL only reports the size and samples.
 * e8g_progressive_load puts a saved state back (same scene, same parameters), after which
 * progressive calls continue the sample sequence where the saved one stopped: the resumed image
 * equals the uninterrupted one up to the order of float additions. */
e8g_status e8g_progressive_save(e8g_ctx *ctx, float *accum, uint32_t *width, uint32_t *height, uint64_t *spp);
e8g_status e8g_progressive_load(e8g_ctx *ctx, const float *accum, uint32_t width, uint32_t height, uint64_t spp);

/* Wavefront autotuner: times the wavefront integrator for each candidate slot capacity
 * {2^20 .. 2^24}, bounces per graph {2, 4} and warp refill threshold {4, 8, 12, 16, 24} (the
 * number of idle lanes at which a trace kernel hands its idle lanes new rays) on a short render
 * of `params` (at most 8 spp), then each capacity's fastest pair again on a render of at most 64
 * spp (long renders favour large slot pools), and keeps the fastest of those for this context
 * and its current tree. cand_ms are the short renders' times. Without it: 2^21 slots, 4 bounces
 * per graph, threshold 16. */
#define E8G_TUNE_MAX_CANDIDATES 64
typedef struct e8g_tune_result {
    uint32_t capacity;          /* chosen number of path slots */
    uint32_t bounces_per_graph; /* chosen bounces captured in one CUDA graph */
    uint32_t threshold;         /* chosen warp refill threshold of the trace kernels (0 = off) */
    uint32_t num_candidates;
    uint32_t cand_capacity[E8G_TUNE_MAX_CANDIDATES];
    uint32_t cand_bounces[E8G_TUNE_MAX_CANDIDATES];
    uint32_t cand_threshold[E8G_TUNE_MAX_CANDIDATES];
    double cand_ms[E8G_TUNE_MAX_CANDIDATES];
    uint32_t shade_variant;     /* chosen shape of the shading kernel (0 .. num_shade - 1) */
    uint32_t num_shade;         /* shapes timed */
    double shade_ms[8];         /* device time of the render with each shape */
    uint32_t from_cache;        /* e8g_wavefront_tune_cached: 1 when the choice came from the file */
    uint32_t concurrent;        /* chosen: 1 = two slot pools interleaving on two streams */
    double concurrent_ms[2];    /* device time of the render with one pool and with two */
} e8g_tune_result;
e8g_status e8g_wavefront_tune(e8g_ctx *ctx, const e8g_render_params *params, e8g_tune_result *result);
/* Sets the wavefront configuration directly: slot capacity (1024 .. 2^26), bounces captured per
 * graph (1 .. 16) and warp refill threshold (0 .. 32). */
e8g_status e8g_wavefront_set(e8g_ctx *ctx, uint32_t capacity, uint32_t bounces_per_graph, uint32_t threshold);
/* Shape of the wavefront's shading kernel (threads x resident blocks per SM, register cap, the
 * materials' code inlined or out of line): 0 = 256 x 4 (64 registers), 1 = 256 x 3 (80),
 * 2 = 256 x 4 out of line, 3 = 256 x 3 out of line, 4 = 256 x 5 (48) out of line, 5 = 128 x 8 (64)
 * out of line; 6 = 256 x 4 and 7 = 256 x 5 in the split form, where a small kernel first turns
 * the extension hits into vertices and adds their emission, and the shading kernel reads them. */
e8g_status e8g_wavefront_set_shade(e8g_ctx *ctx, uint32_t variant);
/* Nonzero: the wavefront splits its slots into two pools that interleave on two streams, one
 * pool shading while the other traces, each kernel at half of an SM's residency, so shading
 * (latency-bound) and tracing (issue-bound) overlap on every SM. The same paths and image. */
e8g_status e8g_wavefront_set_concurrent(e8g_ctx *ctx, int on);
/* e8g_wavefront_tune with a cache of choices in a JSON file (`cache_path`): the key is the scene
 * and frame size bucket (tree layout, stream kind, log2 of the triangle count, of the pixels and of
 * min(spp, 64)). A key found in the file sets its configuration without tuning (result->from_cache
 * = 1); otherwise the tuner runs and its choice is added to the file (written to a temporary file
 * and renamed over it). A missing or unreadable file counts as empty. No counterpart in the
 * reference. */
e8g_status e8g_wavefront_tune_cached(e8g_ctx *ctx, const e8g_render_params *params, const char *cache_path,
                                     e8g_tune_result *result);

/* Largest image (width * height) e8g_render_dev_noalloc accepts. */
#define E8G_NOALLOC_MAX_PIXELS 65536u

/* Same render as e8g_render_dev, but it allocates no device memory: its scratch (first-hit cache,
 * accumulator, counters) lives in one statically sized device array, 4 MiB held on every GPU
 * that loads the library until exit. For callers that cannot call cudaMalloc at render time
 * (cudaMalloc synchronises the device and can fail once a process has budgeted all of its device
 * memory up front). No counterpart in the reference.
 *   - width * height must not exceed E8G_NOALLOC_MAX_PIXELS (else E8G_ERR_INVALID_ARG);
 *   - the scene must already be uploaded and built (those calls allocate, once, beforehand);
 *   - the first call on a device looks up the array's device address: make it before any
 *     stream capture;
 *   - all calls share the one array: calls that overlap on the GPU race, so serialise them;
 *   - E8G_INTEGRATOR_WAVEFRONT renders with the persistent megakernel here, and
 *     E8G_MODE_BDPT_POWER with its one-thread-per-path kernel (the slot pool and the subpath
 *     buffers would need memory); the paths, and so the image, are the same;
 *     E8G_INTEGRATOR_PLAIN runs the plain kernel; the firefly clamp is refused
 *     (E8G_ERR_UNSUPPORTED);
 *   - the array's address is cached per device: a cudaDeviceReset frees the array with every
 *     other allocation of that device, and the library must not be called on that device again
 *     in this process.
 * Asynchronous on `stream` (NULL = the context's stream); the caller synchronises. */
e8g_status e8g_render_dev_noalloc(e8g_ctx *ctx, const e8g_render_params *params, float *d_rgba_out,
                                  void *stream);
/* Runs the render once with traversal counters on (not for timing) and returns the number of
 * rays traced, BVH nodes whose box was fetched and triangles tested. Every mode but
 * E8G_MODE_REF_LT2 (E8G_ERR_UNSUPPORTED); the wavefront integrator is counted through the
 * megakernel, which traces the same rays. */
e8g_status e8g_count_traversal(e8g_ctx *ctx, const e8g_render_params *params, e8g_render_stats *stats);

/* Per-path radiance for explicit primary rays (if_path_tracer::sample, pathtracer.h:59-63): path i
 * starts at ray i, whose first hit is traced as compute_first_hit traces it (back-facing hits are
 * misses, pathtracer.cpp:456-472), and draws from the stream of (params->seed, i,
 * params->sample_offset). params->width and height are ignored. rgb_out is 3*n floats. */
e8g_status e8g_render_rays(e8g_ctx *ctx, const e8g_render_params *params, const e8g_ray *rays, uint32_t n,
                           float *rgb_out);

/* Per-path radiance for an explicit list of (pixel, sample) pairs: rgb_out is 3*n floats. */
e8g_status e8g_render_paths(e8g_ctx *ctx, const e8g_render_params *params, const uint32_t *pixel,
                            const uint32_t *sample, uint32_t n, float *rgb_out);

/* Differentiable render (path-replay adjoint). e8g_forward renders like e8g_render and keeps
 * the parameters; e8g_backward replays every path and accumulates dLoss/d(albedo) (3 floats per
 * material) and dLoss/d(roughness) (1 float per material) given dLoss/d(image) (width*height*3).
 * Gradients are with respect to e8g_material::albedo and e8g_material::roughness. */
e8g_status e8g_forward(e8g_ctx *ctx, const e8g_render_params *params, float *rgba_out);
e8g_status e8g_backward(e8g_ctx *ctx, const float *dl_dimage, float *d_albedo, float *d_roughness);
/* Overwrite material parameters of the uploaded scene without re-uploading geometry. */
e8g_status e8g_set_materials(e8g_ctx *ctx, const e8g_material *materials, uint32_t n);

/* Composite a float RGBA image (width*height*4) into 8-bit RGBA pixels (width*height*4 bytes).
 * _dev: device buffers on `stream` (the caller synchronises); the host form copies in and out.
 * Replaces aces_compositor / clamp_compositor::commit into an if_frame (compositor.cpp:49-69). */
e8g_status e8g_composite(e8g_ctx *ctx, const float *rgba, uint32_t width, uint32_t height,
                         const e8g_composite_params *params, uint8_t *pixels_out);
e8g_status e8g_composite_dev(e8g_ctx *ctx, const float *d_rgba, uint32_t width, uint32_t height,
                             const e8g_composite_params *params, uint8_t *d_pixels_out, void *stream);

/* Render many independent scenes together; each item has its own scene, parameters and output.
 * When every item asks for E8G_INTEGRATOR_WAVEFRONT with E8G_MODE_MIS and the same stream kind,
 * the scenes get eight-wide trees and share the wavefront's path slots (one graph-captured
 * bounce loop over all scenes, with the context's wavefront settings); otherwise one persistent
 * megakernel launch runs every path on SAH-pair trees. Unidirectional modes only; no firefly
 * clamp. The scenes stay independent of the context's uploaded scene. */
e8g_status e8g_batch_render(e8g_ctx *ctx, const e8g_batch_item *items, uint32_t n,
                            e8g_render_stats *stats);

/* ------------------------------------------------- incremental updates ---- */

/* Scene changes between renders without a new e8g_scene_upload: the counterpart of
 * objdb::push_updates (objdb.cpp:59-87), which unloads and reloads every dirty object through its
 * actuator and then commits (bvh_path_space_layout::commit rebuilds the whole tree). Here only the
 * changed meshes travel to the device, and e8g_scene_commit brings the tree up to date on the
 * device. Meshes keep their vertex and triangle counts; a different topology needs an upload.
 * After any of these calls renders and traces fail with E8G_ERR_NOT_BUILT until the next
 * e8g_scene_commit (or e8g_scene_build_bvh). */

/* Replaces the vertex positions (3 floats per vertex of the mesh) and, unless normals is NULL,
 * the normals of mesh `mesh`: the mesh's new blueprint. Its area, the light powers and the light
 * CDF are recomputed as e8g_scene_upload computes them (trimesh::update, geometry.cpp:105-124;
 * basic_light_sources::commit, lightsources.cpp:45-52), so update + commit renders what an upload
 * of the changed scene renders. */
e8g_status e8g_scene_update_mesh(e8g_ctx *ctx, uint32_t mesh, const float *positions, const float *normals);

/* trimesh::transform (geometry.cpp:76-87) of mesh `mesh` on the device, from its blueprint (the
 * vertices of the last upload or e8g_scene_update_mesh; transforms do not compound). m is the 4x4
 * matrix, row-major (m[4*i + j] = row i, column j). Positions become (m * (v, 1)).cart(); normals
 * become (~(m ^ -1) * (n, 1)).cart() with the reference's cofactor inverse, a w divide included
 * (flags 0), or the inverse transpose applied to (n, 0) (flags E8G_XFORM_NORMALS_AS_DIRECTIONS).
 * The mesh keeps its blueprint area for light sampling, as the reference's transformed copy does
 * (transform calls update_aabb only). |det m| <= 1e-5 is E8G_ERR_INVALID_ARG, the reference's
 * "matrix not invertible" (tensor.h:511-540). */
enum { E8G_XFORM_REFERENCE = 0, E8G_XFORM_NORMALS_AS_DIRECTIONS = 1 };
e8g_status e8g_scene_transform_mesh(e8g_ctx *ctx, uint32_t mesh, const float m[16], uint32_t flags);

/* Replaces the camera (camera_container::load after pinhole_camera::transform, camera.cpp:63-71).
 * The tree is unaffected: no commit needed. */
e8g_status e8g_scene_set_camera(e8g_ctx *ctx, const e8g_camera *camera);

/* Reads back a mesh's current world-space vertices (3 floats per vertex each; either may be NULL). */
e8g_status e8g_scene_get_mesh(e8g_ctx *ctx, uint32_t mesh, float *positions, float *normals);

/* Brings the tree up to date with the changed meshes.
 * E8G_COMMIT_REFIT keeps the tree's topology and recomputes, on the device, every triangle record
 * and every box bottom-up (one pass; a refit of an unchanged scene writes exactly the bytes of the
 * build). The tree's quality degrades as geometry moves far from where it was built; rebuild then.
 * E8G_COMMIT_REBUILD builds a new tree on the host with the last build options.
 * The reference layout (E8G_BVH_REFERENCE) always rebuilds, as the reference does on every commit,
 * so its hit identities stay the reference's; the linear layout rewrites its triangle records. stats (may be NULL) receives the tree's statistics;
 * its build_ms is the commit's time. */
enum { E8G_COMMIT_REFIT = 0, E8G_COMMIT_REBUILD = 1 };
e8g_status e8g_scene_commit(e8g_ctx *ctx, uint32_t mode, e8g_bvh_stats *stats);

/* -------------------------------------------------------------- pipeline ---- */

/* One frame of the render pipeline (pt_render_pipeline::render_frame, pipeline.cpp:73-101): the
 * scene changes since the last frame committed (objdb::push_updates: a refit, or a build when the
 * layout changed), samples_per_frame samples rendered, the ACES compositor applied
 * (aces_compositor, compositor.cpp:71-98), 8-bit RGBA returned. The reference re-renders every
 * frame from the same streams; with `progressive` the frames instead continue the sample sequence
 * and accumulate until the scene, the camera or the settings change. */
typedef struct e8g_pipeline_config {
    uint32_t mode;              /* "path_tracer" */
    uint32_t layout;            /* "path_space" */
    uint32_t samples_per_frame; /* "samples_per_frame" */
    uint32_t firefly_filter;    /* "firefly_filter" */
    uint32_t auto_exposure;     /* "auto_exposure" */
    float exposure;             /* "exposure" */
    uint32_t num_threads;       /* "num_threads": host build threads, 0 = all */
    uint32_t progressive;       /* "progressive" (new) */
    uint32_t integrator;        /* "integrator" (new): megakernel, wavefront or plain */
    uint64_t seed;              /* "seed" (new) */
} e8g_pipeline_config;

/* The reference's defaults (pt_render_pipeline::config_protocol, pipeline.cpp:103-121):
 * unidirectional, static_bvh, 64 samples per frame, no firefly filter, fixed exposure 1. */
void e8g_pipeline_config_default(e8g_pipeline_config *cfg);

/* flex_config-style setting by name and value (pipeline.cpp:123-185):
 *   path_tracer        normal | position | direct | unidirectional | unidirectional_lt1 |
 *                      bidirectional_lt2 | bidirectional_mis, and mis | bidirectional_power (new)
 *   path_space         static_bvh (SAH pairs), linear (E8G_BVH_LINEAR), reference_bvh,
 *                      wide_bvh (new)
 *   light_sources      basic
 *   auto_exposure, firefly_filter, progressive       true | false | 1 | 0
 *   exposure (float), samples_per_frame (> 0), num_threads, super_samples (accepted, unused, as
 *   in the reference), seed, integrator (megakernel | wavefront | plain)
 * Anything else is E8G_ERR_INVALID_ARG ("scene_file": scenes come from e8g_obj_load or
 * e8g_gen_scene and e8g_scene_upload). */
e8g_status e8g_pipeline_config_set(e8g_pipeline_config *cfg, const char *key, const char *value);

/* pixels_out: host, width*height*4 bytes; rgba_out (may be NULL): host, the float image before
 * compositing. */
e8g_status e8g_pipeline_frame(e8g_ctx *ctx, const e8g_pipeline_config *cfg, uint32_t width, uint32_t height,
                              uint8_t *pixels_out, float *rgba_out);

/* ------------------------------------------------------------- OBJ ingest ---- */

/* One triangle mesh read from a Wavefront OBJ file with the reference's rules
 * (wavefront_obj::load_geometry, resource.cpp:137-255): "v", "vn", "vt" and triangular "f a/b/c"
 * lines, matched as the reference's regular expressions match them (other lines are ignored;
 * polygons with more corners are errors); per vertex, the normal and texcoord of the last face
 * corner naming it, zero when none does. A file whose faces omit a texcoord or normal index,
 * which the reference reads out of bounds, is refused. Host memory owned by the library. */
typedef struct e8g_host_mesh e8g_host_mesh;
typedef struct e8g_mesh_data {
    uint32_t num_vertices;
    uint32_t num_triangles;
    const float *positions;    /* 3 * num_vertices */
    const float *normals;      /* 3 * num_vertices */
    const float *texcoords;    /* 2 * num_vertices */
    const uint32_t *triangles; /* 3 * num_triangles, 0-based */
} e8g_mesh_data;
/* err (may be NULL) receives a message of at most err_len bytes on failure. */
e8g_status e8g_obj_load(const char *path, e8g_host_mesh **out, char *err, size_t err_len);
e8g_status e8g_obj_parse(const char *text, size_t len, e8g_host_mesh **out, char *err, size_t err_len);
e8g_status e8g_host_mesh_data(const e8g_host_mesh *mesh, e8g_mesh_data *data);
void e8g_host_mesh_free(e8g_host_mesh *mesh);

/* Host-side scene generators (no GPU needed): fill a scene owned by the library. */
typedef struct e8g_host_scene e8g_host_scene;
enum {
    E8G_GEN_CORNELL = 0,        /* unit Cornell box, two rotated boxes, 0.25^2 light */
    E8G_GEN_DISPLACED_ICO = 1,  /* displaced icosphere on a ground plane, 4 quad lights */
    E8G_GEN_SOUP = 2,           /* random triangle soup in an enclosing box */
    E8G_GEN_FURNACE = 3         /* inward uv_sphere, Lambert 0.7, L = 1 (tst_pathtracer.cpp:24-56) */
};
typedef struct e8g_gen_opts {
    uint32_t kind;
    uint64_t seed;
    uint32_t level;         /* icosphere subdivision level / uv_sphere resolution */
    uint32_t num_tris;      /* soup size */
    uint32_t num_materials; /* icosphere materials */
    float amplitude;        /* displacement amplitude */
    float roughness_lo, roughness_hi;
    uint32_t width, height; /* camera aspect */
} e8g_gen_opts;
e8g_status e8g_gen_scene(const e8g_gen_opts *opts, e8g_host_scene **out);
e8g_status e8g_host_scene_desc(const e8g_host_scene *s, e8g_scene_desc *desc);
void e8g_host_scene_free(e8g_host_scene *s);

#ifdef __cplusplus
}
#endif

#endif /* E8G_H */
