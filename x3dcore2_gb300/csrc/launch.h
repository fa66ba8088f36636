// Kernel launchers (defined in the .cu files, called by the C ABI in api.cu).
#pragma once

#include "../../include/e8g.h"
#include "device.cuh"

namespace e8g {

struct LaunchCfg {
    int grid;
    cudaStream_t stream;
};

void launch_first_hits(DevScene const &S, uint32_t w, uint32_t h, FirstHit *out, cudaStream_t st);
void launch_camera_rays(DevScene const &S, uint32_t w, uint32_t h, float *rays6, cudaStream_t st);
// First hits of explicit rays (ray i into out[i]) and the lists that make path i start there:
// pixel[i] = i, samples[i] = sample.
void launch_first_hits_rays(DevScene const &S, float const *rays6, uint32_t n, FirstHit *out, uint32_t sample,
                            uint32_t *pixel, uint32_t *samples, cudaStream_t st);
void launch_trace_closest(DevScene const &S, float const *rays6, uint32_t n, float *hits5, cudaStream_t st);
void launch_trace_any(DevScene const &S, float const *rays6, float const *tmin, float const *tmax, uint32_t n,
                      uint8_t *occ, cudaStream_t st);
void launch_trace_closest_counted(DevScene const &S, float const *rays6, uint32_t n, float *hits5,
                                  unsigned long long *counters, cudaStream_t st);
void launch_resolve(float4 const *accum, uint32_t npix, float inv_spp, float *rgba, cudaStream_t st);
// Firefly clamp of K sample-major per-sample images (W*H rgb each), added to accum in sample order.
void launch_firefly(float const *est, uint32_t K, uint32_t w, uint32_t h, float4 *accum, cudaStream_t st);

// Megakernel integrator (one thread per path, persistent threads refilled warp-wide).
// counters (when non-null): [0] rays, [1] nodes, [2] tris.
// plain: the baseline one-thread-per-path kernel instead (E8G_INTEGRATOR_PLAIN; not with counters).
void launch_megakernel(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                       unsigned long long *work, unsigned long long *counters, int grid, cudaStream_t st,
                       bool plain = false);
int megakernel_blocks_per_sm();
// The same for one tree layout (mega_l0.cu: SAH pairs, mega_l1.cu: reference, mega_l2.cu: wide,
// mega_l3.cu: linear).
void launch_mega_l0(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                    unsigned long long *work, unsigned long long *counters, int grid, bool plain, cudaStream_t st);
void launch_mega_l1(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                    unsigned long long *work, unsigned long long *counters, int grid, bool plain, cudaStream_t st);
void launch_mega_l2(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                    unsigned long long *work, unsigned long long *counters, int grid, bool plain, cudaStream_t st);
void launch_mega_l3(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                    unsigned long long *work, unsigned long long *counters, int grid, bool plain, cudaStream_t st);

// Many scenes, one persistent launch (SAH-pair or eight-wide trees, any stream kind).
struct BatchDev {
    DevScene const *scenes;      // per scene
    RenderArgs const *args;      // per scene
    uint64_t const *path_prefix; // n + 1 prefix sums of each scene's path count
    uint64_t const *pix_prefix;  // n + 1 prefix sums of each scene's pixel count
    uint32_t n;
    uint64_t total_paths;
};
// rng_kinds: bit (1 << E8G_RNG_*) set for every stream kind some scene of the batch uses.
void launch_megakernel_batch(BatchDev const &B, FirstHit const *fh_all, float4 *accum_all, unsigned long long *work,
                             uint32_t rng_kinds, int grid, cudaStream_t st);
int megakernel_batch_blocks_per_sm(uint32_t rng_kinds);
void launch_first_hits_batch(BatchDev const &B, DevScene const *h_scenes, RenderArgs const *h_args,
                             uint64_t const *h_pix_prefix, FirstHit *fh_all, cudaStream_t st);
void launch_resolve_batch(BatchDev const &B, uint64_t total_pix, float4 const *accum_all, float *rgba_all,
                          cudaStream_t st);

// Compositing of a device float RGBA image into 8-bit pixels (composite.cu); d_scratch holds 8
// doubles for the exposure sum.
cudaError_t launch_composite(float const *d_rgba, uint32_t w, uint32_t h, e8g_composite_params const &cp,
                             uint8_t *d_out, double *d_scratch, cudaStream_t st);

// Bidirectional path tracing (uniform or power-heuristic weights), one thread per path.
// counters (or null): the instrumented run (bidirectional modes; rays, node boxes, triangles).
void launch_bdpt(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                 unsigned long long *work, int grid, cudaStream_t st, unsigned long long *counters = nullptr);
int bdpt_blocks_per_sm();

// The split form of E8G_MODE_BDPT_POWER (E8G_INTEGRATOR_WAVEFRONT): a chunk of `count` paths
// starting at path index `first` (at most kBdwMaxChunk), subpaths of at most max_len vertices.
constexpr uint32_t kBdwMaxChunk = 1u << 26; // keeps a chunk's connection count within 32 bits
struct BdwChunk {
    float4 *vtx;      // per path: max_len camera then max_len light vertices, three float4 each
    int4 *info;       // per path: (clen | llen << 8, light, output index, 0)
    float4 *o0;       // per path: the direction back along the camera ray
    uint64_t *conn;   // connection entries: path << 10 | (t - 1) << 5 | s
    uint32_t *conn_n; // entry count (zeroed before each chunk)
    uint32_t max_len;
    uint32_t count;
    uint64_t first;
};

} // namespace e8g
