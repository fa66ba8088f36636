// Wavefront integrator: slot arrays, queues and the per-bounce kernels (wavefront.cu).
#pragma once

#include "device.cuh"
#include "launch.h"

namespace e8g {

struct WfSlots {
    uint32_t capacity;
    uint32_t *state, *pixel, *sample, *out, *rng, *sid; // sid: scene index (many-scene wavefront)
    float4 *beta_pdf, *o, *hit; // o: direction towards the previous vertex | depth
    float4 *sh_o, *sh_d, *sh_c; // shadow queue: origin | out, direction | tmax, contribution
    float4 *ext_o, *ext_d;      // extension queue: origin | slot, direction
    float4 *vp, *vn;            // split form: completed vertex (position | mesh, normal | depth)
    void *counters;
    unsigned long long *next_path; // the path counter refills draw from (shared by the pools of a
                                   // concurrent wavefront; the pool's own counter otherwise)
};

size_t wf_total_bytes(uint32_t capacity);
WfSlots wf_carve(void *base, uint32_t capacity);
cudaError_t wf_init(WfSlots const &W, cudaStream_t st);
int wf_trace_blocks_per_sm(uint32_t layout, uint32_t threshold);
// threshold > 0: trace kernels refill idle lanes with new rays during traversal once that many
// lanes of a warp are idle; 0: one ray per thread.
// B: the scene table of a many-scene wavefront (eight-wide trees, threshold > 0), or null.
void wf_enqueue_bounce(DevScene const &S, RenderArgs const &A, FirstHit const *fh, WfSlots const &W, float4 *accum,
                       float *path_rgb, int shade_grid, int trace_grid, uint32_t threshold, uint64_t total_paths,
                       BatchDev const *B, cudaStream_t st, cudaEvent_t const *timing = nullptr,
                       uint32_t shade_variant = 0);
// Block shapes of the shading kernel (the tuner's choice): the number of them, the threads of
// one, and the grid of a bounce over `capacity` slots.
constexpr uint32_t kWfShadeVariants = 8;
int wf_shade_threads(uint32_t variant);
int wf_shade_grid(uint32_t variant, uint32_t capacity, int num_sms);
uint32_t *wf_busy_ptr(WfSlots const &W);
unsigned long long *wf_next_ptr(WfSlots const &W);
// The two halves of a bounce, for pools that interleave on two streams (concurrent wavefront):
// queue reset + shading, and the trace kernel(s); grids are given for the residency wanted.
void wf_enqueue_shade(DevScene const &S, RenderArgs const &A, FirstHit const *fh, WfSlots const &W, float4 *accum,
                      float *path_rgb, int shade_grid, uint64_t total_paths, cudaStream_t st, uint32_t shade_variant);
void wf_enqueue_trace(DevScene const &S, RenderArgs const &A, WfSlots const &W, float4 *accum, float *path_rgb,
                      int trace_grid, uint32_t threshold, cudaStream_t st);
// Shading block shape's resident blocks per SM.
int wf_shade_blocks(uint32_t variant);

} // namespace e8g
