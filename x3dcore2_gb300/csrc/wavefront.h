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

// A path's stream kept in a slot between bounces: minstd keeps its state word, Philox the number
// of draws taken (its 4-word block is regenerated on resume).
template <class R> struct RngSlot;
template <> struct RngSlot<RngMinstd> {
    __device__ static RngMinstd load(RenderArgs const &, uint32_t, uint32_t, uint32_t word) {
        RngMinstd r;
        r.x = word;
        return r;
    }
    __device__ static uint32_t store(RngMinstd const &r) { return r.x; }
    __device__ static RngMinstd fresh(RenderArgs const &, uint64_t mix, uint32_t px, uint32_t s) {
        RngMinstd r;
        r.seed(path_seed(mix, px, s));
        return r;
    }
};
template <> struct RngSlot<RngPhilox> {
    // the slot keeps the number of draws taken; the 4-word block is regenerated on resume
    __device__ static RngPhilox load(RenderArgs const &A, uint32_t px, uint32_t s, uint32_t drawn) {
        RngPhilox r;
        r.seed(A.seed, px, s);
        r.block = drawn >> 2;
        uint32_t skip = drawn & 3u;
        if (skip) {
            r.refill();
            for (uint32_t k = 0; k < skip; k++) {
                r.buf[0] = r.buf[1];
                r.buf[1] = r.buf[2];
                r.buf[2] = r.buf[3];
            }
            r.lane = skip;
        }
        return r;
    }
    __device__ static uint32_t store(RngPhilox const &r) { return r.lane == 4 ? r.block * 4 : (r.block - 1) * 4 + r.lane; }
    __device__ static RngPhilox fresh(RenderArgs const &A, uint64_t, uint32_t px, uint32_t s) {
        RngPhilox r;
        r.seed(A.seed, px, s);
        return r;
    }
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
// The queue counters' size, and the shadow queue's length in them: a producer outside the
// bounce loop (the split bidirectional form) fills sh_o / sh_d / sh_c and the count, then traces
// the queue with wf_enqueue_trace.
size_t wf_counters_bytes();
uint32_t *wf_shadow_count_ptr(WfSlots const &W);
uint32_t *wf_ext_count_ptr(WfSlots const &W);
// Zeroes the queue lengths, fetch heads and busy count (not the path counter) before a bounce.
void wf_enqueue_reset(WfSlots const &W, cudaStream_t st);

// The split form of E8G_MODE_BDPT_POWER (bdpt.cu). The walk: one bounce over the slots of W
// (advance every slot's path by one subpath vertex, refill finished slots from the chunk), whose
// extension queue wf_enqueue_trace then traces; range: the chunk's first path index and path
// count in device memory. The connections: one thread per entry [first, first + n) of the chunk's
// list into the shadow queue of Q (its counters zeroed beforehand, sh_* arrays sized for n
// entries), which wf_enqueue_trace then drains.
void launch_bdpt_walk(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float *path_rgb, BdwChunk const &C,
                      WfSlots const &W, uint64_t const *range, int grid, cudaStream_t st);
void launch_bdpt_eval(DevScene const &S, float4 *accum, float *path_rgb, BdwChunk const &C, WfSlots const &Q,
                      uint32_t first, uint32_t n, int grid, cudaStream_t st);
int bdpt_eval_blocks_per_sm();
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
