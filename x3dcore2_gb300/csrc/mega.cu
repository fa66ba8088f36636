// Megakernel dispatch and the many-scene megakernel (e8g_batch_render); the per-layout
// integrator kernels are instantiated in mega_l0.cu (SAH pairs), mega_l1.cu (reference tree)
// and mega_l2.cu (eight-wide).
#include "mega.cuh"

namespace e8g {

// rng_kinds: bit E8G_RNG_MINSTD / bit E8G_RNG_PHILOX set when some scene of the batch uses it.
void launch_megakernel_batch(BatchDev const &B, FirstHit const *fh_all, float4 *accum_all, unsigned long long *work,
                             uint32_t rng_kinds, int grid, cudaStream_t st) {
    if (rng_kinds == (1u << E8G_RNG_PHILOX))
        k_mega_batch<RngPhilox><<<grid, kBlock, 0, st>>>(B, fh_all, accum_all, work);
    else if (rng_kinds == (1u << E8G_RNG_MINSTD))
        k_mega_batch<RngMinstd><<<grid, kBlock, 0, st>>>(B, fh_all, accum_all, work);
    else
        k_mega_batch<RngAny><<<grid, kBlock, 0, st>>>(B, fh_all, accum_all, work);
}

int megakernel_batch_blocks_per_sm(uint32_t rng_kinds) {
    int n = 0;
    if (rng_kinds == (1u << E8G_RNG_PHILOX))
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mega_batch<RngPhilox>, kBlock, 0);
    else if (rng_kinds == (1u << E8G_RNG_MINSTD))
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mega_batch<RngMinstd>, kBlock, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mega_batch<RngAny>, kBlock, 0);
    return n > 0 ? n : 1;
}


void launch_megakernel(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                       unsigned long long *work, unsigned long long *counters, int grid, cudaStream_t st, bool plain) {
    if (S.layout == 1)
        launch_mega_l1(S, A, fh, accum, path_rgb, work, counters, grid, plain, st);
    else if (S.layout == 2)
        launch_mega_l2(S, A, fh, accum, path_rgb, work, counters, grid, plain, st);
    else if (S.layout == 3)
        launch_mega_l3(S, A, fh, accum, path_rgb, work, counters, grid, plain, st);
    else
        launch_mega_l0(S, A, fh, accum, path_rgb, work, counters, grid, plain, st);
}

} // namespace e8g
