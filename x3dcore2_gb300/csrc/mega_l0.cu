// Megakernel instantiations for SAH child pairs (layout 0).
#include "mega.cuh"

namespace e8g {

void launch_mega_l0(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                    unsigned long long *work, unsigned long long *counters, int grid, bool plain, cudaStream_t st) {
    launch_layout<0>(S, A, fh, accum, path_rgb, work, counters, grid, plain, st);
}

int megakernel_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mega<RngPhilox, false, 0>, kBlock, 0);
    return n > 0 ? n : 1;
}

} // namespace e8g
