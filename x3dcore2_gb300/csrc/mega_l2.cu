// Megakernel instantiations for the eight-wide tree (layout 2).
#include "mega.cuh"

namespace e8g {

void launch_mega_l2(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                    unsigned long long *work, unsigned long long *counters, int grid, bool plain, cudaStream_t st) {
    launch_layout<2>(S, A, fh, accum, path_rgb, work, counters, grid, plain, st);
}

} // namespace e8g
