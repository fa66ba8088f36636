// Megakernel instantiations for the linear layout (layout 3: every triangle, in order).
#include "mega.cuh"

namespace e8g {

void launch_mega_l3(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                    unsigned long long *work, unsigned long long *counters, int grid, bool plain, cudaStream_t st) {
    launch_layout<3>(S, A, fh, accum, path_rgb, work, counters, grid, plain, st);
}

} // namespace e8g
