// Path-replay adjoint (adjoint.cu).
#pragma once

#include "device.cuh"

namespace e8g {

// Accumulates dLoss/d(albedo) (3 per material) and dLoss/d(roughness) into device arrays given
// dLoss/d(image) (3 floats per pixel); path_rgb (optional) receives each path's radiance.
cudaError_t launch_adjoint(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float const *dl_dimage,
                           float inv_spp, unsigned long long *work, float *d_albedo, float *d_rough, float *path_rgb,
                           int num_sms, cudaStream_t st);

} // namespace e8g
