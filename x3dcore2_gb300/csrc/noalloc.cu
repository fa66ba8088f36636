// e8g_render_dev_noalloc: an image render that allocates no device memory.
//
// Why it exists: e8g_render and e8g_render_dev grow per-context scratch buffers (the per-pixel
// first-hit cache and the radiance accumulator) with cudaMalloc the first time an image of a
// given size is rendered. Some callers cannot allow that at render time: cudaMalloc synchronises
// the whole device and can fail when the process has already budgeted every byte of device
// memory up front (a real-time viewer holding a fixed pool, a host that shares the GPU with an
// allocator it does not own, a frame loop that must never stall on a device-wide sync). For
// them, this entry point keeps its scratch in one statically sized __device__ array that exists
// from module load until process exit, so a render never asks the driver for memory.
//
// Limits and rules:
//  * width * height <= E8G_NOALLOC_MAX_PIXELS (65,536 pixels, e.g. 256 x 256); larger images are
//    rejected with E8G_ERR_INVALID_ARG. The array is 64 bytes per pixel plus 256 bytes of
//    counters: 4 MiB held on every GPU that loads the library, until exit.
//  * Inputs (the scene uploaded with e8g_scene_upload / e8g_scene_build_bvh, which do allocate,
//    once, ahead of time) and the output (d_rgba_out, caller-owned device memory) stay the
//    caller's.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (host code may not use the array's name as a device pointer); make
//    that first call before any stream capture.
//  * Every call on a device shares the one array and leaves the last call's contents in it; each
//    call clears what must start at zero. Two calls that overlap on the GPU (other streams,
//    other contexts on the same device, other host threads) race on the array: serialise them.
//  * E8G_INTEGRATOR_WAVEFRONT runs as the persistent megakernel, and E8G_MODE_BDPT_POWER as its
//    one-thread-per-path kernel (the wavefront's slot pool and the split form's subpath buffers
//    are allocated memory); they render the same paths from the same streams, so the image is
//    the same. E8G_INTEGRATOR_PLAIN runs the plain kernel.
//  * The address looked up per device stays cached for the life of the process. A
//    cudaDeviceReset frees the array with every other allocation on that device; after one, the
//    library must not be used on that device again.
#include "api_internal.h"

#include <mutex>

namespace e8g {
namespace {

constexpr size_t kNoallocPixels = E8G_NOALLOC_MAX_PIXELS;
constexpr size_t kCounterBytes = 256;
constexpr size_t kScratchBytes = kCounterBytes + kNoallocPixels * (sizeof(FirstHit) + sizeof(float4));

// The scratch: [work counter | first hits | accumulator], 256-byte aligned.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
unsigned char *g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

// Device address of the scratch on the current device (looked up once per device).
cudaError_t scratch_address(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return e;
        g_scratch_ptr[device] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[device];
    return cudaSuccess;
}

} // namespace
} // namespace e8g

using namespace e8g;

extern "C" e8g_status e8g_render_dev_noalloc(e8g_ctx *c, e8g_render_params const *p, float *d_rgba_out,
                                             void *stream) {
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, p);
    if (s != E8G_OK)
        return s;
    if (!d_rgba_out)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL output");
    size_t npix = static_cast<size_t>(p->width) * p->height;
    if (npix > kNoallocPixels)
        return fail(c, E8G_ERR_INVALID_ARG, "e8g_render_dev_noalloc: image larger than E8G_NOALLOC_MAX_PIXELS (65536)");
    if (p->firefly)
        return fail(c, E8G_ERR_UNSUPPORTED, "e8g_render_dev_noalloc: the firefly clamp needs per-sample image buffers");
    cudaError_t e = cudaSetDevice(c->device);
    unsigned char *base = nullptr;
    if (e == cudaSuccess)
        e = scratch_address(c->device, &base);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "no-alloc scratch");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    auto *work = reinterpret_cast<unsigned long long *>(base);
    auto *fh = reinterpret_cast<FirstHit *>(base + kCounterBytes);
    auto *accum = reinterpret_cast<float4 *>(base + kCounterBytes + kNoallocPixels * sizeof(FirstHit));

    e = cudaMemsetAsync(work, 0, kCounterBytes, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(accum, 0, npix * sizeof(float4), st);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "no-alloc clear");
    launch_first_hits(c->dev, p->width, p->height, fh, st);
    RenderArgs A = make_args(p);
    if (A.mode == E8G_MODE_REF_BDPT || A.mode == E8G_MODE_BDPT_POWER || A.mode == E8G_MODE_REF_LT2)
        launch_bdpt(c->dev, A, fh, accum, nullptr, work, persistent_grid(c, bdpt_blocks_per_sm()), st);
    else
        launch_megakernel(c->dev, A, fh, accum, nullptr, work, nullptr, persistent_grid(c, megakernel_blocks_per_sm()),
                          st, p->integrator == E8G_INTEGRATOR_PLAIN);
    launch_resolve(accum, static_cast<uint32_t>(npix), p->spp ? 1.0f / static_cast<float>(p->spp) : 0.0f,
                   d_rgba_out, st);
    e = cudaGetLastError();
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "no-alloc render launch");
}
