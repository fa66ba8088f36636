// Compositing on the device (if_compositor::commit, compositor.cpp:29-98): the float image a
// render leaves in device memory becomes 8-bit RGBA without a round trip through the host.
//   k_log_luminance  aces_compositor::exposure: sum of log(luminance + 1e-3) and the count over
//                    pixels that are not all-zero (double accumulators, one atomic per warp)
//   k_composite      per pixel: clamp, or exposure + ACES filmic curve; then pow 1/2.2 * 255
// The reference sums the log-luminances sequentially in float; the device sums them in double
// in another order, so the exposure can differ in its last bits and a pixel on a rounding edge
// by one 8-bit step.
#include "../../include/e8g.h"
#include "api_internal.h"

namespace e8g {
namespace {

__device__ __forceinline__ bool all_zero(float4 c) { // vec == 0.0f, epsilon 1e-5 (tensor.h:14-16)
    return fabsf(c.x - 0.0f) <= 1e-5f && fabsf(c.y - 0.0f) <= 1e-5f && fabsf(c.z - 0.0f) <= 1e-5f &&
           fabsf(c.w - 0.0f) <= 1e-5f;
}

__global__ void k_log_luminance(float4 const *__restrict__ rgba, uint32_t npix, double *sum, unsigned long long *count) {
    double s = 0.0;
    unsigned long long n = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
        float4 c = rgba[i];
        if (!all_zero(c)) {
            float lum = c.x * 0.299f + c.y * 0.587f + c.z * 0.114f; // luminance, compositor.cpp:83-85
            s += static_cast<double>(logf(lum + 1e-3f));
            n++;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(~0u, s, off);
        n += __shfl_down_sync(~0u, n, off);
    }
    if ((threadIdx.x & 31u) == 0 && n) {
        atomicAdd(sum, s);
        atomicAdd(count, n);
    }
}

__device__ __forceinline__ unsigned char channel8(float c) { // pixel_of, compositor.cpp:29-38
    float x = c < 0.0f ? 0.0f : (c > 1.0f ? 1.0f : c);
    return static_cast<unsigned char>(__float2uint_rz(powf(x, 1.0f / 2.2f) * 255.0f));
}

__global__ void k_composite(float4 const *__restrict__ rgba, uint32_t npix, uint32_t tonemap, float exposure,
                            double const *sum, unsigned long long const *count, uchar4 *out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix)
        return;
    float e = exposure;
    if (sum) { // auto exposure: exp(sum / n), the mean taken in float as the reference does
        float m = static_cast<float>(*sum) / static_cast<float>(*count);
        e = expf(m);
    }
    float4 c = rgba[i];
    float v[4];
    if (tonemap == E8G_TONEMAP_ACES) { // aces_tonemap, compositor.cpp:71-81
        const float A = 2.51f, B = 0.03f, C = 2.43f, D = 0.59f, E = 0.14f;
        float in[3] = {c.x, c.y, c.z};
        for (int k = 0; k < 3; k++) {
            float x = in[k] * e;
            v[k] = x * (x * A + B) / (x * (x * C + D) + E);
        }
        v[3] = c.w;
    } else { // clamp_compositor: at_least(0).at_most(1) (tensor.h:277-289)
        float in[4] = {c.x, c.y, c.z, c.w};
        for (int k = 0; k < 4; k++) {
            float x = 0.0f > in[k] ? 0.0f : in[k];
            v[k] = 1.0f < x ? 1.0f : x;
        }
    }
    out[i] = make_uchar4(channel8(v[0]), channel8(v[1]), channel8(v[2]),
                         static_cast<unsigned char>(__float2uint_rz(v[3] * 255.0f)));
}

} // namespace

cudaError_t launch_composite(float const *d_rgba, uint32_t w, uint32_t h, e8g_composite_params const &cp,
                             uint8_t *d_out, double *d_scratch, cudaStream_t st) {
    uint32_t npix = w * h;
    double *sum = nullptr;
    unsigned long long *count = nullptr;
    auto const *in = reinterpret_cast<float4 const *>(d_rgba);
    if (cp.tonemap == E8G_TONEMAP_ACES && cp.auto_exposure) {
        sum = d_scratch;
        count = reinterpret_cast<unsigned long long *>(d_scratch + 1);
        cudaError_t e = cudaMemsetAsync(d_scratch, 0, 2 * sizeof(double), st);
        if (e != cudaSuccess)
            return e;
        int blocks = static_cast<int>(std::min<uint32_t>((npix + 255) / 256, 1024));
        k_log_luminance<<<blocks, 256, 0, st>>>(in, npix, sum, count);
    }
    k_composite<<<(npix + 255) / 256, 256, 0, st>>>(in, npix, cp.tonemap, cp.exposure, sum, count,
                                                     reinterpret_cast<uchar4 *>(d_out));
    return cudaGetLastError();
}

} // namespace e8g

using namespace e8g;

static e8g_status check_composite(e8g_ctx *c, float const *rgba, uint32_t w, uint32_t h, e8g_composite_params const *cp,
                                  void const *out) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    if (!rgba || !cp || !out)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL argument");
    if (w == 0 || h == 0 || static_cast<uint64_t>(w) * h > (1ull << 28))
        return fail(c, E8G_ERR_INVALID_ARG, "bad image size");
    if (cp->tonemap > E8G_TONEMAP_ACES)
        return fail(c, E8G_ERR_INVALID_ARG, "unknown tone map");
    return E8G_OK;
}

extern "C" e8g_status e8g_composite_dev(e8g_ctx *c, float const *d_rgba, uint32_t w, uint32_t h,
                                        e8g_composite_params const *cp, uint8_t *d_out, void *stream) {
    e8g_status s = check_composite(c, d_rgba, w, h, cp, d_out);
    if (s != E8G_OK)
        return s;
    cudaSetDevice(c->device);
    cudaError_t e = c->b_counts.reserve(64);
    if (e == cudaSuccess)
        e = launch_composite(d_rgba, w, h, *cp, d_out, static_cast<double *>(c->b_counts.ptr),
                             stream ? static_cast<cudaStream_t>(stream) : c->stream);
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "composite");
}

extern "C" e8g_status e8g_composite(e8g_ctx *c, float const *rgba, uint32_t w, uint32_t h,
                                    e8g_composite_params const *cp, uint8_t *out) {
    e8g_status s = check_composite(c, rgba, w, h, cp, out);
    if (s != E8G_OK)
        return s;
    cudaSetDevice(c->device);
    size_t npix = static_cast<size_t>(w) * h;
    cudaError_t e = c->b_io0.reserve(npix * 16);
    if (e == cudaSuccess)
        e = c->b_io1.reserve(npix * 4);
    if (e == cudaSuccess)
        e = c->b_counts.reserve(64);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->b_io0.ptr, rgba, npix * 16, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = launch_composite(static_cast<float const *>(c->b_io0.ptr), w, h, *cp, static_cast<uint8_t *>(c->b_io1.ptr),
                             static_cast<double *>(c->b_counts.ptr), c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, c->b_io1.ptr, npix * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "composite");
}
