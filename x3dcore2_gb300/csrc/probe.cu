// Measurement aid: the L2 read bandwidth of this GPU, measured with a plain streaming kernel, as
// the second denominator of the traversal roofline. Tree nodes and triangles are read through
// L1/L2 (ld.global.nc); most of them hit L2, whose bandwidth, not HBM's, bounds a traversal whose
// working set fits there. No counterpart in the reference.
#include "api_internal.h"

namespace e8g {
namespace {

// Every thread streams 16-byte words of a buffer that fits in L2 with loads cached in L2 only
// (ld.global.cg: L1 would serve a block's repeated reads), four independent loads in flight.
// Pass r starts each block at another offset so that blocks do not walk the buffer in lockstep.
__global__ void __launch_bounds__(256) k_l2_read(uint4 const *__restrict__ buf, size_t n16, int reps,
                                                 unsigned *sink) {
    uint32_t acc = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (int r = 0; r < reps; r++) {
        size_t start = (static_cast<size_t>(blockIdx.x) * blockDim.x * 4 + static_cast<size_t>(r) * 7919 * 256) % n16;
        size_t i = start + threadIdx.x;
        for (size_t k = 0; k < n16; k += 4 * stride) {
            uint4 a[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                size_t j = i + k + u * stride;
                j = j >= n16 ? j - n16 : j;
                j = j >= n16 ? j % n16 : j;
                a[u] = __ldcg(buf + j);
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                acc ^= a[u].x ^ a[u].y ^ a[u].z ^ a[u].w;
        }
    }
    if (acc == 0x9E3779B9u) // keeps the loads; practically never true
        atomicAdd(sink, 1u);
}

__global__ void k_fill(uint4 *buf, size_t n16) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n16;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        buf[i] = make_uint4(static_cast<uint32_t>(i), static_cast<uint32_t>(i * 3), static_cast<uint32_t>(i * 5),
                            static_cast<uint32_t>(i * 7));
}

} // namespace
} // namespace e8g

using namespace e8g;

extern "C" e8g_status e8g_l2_read_bandwidth(e8g_ctx *c, uint64_t bytes, uint32_t reps, double *gbs) {
    if (!c || !gbs || bytes < (1u << 20) || reps == 0 || reps > 1000)
        return E8G_ERR_INVALID_ARG;
    *gbs = 0;
    cudaError_t e = cudaSetDevice(c->device);
    size_t n16 = bytes / 16;
    void *buf = nullptr;
    if (e == cudaSuccess)
        e = cudaMalloc(&buf, n16 * 16 + 256);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "L2 probe buffer");
    auto *b = static_cast<uint4 *>(buf);
    auto *sink = reinterpret_cast<unsigned *>(static_cast<char *>(buf) + n16 * 16);
    int grid = c->num_sms * 8;
    k_fill<<<grid, 256, 0, c->stream>>>(b, n16);
    k_l2_read<<<grid, 256, 0, c->stream>>>(b, n16, 2, sink); // brings the buffer into L2
    cudaEventRecord(c->ev0, c->stream);
    k_l2_read<<<grid, 256, 0, c->stream>>>(b, n16, static_cast<int>(reps), sink);
    cudaEventRecord(c->ev1, c->stream);
    e = cudaEventSynchronize(c->ev1);
    float ms = 0;
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    cudaFree(buf);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "L2 probe");
    // every pass loads ceil(n16 / (4 * threads)) * 4 words per thread (the last round wraps)
    size_t threads = static_cast<size_t>(grid) * 256;
    double words = static_cast<double>((n16 + 4 * threads - 1) / (4 * threads) * 4 * threads);
    *gbs = words * 16.0 * reps / (ms * 1e-3) / 1e9;
    return E8G_OK;
}
