// Primary-hit, ray-batch traversal and resolve kernels.
#include "launch.h"

namespace e8g {

// compute_first_hit (pathtracer.cpp:456-472): camera ray, closest hit, back-facing hits become
// misses, emitter lookup.
__global__ void __launch_bounds__(kBlock) k_first_hits(DevScene S, uint32_t w, uint32_t h, FirstHit *out) {
    __shared__ uint32_t stk[kStackWords * kBlock];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h)
        return;
    float3 o, d;
    camera_ray(S.cam, i % w, i / w, w, h, o, d);
    Hit hit = trace_closest<false>(S, o, d, stk + threadIdx.x, nullptr);
    FirstHit f;
    f.d = make_float4(d.x, d.y, d.z, 0.0f);
    int32_t mesh = -1, light = -1;
    float3 p = f3(0, 0, 0), n = f3(0, 0, 0);
    if (hit.tri != 0xFFFFFFFFu) {
        Vert v = make_vert(S, hit);
        if (dot(v.n, neg(d)) > 0) {
            mesh = v.mesh;
            p = v.p;
            n = v.n;
            light = __ldg(&S.mesh_light[mesh]);
        }
    }
    f.p = make_float4(p.x, p.y, p.z, __int_as_float(mesh));
    f.n = make_float4(n.x, n.y, n.z, __int_as_float(light));
    out[i] = f;
}

// compute_first_hit for explicit rays: ray i's first hit into out[i].
__global__ void __launch_bounds__(kBlock) k_first_hits_rays(DevScene S, float const *rays6, uint32_t n,
                                                             FirstHit *out) {
    __shared__ uint32_t stk[kStackWords * kBlock];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float3 o = f3(rays6[6 * i], rays6[6 * i + 1], rays6[6 * i + 2]);
    float3 d = f3(rays6[6 * i + 3], rays6[6 * i + 4], rays6[6 * i + 5]);
    Hit hit = trace_closest<false>(S, o, d, stk + threadIdx.x, nullptr);
    FirstHit f;
    f.d = make_float4(d.x, d.y, d.z, 0.0f);
    int32_t mesh = -1, light = -1;
    float3 p = f3(0, 0, 0), nn = f3(0, 0, 0);
    if (hit.tri != 0xFFFFFFFFu) {
        Vert v = make_vert(S, hit);
        if (dot(v.n, neg(d)) > 0) {
            mesh = v.mesh;
            p = v.p;
            nn = v.n;
            light = __ldg(&S.mesh_light[mesh]);
        }
    }
    f.p = make_float4(p.x, p.y, p.z, __int_as_float(mesh));
    f.n = make_float4(nn.x, nn.y, nn.z, __int_as_float(light));
    out[i] = f;
}

// Identity pixel list and a constant sample list for explicit rays.
__global__ void k_ray_lists(uint32_t n, uint32_t sample, uint32_t *pixel, uint32_t *samples) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        pixel[i] = i;
        samples[i] = sample;
    }
}

__global__ void k_camera_rays(DevScene S, uint32_t w, uint32_t h, float *rays6) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h)
        return;
    float3 o, d;
    camera_ray(S.cam, i % w, i / w, w, h, o, d);
    float *r = rays6 + 6 * static_cast<size_t>(i);
    r[0] = o.x;
    r[1] = o.y;
    r[2] = o.z;
    r[3] = d.x;
    r[4] = d.y;
    r[5] = d.z;
}

template <bool COUNT>
__global__ void __launch_bounds__(kBlock) k_trace_closest(DevScene S, float const *rays6, uint32_t n, float *hits5,
                                                          unsigned long long *counters) {
    __shared__ uint32_t stk[kStackWords * kBlock];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    TraceCounters c{0, 0};
    if (i < n) {
        float const *r = rays6 + 6 * static_cast<size_t>(i);
        float3 o = f3(r[0], r[1], r[2]), d = f3(r[3], r[4], r[5]);
        Hit h = trace_closest<COUNT>(S, o, d, stk + threadIdx.x, &c);
        float *out = hits5 + 5 * static_cast<size_t>(i);
        if (h.tri == 0xFFFFFFFFu) {
            out[0] = 0.0f;
            out[1] = __int_as_float(-1);
            out[2] = __int_as_float(-1);
            out[3] = 0.0f;
            out[4] = 0.0f;
        } else {
            uint4 ti = __ldg(&S.tidx[h.tri]);
            out[0] = h.t;
            out[1] = __int_as_float(static_cast<int>(ti.w));
            out[2] = __int_as_float(static_cast<int>(h.tri - __ldg(&S.mesh_toff[ti.w])));
            out[3] = h.b1;
            out[4] = h.b2;
        }
    }
    if (COUNT) {
        unsigned long long a = c.nodes, b = c.tris;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_down_sync(~0u, a, off);
            b += __shfl_down_sync(~0u, b, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&counters[1], a);
            atomicAdd(&counters[2], b);
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_trace_any(DevScene S, float const *rays6, float const *tmin,
                                                      float const *tmax, uint32_t n, uint8_t *occ) {
    __shared__ uint32_t stk[kStackWords * kBlock];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float const *r = rays6 + 6 * static_cast<size_t>(i);
    float3 o = f3(r[0], r[1], r[2]), d = f3(r[3], r[4], r[5]);
    occ[i] = trace_any<false>(S, o, d, tmin[i], tmax[i], stk + threadIdx.x, nullptr) ? 1 : 0;
}

__global__ void k_resolve(float4 const *accum, uint32_t npix, float inv_spp, float *rgba) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix)
        return;
    float4 a = accum[i];
    reinterpret_cast<float4 *>(rgba)[i] = make_float4(a.x * inv_spp, a.y * inv_spp, a.z * inv_spp, 1.0f);
}

// pt_image_renderer's firefly clamp (renderer.cpp:46-83) over K per-sample images est
// (sample-major, W*H rgb each), accumulated per pixel in sample order like the reference's task
// estimate: an interior pixel whose squared norm exceeds each of its 8 neighbours' by more than
// 1.5 (renderer.h:118) has every channel capped at the neighbours' mean squared norm plus 1.5.
__device__ __forceinline__ float sqnorm(float const *v) {
    float r = 0.0f;
    r += v[0] * v[0];
    r += v[1] * v[1];
    r += v[2] * v[2];
    return r;
}

__global__ void k_firefly(float const *__restrict__ est, uint32_t K, uint32_t w, uint32_t h, float4 *accum) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t npix = w * h;
    if (i >= npix)
        return;
    uint32_t x = i % w, y = i / w;
    bool inner = x > 0 && x < w - 1 && y > 0 && y < h - 1;
    const float diff = 1.5f;
    float4 a = accum[i];
    for (uint32_t k = 0; k < K; k++) {
        float const *e = est + 3 * (static_cast<size_t>(k) * npix + i);
        float v0 = e[0], v1 = e[1], v2 = e[2];
        if (inner) {
            size_t row = 3 * static_cast<size_t>(w);
            float r00 = sqnorm(e - row - 3), r10 = sqnorm(e - row), r20 = sqnorm(e - row + 3);
            float r01 = sqnorm(e - 3), r11 = sqnorm(e), r21 = sqnorm(e + 3);
            float r02 = sqnorm(e + row - 3), r12 = sqnorm(e + row), r22 = sqnorm(e + row + 3);
            bool ff = (r11 - r00) > diff && (r11 - r10) > diff && (r11 - r20) > diff && (r11 - r01) > diff &&
                      (r11 - r21) > diff && (r11 - r02) > diff && (r11 - r12) > diff && (r11 - r22) > diff;
            if (ff) {
                float cap = 1.0f / 8.0f * (r00 + r10 + r20 + r01 + r21 + r02 + r12 + r22) + diff;
                v0 = cap < v0 ? cap : v0;
                v1 = cap < v1 ? cap : v1;
                v2 = cap < v2 ? cap : v2;
            }
        }
        a.x += v0;
        a.y += v1;
        a.z += v2;
    }
    accum[i] = a;
}

static inline int blocks(uint32_t n, int b) { return static_cast<int>((n + b - 1) / b); }

void launch_first_hits(DevScene const &S, uint32_t w, uint32_t h, FirstHit *out, cudaStream_t st) {
    k_first_hits<<<blocks(w * h, kBlock), kBlock, 0, st>>>(S, w, h, out);
}
void launch_first_hits_rays(DevScene const &S, float const *rays6, uint32_t n, FirstHit *out, uint32_t sample,
                            uint32_t *pixel, uint32_t *samples, cudaStream_t st) {
    if (!n)
        return;
    k_first_hits_rays<<<blocks(n, kBlock), kBlock, 0, st>>>(S, rays6, n, out);
    k_ray_lists<<<blocks(n, 256), 256, 0, st>>>(n, sample, pixel, samples);
}
void launch_camera_rays(DevScene const &S, uint32_t w, uint32_t h, float *rays6, cudaStream_t st) {
    k_camera_rays<<<blocks(w * h, 256), 256, 0, st>>>(S, w, h, rays6);
}
void launch_trace_closest(DevScene const &S, float const *rays6, uint32_t n, float *hits5, cudaStream_t st) {
    if (n)
        k_trace_closest<false><<<blocks(n, kBlock), kBlock, 0, st>>>(S, rays6, n, hits5, nullptr);
}
void launch_trace_closest_counted(DevScene const &S, float const *rays6, uint32_t n, float *hits5,
                                  unsigned long long *counters, cudaStream_t st) {
    if (n)
        k_trace_closest<true><<<blocks(n, kBlock), kBlock, 0, st>>>(S, rays6, n, hits5, counters);
}
void launch_trace_any(DevScene const &S, float const *rays6, float const *tmin, float const *tmax, uint32_t n,
                      uint8_t *occ, cudaStream_t st) {
    if (n)
        k_trace_any<<<blocks(n, kBlock), kBlock, 0, st>>>(S, rays6, tmin, tmax, n, occ);
}
void launch_resolve(float4 const *accum, uint32_t npix, float inv_spp, float *rgba, cudaStream_t st) {
    k_resolve<<<blocks(npix, 256), 256, 0, st>>>(accum, npix, inv_spp, rgba);
}
void launch_firefly(float const *est, uint32_t K, uint32_t w, uint32_t h, float4 *accum, cudaStream_t st) {
    k_firefly<<<blocks(w * h, 256), 256, 0, st>>>(est, K, w, h, accum);
}

} // namespace e8g

namespace e8g {

// Batched first hits: the pixel index runs over every scene's pixels.
__global__ void __launch_bounds__(kBlock) k_first_hits_batch(BatchDev B, uint64_t total_pix, FirstHit *out) {
    __shared__ uint32_t stk[kStackWords * kBlock];
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= total_pix)
        return;
    uint32_t lo = 0, hi = B.n;
    while (hi - lo > 1) {
        uint32_t mi = (lo + hi) >> 1;
        if (B.pix_prefix[mi] <= i)
            lo = mi;
        else
            hi = mi;
    }
    DevScene const &S = B.scenes[lo];
    RenderArgs const &A = B.args[lo];
    uint32_t px = static_cast<uint32_t>(i - B.pix_prefix[lo]);
    float3 o, d;
    camera_ray(S.cam, px % A.width, px / A.width, A.width, A.height, o, d);
    Hit hit = trace_closest<false>(S, o, d, stk + threadIdx.x, nullptr); // the scene's own layout
    FirstHit f;
    f.d = make_float4(d.x, d.y, d.z, 0.0f);
    int32_t mesh = -1, light = -1;
    float3 p = f3(0, 0, 0), n = f3(0, 0, 0);
    if (hit.tri != 0xFFFFFFFFu) {
        Vert v = make_vert(S, hit);
        if (dot(v.n, neg(d)) > 0) {
            mesh = v.mesh;
            p = v.p;
            n = v.n;
            light = __ldg(&S.mesh_light[mesh]);
        }
    }
    f.p = make_float4(p.x, p.y, p.z, __int_as_float(mesh));
    f.n = make_float4(n.x, n.y, n.z, __int_as_float(light));
    out[i] = f;
}

__global__ void k_resolve_batch(BatchDev B, uint64_t total_pix, float4 const *accum, float *rgba) {
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= total_pix)
        return;
    uint32_t lo = 0, hi = B.n;
    while (hi - lo > 1) {
        uint32_t mi = (lo + hi) >> 1;
        if (B.pix_prefix[mi] <= i)
            lo = mi;
        else
            hi = mi;
    }
    uint32_t spp = B.args[lo].spp;
    float inv = spp ? 1.0f / static_cast<float>(spp) : 0.0f;
    float4 a = accum[i];
    reinterpret_cast<float4 *>(rgba)[i] = make_float4(a.x * inv, a.y * inv, a.z * inv, 1.0f);
}

void launch_first_hits_batch(BatchDev const &B, DevScene const *, RenderArgs const *, uint64_t const *h_pix_prefix,
                             FirstHit *fh_all, cudaStream_t st) {
    uint64_t total = h_pix_prefix[B.n];
    if (total)
        k_first_hits_batch<<<static_cast<unsigned>((total + kBlock - 1) / kBlock), kBlock, 0, st>>>(B, total, fh_all);
}

void launch_resolve_batch(BatchDev const &B, uint64_t total_pix, float4 const *accum_all, float *rgba_all,
                          cudaStream_t st) {
    if (total_pix)
        k_resolve_batch<<<static_cast<unsigned>((total_pix + 255) / 256), 256, 0, st>>>(B, total_pix, accum_all, rgba_all);
}

} // namespace e8g
