// Megakernel integrators (templates; mega_l0/l1/l2.cu instantiate one tree layout each so the
// three compile in parallel, mega.cu holds the many-scene kernel and the dispatch).
//
// One thread carries one path at a time; threads are persistent and a
// lane whose path ended takes the next path in the same loop iteration, the lanes of a warp
// fetching new work together with one atomic (ballot + popc). Each loop iteration advances
// every live path by one vertex: [Russian roulette] [next-event estimation + shadow ray]
// [BSDF sample + extension ray], so lanes stay converged whatever their path depths.
//
// Reference integrators reproduced (mode):
//   E8G_MODE_REF_UNI     unidirect_path_tracer::sample_indirect_illum   pathtracer.cpp:528-585
//   E8G_MODE_REF_LT1     unidirect_lt1_path_tracer                      pathtracer.cpp:587-653
//   E8G_MODE_REF_DIRECT  direct_path_tracer                             pathtracer.cpp:508-526
//   E8G_MODE_NORMAL / E8G_MODE_POSITION                                 pathtracer.cpp:474-506
// plus the product estimator E8G_MODE_MIS (NEE + BSDF sampling, power heuristic).
// The per-vertex draw order equals the reference's recursion order, so a path fed the
// reference's draw stream reproduces the reference's radiance.
#pragma once

#include "../../include/e8g.h"
#include "launch.h"

namespace e8g {

namespace {

struct PathState {
    float3 L, beta, p, n, o;
    int32_t mesh;
    uint32_t depth;
    uint32_t pixel, out; // out: pixel (image) or list index (per-path output)
};


template <class R> __device__ __forceinline__ void seed_rng(R &rng, RenderArgs const &A, uint64_t mix, uint32_t px, uint32_t s);
template <> __device__ __forceinline__ void seed_rng<RngMinstd>(RngMinstd &rng, RenderArgs const &, uint64_t mix,
                                                               uint32_t px, uint32_t s) {
    rng.seed(path_seed(mix, px, s));
}
template <> __device__ __forceinline__ void seed_rng<RngPhilox>(RngPhilox &rng, RenderArgs const &A, uint64_t,
                                                               uint32_t px, uint32_t s) {
    rng.seed(A.seed, px, s);
}

// Either stream, chosen per path from its scene's RenderArgs: batches whose scenes mix the
// reference's minstd streams and Philox.
struct RngAny {
    RngPhilox p;
    RngMinstd m;
    bool philox;
    __device__ __forceinline__ float next() { return philox ? p.next() : m.next(); }
};
template <> __device__ __forceinline__ void seed_rng<RngAny>(RngAny &rng, RenderArgs const &A, uint64_t mix,
                                                            uint32_t px, uint32_t s) {
    rng.philox = A.rng == E8G_RNG_PHILOX;
    if (rng.philox)
        rng.p.seed(A.seed, px, s);
    else
        rng.m.seed(path_seed(mix, px, s));
}

__device__ __forceinline__ void emit(RenderArgs const &A, float4 *accum, float *path_rgb, uint32_t out, float3 L) {
    if (path_rgb) {
        path_rgb[3 * static_cast<size_t>(out)] = L.x;
        path_rgb[3 * static_cast<size_t>(out) + 1] = L.y;
        path_rgb[3 * static_cast<size_t>(out) + 2] = L.z;
    } else {
        atomicAdd(&accum[out], make_float4(L.x, L.y, L.z, 0.0f));
    }
}

// Starts a path at its cached first hit. Returns false when the path is already complete
// (no valid first hit, or a tracer without random walk, whose value it emits itself).
template <class R>
__device__ __forceinline__ bool mega_start(DevScene const &S, RenderArgs const &A, uint64_t mix, FirstHit const &f,
                                           uint32_t pixel, uint32_t sample, uint32_t out, PathState &ps, R &rng,
                                           float4 *accum, float *path_rgb) {
    int32_t mesh = __float_as_int(f.p.w);
    if (mesh < 0) {
        if (path_rgb)
            emit(A, accum, path_rgb, out, f3(0, 0, 0));
        return false;
    }
    ps.p = xyz(f.p);
    ps.n = xyz(f.n);
    ps.o = neg(xyz(f.d));
    ps.mesh = mesh;
    ps.depth = 0;
    ps.pixel = pixel;
    ps.out = out;
    ps.beta = f3(1.0f, 1.0f, 1.0f);
    ps.L = f3(0, 0, 0);
    int32_t light = __float_as_int(f.n.w);
    if (A.mode == E8G_MODE_MIS && light >= 0)
        ps.L = light_radiance(S, light, ps.o, ps.n);
    seed_rng(rng, A, mix, pixel, sample);
    if (A.mode == E8G_MODE_NORMAL) { // normal_tracer
        emit(A, accum, path_rgb, out, divs(add(ps.n, f3(1.0f, 1.0f, 1.0f)), 2.0f));
        return false;
    }
    if (A.mode == E8G_MODE_POSITION) { // position_tracer
        float3 bmin = f3(S.bmin[0], S.bmin[1], S.bmin[2]);
        float3 rg = sub(f3(S.bmax[0], S.bmax[1], S.bmax[2]), bmin);
        float3 q = sub(ps.p, bmin);
        emit(A, accum, path_rgb, out, f3(q.x / rg.x, q.y / rg.y, q.z / rg.z));
        return false;
    }
    return true;
}

// One vertex of a path: returns true when the path is finished.
// The vertex first draws everything it needs in the reference's order (Russian roulette, the
// light sample, the BSDF sample), then traces its two rays, the shadow ray and the extension
// ray, through one traversal call site, so the kernel holds a single inlined traversal.
template <class R, bool COUNT, int LAYOUT>
__device__ __forceinline__ bool mega_step(DevScene const &S, RenderArgs const &A, PathState &ps, R &rng, uint32_t *sn,
                                          TraceCounters *cnt, uint32_t &rays) {
    const DevMaterial &m = vert_mat(S, ps.mesh);
    const bool ref_nee = A.mode == E8G_MODE_REF_DIRECT || A.mode == E8G_MODE_REF_LT1;
    float3 bl = ps.beta;
    if (A.mode != E8G_MODE_REF_DIRECT) {
        if ((A.max_depth && ps.depth >= A.max_depth) || ps.depth >= kHardDepth)
            return true;
        float surv = A.rr_prob;
        if (ps.depth >= A.rr_start) {
            if (rng.next() >= surv)
                return true;
        }
        if (A.mode == E8G_MODE_MIS) {
            if (ps.depth >= A.rr_start)
                ps.beta = divs(ps.beta, surv);
            bl = ps.beta;
        } else {
            bl = divs(ps.beta, ps.depth >= A.rr_start ? surv : 1.0f);
        }
    }
    // --- next-event estimation: the shadow query and what it adds when unoccluded
    bool shadow = false;
    float3 sh_d = f3(0, 0, 1), sh_vis = f3(0, 0, 0);
    float sh_tmax = 0.0f, sh_ad = 1.0f; // sh_ad: the light sample's area density (reference NEE)
    if (ref_nee) { // transport_direct_illum with one light sample (pathtracer.cpp:152-242)
        float pmf;
        int light = sample_light(S, rng, pmf);
        Surf ls = mesh_sample(S, __ldg(&S.light_mesh[light]), rng, false);
        ls.area_dens *= pmf;
        float3 l = sub(ps.p, ls.p);
        float3 illum = light_eval(S, light, l, ls.n, ps.n);
        sh_ad = ls.area_dens;
        if (!vequals0(illum)) {
            float dist = norm(l);
            sh_d = divs(neg(l), dist);
            sh_tmax = dist - 1e-3f;
            sh_vis = divs(divs(mul(illum, bsdf_eval(S, m, ps.n, ps.o, sh_d)), ls.area_dens), 1.0f);
            shadow = true;
        }
    } else if (A.mode == E8G_MODE_MIS) {
        float pmf;
        int light = sample_light(S, rng, pmf);
        Surf ls = mesh_sample(S, __ldg(&S.light_mesh[light]), rng, true);
        float3 l = sub(ps.p, ls.p);
        float r2 = dot(l, l);
        float dist = sqrtf(r2);
        float3 ln = divs(l, dist);
        float cos_l = dot(ls.n, ln);
        float3 wi = neg(ln);
        float cos_x = dot(ps.n, wi);
        if (cos_l > 0.0f && cos_x > 0.0f) {
            float3 f = bsdf_eval(S, m, ps.n, ps.o, wi);
            if (!vequals0(f)) {
                float p_l = pmf * ls.area_dens * r2 / cos_l;
                float p_b = bsdf_pdf(S, m, ps.n, ps.o, wi);
                float w = power_heuristic(p_l, p_b);
                sh_vis = scale(mul(mul(ps.beta, f), light_rad(S, light)), cos_x * w / p_l);
                sh_d = wi;
                sh_tmax = dist - 1e-3f;
                shadow = true;
            }
        }
    } else if (A.mode == E8G_MODE_REF_UNI) { // emission at every vertex (pathtracer.cpp:543-547)
        int32_t light = __ldg(&S.mesh_light[ps.mesh]);
        if (light >= 0)
            ps.L = add(ps.L, mul(bl, light_radiance(S, light, ps.o, ps.n)));
    }
    // --- the BSDF sample: the extension query
    bool extend = false;
    float pdf = 0.0f;
    float3 i = f3(0, 0, 1);
    if (A.mode == E8G_MODE_REF_LT1 || A.mode == E8G_MODE_REF_UNI) {
        i = bsdf_sample_ref(S, m, rng, pdf, ps.n, ps.o);
        extend = pdf != 0.0f;
    } else if (A.mode == E8G_MODE_MIS) {
        i = bsdf_sample_mis(S, m, rng, pdf, ps.n, ps.o);
        if (pdf > 0.0f) {
            float cw = dot(ps.n, i);
            if (cw > 0.0f) {
                float3 f = bsdf_eval(S, m, ps.n, ps.o, i);
                ps.beta = mul(ps.beta, scale(f, cw / pdf));
                extend = true;
            }
        }
    }
    // --- trace: shadow ray (q = 0) then extension ray (q = 1), one call site
    bool visible = false;
    Hit h;
    h.tri = 0xFFFFFFFFu;
    h.t = INFINITY;
    h.b1 = h.b2 = 0.0f;
#pragma unroll 1
    for (uint32_t q = shadow ? 0u : 1u; q < (extend ? 2u : 1u); q++) {
        bool any = q == 0;
        if (COUNT)
            rays++;
        Hit r = trace_l<LAYOUT, COUNT>(S, ps.p, any ? sh_d : i, 1e-4f, any ? sh_tmax : 1000.0f, any, sn, cnt);
        if (any)
            visible = r.tri == 0xFFFFFFFFu;
        else
            h = r;
    }
    if (ref_nee) {
        float3 r = shadow && visible ? sh_vis : divs(divs(f3(0, 0, 0), sh_ad), 1.0f);
        if (A.mode == E8G_MODE_REF_DIRECT) {
            int32_t light = __ldg(&S.mesh_light[ps.mesh]);
            if (light >= 0)
                r = add(r, light_projected(S, light, ps.o, ps.n));
            ps.L = r;
            return true;
        }
        ps.L = add(ps.L, mul(bl, r));
    } else if (shadow && visible) {
        ps.L = add(ps.L, sh_vis);
    }
    if (!extend || h.tri == 0xFFFFFFFFu)
        return true;
    Vert nv = make_vert(S, h);
    if (dot(nv.n, neg(i)) <= 0.0f)
        return true;
    if (A.mode == E8G_MODE_MIS) {
        int32_t hl = __ldg(&S.mesh_light[nv.mesh]);
        if (hl >= 0) {
            float cos_l2 = dot(nv.n, neg(i));
            float pl = __ldg(&S.light_pnorm[hl]) / S.total_power;
            float inv_area = 1.0f / __ldg(&S.mesh_area[__ldg(&S.light_mesh[hl])]);
            float p_l = pl * inv_area * (nv.t * nv.t) / cos_l2;
            float w = power_heuristic(pdf, p_l);
            ps.L = add(ps.L, scale(mul(ps.beta, light_rad(S, hl)), w));
        }
    } else {
        float3 f = bsdf_eval(S, m, ps.n, ps.o, i);
        float cw = dot(ps.n, i);
        ps.beta = divs(scale(mul(bl, f), cw), pdf);
    }
    ps.p = nv.p;
    ps.n = nv.n;
    ps.mesh = nv.mesh;
    ps.o = neg(i);
    ps.depth++;
    return false;
}

// Radiance of a finished path: lt1 adds the first hit's emission last (pathtracer.cpp:644-646).
__device__ __forceinline__ float3 mega_final(DevScene const &S, RenderArgs const &A, PathState const &ps,
                                             FirstHit const *fh) {
    float3 L = ps.L;
    if (A.mode == E8G_MODE_REF_LT1) {
        FirstHit f = fh[ps.pixel];
        int32_t light = __float_as_int(f.n.w);
        if (light >= 0)
            L = add(L, light_radiance(S, light, neg(xyz(f.d)), xyz(f.n)));
    }
    return L;
}

// Six resident blocks per SM (24 warps) cap the megakernels at 80 registers. Traversal waits on
// L1/L2 loads most of the time, so the extra warps (instead of 5 blocks at ~88 registers) hide
// more latency than the few spilled registers cost: 13% more paths/s on the 1.3M-triangle frame.
constexpr int kMegaBlocksPerSm = 6;

template <class R, bool COUNT, int LAYOUT>
__global__ void __launch_bounds__(kBlock, kMegaBlocksPerSm) k_mega(DevScene S, RenderArgs A, FirstHit const *__restrict__ fh,
                                                 float4 *accum, float *path_rgb, unsigned long long *work,
                                                 unsigned long long *counters) {
    __shared__ uint32_t stk_all[kStackWords * kBlock];
    uint32_t *sn = stk_all + threadIdx.x;
    TraceCounters cnt{0, 0};
    uint32_t rays = 0;
    const uint64_t mix = splitmix64(A.seed);
    const uint32_t lane = lane_id();
    bool active = false, done = false;
    PathState ps;
    R rng;
    while (true) {
        // refill: lanes without a path keep drawing until they hold one with a valid first hit
        // (sky pixels end at once) or the work is exhausted; one atomic per warp per round
        while (true) {
            uint32_t need = __ballot_sync(~0u, !active && !done);
            if (!need)
                break;
            int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (static_cast<int>(lane) == leader)
                base = atomicAdd(work, static_cast<unsigned long long>(__popc(need)));
            base = __shfl_sync(~0u, base, leader);
            if (!active && !done) {
                uint64_t idx = base + __popc(need & ((1u << lane) - 1u));
                uint32_t pixel, sample, out;
                if (idx >= A.total_paths)
                    done = true;
                else if (path_coords(A, idx, pixel, sample, out))
                    active = mega_start(S, A, mix, fh[pixel], pixel, sample, out, ps, rng, accum, path_rgb);
            }
        }
        if (__all_sync(~0u, done))
            break;
        if (!active)
            continue;
        if (mega_step<R, COUNT, LAYOUT>(S, A, ps, rng, sn, &cnt, rays)) {
            emit(A, accum, path_rgb, ps.out, mega_final(S, A, ps, fh));
            active = false;
        }
    }
    if (COUNT) {
        unsigned long long a = rays, b = cnt.nodes, c = cnt.tris;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_down_sync(~0u, a, off);
            b += __shfl_down_sync(~0u, b, off);
            c += __shfl_down_sync(~0u, c, off);
        }
        if (lane == 0) {
            atomicAdd(&counters[0], a);
            atomicAdd(&counters[1], b);
            atomicAdd(&counters[2], c);
        }
    }
}

// The baseline per-path kernel (E8G_INTEGRATOR_PLAIN): one thread per path index, the thread
// walks its path to the end; a warp runs as long as its longest path and no lane is refilled.
template <class R, int LAYOUT>
__global__ void __launch_bounds__(kBlock, kMegaBlocksPerSm) k_plain(DevScene S, RenderArgs A, FirstHit const *__restrict__ fh,
                                                                   float4 *accum, float *path_rgb) {
    __shared__ uint32_t stk_all[kStackWords * kBlock];
    uint32_t *sn = stk_all + threadIdx.x;
    uint64_t idx = static_cast<uint64_t>(blockIdx.x) * kBlock + threadIdx.x;
    uint32_t pixel, sample, out;
    if (idx >= A.total_paths || !path_coords(A, idx, pixel, sample, out))
        return;
    TraceCounters cnt{0, 0};
    uint32_t rays = 0;
    PathState ps;
    R rng;
    if (!mega_start(S, A, splitmix64(A.seed), fh[pixel], pixel, sample, out, ps, rng, accum, path_rgb))
        return;
    while (!mega_step<R, false, LAYOUT>(S, A, ps, rng, sn, &cnt, rays)) {
    }
    emit(A, accum, path_rgb, ps.out, mega_final(S, A, ps, fh));
}

// Many scenes in one persistent launch: the path index runs over the concatenation of every
// scene's paths; a lane that takes a path looks up its scene (binary search over the path
// prefix) and keeps that scene's record for the path's lifetime.
template <class R>
__global__ void __launch_bounds__(kBlock, kMegaBlocksPerSm) k_mega_batch(BatchDev B, FirstHit const *__restrict__ fh_all, float4 *accum_all,
                                                       unsigned long long *work) {
    __shared__ uint32_t stk_all[kStackWords * kBlock];
    uint32_t *sn = stk_all + threadIdx.x;
    TraceCounters cnt{0, 0};
    uint32_t rays = 0;
    const uint32_t lane = lane_id();
    bool active = false, done = false;
    PathState ps;
    uint32_t sid = 0;
    R rng;
    while (true) {
        while (true) {
            uint32_t need = __ballot_sync(~0u, !active && !done);
            if (!need)
                break;
            int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (static_cast<int>(lane) == leader)
                base = atomicAdd(work, static_cast<unsigned long long>(__popc(need)));
            base = __shfl_sync(~0u, base, leader);
            if (!active && !done) {
                uint64_t idx = base + __popc(need & ((1u << lane) - 1u));
                if (idx >= B.total_paths) {
                    done = true;
                } else {
                    uint32_t lo = 0, hi = B.n;
                    while (hi - lo > 1) {
                        uint32_t mi = (lo + hi) >> 1;
                        if (B.path_prefix[mi] <= idx)
                            lo = mi;
                        else
                            hi = mi;
                    }
                    sid = lo;
                    RenderArgs const &A = B.args[sid];
                    DevScene const &S = B.scenes[sid];
                    uint32_t pixel, sample, out;
                    if (path_coords(A, idx - B.path_prefix[sid], pixel, sample, out)) {
                        FirstHit const *fh = fh_all + B.pix_prefix[sid];
                        active = mega_start(S, A, splitmix64(A.seed), fh[pixel], pixel, sample, out, ps, rng,
                                            accum_all + B.pix_prefix[sid], nullptr);
                    }
                }
            }
        }
        if (__all_sync(~0u, done))
            break;
        if (!active)
            continue;
        DevScene const &S = B.scenes[sid];
        RenderArgs const &A = B.args[sid];
        if (mega_step<R, false, 0>(S, A, ps, rng, sn, &cnt, rays)) { // batch scenes use the SAH pairs
            emit(A, accum_all + B.pix_prefix[sid], nullptr, ps.out, mega_final(S, A, ps, fh_all + B.pix_prefix[sid]));
            active = false;
        }
    }
}

} // namespace

template <int LAYOUT>
inline void launch_layout(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                          unsigned long long *work, unsigned long long *counters, int grid, bool plain,
                          cudaStream_t st) {
    bool minstd = A.rng == E8G_RNG_MINSTD;
    if (plain && !counters) {
        unsigned blocks = static_cast<unsigned>((A.total_paths + kBlock - 1) / kBlock);
        if (blocks == 0)
            return;
        if (minstd)
            k_plain<RngMinstd, LAYOUT><<<blocks, kBlock, 0, st>>>(S, A, fh, accum, path_rgb);
        else
            k_plain<RngPhilox, LAYOUT><<<blocks, kBlock, 0, st>>>(S, A, fh, accum, path_rgb);
        return;
    }
    if (counters) {
        if (minstd)
            k_mega<RngMinstd, true, LAYOUT><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, counters);
        else
            k_mega<RngPhilox, true, LAYOUT><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, counters);
    } else {
        if (minstd)
            k_mega<RngMinstd, false, LAYOUT><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, nullptr);
        else
            k_mega<RngPhilox, false, LAYOUT><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, nullptr);
    }
}

} // namespace e8g
