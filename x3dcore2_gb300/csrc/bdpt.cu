// Bidirectional integrators, one thread per path (persistent threads, warp-wide refill).
//
// E8G_MODE_REF_BDPT reproduces bidirect_mis_path_tracer (pathtracer.cpp:12-137, :247-452,
// :754-803): a camera subpath from the cached first hit, a light subpath from an emission
// sample, every (camera length, light length) connection of each total length with a shadow
// ray, and uniform weights over the strategies evaluated for that length (occluded ones count).
// Draw order per path: camera subpath BSDF samples, light pick (1), light point (3), emission
// direction (2), light subpath BSDF samples — the reference's order.
#include "../../include/e8g.h"
#include "launch.h"

namespace e8g {

namespace {

constexpr int kMaxSub = 16; // longest subpath the ABI accepts (bdpt_max_len <= 16)

struct PV { // sampled_pathlet (pathtracer.cpp:12-40)
    float3 v;   // towards the previous vertex
    float dens;
    float3 p, n;
    int32_t mesh;
    int32_t light;
};

template <class R>
__device__ __forceinline__ uint32_t sample_subpath(DevScene const &S, R &rng, PV *path, uint32_t depth,
                                                   uint32_t max_len, uint32_t *stk) {
    while (depth != max_len) { // sample_path, pathtracer.cpp:73-95
        PV const &prev = path[depth - 1];
        float w_dens;
        float3 i = bsdf_sample_ref(S, vert_mat(S, prev.mesh), rng, w_dens, prev.n, prev.v);
        if (feq0(w_dens))
            return depth;
        Hit h = trace_closest<false>(S, prev.p, i, stk, nullptr);
        if (h.tri == 0xFFFFFFFFu)
            return depth;
        Vert nv = make_vert(S, h);
        if (!(dot(nv.n, neg(i)) > 0))
            return depth;
        PV &cur = path[depth];
        cur.v = neg(i);
        cur.dens = w_dens;
        cur.p = nv.p;
        cur.n = nv.n;
        cur.mesh = nv.mesh;
        cur.light = -1;
        depth++;
    }
    return depth;
}

// transport_illum_source (pathtracer.cpp:152-176)
__device__ __forceinline__ float3 illum_source(DevScene const &S, int light, float3 pl, float3 nl, PV const &tv,
                                               uint32_t *stk) {
    float3 l = sub(tv.p, pl);
    float3 illum = light_eval(S, light, l, nl, tv.n);
    if (vequals0(illum))
        return f3(0, 0, 0);
    float dist = norm(l);
    float3 i = divs(neg(l), dist);
    if (!trace_any<false>(S, tv.p, i, 1e-4f, dist - 1e-3f, stk, nullptr))
        return mul(illum, bsdf_eval(S, vert_mat(S, tv.mesh), tv.n, tv.v, i));
    return f3(0, 0, 0);
}

// transport_all_connectible_subpaths (pathtracer.cpp:351-452)
__device__ float3 connect_all(DevScene const &S, PV const *cam, uint32_t clen, PV const *lp, uint32_t llen, float3 em_p,
                              float3 em_n, float em_area_dens, int light, uint32_t *stk) {
    if (clen == 0)
        return f3(0, 0, 0);
    float3 cam_pre[kMaxSub], light_pre[kMaxSub];
    float3 tr = f3(1.0f, 1.0f, 1.0f);
    cam_pre[0] = tr;
    for (uint32_t k = 0; k + 1 < clen; k++) { // projected_adjoint_brdf (:62-68)
        float3 towards = neg(cam[k + 1].v);
        float cw = dot(cam[k].n, towards);
        float3 f = scale(bsdf_eval(S, vert_mat(S, cam[k].mesh), cam[k].n, cam[k].v, towards), cw);
        tr = mul(tr, divs(f, cam[k + 1].dens));
        cam_pre[k + 1] = tr;
    }
    tr = f3(1.0f, 1.0f, 1.0f);
    light_pre[0] = tr;
    for (uint32_t k = 0; k + 1 < llen; k++) { // projected_brdf (:54-60)
        float3 towards = neg(lp[k + 1].v);
        float cw = dot(lp[k].n, towards);
        float3 f = scale(bsdf_eval(S, vert_mat(S, lp[k].mesh), lp[k].n, towards, lp[k].v), cw);
        tr = mul(tr, divs(f, lp[k + 1].dens));
        light_pre[k + 1] = tr;
    }
    float3 rad = f3(0, 0, 0);
    for (uint32_t plen = 1; plen <= clen + llen + 1; plen++) {
        uint32_t cam_plen = plen - 1 < clen ? plen - 1 : clen;
        uint32_t light_plen = plen - 1 - cam_plen;
        float3 psum = f3(0, 0, 0);
        float wsum = 0.0f;
        const float cw = 1.0f;
        while (static_cast<int>(cam_plen) >= 0 && light_plen <= llen) {
            if (light_plen == 0 && cam_plen == 0) {
                if (cam[0].light >= 0)
                    psum = add(psum, scale(light_radiance(S, cam[0].light, cam[0].v, cam[0].n), cw));
                wsum += cw;
            } else if (light_plen == 0) {
                PV const &cj = cam[cam_plen - 1];
                float3 ti = divs(illum_source(S, light, em_p, em_n, cj, stk), em_area_dens);
                float3 pr = divs(mul(ti, cam_pre[cam_plen - 1]), cam[0].dens);
                psum = add(psum, scale(pr, cw));
                wsum += cw;
            } else if (cam_plen != 0) {
                PV const &lj = lp[light_plen - 1];
                PV const &cj = cam[cam_plen - 1];
                float3 join = sub(cj.p, lj.p);
                float jd = norm(join);
                join = divs(join, jd);
                float cos_wo = dot(lj.n, join);
                float cos_wi = dot(cj.n, neg(join));
                if (cos_wo > 0.0f && cos_wi > 0.0f && !trace_any<false>(S, lj.p, join, 1e-3f, jd - 1e-3f, stk, nullptr)) {
                    float3 le = divs(light_projected(S, light, neg(lp[0].v), em_n), lp[0].dens * em_area_dens);
                    float3 lsi = mul(le, light_pre[light_plen - 1]);
                    float to_area = cos_wi * cos_wo / (jd * jd);
                    float3 ljw = bsdf_eval(S, vert_mat(S, lj.mesh), lj.n, join, lj.v);
                    float3 cjw = bsdf_eval(S, vert_mat(S, cj.mesh), cj.n, cj.v, neg(join));
                    float3 ti = scale(mul(mul(lsi, ljw), cjw), to_area);
                    float3 csr = divs(mul(ti, cam_pre[cam_plen - 1]), cam[0].dens);
                    psum = add(psum, scale(csr, cw));
                }
                wsum += cw;
            }
            light_plen++;
            cam_plen--;
        }
        if (wsum > 0)
            rad = add(rad, divs(psum, wsum));
    }
    return rad;
}

template <class R> __device__ __forceinline__ void seed_path(R &rng, RenderArgs const &A, uint64_t mix, uint32_t px, uint32_t s);
template <> __device__ __forceinline__ void seed_path<RngMinstd>(RngMinstd &rng, RenderArgs const &, uint64_t mix,
                                                                uint32_t px, uint32_t s) {
    rng.seed(path_seed(mix, px, s));
}
template <> __device__ __forceinline__ void seed_path<RngPhilox>(RngPhilox &rng, RenderArgs const &A, uint64_t,
                                                                uint32_t px, uint32_t s) {
    rng.seed(A.seed, px, s);
}

__device__ __forceinline__ bool coords(RenderArgs const &A, uint64_t idx, uint32_t &pixel, uint32_t &sample,
                                       uint32_t &out) {
    if (A.list_pixel) {
        pixel = A.list_pixel[idx];
        sample = A.list_sample[idx];
        out = static_cast<uint32_t>(idx);
        return true;
    }
    uint32_t s = static_cast<uint32_t>(idx / A.paths_per_sample);
    uint32_t j = static_cast<uint32_t>(idx - static_cast<uint64_t>(s) * A.paths_per_sample);
    uint32_t tile = j >> 5, w = j & 31u;
    uint32_t x = (tile % A.tiles_x) * 8 + (w & 7u), y = (tile / A.tiles_x) * 4 + (w >> 3);
    if (x >= A.width || y >= A.height)
        return false;
    pixel = y * A.width + x;
    sample = A.sample_offset + s;
    out = pixel;
    return true;
}

template <class R>
__global__ void __launch_bounds__(kBlock) k_bdpt_ref(DevScene S, RenderArgs A, FirstHit const *__restrict__ fh,
                                                     float4 *accum, float *path_rgb, unsigned long long *work) {
    __shared__ uint32_t stk_all[kStackWords * kBlock];
    uint32_t *stk = stk_all + threadIdx.x;
    const uint64_t mix = splitmix64(A.seed);
    const uint32_t lane = lane_id();
    const uint32_t max_len = A.bdpt_max_len < kMaxSub ? A.bdpt_max_len : kMaxSub;
    PV cam[kMaxSub], lp[kMaxSub];
    while (true) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32ull);
        base = __shfl_sync(~0u, base, 0);
        if (base >= A.total_paths)
            break;
        uint64_t idx = base + lane;
        uint32_t pixel, sample, out;
        if (idx < A.total_paths && coords(A, idx, pixel, sample, out)) {
            R rng;
            seed_path(rng, A, mix, pixel, sample);
            FirstHit f = fh[pixel];
            uint32_t clen = 0;
            int32_t mesh = __float_as_int(f.p.w);
            if (mesh >= 0 && max_len != 0) { // sample_path with the cached first hit (:127-137)
                cam[0].v = neg(xyz(f.d));
                cam[0].dens = 1.0f;
                cam[0].p = xyz(f.p);
                cam[0].n = xyz(f.n);
                cam[0].mesh = mesh;
                cam[0].light = __float_as_int(f.n.w);
                clen = sample_subpath(S, rng, cam, 1, max_len, stk);
            }
            // sample_illum_source (:754-767), area_light::sample_emssion (light.cpp:26-32)
            float pmf;
            int light = sample_light(S, rng, pmf);
            Surf em = mesh_sample(S, __ldg(&S.light_mesh[light]), rng, false);
            float3 w = cos_hemisphere(em.n, rng);
            float sa_dens = dot(em.n, w) / kPi;
            em.area_dens *= pmf;
            uint32_t llen = 0;
            Hit h = trace_closest<false>(S, em.p, w, stk, nullptr); // sample_path from r0 (:109-120)
            if (h.tri != 0xFFFFFFFFu && max_len != 0) {
                Vert v0 = make_vert(S, h);
                if (!(dot(v0.n, neg(w)) <= 0.0f)) {
                    lp[0].v = neg(w);
                    lp[0].dens = sa_dens;
                    lp[0].p = v0.p;
                    lp[0].n = v0.n;
                    lp[0].mesh = v0.mesh;
                    lp[0].light = -1;
                    llen = sample_subpath(S, rng, lp, 1, max_len, stk);
                }
            }
            float3 L = connect_all(S, cam, clen, lp, llen, em.p, em.n, em.area_dens, light, stk);
            if (path_rgb) {
                path_rgb[3 * static_cast<size_t>(out)] = L.x;
                path_rgb[3 * static_cast<size_t>(out) + 1] = L.y;
                path_rgb[3 * static_cast<size_t>(out) + 2] = L.z;
            } else {
                atomicAdd(&accum[out], make_float4(L.x, L.y, L.z, 0.0f));
            }
        }
    }
}

} // namespace

int bdpt_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_bdpt_ref<RngMinstd>, kBlock, 0);
    return n > 0 ? n : 1;
}

void launch_bdpt(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                 unsigned long long *work, int grid, cudaStream_t st) {
    if (A.rng == E8G_RNG_MINSTD)
        k_bdpt_ref<RngMinstd><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work);
    else
        k_bdpt_ref<RngPhilox><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work);
}

} // namespace e8g
