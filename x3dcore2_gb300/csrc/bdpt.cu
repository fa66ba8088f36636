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
#include "wavefront.h"

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

template <bool COUNT, class R>
__device__ __forceinline__ uint32_t sample_subpath(DevScene const &S, R &rng, PV *path, uint32_t depth,
                                                   uint32_t max_len, uint32_t *stk, TraceCounters *cnt) {
    while (depth != max_len) { // sample_path, pathtracer.cpp:73-95
        PV const &prev = path[depth - 1];
        float w_dens;
        float3 i = bsdf_sample_ref<true>(S, vert_mat(S, prev.mesh), rng, w_dens, prev.n, prev.v);
        if (feq0(w_dens))
            return depth;
        if (COUNT)
            cnt->rays++;
        Hit h = trace_closest<COUNT>(S, prev.p, i, stk, cnt);
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
template <bool COUNT>
__device__ __forceinline__ float3 illum_source(DevScene const &S, int light, float3 pl, float3 nl, PV const &tv,
                                               uint32_t *stk, TraceCounters *cnt) {
    float3 l = sub(tv.p, pl);
    float3 illum = light_eval(S, light, l, nl, tv.n);
    if (vequals0(illum))
        return f3(0, 0, 0);
    float dist = norm(l);
    float3 i = divs(neg(l), dist);
    if (COUNT)
        cnt->rays++;
    if (!trace_any<COUNT>(S, tv.p, i, 1e-4f, dist - 1e-3f, stk, cnt))
        return mul(illum, bsdf_eval<true>(S, vert_mat(S, tv.mesh), tv.n, tv.v, i));
    return f3(0, 0, 0);
}

// transport_all_connectible_subpaths (pathtracer.cpp:351-452)
template <bool COUNT>
__device__ float3 connect_all(DevScene const &S, PV const *cam, uint32_t clen, PV const *lp, uint32_t llen, float3 em_p,
                              float3 em_n, float em_area_dens, int light, uint32_t *stk, TraceCounters *cnt) {
    if (clen == 0)
        return f3(0, 0, 0);
    float3 cam_pre[kMaxSub], light_pre[kMaxSub];
    float3 tr = f3(1.0f, 1.0f, 1.0f);
    cam_pre[0] = tr;
    for (uint32_t k = 0; k + 1 < clen; k++) { // projected_adjoint_brdf (:62-68)
        float3 towards = neg(cam[k + 1].v);
        float cw = dot(cam[k].n, towards);
        float3 f = scale(bsdf_eval<true>(S, vert_mat(S, cam[k].mesh), cam[k].n, cam[k].v, towards), cw);
        tr = mul(tr, divs(f, cam[k + 1].dens));
        cam_pre[k + 1] = tr;
    }
    tr = f3(1.0f, 1.0f, 1.0f);
    light_pre[0] = tr;
    for (uint32_t k = 0; k + 1 < llen; k++) { // projected_brdf (:54-60)
        float3 towards = neg(lp[k + 1].v);
        float cw = dot(lp[k].n, towards);
        float3 f = scale(bsdf_eval<true>(S, vert_mat(S, lp[k].mesh), lp[k].n, towards, lp[k].v), cw);
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
                float3 ti = divs(illum_source<COUNT>(S, light, em_p, em_n, cj, stk, cnt), em_area_dens);
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
                if (COUNT && cos_wo > 0.0f && cos_wi > 0.0f)
                    cnt->rays++;
                if (cos_wo > 0.0f && cos_wi > 0.0f && !trace_any<COUNT>(S, lj.p, join, 1e-3f, jd - 1e-3f, stk, cnt)) {
                    float3 le = divs(light_projected(S, light, neg(lp[0].v), em_n), lp[0].dens * em_area_dens);
                    float3 lsi = mul(le, light_pre[light_plen - 1]);
                    float to_area = cos_wi * cos_wo / (jd * jd);
                    float3 ljw = bsdf_eval<true>(S, vert_mat(S, lj.mesh), lj.n, join, lj.v);
                    float3 cjw = bsdf_eval<true>(S, vert_mat(S, cj.mesh), cj.n, cj.v, neg(join));
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

// ---- E8G_MODE_BDPT_POWER: bidirectional with power-heuristic MIS (product mode) ----
// Camera subpath from the cached first hit, light subpath from an area-weighted emission sample
// with a cosine direction, every (s, t >= 1) connection, weighted by the power heuristic over the
// strategies that could produce the same path under the subpath caps. Per vertex: throughput and
// the forward / reverse densities in area measure; a connection updates the four densities it
// changes and restores them afterwards (Veach's recurrence).

struct BV {
    float3 p, n;
    int32_t mesh;
    float3 beta;
    float fwd, rev;
};

__device__ __forceinline__ float to_area(float pdf_w, float3 from, float3 to, float3 n_to) {
    float3 d = sub(to, from);
    float d2 = dot(d, d);
    if (d2 <= 0.0f)
        return 0.0f;
    float c = fabsf(dot(n_to, d)) / sqrtf(d2);
    return pdf_w * c / d2;
}

__device__ __forceinline__ float vpdf(DevScene const &S, BV const &v, float3 wo, float3 wi) {
    return bsdf_pdf<true>(S, vert_mat(S, v.mesh), v.n, wo, wi);
}

template <bool COUNT, class R>
__device__ uint32_t bdp_walk(DevScene const &S, R &rng, BV *path, uint32_t len, uint32_t max_len, float3 wo,
                             uint32_t *stk, TraceCounters *cnt) {
    while (len < max_len) {
        BV &cur = path[len - 1];
        const DevMaterial &m = vert_mat(S, cur.mesh);
        float pdf;
        float3 i = bsdf_sample_mis<true>(S, m, rng, pdf, cur.n, wo);
        if (!(pdf > 0.0f))
            break;
        float cw = dot(cur.n, i);
        if (cw <= 0.0f)
            break;
        float3 f = bsdf_eval<true>(S, m, cur.n, wo, i);
        if (COUNT)
            cnt->rays++;
        Hit h = trace_closest<COUNT>(S, cur.p, i, stk, cnt);
        if (h.tri == 0xFFFFFFFFu)
            break;
        Vert nv = make_vert(S, h);
        if (dot(nv.n, neg(i)) <= 0.0f)
            break;
        BV &nx = path[len];
        nx.p = nv.p;
        nx.n = nv.n;
        nx.mesh = nv.mesh;
        nx.beta = mul(cur.beta, scale(f, cw / pdf));
        nx.fwd = to_area(pdf, cur.p, nx.p, nx.n);
        nx.rev = 0.0f;
        float prev_w = vpdf(S, cur, i, wo);
        if (len >= 2)
            path[len - 2].rev = to_area(prev_w, cur.p, path[len - 2].p, path[len - 2].n);
        wo = neg(i);
        len++;
    }
    return len;
}

template <bool COUNT>
__device__ float3 connect_power(DevScene const &S, BV *cam, uint32_t clen, BV *lp, uint32_t llen, uint32_t maxlen,
                                float3 o0, int light, uint32_t *stk, TraceCounters *cnt) {
    float3 L = f3(0, 0, 0);
    for (uint32_t t = 1; t <= clen; t++) {
        for (uint32_t sl = 0; sl <= llen; sl++) {
            BV &cv = cam[t - 1];
            float3 wo_c = t >= 2 ? normalize(sub(cam[t - 2].p, cv.p)) : o0;
            float3 contrib;
            float save_c_rev = cv.rev, save_c2_rev = t >= 2 ? cam[t - 2].rev : 0.0f;
            float save_l_rev = sl >= 1 ? lp[sl - 1].rev : 0.0f, save_l2_rev = sl >= 2 ? lp[sl - 2].rev : 0.0f;
            if (sl == 0) {
                int hl = __ldg(&S.mesh_light[cv.mesh]);
                if (hl < 0)
                    continue;
                float3 le = light_radiance(S, hl, wo_c, cv.n);
                if (vequals0(le))
                    continue;
                contrib = mul(cv.beta, le);
                float pl = __ldg(&S.light_pnorm[hl]) / S.total_power;
                cv.rev = pl * (1.0f / __ldg(&S.mesh_area[__ldg(&S.light_mesh[hl])]));
                if (t >= 2) {
                    float ew = fmaxf(dot(cv.n, wo_c), 0.0f) / kPi;
                    cam[t - 2].rev = to_area(ew, cv.p, cam[t - 2].p, cam[t - 2].n);
                }
            } else {
                BV &lv = lp[sl - 1];
                float3 d = sub(lv.p, cv.p);
                float d2 = dot(d, d);
                if (d2 <= 0.0f)
                    continue;
                float dist = sqrtf(d2);
                float3 dir = divs(d, dist);
                float cos_c = dot(cv.n, dir);
                float cos_l = dot(lv.n, neg(dir));
                if (cos_c <= 0.0f || cos_l <= 0.0f)
                    continue;
                float3 fc = bsdf_eval<true>(S, vert_mat(S, cv.mesh), cv.n, wo_c, dir);
                if (vequals0(fc))
                    continue;
                float3 fl, wo_l = f3(0, 0, 0);
                if (sl == 1) {
                    fl = light_radiance(S, light, neg(dir), lv.n);
                } else {
                    wo_l = normalize(sub(lp[sl - 2].p, lv.p));
                    fl = bsdf_eval<true>(S, vert_mat(S, lv.mesh), lv.n, neg(dir), wo_l);
                }
                if (vequals0(fl))
                    continue;
                if (COUNT)
                    cnt->rays++;
                if (trace_any<COUNT>(S, cv.p, dir, 1e-4f, dist - 1e-3f, stk, cnt))
                    continue;
                float G = cos_c * cos_l / d2;
                contrib = scale(mul(mul(mul(cv.beta, fc), fl), lv.beta), G);
                float pc = vpdf(S, cv, wo_c, dir);
                lv.rev = to_area(pc, cv.p, lv.p, lv.n);
                if (sl == 1)
                    cv.rev = to_area(cos_l / kPi, lv.p, cv.p, cv.n);
                else
                    cv.rev = to_area(vpdf(S, lv, wo_l, neg(dir)), lv.p, cv.p, cv.n);
                if (t >= 2)
                    cam[t - 2].rev = to_area(vpdf(S, cv, dir, wo_c), cv.p, cam[t - 2].p, cam[t - 2].n);
                if (sl >= 2)
                    lp[sl - 2].rev = to_area(vpdf(S, lv, neg(dir), wo_l), lv.p, lp[sl - 2].p, lp[sl - 2].n);
            }
            // single precision (FP64 issues at a small fraction of the FP32 rate on this GPU): a
            // ratio product whose square overflows gives weight 0, where FP64 would give < 1e-38
            float sum = 0.0f, ri = 1.0f;
            for (int i = static_cast<int>(t) - 1; i >= 1; i--) {
                if (sl + t - static_cast<uint32_t>(i) > maxlen)
                    break;
                ri *= (cam[i].fwd > 0.0f) ? cam[i].rev / cam[i].fwd : 0.0f;
                sum += ri * ri;
            }
            ri = 1.0f;
            for (int i = static_cast<int>(sl) - 1; i >= 0; i--) {
                if (t + sl - static_cast<uint32_t>(i) > maxlen)
                    break;
                ri *= (lp[i].fwd > 0.0f) ? lp[i].rev / lp[i].fwd : 0.0f;
                sum += ri * ri;
            }
            float wgt = 1.0f / (1.0f + sum);
            L = add(L, scale(contrib, wgt));
            cv.rev = save_c_rev;
            if (t >= 2)
                cam[t - 2].rev = save_c2_rev;
            if (sl >= 1)
                lp[sl - 1].rev = save_l_rev;
            if (sl >= 2)
                lp[sl - 2].rev = save_l2_rev;
        }
    }
    return L;
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


// Adds a thread's traversal counts (rays traced, node boxes fetched, triangles tested) to the
// three device counters, one atomic per warp and counter.
__device__ __forceinline__ void flush_counts(TraceCounters const &cnt, unsigned long long *counters) {
    unsigned long long a = cnt.rays, b = cnt.nodes, c = cnt.tris;
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(~0u, a, off);
        b += __shfl_down_sync(~0u, b, off);
        c += __shfl_down_sync(~0u, c, off);
    }
    if (lane_id() == 0) {
        atomicAdd(&counters[0], a);
        atomicAdd(&counters[1], b);
        atomicAdd(&counters[2], c);
    }
}

// COUNT: the instrumented instantiation that counts traversal work into counters[0..2].
template <class R, bool COUNT>
__global__ void __launch_bounds__(kBlock) k_bdpt_ref(DevScene S, RenderArgs A, FirstHit const *__restrict__ fh,
                                                     float4 *accum, float *path_rgb, unsigned long long *work,
                                                     unsigned long long *counters) {
    TraceCounters cnt{0, 0, 0};
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
        if (idx < A.total_paths && path_coords(A, idx, pixel, sample, out)) {
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
                clen = sample_subpath<COUNT>(S, rng, cam, 1, max_len, stk, &cnt);
            }
            // sample_illum_source (:754-767), area_light::sample_emssion (light.cpp:26-32)
            float pmf;
            int light = sample_light(S, rng, pmf);
            Surf em = mesh_sample(S, __ldg(&S.light_mesh[light]), rng, false);
            float3 w = cos_hemisphere(em.n, rng);
            float sa_dens = dot(em.n, w) / kPi;
            em.area_dens *= pmf;
            uint32_t llen = 0;
            if (COUNT)
                cnt.rays++;
            Hit h = trace_closest<COUNT>(S, em.p, w, stk, &cnt); // sample_path from r0 (:109-120)
            if (h.tri != 0xFFFFFFFFu && max_len != 0) {
                Vert v0 = make_vert(S, h);
                if (!(dot(v0.n, neg(w)) <= 0.0f)) {
                    lp[0].v = neg(w);
                    lp[0].dens = sa_dens;
                    lp[0].p = v0.p;
                    lp[0].n = v0.n;
                    lp[0].mesh = v0.mesh;
                    lp[0].light = -1;
                    llen = sample_subpath<COUNT>(S, rng, lp, 1, max_len, stk, &cnt);
                }
            }
            float3 L = connect_all<COUNT>(S, cam, clen, lp, llen, em.p, em.n, em.area_dens, light, stk, &cnt);
            if (path_rgb) {
                path_rgb[3 * static_cast<size_t>(out)] = L.x;
                path_rgb[3 * static_cast<size_t>(out) + 1] = L.y;
                path_rgb[3 * static_cast<size_t>(out) + 2] = L.z;
            } else {
                atomicAdd(&accum[out], make_float4(L.x, L.y, L.z, 0.0f));
            }
        }
    }
    if (COUNT)
        flush_counts(cnt, counters);
}

// Both subpaths of one path (the draw order of k_bdpt_power): the camera subpath from the cached
// first hit f, then the light pick, the emission point and direction and the light subpath.
// Returns the light's index; clen = 0 when the camera ray missed.
template <bool COUNT, class R>
__device__ __forceinline__ int sample_subpaths(DevScene const &S, R &rng, FirstHit const &f, uint32_t max_len, BV *cam,
                                               BV *lp, uint32_t &clen, uint32_t &llen, uint32_t *stk,
                                               TraceCounters *cnt) {
    int32_t mesh = __float_as_int(f.p.w);
    float3 o0 = neg(xyz(f.d));
    clen = 0;
    llen = 0;
    if (mesh >= 0 && max_len) {
        cam[0].p = xyz(f.p);
        cam[0].n = xyz(f.n);
        cam[0].mesh = mesh;
        cam[0].beta = f3(1.0f, 1.0f, 1.0f);
        cam[0].fwd = 1.0f;
        cam[0].rev = 0.0f;
        clen = bdp_walk<COUNT>(S, rng, cam, 1, max_len, o0, stk, cnt);
    }
    float pmf;
    int light = sample_light(S, rng, pmf);
    uint32_t lmesh = __ldg(&S.light_mesh[light]);
    Surf em = mesh_sample(S, lmesh, rng, true);
    float3 w = cos_hemisphere(em.n, rng);
    float pdf_w = dot(em.n, w) / kPi;
    if (max_len) {
        lp[0].p = em.p;
        lp[0].n = em.n;
        lp[0].mesh = static_cast<int32_t>(lmesh);
        lp[0].fwd = pmf * em.area_dens;
        lp[0].rev = 0.0f;
        float ib = 1.0f / lp[0].fwd;
        lp[0].beta = f3(ib, ib, ib);
        llen = 1;
        if (pdf_w > 0.0f && max_len > 1) {
            if (COUNT)
                cnt->rays++;
            Hit h = trace_closest<COUNT>(S, em.p, w, stk, cnt);
            if (h.tri != 0xFFFFFFFFu) {
                Vert v0 = make_vert(S, h);
                if (dot(v0.n, neg(w)) > 0.0f) {
                    lp[1].p = v0.p;
                    lp[1].n = v0.n;
                    lp[1].mesh = v0.mesh;
                    lp[1].beta = scale(light_rad(S, light), dot(em.n, w) / (pdf_w * lp[0].fwd));
                    lp[1].fwd = to_area(pdf_w, em.p, lp[1].p, lp[1].n);
                    lp[1].rev = 0.0f;
                    llen = bdp_walk<COUNT>(S, rng, lp, 2, max_len, neg(w), stk, cnt);
                }
            }
        }
    }
    return light;
}

template <class R, bool COUNT>
__global__ void __launch_bounds__(kBlock) k_bdpt_power(DevScene S, RenderArgs A, FirstHit const *__restrict__ fh,
                                                       float4 *accum, float *path_rgb, unsigned long long *work,
                                                       unsigned long long *counters) {
    TraceCounters cnt{0, 0, 0};
    __shared__ uint32_t stk_all[kStackWords * kBlock];
    uint32_t *stk = stk_all + threadIdx.x;
    const uint64_t mix = splitmix64(A.seed);
    const uint32_t lane = lane_id();
    const uint32_t max_len = A.bdpt_max_len < kMaxSub ? A.bdpt_max_len : kMaxSub;
    BV cam[kMaxSub], lp[kMaxSub];
    while (true) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32ull);
        base = __shfl_sync(~0u, base, 0);
        if (base >= A.total_paths)
            break;
        uint64_t idx = base + lane;
        uint32_t pixel, sample, out;
        if (idx < A.total_paths && path_coords(A, idx, pixel, sample, out)) {
            R rng;
            seed_path(rng, A, mix, pixel, sample);
            FirstHit f = fh[pixel];
            uint32_t clen, llen;
            int light = sample_subpaths<COUNT>(S, rng, f, max_len, cam, lp, clen, llen, stk, &cnt);
            float3 L = clen ? connect_power<COUNT>(S, cam, clen, lp, llen, max_len, neg(xyz(f.d)), light, stk, &cnt)
                            : f3(0, 0, 0);
            if (path_rgb) {
                path_rgb[3 * static_cast<size_t>(out)] = L.x;
                path_rgb[3 * static_cast<size_t>(out) + 1] = L.y;
                path_rgb[3 * static_cast<size_t>(out) + 2] = L.z;
            } else {
                atomicAdd(&accum[out], make_float4(L.x, L.y, L.z, 0.0f));
            }
        }
    }
    if (COUNT)
        flush_counts(cnt, counters);
}

// ---- E8G_MODE_BDPT_POWER, split form (E8G_INTEGRATOR_WAVEFRONT) ----
// One thread per path of k_bdpt_power waits, with its warp, for the path with the longest
// subpaths and the most connections (every (t, s) pair traces a shadow ray), and its lanes diverge
// on every early exit and traversal. The split form runs the same estimator per chunk of paths as
// two wavefronts:
//   the walk     path slots (WfSlots) advance both subpaths of their paths one vertex per
//                bounce: k_bdw_walk shades (completes the last ray's vertex, samples the next
//                direction, the same draws in the same order as sample_subpaths), the wavefront's
//                trace kernel traces the extension queue; a finished path stores its record and
//                appends one entry per (t, s) strategy that can contribute (s = 0 only when the
//                camera vertex lies on a light), and its slot takes the next path;
//   connections  k_bdw_eval evaluates one entry per thread without tracing (BSDFs, geometry
//                term, the power-heuristic weight from the stored densities with the four it
//                changes); s = 0 terms go to the output at once, the others become shadow rays
//                carrying their weighted contribution, which the wavefront's trace kernel drains.
// A path's radiance is the same sum of the same terms, added in another order.

// Stored vertex: three float4 (p | mesh), (n | fwd), (beta | rev).
__device__ __forceinline__ void bdw_store(float4 *dst, BV const &v) {
    dst[0] = make_float4(v.p.x, v.p.y, v.p.z, __int_as_float(v.mesh));
    dst[1] = make_float4(v.n.x, v.n.y, v.n.z, v.fwd);
    dst[2] = make_float4(v.beta.x, v.beta.y, v.beta.z, v.rev);
}
__device__ __forceinline__ BV bdw_load(float4 const *src) {
    float4 a = src[0], b = src[1], c = src[2];
    BV v;
    v.p = xyz(a);
    v.mesh = __float_as_int(a.w);
    v.n = xyz(b);
    v.fwd = b.w;
    v.beta = xyz(c);
    v.rev = c.w;
    return v;
}

// One step of a subpath walk at its last vertex cur (the loop body of bdp_walk up to the trace):
// samples the next direction; false when the walk ends there. On true: the ray, the throughput of
// the vertex it will make, the sampling density and the reverse density at the current vertex.
template <class R>
__device__ __forceinline__ bool walk_sample(DevScene const &S, R &rng, BV const &cur, float3 wo, float3 &org,
                                            float3 &dir, float3 &beta_next, float &pdf, float &prev_w) {
    const DevMaterial &m = vert_mat(S, cur.mesh);
    float3 i = bsdf_sample_mis<true>(S, m, rng, pdf, cur.n, wo);
    if (!(pdf > 0.0f))
        return false;
    float cw = dot(cur.n, i);
    if (cw <= 0.0f)
        return false;
    float3 f = bsdf_eval<true>(S, m, cur.n, wo, i);
    beta_next = mul(cur.beta, scale(f, cw / pdf));
    prev_w = bsdf_pdf<true>(S, m, cur.n, i, wo); // vpdf(cur, i, wo)
    org = cur.p;
    dir = i;
    return true;
}

// The rest of the step once the ray's hit is known: stores vertex len (also into nx) and the
// reverse density of vertex len-2; false when the walk ends (miss or back face). cp: the ray's
// origin, vertex len-1.
__device__ __forceinline__ bool walk_complete(DevScene const &S, float4 *sub, uint32_t len, Hit const &h, float3 cp,
                                              float3 dir, float3 beta_next, float pdf, float prev_w, BV &nx) {
    if (h.tri == 0xFFFFFFFFu)
        return false;
    Vert nv = make_vert(S, h);
    if (dot(nv.n, neg(dir)) <= 0.0f)
        return false;
    nx.p = nv.p;
    nx.n = nv.n;
    nx.mesh = nv.mesh;
    nx.beta = beta_next;
    nx.fwd = to_area(pdf, cp, nx.p, nx.n);
    nx.rev = 0.0f;
    bdw_store(sub + 3 * len, nx);
    if (len >= 2) {
        float4 pp = sub[3 * (len - 2)], pn = sub[3 * (len - 2) + 1];
        reinterpret_cast<float *>(sub + 3 * (len - 2) + 2)[3] = to_area(prev_w, cp, xyz(pp), xyz(pn));
    }
    return true;
}

// Slot state of the walk: stage in bits 0-1 (kWkEmpty, kWkCam: a camera-subpath ray is pending,
// kWkLight: a light-subpath ray is pending), the current subpath's stored vertices in bits 2-6,
// the camera subpath's length in bits 7-11.
enum : uint32_t { kWkEmpty = 0, kWkCam = 1, kWkLight = 2 };
constexpr int kWalkRounds = 4; // paths a slot may start and finish without a ray in one bounce

// One bounce of the walk over every slot. range: the chunk's first path index and path count
// (device memory, so one captured graph serves every chunk). W.next_path: the chunk's path
// counter; W.sid: the slot's path (index in the chunk), W.out: its light, W.beta_pdf: throughput
// of the pending vertex | sampling density, W.o: ray direction | reverse density.
// The materials' code is out of line and the kernel held to 64 registers (four blocks of 256 per
// SM): the walk stalled on instruction fetch with it inlined, and at three blocks per SM (80
// registers, no spills) it took 52.1 ms per 1280x720, 32-spp frame against 47.6 ms at four.
template <class R>
__global__ void __launch_bounds__(256, 4)
    k_bdw_walk(DevScene S, RenderArgs A, FirstHit const *__restrict__ fh, float *path_rgb, BdwChunk C, WfSlots W,
               uint64_t const *range, uint32_t *ext_n, uint32_t *busy) {
    const uint64_t mix = splitmix64(A.seed);
    const uint32_t max_len = C.max_len;
    const uint64_t first = range[0];
    const uint32_t count = static_cast<uint32_t>(range[1]);
    const uint32_t lane = lane_id();
    uint32_t busy_local = 0;
    for (uint32_t s0 = blockIdx.x * blockDim.x; s0 < W.capacity; s0 += gridDim.x * blockDim.x) {
        const uint32_t s = s0 + threadIdx.x;
        const bool in = s < W.capacity;
        const uint32_t st = in ? W.state[s] : kWkEmpty;
        uint32_t stage = st & 3u, len = (st >> 2) & 31u, clen = (st >> 7) & 31u;
        uint32_t path = 0, pixel = 0, sample = 0, light = 0;
        R rng;
        float3 wo = f3(0, 0, 0), org = f3(0, 0, 0), dir = f3(0, 0, 0), beta_next = f3(0, 0, 0);
        float pdf = 0.0f, prev_w = 0.0f;
        bool at_vertex = false; // at stored vertex len-1 (cur) with the walk going on (else it ended)
        BV cur{};
        if (stage != kWkEmpty) { // complete the pending ray
            path = W.sid[s];
            pixel = W.pixel[s];
            sample = W.sample[s];
            light = W.out[s];
            rng = RngSlot<R>::load(A, pixel, sample, W.rng[s]);
            float4 hv = W.hit[s], od = W.o[s], bp = W.beta_pdf[s];
            Hit h;
            h.t = hv.x;
            h.tri = __float_as_uint(hv.y);
            h.b1 = hv.z;
            h.b2 = hv.w;
            float4 *sub = C.vtx + static_cast<size_t>(path) * 6 * max_len + (stage == kWkLight ? 3 * max_len : 0);
            if (walk_complete(S, sub, len, h, xyz(sub[3 * (len - 1)]), xyz(od), xyz(bp), bp.w, od.w, cur)) {
                len++;
                wo = neg(xyz(od));
                at_vertex = true;
            }
        }
        // once the chunk's path counter has passed its last path (it only grows), no slot takes a
        // path for the rest of the chunk: the tail bounces skip the refill atomics
        bool emitted = false, paths_left = __ldcg(W.next_path) < count;
        for (int round = 0; round < kWalkRounds; round++) {
            // a new path for every empty slot, one atomic per warp
            bool want = in && stage == kWkEmpty && paths_left;
            uint32_t mask = __ballot_sync(~0u, want);
            if (mask) {
                int leader = __ffs(mask) - 1;
                unsigned long long base = 0;
                if (static_cast<int>(lane) == leader)
                    base = atomicAdd(W.next_path, static_cast<unsigned long long>(__popc(mask)));
                base = __shfl_sync(~0u, base, leader);
                if (want) {
                    uint64_t idx = base + __popc(mask & ((1u << lane) - 1u));
                    uint32_t out;
                    if (idx >= count) {
                        paths_left = false;
                    } else if (path_coords(A, first + idx, pixel, sample, out)) {
                        path = static_cast<uint32_t>(idx);
                        seed_path(rng, A, mix, pixel, sample);
                        FirstHit f = fh[pixel];
                        const float3 o0 = neg(xyz(f.d));
                        C.o0[path] = make_float4(o0.x, o0.y, o0.z, 0.0f);
                        stage = kWkCam;
                        len = 0;
                        at_vertex = false;
                        int32_t mesh = __float_as_int(f.p.w);
                        if (mesh >= 0 && max_len) {
                            BV v0;
                            v0.p = xyz(f.p);
                            v0.n = xyz(f.n);
                            v0.mesh = mesh;
                            v0.beta = f3(1.0f, 1.0f, 1.0f);
                            v0.fwd = 1.0f;
                            v0.rev = 0.0f;
                            bdw_store(C.vtx + static_cast<size_t>(path) * 6 * max_len, v0);
                            cur = v0;
                            len = 1;
                            wo = o0;
                            at_vertex = true;
                        }
                    }
                }
            }
            // advance the lane's path until it waits for a ray or is finished
            bool done = false;
            for (int k = 0; k < 3 && !emitted && !done && stage != kWkEmpty; k++) {
                if (at_vertex && len < max_len && walk_sample(S, rng, cur, wo, org, dir, beta_next, pdf, prev_w)) {
                    emitted = true;
                    break;
                }
                at_vertex = false;
                if (stage == kWkLight) { // the light subpath ended: len vertices
                    done = true;
                    break;
                }
                // the camera subpath ended: the light's emission sample (sample_subpaths' order)
                clen = len;
                float pmf;
                int li = sample_light(S, rng, pmf);
                light = static_cast<uint32_t>(li);
                uint32_t lmesh = __ldg(&S.light_mesh[li]);
                Surf em = mesh_sample(S, lmesh, rng, true);
                float3 w = cos_hemisphere(em.n, rng);
                float pdf_w = dot(em.n, w) / kPi;
                stage = kWkLight;
                len = 0;
                if (max_len) {
                    BV l0;
                    l0.p = em.p;
                    l0.n = em.n;
                    l0.mesh = static_cast<int32_t>(lmesh);
                    l0.fwd = pmf * em.area_dens;
                    l0.rev = 0.0f;
                    float ib = 1.0f / l0.fwd;
                    l0.beta = f3(ib, ib, ib);
                    bdw_store(C.vtx + static_cast<size_t>(path) * 6 * max_len + 3 * max_len, l0);
                    len = 1;
                    if (pdf_w > 0.0f && max_len > 1) {
                        org = em.p;
                        dir = w;
                        beta_next = scale(light_rad(S, li), dot(em.n, w) / (pdf_w * l0.fwd));
                        pdf = pdf_w;
                        prev_w = 0.0f;
                        emitted = true;
                        break;
                    }
                }
                done = true; // a light subpath of at most one vertex
            }
            // finished paths: record, output cleared, connection entries (one atomic per warp)
            uint32_t n_conn = 0;
            float4 const *cam = C.vtx + static_cast<size_t>(path) * 6 * max_len;
            if (done) {
                uint32_t px, smp, out = 0;
                path_coords(A, first + path, px, smp, out);
                C.info[path] = make_int4(static_cast<int>(clen | len << 8), static_cast<int>(light),
                                         static_cast<int>(out), 0);
                if (path_rgb) {
                    path_rgb[3 * static_cast<size_t>(out)] = 0.0f;
                    path_rgb[3 * static_cast<size_t>(out) + 1] = 0.0f;
                    path_rgb[3 * static_cast<size_t>(out) + 2] = 0.0f;
                }
                for (uint32_t t = 1; t <= clen; t++)
                    n_conn += len + (__ldg(&S.mesh_light[__float_as_int(cam[3 * (t - 1)].w)]) >= 0 ? 1u : 0u);
            }
            uint32_t incl = n_conn;
            for (int off = 1; off < 32; off <<= 1) {
                uint32_t y = __shfl_up_sync(~0u, incl, off);
                if (static_cast<int>(lane) >= off)
                    incl += y;
            }
            uint32_t total = __shfl_sync(~0u, incl, 31), start = 0;
            if (lane == 31 && total)
                start = atomicAdd(C.conn_n, total);
            start = __shfl_sync(~0u, start, 31);
            if (n_conn) {
                uint32_t pos = start + incl - n_conn;
                for (uint32_t t = 1; t <= clen; t++) {
                    uint32_t sl0 = __ldg(&S.mesh_light[__float_as_int(cam[3 * (t - 1)].w)]) >= 0 ? 0u : 1u;
                    for (uint32_t sl = sl0; sl <= len; sl++)
                        C.conn[pos++] = static_cast<uint64_t>(path) << 10 | (t - 1) << 5 | sl;
                }
            }
            if (done) {
                stage = kWkEmpty;
                len = clen = 0;
            }
            if (__ballot_sync(~0u, in && stage == kWkEmpty && paths_left) == 0)
                break;
        }
        // the slot's ray to the extension queue, one atomic per warp
        uint32_t mask = __ballot_sync(~0u, emitted);
        uint32_t base = 0;
        if (mask) {
            int leader = __ffs(mask) - 1;
            if (static_cast<int>(lane) == leader)
                base = atomicAdd(ext_n, static_cast<uint32_t>(__popc(mask)));
            base = __shfl_sync(~0u, base, leader);
        }
        if (in) {
            if (emitted) {
                uint32_t q = base + __popc(mask & ((1u << lane) - 1u));
                if (E8G_CHK(S.check, q < W.capacity, kChkQueue, q)) {
                    W.ext_o[q] = make_float4(org.x, org.y, org.z, __uint_as_float(s));
                    W.ext_d[q] = make_float4(dir.x, dir.y, dir.z, 0.0f);
                }
                W.state[s] = stage | len << 2 | clen << 7;
                W.sid[s] = path;
                W.pixel[s] = pixel;
                W.sample[s] = sample;
                W.out[s] = light;
                W.rng[s] = RngSlot<R>::store(rng);
                W.beta_pdf[s] = make_float4(beta_next.x, beta_next.y, beta_next.z, pdf);
                W.o[s] = make_float4(dir.x, dir.y, dir.z, prev_w);
                busy_local++;
            } else {
                W.state[s] = kWkEmpty;
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1)
        busy_local += __shfl_down_sync(~0u, busy_local, off);
    if (lane == 0 && busy_local)
        atomicAdd(busy, busy_local);
}

// Power-heuristic density of the BSDF at a stored vertex (vpdf on its mesh and normal).
__device__ __forceinline__ float bdw_pdf(DevScene const &S, int32_t mesh, float3 n, float3 wo, float3 wi) {
    return bsdf_pdf<true>(S, vert_mat(S, mesh), n, wo, wi);
}

// Held to 80 registers (six blocks of 128 per SM; 42.7 against 43.0 ms per frame at 96 registers).
__global__ void __launch_bounds__(kBlock, 6) k_bdw_eval(DevScene S, float4 *accum, float *path_rgb, BdwChunk C,
                                                     WfSlots W, uint32_t *shadow_n, uint32_t first, uint32_t n) {
    const uint32_t maxlen = C.max_len;
    const uint32_t lane = lane_id();
    // warp-uniform loop: every lane reaches the shadow-queue append
    for (uint32_t q0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); q0 < n; q0 += gridDim.x * blockDim.x) {
        const uint32_t q = q0 + lane;
        const uint32_t entry = first + q;
        bool push = false;
        float3 org = f3(0, 0, 0), dir = f3(0, 0, 0), L = f3(0, 0, 0);
        float tmax = 0.0f;
        uint32_t out = 0;
        do {
            if (q >= n)
                break;
            const uint64_t e = C.conn[entry];
            const uint32_t path = static_cast<uint32_t>(e >> 10), t = ((e >> 5) & 31u) + 1u,
                           sl = static_cast<uint32_t>(e & 31u);
            const int4 inf = C.info[path];
            out = static_cast<uint32_t>(inf.z);
            float4 const *cam = C.vtx + static_cast<size_t>(path) * 6 * maxlen;
            float4 const *lpv = cam + 3 * maxlen;
            const BV cv = bdw_load(cam + 3 * (t - 1));
            BV c2{};
            if (t >= 2)
                c2 = bdw_load(cam + 3 * (t - 2));
            const float3 wo_c = t >= 2 ? normalize(sub(c2.p, cv.p)) : xyz(C.o0[path]);
            // the densities this connection changes: camera vertices t-1, t-2; light vertices s-1, s-2
            float rc1 = cv.rev, rc2 = c2.rev, rl1 = 0.0f, rl2 = 0.0f;
            float3 contrib;
            if (sl == 0) {
                int hl = __ldg(&S.mesh_light[cv.mesh]);
                if (hl < 0)
                    break;
                float3 le = light_radiance(S, hl, wo_c, cv.n);
                if (vequals0(le))
                    break;
                contrib = mul(cv.beta, le);
                float pl = __ldg(&S.light_pnorm[hl]) / S.total_power;
                rc1 = pl * (1.0f / __ldg(&S.mesh_area[__ldg(&S.light_mesh[hl])]));
                if (t >= 2) {
                    float ew = fmaxf(dot(cv.n, wo_c), 0.0f) / kPi;
                    rc2 = to_area(ew, cv.p, c2.p, c2.n);
                }
            } else {
                const BV lv = bdw_load(lpv + 3 * (sl - 1));
                float3 d = sub(lv.p, cv.p);
                float d2 = dot(d, d);
                if (d2 <= 0.0f)
                    break;
                float dist = sqrtf(d2);
                dir = divs(d, dist);
                float cos_c = dot(cv.n, dir);
                float cos_l = dot(lv.n, neg(dir));
                if (cos_c <= 0.0f || cos_l <= 0.0f)
                    break;
                float3 fc = bsdf_eval<true>(S, vert_mat(S, cv.mesh), cv.n, wo_c, dir);
                if (vequals0(fc))
                    break;
                float3 fl, wo_l = f3(0, 0, 0);
                float4 l2p = make_float4(0, 0, 0, 0), l2n = make_float4(0, 0, 0, 0);
                if (sl == 1) {
                    fl = light_radiance(S, inf.y, neg(dir), lv.n);
                } else {
                    l2p = lpv[3 * (sl - 2)];
                    l2n = lpv[3 * (sl - 2) + 1];
                    wo_l = normalize(sub(xyz(l2p), lv.p));
                    fl = bsdf_eval<true>(S, vert_mat(S, lv.mesh), lv.n, neg(dir), wo_l);
                }
                if (vequals0(fl))
                    break;
                float G = cos_c * cos_l / d2;
                contrib = scale(mul(mul(mul(cv.beta, fc), fl), lv.beta), G);
                float pc = bdw_pdf(S, cv.mesh, cv.n, wo_c, dir);
                rl1 = to_area(pc, cv.p, lv.p, lv.n);
                if (sl == 1)
                    rc1 = to_area(cos_l / kPi, lv.p, cv.p, cv.n);
                else
                    rc1 = to_area(bdw_pdf(S, lv.mesh, lv.n, wo_l, neg(dir)), lv.p, cv.p, cv.n);
                if (t >= 2)
                    rc2 = to_area(bdw_pdf(S, cv.mesh, cv.n, dir, wo_c), cv.p, c2.p, c2.n);
                if (sl >= 2)
                    rl2 = to_area(bdw_pdf(S, lv.mesh, lv.n, neg(dir), wo_l), lv.p, xyz(l2p), xyz(l2n));
                org = cv.p;
                tmax = dist - 1e-3f;
            }
            // the weight of connect_power, densities read from the stored subpaths
            float sum = 0.0f, ri = 1.0f;
            for (int i = static_cast<int>(t) - 1; i >= 1; i--) {
                if (sl + t - static_cast<uint32_t>(i) > maxlen)
                    break;
                float fwd = cam[3 * i + 1].w;
                float rev = i == static_cast<int>(t) - 1 ? rc1 : i == static_cast<int>(t) - 2 ? rc2 : cam[3 * i + 2].w;
                ri *= (fwd > 0.0f) ? rev / fwd : 0.0f;
                sum += ri * ri;
            }
            ri = 1.0f;
            for (int i = static_cast<int>(sl) - 1; i >= 0; i--) {
                if (t + sl - static_cast<uint32_t>(i) > maxlen)
                    break;
                float fwd = lpv[3 * i + 1].w;
                float rev = i == static_cast<int>(sl) - 1 ? rl1 : i == static_cast<int>(sl) - 2 ? rl2 : lpv[3 * i + 2].w;
                ri *= (fwd > 0.0f) ? rev / fwd : 0.0f;
                sum += ri * ri;
            }
            L = scale(contrib, 1.0f / (1.0f + sum));
            if (sl == 0) { // no shadow ray: the camera subpath itself reached a light
                if (path_rgb) {
                    atomicAdd(&path_rgb[3 * static_cast<size_t>(out)], L.x);
                    atomicAdd(&path_rgb[3 * static_cast<size_t>(out) + 1], L.y);
                    atomicAdd(&path_rgb[3 * static_cast<size_t>(out) + 2], L.z);
                } else {
                    atomicAdd(&accum[out], make_float4(L.x, L.y, L.z, 0.0f));
                }
            } else {
                push = true;
            }
        } while (false);
        // warp-aggregated append to the shadow queue
        uint32_t mask = __ballot_sync(~0u, push);
        uint32_t base = 0;
        if (mask) {
            int leader = __ffs(mask) - 1;
            if (static_cast<int>(lane) == leader)
                base = atomicAdd(shadow_n, static_cast<uint32_t>(__popc(mask)));
            base = __shfl_sync(~0u, base, leader);
        }
        if (push) {
            uint32_t slot = base + __popc(mask & ((1u << lane) - 1u));
            if (E8G_CHK(S.check, slot < W.capacity, kChkQueue, slot)) {
                W.sh_o[slot] = make_float4(org.x, org.y, org.z, __uint_as_float(out));
                W.sh_d[slot] = make_float4(dir.x, dir.y, dir.z, tmax);
                W.sh_c[slot] = make_float4(L.x, L.y, L.z, 0.0f);
            }
        }
    }
}

} // namespace

int bdpt_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_bdpt_ref<RngMinstd, false>, kBlock, 0);
    return n > 0 ? n : 1;
}

// ---- bidirect_lt2_path_tracer (pathtracer.cpp:655-752) ----

// join_with_light_paths (pathtracer.cpp:655-699): one light sample (transport_direct_illum)
// plus a one-vertex light path joined to tv; a light ray that misses drops both terms.
template <class R>
__device__ __forceinline__ float3 lt2_join(DevScene const &S, R &rng, PV const &tv, uint32_t cam_len, uint32_t *stk) {
    float pmf;
    int light = sample_light(S, rng, pmf);
    Surf ls = mesh_sample(S, __ldg(&S.light_mesh[light]), rng, false);
    ls.area_dens *= pmf;
    float3 p1 = divs(add(f3(0, 0, 0), divs(illum_source<false>(S, light, ls.p, ls.n, tv, stk, nullptr), ls.area_dens)), 1.0f);
    float pmf2;
    int light2 = sample_light(S, rng, pmf2);
    Surf em = mesh_sample(S, __ldg(&S.light_mesh[light2]), rng, false); // area_light::sample_emssion
    float3 w = cos_hemisphere(em.n, rng);
    float sa_dens = dot(em.n, w) / kPi;
    Hit lh = trace_closest<false>(S, em.p, w, stk, nullptr);
    if (lh.tri == 0xFFFFFFFFu)
        return f3(0, 0, 0);
    float3 illum = divs(light_projected(S, light2, w, em.n), pmf2 * em.area_dens * sa_dens);
    Vert term = make_vert(S, lh);
    float3 tray = neg(w);
    float3 join = sub(tv.p, term.p);
    float dist = norm(join);
    join = divs(join, dist);
    float cos_w2 = dot(term.n, tray);
    float cos_wo = dot(term.n, join);
    float cos_wi = dot(tv.n, neg(join));
    if (cos_wo > 0.0f && cos_wi > 0.0f && cos_w2 > 0.0f &&
        !trace_any<false>(S, term.p, join, 1e-4f, dist - 1e-3f, stk, nullptr)) {
        float3 f2 = scale(mul(illum, bsdf_eval<true>(S, vert_mat(S, term.mesh), term.n, join, tray)), cos_w2);
        float3 p2 = scale(mul(divs(scale(f2, cos_wo), dist * dist), bsdf_eval<true>(S, vert_mat(S, tv.mesh), tv.n, tv.v, neg(join))),
                          cos_wi);
        return cam_len == 0 ? add(p1, scale(p2, 0.5f)) : scale(add(p1, p2), 0.5f);
    }
    return p1;
}

// One thread per path. The reference recurses, value(v) = (join(v) + g(v) value(next)) / survive
// with g = f cos / pdf (sample_indirect_illum, :701-729); the kernel walks forwards with the
// throughput beta and adds beta / survive x join(v) at each vertex. Russian roulette from depth
// rr_start (the reference's mutate_depth = 1, e8g_default_params' value for this mode); a
// continuation whose ray hits nothing keeps the vertex's join term, one that leaves below the
// surface drops it and ends the path; the continuation's hit is not tested for back faces.
template <class R>
__global__ void __launch_bounds__(kBlock) k_lt2(DevScene S, RenderArgs A, FirstHit const *__restrict__ fh,
                                                float4 *accum, float *path_rgb, unsigned long long *work) {
    __shared__ uint32_t stk_all[kStackWords * kBlock];
    uint32_t *stk = stk_all + threadIdx.x;
    const uint64_t mix = splitmix64(A.seed);
    const uint32_t lane = lane_id();
    while (true) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32ull);
        base = __shfl_sync(~0u, base, 0);
        if (base >= A.total_paths)
            break;
        uint64_t idx = base + lane;
        uint32_t pixel, sample, out;
        if (idx < A.total_paths && path_coords(A, idx, pixel, sample, out)) {
            R rng;
            seed_path(rng, A, mix, pixel, sample);
            FirstHit f = fh[pixel];
            float3 L = f3(0, 0, 0);
            int32_t fmesh = __float_as_int(f.p.w);
            if (fmesh >= 0) {
                PV tv;
                tv.v = neg(xyz(f.d));
                tv.p = xyz(f.p);
                tv.n = xyz(f.n);
                tv.mesh = fmesh;
                tv.light = -1;
                tv.dens = 1.0f;
                float3 beta = f3(1.0f, 1.0f, 1.0f);
                for (uint32_t depth = 0; depth < kHardDepth; depth++) {
                    if (A.max_depth && depth >= A.max_depth)
                        break;
                    float surv = 1.0f;
                    if (depth >= A.rr_start) {
                        if (rng.next() >= A.rr_prob)
                            break;
                        surv = A.rr_prob;
                    }
                    float3 bid = lt2_join(S, rng, tv, depth, stk);
                    float pdf;
                    float3 i = bsdf_sample_ref<true>(S, vert_mat(S, tv.mesh), rng, pdf, tv.n, tv.v);
                    Hit h = trace_closest<false>(S, tv.p, i, stk, nullptr);
                    float3 bl = divs(beta, surv);
                    if (h.tri == 0xFFFFFFFFu) {
                        L = add(L, mul(bl, bid));
                        break;
                    }
                    float cw = dot(tv.n, i);
                    if (cw < 0.0f)
                        break;
                    L = add(L, mul(bl, bid));
                    float3 fv = bsdf_eval<true>(S, vert_mat(S, tv.mesh), tv.n, tv.v, i);
                    beta = divs(scale(mul(bl, fv), cw), pdf);
                    Vert nv = make_vert(S, h);
                    tv.v = neg(i);
                    tv.p = nv.p;
                    tv.n = nv.n;
                    tv.mesh = nv.mesh;
                }
                int32_t fl = __float_as_int(f.n.w);
                if (fl >= 0)
                    L = add(L, light_projected(S, fl, neg(xyz(f.d)), xyz(f.n)));
            }
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

int bdpt_eval_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_bdw_eval, kBlock, 0);
    return n > 0 ? n : 1;
}

void launch_bdpt_walk(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float *path_rgb, BdwChunk const &C,
                      WfSlots const &W, uint64_t const *range, int grid, cudaStream_t st) {
    if (A.rng == E8G_RNG_MINSTD)
        k_bdw_walk<RngMinstd><<<grid, 256, 0, st>>>(S, A, fh, path_rgb, C, W, range, wf_ext_count_ptr(W), wf_busy_ptr(W));
    else
        k_bdw_walk<RngPhilox><<<grid, 256, 0, st>>>(S, A, fh, path_rgb, C, W, range, wf_ext_count_ptr(W), wf_busy_ptr(W));
}

void launch_bdpt_eval(DevScene const &S, float4 *accum, float *path_rgb, BdwChunk const &C, WfSlots const &Q,
                      uint32_t first, uint32_t n, int grid, cudaStream_t st) {
    k_bdw_eval<<<grid, kBlock, 0, st>>>(S, accum, path_rgb, C, Q, wf_shadow_count_ptr(Q), first, n);
}

void launch_bdpt(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float4 *accum, float *path_rgb,
                 unsigned long long *work, int grid, cudaStream_t st, unsigned long long *counters) {
    bool minstd = A.rng == E8G_RNG_MINSTD;
    if (A.mode == E8G_MODE_BDPT_POWER) {
        if (counters && minstd)
            k_bdpt_power<RngMinstd, true><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, counters);
        else if (counters)
            k_bdpt_power<RngPhilox, true><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, counters);
        else if (minstd)
            k_bdpt_power<RngMinstd, false><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, nullptr);
        else
            k_bdpt_power<RngPhilox, false><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, nullptr);
        return;
    }
    if (A.mode == E8G_MODE_REF_LT2) {
        if (minstd)
            k_lt2<RngMinstd><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work);
        else
            k_lt2<RngPhilox><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work);
        return;
    }
    if (counters && minstd)
        k_bdpt_ref<RngMinstd, true><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, counters);
    else if (counters)
        k_bdpt_ref<RngPhilox, true><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, counters);
    else if (minstd)
        k_bdpt_ref<RngMinstd, false><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, nullptr);
    else
        k_bdpt_ref<RngPhilox, false><<<grid, kBlock, 0, st>>>(S, A, fh, accum, path_rgb, work, nullptr);
}

} // namespace e8g
