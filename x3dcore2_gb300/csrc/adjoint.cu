// Path-replay adjoint of the product estimator (E8G_MODE_MIS): gradients of a loss on the image
// with respect to every material's albedo (3 channels) and GGX roughness.
//
// Each path is recomputed from its counter-based (Philox) stream; nothing is stored between the
// forward render and the adjoint. The BSDF value f_j used for the continuation at vertex j
// multiplies every contribution gathered after it, i.e. L - L_j with L the path's radiance and
// L_j the radiance gathered before that scatter; the BSDF value of the light sample at vertex j
// multiplies that sample's contribution only. Sampling densities and MIS weights are held fixed
// (weights still sum to one, so the gradient estimate stays unbiased), and since f is linear in
// albedo and d ln f / d r follows from GGX's D and G, each vertex adds
//     dL/d albedo_c += w_c (C_c / albedo_c)        dL/d r += (w . C) d ln f / d r
// with C the contribution it multiplies and w the upstream gradient of the path's pixel / spp.
// One walk does it: light-sample terms are added at once, and the first kScatterList scatters
// are recorded as (material, d ln f / d r, L_j) and added when the walk ends and L is known.
// A path with more scatters than that is walked a second time for the rest (the classic
// two-pass replay), which only paths longer than kScatterList vertices pay.
// Gradients are summed per block in shared memory and flushed with one atomic per material.
// Materials whose parameters do not enter f linearly (mixtures, the fail-safe material) and the
// Oren-Nayar sigma receive no gradient.
#include "../../include/e8g.h"
#include "adjoint.h"

namespace e8g {

namespace {

// d ln f / d r of cook_torr at (n, o, i), f = F D G / (4 cos_i cos_o) with alpha^2 = 2 r^2.
__device__ __forceinline__ float ct_dlog_dr(const DevMaterial &m, float3 n, float3 o, float3 i) {
    float3 h = add(i, o);
    if (vequals0(h))
        return 0.0f;
    h = normalize(h);
    float a2 = m.alpha2;
    float ch = dot(n, h);
    float c2 = ch * ch;
    float t2 = (1.0f - c2) / c2;
    float k = 1.0f + t2 / a2;
    float dlnD = -1.0f / a2 + 2.0f * t2 / (a2 * a2 * k);
    float ci = dot(n, i), co = dot(n, o);
    float ti = (1.0f - ci * ci) / (ci * ci), to = (1.0f - co * co) / (co * co);
    float si = sqrtf(1.0f + a2 * ti), so = sqrtf(1.0f + a2 * to);
    float li = (-1.0f + si) / 2.0f, lo = (-1.0f + so) / 2.0f;
    float dli = ti / (4.0f * si), dlo = to / (4.0f * so);
    float dlnG = -(dli + dlo) / (1.0f + li + lo);
    return (dlnD + dlnG) * 4.0f * m.rough;
}

struct GradAcc {
    float *a; // 3 per material (shared memory)
    float *r; // 1 per material
    uint32_t nmat;
};

constexpr uint32_t kScatterList = 8;

struct ScatterRec {
    int32_t mat;  // -1: no gradient (other material types)
    float dlog;   // d ln f / d r (cook_torr), else 0
    float3 L;     // radiance gathered before the scatter
};

// Material index receiving gradients at a vertex of this mesh, or -1.
__device__ __forceinline__ int32_t grad_mat(DevScene const &S, uint32_t nmat, int32_t mesh) {
    int32_t mi = __ldg(&S.mesh_mat[mesh]);
    if (mi < 0 || static_cast<uint32_t>(mi) >= nmat)
        return -1;
    uint32_t t = S.mats[mi].type;
    return (t == E8G_MAT_OREN_NAYAR || t == E8G_MAT_COOK_TORR) ? mi : -1;
}

__device__ __forceinline__ void add_grad_m(GradAcc &g, DevScene const &S, int32_t mi, float dlog, float3 C, float3 w) {
    const DevMaterial &m = S.mats[mi];
    if (m.albedo[0] > 0.0f)
        atomicAdd(&g.a[3 * mi], w.x * C.x / m.albedo[0]);
    if (m.albedo[1] > 0.0f)
        atomicAdd(&g.a[3 * mi + 1], w.y * C.y / m.albedo[1]);
    if (m.albedo[2] > 0.0f)
        atomicAdd(&g.a[3 * mi + 2], w.z * C.z / m.albedo[2]);
    if (m.type == E8G_MAT_COOK_TORR)
        atomicAdd(&g.r[mi], dot(w, C) * dlog);
}

__device__ __forceinline__ float grad_dlog(DevScene const &S, int32_t mi, float3 n, float3 o, float3 i) {
    const DevMaterial &m = S.mats[mi];
    return m.type == E8G_MAT_COOK_TORR ? ct_dlog_dr(m, n, o, i) : 0.0f;
}

// One walk of the MIS path in megakernel/oracle order.
// FIRST: adds the light-sample terms, records the first kScatterList scatters in `rec` and
// counts every scatter in *nscatter; returns L. !FIRST (second walk, L = Ltot known): adds the
// terms of scatters kScatterList and later only.
template <bool FIRST, int LAYOUT>
__device__ float3 replay(DevScene const &S, RenderArgs const &A, FirstHit const &f, uint32_t pixel, uint32_t sample,
                         float3 Ltot, float3 w, GradAcc &g, uint32_t *stk, ScatterRec *rec, uint32_t *nscatter) {
    RngPhiloxMem rng;
    rng.seed(A.seed, pixel, sample);
    float3 p = xyz(f.p), n = xyz(f.n), o = neg(xyz(f.d));
    int32_t mesh = __float_as_int(f.p.w);
    float3 L = f3(0, 0, 0);
    int32_t l0 = __float_as_int(f.n.w);
    if (l0 >= 0)
        L = light_radiance(S, l0, o, n);
    float3 beta = f3(1.0f, 1.0f, 1.0f);
    uint32_t scat = 0;
    for (uint32_t depth = 0;; depth++) {
        if ((A.max_depth && depth >= A.max_depth) || depth >= kHardDepth)
            break;
        if (depth >= A.rr_start) {
            if (rng.next() >= A.rr_prob)
                break;
            beta = divs(beta, A.rr_prob);
        }
        const DevMaterial &m = vert_mat(S, mesh);
        float pmf;
        int light = sample_light(S, rng, pmf);
        Surf ls = mesh_sample(S, __ldg(&S.light_mesh[light]), rng, true);
        float3 l = sub(p, ls.p);
        float r2 = dot(l, l);
        float dist = sqrtf(r2);
        float3 ln = divs(l, dist);
        float cos_l = dot(ls.n, ln);
        float3 wi = neg(ln);
        float cos_x = dot(n, wi);
        if (cos_l > 0.0f && cos_x > 0.0f) {
            float3 fv = bsdf_eval(S, m, n, o, wi);
            if (!vequals0(fv)) {
                float p_l = pmf * ls.area_dens * r2 / cos_l;
                float p_b = bsdf_pdf(S, m, n, o, wi);
                if (trace_l<LAYOUT, false>(S, p, wi, 1e-4f, dist - 1e-3f, true, stk, nullptr).tri == 0xFFFFFFFFu) {
                    float wgt = power_heuristic(p_l, p_b);
                    float3 c = scale(mul(mul(beta, fv), light_rad(S, light)), cos_x * wgt / p_l);
                    L = add(L, c);
                    if (FIRST) {
                        int32_t mi = grad_mat(S, g.nmat, mesh);
                        if (mi >= 0)
                            add_grad_m(g, S, mi, grad_dlog(S, mi, n, o, wi), c, w);
                    }
                }
            }
        }
        float pdf;
        float3 i = bsdf_sample_mis(S, m, rng, pdf, n, o);
        if (!(pdf > 0.0f))
            break;
        float cw = dot(n, i);
        if (cw <= 0.0f)
            break;
        float3 fv = bsdf_eval(S, m, n, o, i);
        if (FIRST) {
            if (scat < kScatterList) {
                int32_t mi = grad_mat(S, g.nmat, mesh);
                rec[scat].mat = mi;
                rec[scat].dlog = mi >= 0 ? grad_dlog(S, mi, n, o, i) : 0.0f;
                rec[scat].L = L;
            }
        } else if (scat >= kScatterList) {
            int32_t mi = grad_mat(S, g.nmat, mesh);
            if (mi >= 0)
                add_grad_m(g, S, mi, grad_dlog(S, mi, n, o, i), sub(Ltot, L), w); // gathered after this scatter
        }
        scat++;
        beta = mul(beta, scale(fv, cw / pdf));
        Hit h = trace_l<LAYOUT, false>(S, p, i, 1e-4f, 1000.0f, false, stk, nullptr);
        if (h.tri == 0xFFFFFFFFu)
            break;
        Vert nv = make_vert(S, h);
        if (dot(nv.n, neg(i)) <= 0.0f)
            break;
        int32_t hl = __ldg(&S.mesh_light[nv.mesh]);
        if (hl >= 0) {
            float cos_l2 = dot(nv.n, neg(i));
            float pl = __ldg(&S.light_pnorm[hl]) / S.total_power;
            float inv_area = 1.0f / __ldg(&S.mesh_area[__ldg(&S.light_mesh[hl])]);
            float p_l = pl * inv_area * (nv.t * nv.t) / cos_l2;
            L = add(L, scale(mul(beta, light_rad(S, hl)), power_heuristic(pdf, p_l)));
        }
        p = nv.p;
        n = nv.n;
        mesh = nv.mesh;
        o = neg(i);
    }
    if (FIRST)
        *nscatter = scat;
    return L;
}

template <int LAYOUT>
__global__ void __launch_bounds__(kBlock) k_adjoint(DevScene S, RenderArgs A, FirstHit const *__restrict__ fh,
                                                    float const *__restrict__ dl_dimage, float inv_spp,
                                                    unsigned long long *work, float *d_albedo, float *d_rough,
                                                    float *path_rgb) {
    __shared__ uint32_t stk_all[kStackWords * kBlock];
    extern __shared__ float sgrad[];
    GradAcc g{sgrad, sgrad + 3 * S.nmat, S.nmat};
    for (uint32_t k = threadIdx.x; k < 4 * S.nmat; k += blockDim.x)
        sgrad[k] = 0.0f;
    __syncthreads();
    uint32_t *stk = stk_all + threadIdx.x;
    const uint32_t lane = lane_id();
    while (true) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32ull);
        base = __shfl_sync(~0u, base, 0);
        if (base >= A.total_paths)
            break;
        uint64_t idx = base + lane;
        if (idx < A.total_paths) {
            uint32_t pixel, sample, out;
            bool ok = path_coords(A, idx, pixel, sample, out);
            if (ok) {
                FirstHit f = fh[pixel];
                if (__float_as_int(f.p.w) >= 0) {
                    float3 w = scale(f3(dl_dimage[3 * static_cast<size_t>(pixel)], dl_dimage[3 * static_cast<size_t>(pixel) + 1],
                                        dl_dimage[3 * static_cast<size_t>(pixel) + 2]),
                                     inv_spp);
                    ScatterRec rec[kScatterList];
                    uint32_t ns = 0;
                    float3 Ltot = replay<true, LAYOUT>(S, A, f, pixel, sample, f3(0, 0, 0), w, g, stk, rec, &ns);
                    uint32_t nl = ns < kScatterList ? ns : kScatterList;
                    for (uint32_t j = 0; j < nl; j++)
                        if (rec[j].mat >= 0)
                            add_grad_m(g, S, rec[j].mat, rec[j].dlog, sub(Ltot, rec[j].L), w);
                    if (ns > kScatterList)
                        replay<false, LAYOUT>(S, A, f, pixel, sample, Ltot, w, g, stk, nullptr, nullptr);
                    if (path_rgb) {
                        path_rgb[3 * idx] = Ltot.x;
                        path_rgb[3 * idx + 1] = Ltot.y;
                        path_rgb[3 * idx + 2] = Ltot.z;
                    }
                }
            }
        }
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < 3 * S.nmat; k += blockDim.x)
        if (sgrad[k] != 0.0f)
            atomicAdd(&d_albedo[k], sgrad[k]);
    for (uint32_t k = threadIdx.x; k < S.nmat; k += blockDim.x)
        if (sgrad[3 * S.nmat + k] != 0.0f)
            atomicAdd(&d_rough[k], sgrad[3 * S.nmat + k]);
}

} // namespace

cudaError_t launch_adjoint(DevScene const &S, RenderArgs const &A, FirstHit const *fh, float const *dl_dimage,
                           float inv_spp, unsigned long long *work, float *d_albedo, float *d_rough, float *path_rgb,
                           int num_sms, cudaStream_t st) {
    size_t smem = static_cast<size_t>(S.nmat) * 4 * sizeof(float);
    if (smem + kStackWords * kBlock * sizeof(uint32_t) > 200 * 1024)
        return cudaErrorInvalidValue;
    auto kern = S.layout == 1 ? k_adjoint<1>
                              : (S.layout == 2 ? k_adjoint<2> : (S.layout == 3 ? k_adjoint<3> : k_adjoint<0>));
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, smem);
    int grid = num_sms * (per_sm > 0 ? per_sm : 1);
    kern<<<grid, kBlock, smem, st>>>(S, A, fh, dl_dimage, inv_spp, work, d_albedo, d_rough, path_rgb);
    return cudaGetLastError();
}

} // namespace e8g
