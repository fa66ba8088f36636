// Wavefront integrator for the product estimator (E8G_MODE_MIS).
//
// Path states live in structure-of-arrays slots (capacity Q). One bounce of the whole wavefront
// is three kernels:
//   k_wf_shade   every slot: finish the pending extension hit (emission with MIS weight, or
//                termination), refill empty slots with new paths (warp-aggregated fetch), then
//                shade the vertex: Russian roulette, one light sample whose shadow ray goes to
//                the shadow queue, one BSDF sample whose ray goes to the extension queue;
//   k_wf_shadow  drains the shadow queue: any-hit, adds unoccluded contributions to the image;
//   k_wf_extend  drains the extension queue: closest hit into the slot.
// Queue kernels are persistent (grid = SMs x resident blocks, grid-stride over the device-side
// queue length). The bounce loop is captured once as a CUDA graph of `k` bounces and replayed
// until no slot is busy. Per path, draws happen in the same order as in the megakernel, so
// both integrators produce the same per-path radiance.
#include "../../include/e8g.h"
#include "wavefront.h"

#include <algorithm>

namespace e8g {

namespace {

// kVertexReady: the split form's completion kernel has turned the slot's extension hit into its
// vertex (slot arrays vp, vn) and added the vertex's emission.
enum : uint32_t { kEmpty = 0, kAtVertex = 1, kWaitHit = 2, kVertexReady = 3 };

// Refill rounds per slot and bounce: a lane skips paths whose camera ray missed the scene for at
// most this many rounds (a frame that is half sky leaves a slot empty after 8 rounds with
// probability 1/256).
constexpr int kRefillRounds = 8;

struct Counters {
    unsigned long long next_path; // global path counter
    uint32_t shadow_n, ext_n;      // queue lengths of the current bounce
    uint32_t busy;                 // slots holding a path after the last shade
    uint32_t shadow_head, ext_head; // next queue entry to hand out (dynamic fetch)
    uint32_t pad;
};

__device__ __forceinline__ void emit_to(RenderArgs const &A, float4 *accum, float *path_rgb, uint32_t out, float3 c) {
    if (path_rgb) {
        atomicAdd(&path_rgb[3 * static_cast<size_t>(out)], c.x);
        atomicAdd(&path_rgb[3 * static_cast<size_t>(out) + 1], c.y);
        atomicAdd(&path_rgb[3 * static_cast<size_t>(out) + 2], c.z);
    } else {
        atomicAdd(&accum[out], make_float4(c.x, c.y, c.z, 0.0f));
    }
}

// Warp-aggregated append: one atomic per warp for all lanes with `want`.
__device__ __forceinline__ uint32_t warp_append(uint32_t *counter, bool want) {
    uint32_t mask = __ballot_sync(__activemask(), want);
    if (!want)
        return 0;
    uint32_t lane = lane_id();
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (static_cast<int>(lane) == leader)
        base = atomicAdd(counter, static_cast<uint32_t>(__popc(mask)));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// The scene table of a many-scene wavefront: MULTI kernels look a path's scene and render
// arguments up by its scene index; single-scene kernels use their parameters.
template <bool MULTI>
__device__ __forceinline__ DevScene const &scene_of(DevScene const &S0, BatchDev const &B, uint32_t sid) {
    if constexpr (MULTI)
        return B.scenes[sid];
    else
        return S0;
}
template <bool MULTI>
__device__ __forceinline__ RenderArgs const &args_of(RenderArgs const &A0, BatchDev const &B, uint32_t sid) {
    if constexpr (MULTI)
        return B.args[sid];
    else
        return A0;
}

// Shading of every slot. MULTI: paths of many scenes share the slots; a slot keeps its path's
// scene index, `out` is the path's pixel in the concatenated accumulator and first hits are
// indexed the same way. Shading waits on slot and vertex loads: more resident warps hide more of
// them, fewer registers spill more. The block shape (THREADS, MINB resident blocks per SM, which
// sets the register cap) and OUT (the materials' code out of line, one copy for every call site:
// the inlined form overflows the instruction cache) are one of kShadeShape, chosen by the
// wavefront tuner.
template <class R, bool MULTI, int THREADS, int MINB, bool OUT, bool SPLIT = false>
__global__ void __launch_bounds__(THREADS, MINB)
    k_wf_shade(const __grid_constant__ DevScene S0, const __grid_constant__ RenderArgs A0, BatchDev B,
               FirstHit const *__restrict__ fh, WfSlots W, Counters *cnt, float4 *accum, float *path_rgb,
               uint64_t total_paths) {
    const uint64_t mix0 = MULTI ? 0 : splitmix64(A0.seed);
    // Read once per thread: once the path counter has passed the last path (it only grows), no
    // slot can be refilled for the rest of the frame, and the tail bounces skip the refill atomics
    // (one per warp and slot group on a single address).
    const bool paths_left = __ldcg(W.next_path) < total_paths;
    uint32_t busy_local = 0;
    for (uint32_t s0 = blockIdx.x * blockDim.x; s0 < W.capacity; s0 += gridDim.x * blockDim.x) {
        uint32_t s = s0 + threadIdx.x;
        bool in = s < W.capacity;
        uint32_t state = in ? W.state[s] : kEmpty;
        uint32_t sid = 0, pixel = 0, sample = 0, out = 0;
        float3 beta = f3(0, 0, 0), p = f3(0, 0, 0), n = f3(0, 0, 0), o = f3(0, 0, 0);
        int32_t mesh = 0;
        uint32_t depth = 0;
        float last_pdf = 0.0f;
        R rng;
        if (state != kEmpty) {
            if (MULTI)
                sid = W.sid[s];
            pixel = W.pixel[s];
            sample = W.sample[s];
            out = W.out[s];
            float4 b = W.beta_pdf[s];
            beta = xyz(b);
            last_pdf = b.w;
            // a stored slot always waits for its extension hit: the vertex comes from the hit, so
            // only the direction and the depth travel between bounces
            float4 od = W.o[s];
            o = xyz(od);
            depth = __float_as_uint(od.w);
            rng = RngSlot<R>::load(args_of<MULTI>(A0, B, sid), pixel, sample, W.rng[s]);
        }
        if (SPLIT && state == kVertexReady) { // completed by k_wf_complete
            float4 vp = W.vp[s], vn = W.vn[s];
            p = xyz(vp);
            mesh = __float_as_int(vp.w);
            n = xyz(vn);
            depth = __float_as_uint(vn.w);
            state = kAtVertex;
        }
        if (!SPLIT && state == kWaitHit) { // complete the extension ray shot last bounce
            DevScene const &S = scene_of<MULTI>(S0, B, sid);
            float4 hv = W.hit[s];
            Hit h;
            h.t = hv.x;
            h.tri = __float_as_uint(hv.y);
            h.b1 = hv.z;
            h.b2 = hv.w;
            float3 i = neg(o);
            state = kEmpty;
            if (h.tri != 0xFFFFFFFFu) {
                Vert nv = make_vert(S, h);
                if (dot(nv.n, neg(i)) > 0.0f) {
                    int32_t hl = __ldg(&S.mesh_light[nv.mesh]);
                    if (hl >= 0) {
                        float cos_l2 = dot(nv.n, neg(i));
                        float pl = __ldg(&S.light_pnorm[hl]) / S.total_power;
                        float inv_area = 1.0f / __ldg(&S.mesh_area[__ldg(&S.light_mesh[hl])]);
                        float p_l = pl * inv_area * (nv.t * nv.t) / cos_l2;
                        float w = power_heuristic(last_pdf, p_l);
                        emit_to(A0, accum, path_rgb, out, scale(mul(beta, light_rad(S, hl)), w));
                    }
                    p = nv.p;
                    n = nv.n;
                    mesh = nv.mesh;
                    depth++;
                    state = kAtVertex;
                }
            }
        }
        // refill empty slots, one atomic per warp per round. A path whose camera ray left the
        // scene (its cached first hit is a miss) has no vertex and contributes nothing, so the
        // lane draws again, up to kRefillRounds rounds, instead of leaving the slot idle for the
        // whole bounce; the megakernel's refill does the same.
        bool want = paths_left && in && state == kEmpty;
        bool refilled = false;
        for (int round = 0; round < kRefillRounds; round++) {
            uint32_t mask = __ballot_sync(~0u, want);
            if (!mask)
                break;
            int leader = __ffs(mask) - 1;
            unsigned long long base = 0;
            if (static_cast<int>(lane_id()) == leader)
                base = atomicAdd(W.next_path, static_cast<unsigned long long>(__popc(mask)));
            base = __shfl_sync(~0u, base, leader);
            if (want) {
                uint64_t idx = base + __popc(mask & ((1u << lane_id()) - 1u));
                if (idx >= total_paths) {
                    want = false; // the path counter only grows: nothing left for this lane
                } else {
                    uint32_t nsid = 0;
                    uint64_t local = idx, pbase = 0;
                    if (MULTI) { // the scene whose path range holds idx
                        uint32_t lo = 0, hi = B.n;
                        while (hi - lo > 1) {
                            uint32_t mi = (lo + hi) >> 1;
                            if (B.path_prefix[mi] <= idx)
                                lo = mi;
                            else
                                hi = mi;
                        }
                        nsid = lo;
                        local = idx - B.path_prefix[lo];
                        pbase = B.pix_prefix[lo];
                    }
                    RenderArgs const &A = args_of<MULTI>(A0, B, nsid);
                    if (path_coords(A, local, pixel, sample, out)) {
                        FirstHit f = fh[pbase + pixel];
                        int32_t m = __float_as_int(f.p.w);
                        if (m >= 0) {
                            sid = nsid;
                            out += static_cast<uint32_t>(pbase);
                            p = xyz(f.p);
                            n = xyz(f.n);
                            o = neg(xyz(f.d));
                            mesh = m;
                            depth = 0;
                            beta = f3(1.0f, 1.0f, 1.0f);
                            rng = RngSlot<R>::fresh(A, MULTI ? splitmix64(A.seed) : mix0, pixel, sample);
                            int32_t light = __float_as_int(f.n.w);
                            if (light >= 0)
                                emit_to(A, accum, path_rgb, out,
                                        light_radiance(scene_of<MULTI>(S0, B, sid), light, o, n));
                            state = kAtVertex;
                            refilled = true;
                            want = false;
                        }
                    }
                }
            }
        }
        // shade the vertex
        bool push_shadow = false, push_ext = false;
        float3 sh_dir = f3(0, 0, 0), sh_c = f3(0, 0, 0);
        float sh_tmax = 0.0f;
        if (state == kAtVertex) {
            DevScene const &S = scene_of<MULTI>(S0, B, sid);
            RenderArgs const &A = args_of<MULTI>(A0, B, sid);
            state = kEmpty;
            bool go = !((A.max_depth && depth >= A.max_depth) || depth >= kHardDepth);
            if (go && depth >= A.rr_start) {
                if (rng.next() >= A.rr_prob)
                    go = false;
                else
                    beta = divs(beta, A.rr_prob);
            }
            if (go) {
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
                    float3 f = bsdf_eval<OUT>(S, m, n, o, wi);
                    if (!vequals0(f)) {
                        float p_l = pmf * ls.area_dens * r2 / cos_l;
                        float p_b = bsdf_pdf<OUT>(S, m, n, o, wi);
                        float w = power_heuristic(p_l, p_b);
                        sh_c = scale(mul(mul(beta, f), light_rad(S, light)), cos_x * w / p_l);
                        sh_dir = wi;
                        sh_tmax = dist - 1e-3f;
                        push_shadow = true;
                    }
                }
                float pdf;
                float3 i = bsdf_sample_mis<OUT>(S, m, rng, pdf, n, o);
                if (pdf > 0.0f) {
                    float cw = dot(n, i);
                    if (cw > 0.0f) {
                        float3 f = bsdf_eval<OUT>(S, m, n, o, i);
                        beta = mul(beta, scale(f, cw / pdf));
                        o = neg(i);
                        last_pdf = pdf;
                        push_ext = true;
                        state = kWaitHit;
                    }
                }
            }
        }
        uint32_t sq = warp_append(&cnt->shadow_n, push_shadow);
        if (push_shadow && !E8G_CHK(S0.check, sq < W.capacity, kChkQueue, sq))
            push_shadow = false;
        if (push_shadow) {
            W.sh_o[sq] = make_float4(p.x, p.y, p.z, __uint_as_float(out));
            W.sh_d[sq] = make_float4(sh_dir.x, sh_dir.y, sh_dir.z, sh_tmax);
            W.sh_c[sq] = make_float4(sh_c.x, sh_c.y, sh_c.z, __uint_as_float(sid));
        }
        uint32_t eq = warp_append(&cnt->ext_n, push_ext);
        if (push_ext && !E8G_CHK(S0.check, eq < W.capacity, kChkQueue, eq))
            push_ext = false;
        if (push_ext) {
            W.ext_o[eq] = make_float4(p.x, p.y, p.z, __uint_as_float(s));
            W.ext_d[eq] = make_float4(-o.x, -o.y, -o.z, __uint_as_float(sid));
        }
        if (in) {
            W.state[s] = state;
            if (state != kEmpty) {
                if (refilled) { // a path keeps its pixel, sample, output slot and scene
                    W.pixel[s] = pixel;
                    W.sample[s] = sample;
                    W.out[s] = out;
                    if (MULTI)
                        W.sid[s] = sid;
                }
                W.beta_pdf[s] = make_float4(beta.x, beta.y, beta.z, last_pdf);
                W.o[s] = make_float4(o.x, o.y, o.z, __uint_as_float(depth));
                W.rng[s] = RngSlot<R>::store(rng);
                busy_local++;
            }
        }
    }
    // busy count for the host's termination test
    for (int off = 16; off > 0; off >>= 1)
        busy_local += __shfl_down_sync(~0u, busy_local, off);
    if (lane_id() == 0 && busy_local)
        atomicAdd(&cnt->busy, busy_local);
}

__global__ void __launch_bounds__(kBlock) k_wf_shadow(DevScene S, RenderArgs A, WfSlots W, Counters const *cnt,
                                                      float4 *accum, float *path_rgb) {
    __shared__ uint32_t stk[kStackWords * kBlock];
    uint32_t n = cnt->shadow_n;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        float4 so = W.sh_o[q], sd = W.sh_d[q];
        if (!trace_any<false>(S, xyz(so), xyz(sd), 1e-4f, sd.w, stk + threadIdx.x, nullptr))
            emit_to(A, accum, path_rgb, __float_as_uint(so.w), xyz(W.sh_c[q]));
    }
}

__global__ void __launch_bounds__(kBlock) k_wf_extend(DevScene S, WfSlots W, Counters const *cnt) {
    __shared__ uint32_t stk[kStackWords * kBlock];
    uint32_t n = cnt->ext_n;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        float4 eo = W.ext_o[q];
        Hit h = trace_closest<false>(S, xyz(eo), xyz(W.ext_d[q]), stk + threadIdx.x, nullptr);
        W.hit[__float_as_uint(eo.w)] = make_float4(h.t, __uint_as_float(h.tri), h.b1, h.b2);
    }
}

// The split form's completion of the extension rays traced last bounce, one thread per queue
// entry: the hit becomes the slot's vertex (vp: position | mesh, vn: normal | depth) and its
// emission is added with the MIS weight; a miss or a back-facing hit empties the slot. A small
// kernel of scene gathers, at full residency; the shading kernel then reads the vertex.
__global__ void __launch_bounds__(256, 8)
    k_wf_complete(const __grid_constant__ DevScene S, const __grid_constant__ RenderArgs A, WfSlots W,
                  Counters const *cnt, float4 *accum, float *path_rgb) {
    const uint32_t n = cnt->ext_n;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        uint32_t s = __float_as_uint(W.ext_o[q].w);
        float4 hv = W.hit[s];
        Hit h;
        h.t = hv.x;
        h.tri = __float_as_uint(hv.y);
        h.b1 = hv.z;
        h.b2 = hv.w;
        uint32_t state = kEmpty;
        if (h.tri != 0xFFFFFFFFu) {
            float4 od = W.o[s];
            float3 o = xyz(od);
            Vert nv = make_vert(S, h);
            float cos_l2 = dot(nv.n, o);
            if (cos_l2 > 0.0f) {
                int32_t hl = __ldg(&S.mesh_light[nv.mesh]);
                if (hl >= 0) {
                    float4 b = W.beta_pdf[s];
                    float pl = __ldg(&S.light_pnorm[hl]) / S.total_power;
                    float inv_area = 1.0f / __ldg(&S.mesh_area[__ldg(&S.light_mesh[hl])]);
                    float p_l = pl * inv_area * (nv.t * nv.t) / cos_l2;
                    float w = power_heuristic(b.w, p_l);
                    emit_to(A, accum, path_rgb, W.out[s], scale(mul(xyz(b), light_rad(S, hl)), w));
                }
                W.vp[s] = make_float4(nv.p.x, nv.p.y, nv.p.z, __int_as_float(nv.mesh));
                W.vn[s] = make_float4(nv.n.x, nv.n.y, nv.n.z, __uint_as_float(__float_as_uint(od.w) + 1u));
                state = kVertexReady;
            }
        }
        W.state[s] = state;
    }
}

// Persistent trace kernel with per-lane dynamic fetch: a lane whose ray is finished takes the
// next queue entry; lanes are refilled together (one atomic) once at least `threshold` of them
// are idle, or when none is busy. WIDE: the eight-wide tree (one node visit per step), else the
// SAH child pairs.
// The wide tree's stack takes 2 * kWideStack words per thread (16 KB per block), so its kernels
// fit eight blocks per SM when they are held to 64 registers. Measured on the 1080p, 64-spp
// frame of the 1.3M-triangle scene: 6 blocks (75 registers, no spills) 72.1 ms, 7 (70) 67.9 ms,
// 8 (64) 66.3 ms, 9 (56, 64-byte spills) 69.9 ms, 10 (48) 76.9 ms.
constexpr int kWfWideBlocks = 8;

// Queue entries a warp reserves with one atomic on the queue head; its idle lanes take entries
// from that reserve first. Measured on the 1080p, 64-spp frame: one atomic per refill (the
// entries of that refill only) 39.5 ms of tracing per frame at its best refill threshold (12);
// reserves of 32 entries 37.4 ms at threshold 8 (64: 37.5 ms): fewer atomics on one address
// make refills cheap enough for warps to refill sooner.
constexpr uint32_t kWarpChunk = 32;

template <bool ANY, bool WIDE>
__global__ void __launch_bounds__(kBlock, WIDE ? kWfWideBlocks : 1)
    k_wf_trace_dyn(DevScene S, RenderArgs A, WfSlots W, Counters *cnt, float4 *accum, float *path_rgb,
                   uint32_t threshold) {
    __shared__ uint32_t stk_all[(WIDE ? 2 * kWideStack : kStackWords) * kBlock];
    uint32_t *stk = stk_all + threadIdx.x;
    const uint32_t n = ANY ? cnt->shadow_n : cnt->ext_n;
    uint32_t *head = ANY ? &cnt->shadow_head : &cnt->ext_head;
    const uint32_t lane = lane_id();
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    const WideView WV{S.wnodes, S.tri, S.nnodes, S.ntris, S.check};
    uint32_t q = kNone;
    bool exhausted = false;  // the same in every lane: the queue and the warp's reserve are empty
    uint32_t wb = 0, we = 0; // the warp's reserved entries [wb, we)
    bool gdrained = false;
    uint32_t qw = 0; // the lane's ray's output (shadow) or slot (extension), kept from the refill
    TravState T;
    WideTrav TW;
    while (true) {
        bool idle = q == kNone && !exhausted;
        uint32_t im = __ballot_sync(~0u, idle);
        uint32_t busy = __ballot_sync(~0u, q != kNone);
        if (im && (__popc(im) >= threshold || busy == 0)) {
            const uint32_t k = static_cast<uint32_t>(__popc(im));
            const uint32_t avail = we - wb;
            uint32_t nb = 0, ne = 0;
            if (avail < k && !gdrained) {
                uint32_t want = kWarpChunk > k ? kWarpChunk : k;
                if (lane == 0)
                    nb = atomicAdd(head, want);
                nb = __shfl_sync(~0u, nb, 0);
                ne = nb + want < n ? nb + want : n;
                if (nb >= n) {
                    gdrained = true;
                    ne = nb;
                }
            }
            const uint32_t r = __popc(im & ((1u << lane) - 1u));
            uint32_t qq = kNone;
            if (r < avail)
                qq = wb + r;
            else if (r - avail < ne - nb)
                qq = nb + (r - avail);
            const uint32_t t_old = k < avail ? k : avail;
            wb += t_old;
            if (ne > nb) {
                uint32_t t_new = k - t_old < ne - nb ? k - t_old : ne - nb;
                wb = nb + t_new;
                we = ne;
            }
            exhausted = gdrained && wb >= we;
            if (idle) {
                if (qq != kNone) {
                    q = qq;
                    float3 ro, rd;
                    float tmax;
                    if (ANY) {
                        float4 so = W.sh_o[q], sd = W.sh_d[q];
                        ro = xyz(so);
                        rd = xyz(sd);
                        tmax = sd.w;
                        qw = __float_as_uint(so.w);
                    } else {
                        float4 eo = W.ext_o[q];
                        ro = xyz(eo);
                        rd = xyz(W.ext_d[q]);
                        tmax = 1000.0f;
                        qw = __float_as_uint(eo.w);
                    }
                    if (WIDE)
                        wide_begin(TW, ro, rd, 1e-4f, tmax, ANY);
                    else
                        trav_begin(S, T, ro, rd, 1e-4f, tmax);
                }
            }
            busy = __ballot_sync(~0u, q != kNone);
        }
        if (busy == 0) {
            if (__ballot_sync(~0u, !exhausted) == 0)
                break;
            continue;
        }
        if (q == kNone)
            continue;
        bool done = WIDE ? wide_step(WV, TW, stk, kBlock, nullptr, nullptr) : trav_step<ANY>(S, T, stk);
        if (done) {
            if (ANY) {
                bool occluded = WIDE ? TW.h.tri != 0xFFFFFFFFu : T.found;
                if (!occluded)
                    emit_to(A, accum, path_rgb, qw, xyz(W.sh_c[q]));
            } else {
                Hit b = WIDE ? TW.h : T.best;
                W.hit[qw] = make_float4(b.t, __uint_as_float(b.tri), b.b1, b.b2);
            }
            q = kNone;
        }
    }
}

// Both queues of a bounce in one launch on the eight-wide tree: queue positions below ext_n are
// extension rays (closest hit), the rest shadow rays (any hit), so a bounce has one kernel tail
// instead of two. Per-lane dynamic fetch like k_wf_trace_dyn's, from warp reserves. MULTI: each
// ray carries its scene index (w of its direction or of its contribution) and traces that
// scene's tree.
template <bool MULTI>
__global__ void __launch_bounds__(kBlock, kWfWideBlocks)
    k_wf_trace_wide_both(const __grid_constant__ DevScene S0, RenderArgs A, BatchDev B, WfSlots W, Counters *cnt,
                         float4 *accum, float *path_rgb, uint32_t threshold) {
    __shared__ uint32_t stk_all[2 * kWideStack * kBlock];
    uint32_t *stk = stk_all + threadIdx.x;
    const uint32_t n_ext = cnt->ext_n, n = n_ext + cnt->shadow_n;
    uint32_t *head = &cnt->ext_head;
    const uint32_t lane = lane_id();
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    WideView WV{S0.wnodes, S0.tri, S0.nnodes, S0.ntris, S0.check};
    uint32_t q = kNone;
    bool drained = false; // the same in every lane: the queue had no entry left for this warp
    uint32_t wb = 0, we = 0; // the warp's reserved entries [wb, we) (the same in every lane)
    bool gdrained = false;
    // the lane's ray's slot (extension) or output (shadow), kept from the refill: reading it back
    // from the queue at the ray's end cost 3.6% of the kernel's time
    uint32_t qw = 0;
    WideTrav T;
    while (true) {
        uint32_t busy = __ballot_sync(~0u, q != kNone);
        uint32_t im = drained ? 0u : ~busy; // idle lanes
        if (im && (__popc(im) >= threshold || busy == 0)) {
            const uint32_t k = static_cast<uint32_t>(__popc(im));
            const uint32_t avail = we - wb;
            uint32_t nb = 0, ne = 0;
            if (avail < k && !gdrained) {
                uint32_t want = kWarpChunk > k ? kWarpChunk : k;
                if (lane == 0)
                    nb = atomicAdd(head, want);
                nb = __shfl_sync(~0u, nb, 0);
                ne = nb + want < n ? nb + want : n;
                if (nb >= n) {
                    gdrained = true;
                    ne = nb;
                }
            }
            const uint32_t r = __popc(im & ((1u << lane) - 1u));
            uint32_t qq = kNone;
            if (r < avail)
                qq = wb + r;
            else if (r - avail < ne - nb)
                qq = nb + (r - avail);
            const uint32_t t_old = k < avail ? k : avail;
            wb += t_old;
            if (ne > nb) {
                uint32_t t_new = k - t_old < ne - nb ? k - t_old : ne - nb;
                wb = nb + t_new;
                we = ne;
            }
            drained = gdrained && wb >= we;
            if (q == kNone) {
                if (qq != kNone) {
                    q = qq;
                    uint32_t sid;
                    if (q < n_ext) {
                        float4 ed = W.ext_d[q], eo = W.ext_o[q];
                        sid = __float_as_uint(ed.w);
                        qw = __float_as_uint(eo.w);
                        wide_begin(T, xyz(eo), xyz(ed), 1e-4f, 1000.0f, false);
                    } else {
                        float4 sd = W.sh_d[q - n_ext], so = W.sh_o[q - n_ext];
                        sid = MULTI ? __float_as_uint(W.sh_c[q - n_ext].w) : 0;
                        qw = __float_as_uint(so.w);
                        wide_begin(T, xyz(so), xyz(sd), 1e-4f, sd.w, true);
                    }
                    if (MULTI) {
                        DevScene const &S = B.scenes[sid];
                        WV = WideView{S.wnodes, S.tri, S.nnodes, S.ntris, S.check};
                    }
                }
            }
            busy = __ballot_sync(~0u, q != kNone);
        }
        if (busy == 0) {
            if (drained)
                break;
            continue;
        }
        if (q == kNone)
            continue;
        if (wide_step(WV, T, stk, kBlock, nullptr, nullptr)) {
            if (q < n_ext) {
                uint32_t slot = qw;
                if (E8G_CHK(S0.check, slot < W.capacity, kChkSlot, slot))
                    W.hit[slot] = make_float4(T.h.t, __uint_as_float(T.h.tri), T.h.b1, T.h.b2);
            } else if (T.h.tri == 0xFFFFFFFFu) {
                uint32_t sq = q - n_ext;
                emit_to(A, accum, path_rgb, qw, xyz(W.sh_c[sq]));
            }
            q = kNone;
        }
    }
}

__global__ void k_wf_reset(Counters *cnt) {
    cnt->shadow_n = 0;
    cnt->ext_n = 0;
    cnt->busy = 0;
    cnt->shadow_head = 0;
    cnt->ext_head = 0;
}

} // namespace

// Lays the slot arrays and queues out from `base` (each array 256-byte aligned) and returns
// the bytes used in *total; with a null base it only measures (all pointers null).
static WfSlots carve(char *base, uint32_t capacity, size_t *total) {
    WfSlots W{};
    W.capacity = capacity;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *r = base ? base + off : nullptr;
        off += (bytes + 255) & ~static_cast<size_t>(255);
        return r;
    };
    size_t Q = capacity;
    W.state = reinterpret_cast<uint32_t *>(take(Q * 4));
    W.pixel = reinterpret_cast<uint32_t *>(take(Q * 4));
    W.sample = reinterpret_cast<uint32_t *>(take(Q * 4));
    W.out = reinterpret_cast<uint32_t *>(take(Q * 4));
    W.rng = reinterpret_cast<uint32_t *>(take(Q * 4));
    W.sid = reinterpret_cast<uint32_t *>(take(Q * 4));
    W.beta_pdf = reinterpret_cast<float4 *>(take(Q * 16));
    W.o = reinterpret_cast<float4 *>(take(Q * 16));
    W.hit = reinterpret_cast<float4 *>(take(Q * 16));
    W.sh_o = reinterpret_cast<float4 *>(take(Q * 16));
    W.sh_d = reinterpret_cast<float4 *>(take(Q * 16));
    W.sh_c = reinterpret_cast<float4 *>(take(Q * 16));
    W.ext_o = reinterpret_cast<float4 *>(take(Q * 16));
    W.ext_d = reinterpret_cast<float4 *>(take(Q * 16));
    W.vp = reinterpret_cast<float4 *>(take(Q * 16));
    W.vn = reinterpret_cast<float4 *>(take(Q * 16));
    W.counters = take(sizeof(Counters));
    W.next_path = base ? &reinterpret_cast<Counters *>(W.counters)->next_path : nullptr;
    *total = off;
    return W;
}

WfSlots wf_carve(void *base, uint32_t capacity) {
    size_t total = 0;
    return carve(static_cast<char *>(base), capacity, &total);
}

size_t wf_total_bytes(uint32_t capacity) {
    size_t total = 0;
    carve(nullptr, capacity, &total);
    return total;
}

// Resident blocks per SM of the trace kernels a bounce launches for this tree and threshold.
int wf_trace_blocks_per_sm(uint32_t layout, uint32_t threshold) {
    int a = 0, b = 0;
    if (threshold > 0 && layout == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_wf_trace_dyn<true, false>, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_wf_trace_dyn<false, false>, kBlock, 0);
    } else if (threshold > 0 && layout == 2) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_wf_trace_wide_both<false>, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_wf_trace_wide_both<true>, kBlock, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_wf_extend, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_wf_shadow, kBlock, 0);
    }
    int n = a < b ? a : b;
    return n > 0 ? n : 1;
}

// The shading kernel's shapes: threads per block, resident blocks per SM (the register cap is
// 65536 / (threads x blocks)) and whether the materials' code is out of line.
constexpr int kShadeShape[kWfShadeVariants][3] = {{256, 4, 0}, {256, 3, 0}, {256, 4, 1}, {256, 3, 1},
                                                  {256, 5, 1}, {128, 8, 1}, {256, 4, 0}, {256, 5, 0}};
// Shapes 6 and 7 run the split form: k_wf_complete first, then the shading kernel without the
// hit completion (fewer registers, a smaller instruction footprint).
constexpr bool shade_split(uint32_t v) { return v == 6 || v == 7; }

int wf_shade_threads(uint32_t variant) { return kShadeShape[variant < kWfShadeVariants ? variant : 0][0]; }
int wf_shade_blocks(uint32_t variant) { return kShadeShape[variant < kWfShadeVariants ? variant : 0][1]; }

int wf_shade_grid(uint32_t variant, uint32_t capacity, int num_sms) {
    variant = variant < kWfShadeVariants ? variant : 0;
    int t = kShadeShape[variant][0], b = kShadeShape[variant][1];
    return static_cast<int>(std::min<uint64_t>((capacity + t - 1) / t, static_cast<uint64_t>(num_sms) * b * 2));
}

template <class R>
static void launch_shade(uint32_t variant, int grid, cudaStream_t st, DevScene const &S, RenderArgs const &A,
                         FirstHit const *fh, WfSlots const &W, Counters *cnt, float4 *accum, float *path_rgb,
                         uint64_t total_paths) {
    BatchDev none{};
    switch (variant) {
    case 1:
        k_wf_shade<R, false, 256, 3, false><<<grid, 256, 0, st>>>(S, A, none, fh, W, cnt, accum, path_rgb, total_paths);
        break;
    case 2:
        k_wf_shade<R, false, 256, 4, true><<<grid, 256, 0, st>>>(S, A, none, fh, W, cnt, accum, path_rgb, total_paths);
        break;
    case 3:
        k_wf_shade<R, false, 256, 3, true><<<grid, 256, 0, st>>>(S, A, none, fh, W, cnt, accum, path_rgb, total_paths);
        break;
    case 4:
        k_wf_shade<R, false, 256, 5, true><<<grid, 256, 0, st>>>(S, A, none, fh, W, cnt, accum, path_rgb, total_paths);
        break;
    case 5:
        k_wf_shade<R, false, 128, 8, true><<<grid, 128, 0, st>>>(S, A, none, fh, W, cnt, accum, path_rgb, total_paths);
        break;
    case 6:
        k_wf_shade<R, false, 256, 4, false, true><<<grid, 256, 0, st>>>(S, A, none, fh, W, cnt, accum, path_rgb,
                                                                       total_paths);
        break;
    case 7:
        k_wf_shade<R, false, 256, 5, false, true><<<grid, 256, 0, st>>>(S, A, none, fh, W, cnt, accum, path_rgb,
                                                                       total_paths);
        break;
    default:
        k_wf_shade<R, false, 256, 4, false><<<grid, 256, 0, st>>>(S, A, none, fh, W, cnt, accum, path_rgb, total_paths);
    }
}

// One bounce: reset queue lengths, shade, then the trace kernel(s). B (or null): the scene table
// of a many-scene wavefront (eight-wide trees, dynamic fetch). timing (or null): three events
// recorded at the bounce's start, after its shading and after its trace kernel(s).
void wf_enqueue_bounce(DevScene const &S, RenderArgs const &A, FirstHit const *fh, WfSlots const &W, float4 *accum,
                       float *path_rgb, int shade_grid, int trace_grid, uint32_t threshold, uint64_t total_paths,
                       BatchDev const *B, cudaStream_t st, cudaEvent_t const *timing, uint32_t shade_variant) {
    auto *cnt = reinterpret_cast<Counters *>(W.counters);
    auto mark = [&](int k) {
        if (timing)
            cudaEventRecordWithFlags(timing[k], st, cudaEventRecordExternal);
    };
    mark(0);
    if (!B && shade_split(shade_variant))
        k_wf_complete<<<shade_grid, 256, 0, st>>>(S, A, W, cnt, accum, path_rgb);
    k_wf_reset<<<1, 1, 0, st>>>(cnt);
    if (B) { // the many-scene form shades with the first block shape
        if (A.rng == E8G_RNG_MINSTD)
            k_wf_shade<RngMinstd, true, 256, 4, false><<<shade_grid, 256, 0, st>>>(S, A, *B, fh, W, cnt, accum, nullptr,
                                                                                    total_paths);
        else
            k_wf_shade<RngPhilox, true, 256, 4, false><<<shade_grid, 256, 0, st>>>(S, A, *B, fh, W, cnt, accum, nullptr,
                                                                                    total_paths);
        mark(1);
        k_wf_trace_wide_both<true><<<trace_grid, kBlock, 0, st>>>(S, A, *B, W, cnt, accum, nullptr, threshold);
        mark(2);
        return;
    }
    BatchDev none{};
    if (A.rng == E8G_RNG_MINSTD)
        launch_shade<RngMinstd>(shade_variant, shade_grid, st, S, A, fh, W, cnt, accum, path_rgb, total_paths);
    else
        launch_shade<RngPhilox>(shade_variant, shade_grid, st, S, A, fh, W, cnt, accum, path_rgb, total_paths);
    mark(1);
    if (threshold > 0 && S.layout == 0) {
        k_wf_trace_dyn<true, false><<<trace_grid, kBlock, 0, st>>>(S, A, W, cnt, accum, path_rgb, threshold);
        k_wf_trace_dyn<false, false><<<trace_grid, kBlock, 0, st>>>(S, A, W, cnt, accum, path_rgb, threshold);
    } else if (threshold > 0 && S.layout == 2) {
        k_wf_trace_wide_both<false><<<trace_grid, kBlock, 0, st>>>(S, A, none, W, cnt, accum, path_rgb, threshold);
    } else {
        k_wf_shadow<<<trace_grid, kBlock, 0, st>>>(S, A, W, cnt, accum, path_rgb);
        k_wf_extend<<<trace_grid, kBlock, 0, st>>>(S, W, cnt);
    }
    mark(2);
}

void wf_enqueue_shade(DevScene const &S, RenderArgs const &A, FirstHit const *fh, WfSlots const &W, float4 *accum,
                      float *path_rgb, int shade_grid, uint64_t total_paths, cudaStream_t st, uint32_t shade_variant) {
    auto *cnt = reinterpret_cast<Counters *>(W.counters);
    if (shade_split(shade_variant))
        k_wf_complete<<<shade_grid, 256, 0, st>>>(S, A, W, cnt, accum, path_rgb);
    k_wf_reset<<<1, 1, 0, st>>>(cnt);
    if (A.rng == E8G_RNG_MINSTD)
        launch_shade<RngMinstd>(shade_variant, shade_grid, st, S, A, fh, W, cnt, accum, path_rgb, total_paths);
    else
        launch_shade<RngPhilox>(shade_variant, shade_grid, st, S, A, fh, W, cnt, accum, path_rgb, total_paths);
}

void wf_enqueue_trace(DevScene const &S, RenderArgs const &A, WfSlots const &W, float4 *accum, float *path_rgb,
                      int trace_grid, uint32_t threshold, cudaStream_t st) {
    auto *cnt = reinterpret_cast<Counters *>(W.counters);
    BatchDev none{};
    if (threshold > 0 && S.layout == 0) {
        k_wf_trace_dyn<true, false><<<trace_grid, kBlock, 0, st>>>(S, A, W, cnt, accum, path_rgb, threshold);
        k_wf_trace_dyn<false, false><<<trace_grid, kBlock, 0, st>>>(S, A, W, cnt, accum, path_rgb, threshold);
    } else if (threshold > 0 && S.layout == 2) {
        k_wf_trace_wide_both<false><<<trace_grid, kBlock, 0, st>>>(S, A, none, W, cnt, accum, path_rgb, threshold);
    } else {
        k_wf_shadow<<<trace_grid, kBlock, 0, st>>>(S, A, W, cnt, accum, path_rgb);
        k_wf_extend<<<trace_grid, kBlock, 0, st>>>(S, W, cnt);
    }
}

cudaError_t wf_init(WfSlots const &W, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(W.state, 0, static_cast<size_t>(W.capacity) * 4, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(W.counters, 0, sizeof(Counters), st);
    return e;
}

// Busy slots after the last bounce (read back by the host between graph replays).
uint32_t *wf_busy_ptr(WfSlots const &W) { return &reinterpret_cast<Counters *>(W.counters)->busy; }
size_t wf_counters_bytes() { return sizeof(Counters); }
uint32_t *wf_shadow_count_ptr(WfSlots const &W) { return &reinterpret_cast<Counters *>(W.counters)->shadow_n; }
uint32_t *wf_ext_count_ptr(WfSlots const &W) { return &reinterpret_cast<Counters *>(W.counters)->ext_n; }
void wf_enqueue_reset(WfSlots const &W, cudaStream_t st) { k_wf_reset<<<1, 1, 0, st>>>(reinterpret_cast<Counters *>(W.counters)); }
unsigned long long *wf_next_ptr(WfSlots const &W) { return &reinterpret_cast<Counters *>(W.counters)->next_path; }

} // namespace e8g
