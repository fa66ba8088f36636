// Device-side building blocks of the path-tracing core (sm_103a).
//
// Arithmetic that decides per-path results follows the reference's operation order
// (corelib/src/tensor.h vec ops, material.cpp, light.cpp, geometry.cpp) and the translation units
// that include this header are compiled with --fmad=false, so a kernel fed the same draws as the
// reference reproduces its floating-point results up to the last-ulp differences of CUDA's
// sinf/cosf/atanf against glibc.
#pragma once

#include "layout.h"
#include "wide_trav.h"

#include <cstdint>
#include <cuda_runtime.h>

namespace e8g {

constexpr float kPi = 3.14159274101257324f;    // static_cast<float>(M_PI)
constexpr float kInvPi = 0.318309873342514038f; // 1.0f / static_cast<float>(M_PI), 0x3ea2f983
constexpr int kBlock = 128;                     // threads per block of the traversal kernels
constexpr int kStack = 32;                      // per-thread (node, t) stack of the SAH layout (== kMaxTreeDepth)
constexpr int kStackWords = 2 * kStack;          // shared words per thread: 64 node entries in reference order
static_assert(2 * kWideStack <= kStackWords, "the eight-wide stack must fit the per-thread stack words");
static_assert(kWideStack >= 16, "bvh_wide.h kWideMaxDepth needs 16 stack entries");
constexpr float kOneMinusUlp = 0.999999940395355225f; // nextafter(1.0f, 0.0f)
// Safety stop for any path, whatever the policy (the C ABI rejects policies under which paths
// could approach it: survival <= 0.95 from depth <= 64 leaves a 1e-21 chance of reaching it).
constexpr uint32_t kHardDepth = 1024;

// ------------------------------------------------------------------ data layout ----

struct DevScene {
    const float4 *nlo;      // node min xyz | link
    const float4 *nhi;      // node max xyz | count
    const uint4 *wnodes;    // eight-wide layout: 6 uint4 per node (bvh_wide.h)
    const float4 *tri;      // 3 float4 per BVH position: (v0 | global tri id), (v1 - v0), (v2 - v0)
    const uint4 *tidx;      // per global triangle: global vertex indices, mesh
    const float4 *vpos;     // per vertex
    const float4 *vnrm;     // per vertex
    const float4 *vtx;      // per vertex, for shading: (position, normal.x), (normal.y, normal.z, 0, 0),
                            // one 32-byte sector per vertex instead of one in each array above
    const int32_t *mesh_mat;   // per mesh: material index (fail-safe remapped to nmat)
    const int32_t *mesh_light; // per mesh: light index or -1
    const uint32_t *mesh_toff; // num_meshes + 1
    const float *mesh_area;    // per mesh, trimesh::update_face_cdf (geometry.cpp:105-118)
    const float *tri_cum;      // per global triangle: prefix area inside its mesh
    const DevMaterial *mats;   // nmat + 1 entries, the last one is mat_fail_safe
    const uint32_t *light_mesh;
    const float4 *light_rad;
    const float *light_cum;    // basic_light_sources::commit CDF (lightsources.cpp:45-52)
    const float *light_pnorm;  // |power| per light
    uint32_t nmat, nl, nm, nnodes, ntris;
    uint32_t nverts;              // vertices (bounds checks of the debug build)
    unsigned long long *check;    // check word of the debug build (E8G_CHECKS), or null
    uint32_t layout; // 0: SAH child pairs (ordered traversal), 1: the reference's tree and order,
                     // 2: eight-wide quantized nodes, 3: no tree (every triangle, in order)
    float total_power;
    float bmin[3], bmax[3]; // if_path_space::aabb() for the position tracer
    DevCamera cam;
};

// Render-time arguments shared by every integrator kernel.
struct RenderArgs {
    uint32_t mode, rng, width, height, spp, sample_offset;
    uint64_t seed;
    uint32_t max_depth, rr_start;
    float rr_prob;
    uint32_t bdpt_max_len;
    uint32_t tiles_x, tiles_y;  // 8x4 pixel tiles, one warp's worth of paths per tile
    uint32_t paths_per_sample;  // tiles_x * tiles_y * 32
    uint64_t total_paths;       // paths_per_sample * spp (or the explicit list length)
    const uint32_t *list_pixel; // explicit (pixel, sample) list, or null
    const uint32_t *list_sample;
    uint32_t sample_major;      // image mode: per-path output at (sample - sample_offset) * W * H + pixel
};

// Map a path index to (pixel, sample) and its output slot: the list index (explicit lists), the
// pixel (image accumulation) or sample * W * H + pixel (per-sample images). Consecutive path
// indices cover 8x4 pixel tiles, one warp per tile, so a warp's first hits are neighbours.
// Returns false for padding lanes outside the image.
__device__ __forceinline__ bool path_coords(RenderArgs const &A, uint64_t idx, uint32_t &pixel, uint32_t &sample,
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
    out = A.sample_major ? s * (A.width * A.height) + pixel : pixel;
    return true;
}

// Per-pixel cached primary hit (compute_first_hit, pathtracer.cpp:456-472).
struct FirstHit {
    float4 p;  // vertex | mesh (int bits, -1 = invalid)
    float4 n;  // normal | light (int bits, -1 = none)
    float4 d;  // camera ray direction | unused
};

// ----------------------------------------------------------------- vector math ----
// Component-wise, in the reference's operand order (tensor.h:110-227).

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 add(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 neg(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 mul(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 scale(float3 a, float k) { return f3(k * a.x, k * a.y, k * a.z); }
__device__ __forceinline__ float3 divs(float3 a, float k) { return f3(a.x / k, a.y / k, a.z / k); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float norm(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) {
    float k = 1.0f / norm(a);
    return scale(a, k);
}
__device__ __forceinline__ bool feq0(float a) { return fabsf(a) <= 1e-5f; } // tensor.h:14-16
__device__ __forceinline__ bool vequals0(float3 a) { return feq0(a.x) && feq0(a.y) && feq0(a.z); }
__device__ __forceinline__ float3 xyz(float4 a) { return f3(a.x, a.y, a.z); }
__device__ __forceinline__ float smax(float a, float b) { return a < b ? b : a; }   // std::max
__device__ __forceinline__ float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

// ------------------------------------------------------------------------ random ----

// One std::minstd_rand0 stream per path feeding uniform_real_distribution<float>(0, 1) as
// libstdc++ does (tensor.h:987-1001): x <- 16807 x mod (2^31 - 1); u = float(x - 1) / 2^31,
// clamped below 1.
struct RngMinstd {
    uint32_t x;
    __device__ __forceinline__ void seed(uint32_t s) {
        x = s % 2147483647u;
        if (x == 0)
            x = 1;
    }
    __device__ __forceinline__ float next() {
        uint64_t p = static_cast<uint64_t>(x) * 16807ull; // < 2^46
        uint32_t r = static_cast<uint32_t>(p & 0x7FFFFFFFull) + static_cast<uint32_t>(p >> 31);
        if (r >= 2147483647u)
            r -= 2147483647u;
        x = r;
        float f = __uint2float_rn(r - 1u) * 4.656612873077392578125e-10f; // * 2^-31, exact
        return f >= 1.0f ? kOneMinusUlp : f;
    }
};

// Philox4x32-10 (Salmon et al., SC'11), counter (block, pixel, sample, tag), key = seed.
// Philox4x32-10 block `block` of the stream keyed (k0, k1) at counter (block, pixel, sample, const).
// Out of line: RngPhilox::next() is inlined at every draw site, and one copy of the ten rounds
// serves all of them (the shading kernels' code otherwise overflows the instruction cache). Its
// arguments and result are plain values, so the caller's stream state stays in registers.
static __device__ __noinline__ uint4 philox_block(uint32_t k0, uint32_t k1, uint32_t block, uint32_t pixel,
                                                  uint32_t sample) {
    uint32_t c0 = block, c1 = pixel, c2 = sample, c3 = 0x0E8A0E8Au;
    uint32_t a = k0, b = k1;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ a, n2 = hi0 ^ c3 ^ b;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        a += 0x9E3779B9u;
        b += 0xBB67AE85u;
    }
    return make_uint4(c0, c1, c2, c3);
}

struct RngPhilox {
    uint32_t k0, k1, pixel, sample, block, lane;
    uint32_t buf[4];
    __device__ __forceinline__ void seed(uint64_t s, uint32_t px, uint32_t smp) {
        k0 = static_cast<uint32_t>(s);
        k1 = static_cast<uint32_t>(s >> 32);
        pixel = px;
        sample = smp;
        block = 0;
        lane = 4;
    }
    __device__ __forceinline__ void refill() {
        uint4 r = philox_block(k0, k1, block, pixel, sample);
        buf[0] = r.x;
        buf[1] = r.y;
        buf[2] = r.z;
        buf[3] = r.w;
        block++;
        lane = 0;
    }
    __device__ __forceinline__ float next() {
        if (lane == 4)
            refill();
        uint32_t u = buf[0];
        // rotate so that the register array is indexed statically
        buf[0] = buf[1];
        buf[1] = buf[2];
        buf[2] = buf[3];
        lane++;
        return __uint2float_rz(u >> 8) * (1.0f / 16777216.0f);
    }
};

// The same stream with its state kept in local memory (the out-of-line refill takes the object's
// address): for kernels whose occupancy is held back by registers. The adjoint's replays run at
// five blocks per SM this way against four with the state in registers (backward 15.7 against
// 16.3 ms on the differentiable configuration).
struct RngPhiloxMem : RngPhilox {
    __device__ __noinline__ void refill_mem() {
        uint4 r = philox_block(k0, k1, block, pixel, sample);
        buf[0] = r.x;
        buf[1] = r.y;
        buf[2] = r.z;
        buf[3] = r.w;
        block++;
        lane = 0;
    }
    __device__ __forceinline__ float next() {
        if (lane == 4)
            refill_mem();
        uint32_t u = buf[0];
        buf[0] = buf[1];
        buf[1] = buf[2];
        buf[2] = buf[3];
        lane++;
        return __uint2float_rz(u >> 8) * (1.0f / 16777216.0f);
    }
};

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Seed of the per-path minstd stream (shared with the oracle's o_path_seed).
__host__ __device__ __forceinline__ uint32_t path_seed(uint64_t seed_mix, uint32_t pixel, uint32_t sample) {
    uint64_t z = splitmix64(seed_mix ^ ((static_cast<uint64_t>(pixel) << 32) | sample));
    uint32_t s = static_cast<uint32_t>(z % 2147483647ull);
    return s == 0 ? 1u : s;
}

// ----------------------------------------------------------------- traversal ----

struct TraceCounters {
    uint32_t nodes, tris;
    uint32_t rays; // counted by the callers that trace (the bidirectional kernels)
};

// Slab test of a node box against [tmin, tmax] (aabb::intersect, tensor.h:815-840, with the
// box inflated by the builder so rounding never culls a triangle the exact test would hit).
__device__ __forceinline__ bool slab(float4 lo, float4 hi, float3 o, float3 inv, float tmin, float tmax,
                                     float &tnear) {
    float x0 = (lo.x - o.x) * inv.x, x1 = (hi.x - o.x) * inv.x;
    float y0 = (lo.y - o.y) * inv.y, y1 = (hi.y - o.y) * inv.y;
    float z0 = (lo.z - o.z) * inv.z, z1 = (hi.z - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
    float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tmax));
    tnear = tn;
    return tn <= tf;
}

// ray::intersect (tensor.h:688-725) on a triangle stored as (v0, v1 - v0, v2 - v0).
__device__ __forceinline__ bool tri_test(float3 o, float3 d, float4 a, float4 b, float4 c, float tmin,
                                         float tmax, float &t0, float &b1o, float &b2o) {
    return hd_tri_test(o, d, a, b, c, tmin, tmax, t0, b1o, b2o);
}

// SAH child-pair tree. Closest hit (any = false) with the reference's strict `t0 < t`
// (pathspace.cpp:330-413) or any hit (has_intersect, pathspace.cpp:415-456) on [tmin, tmax]:
// ordered child visits, far children and their entry distances kept on a per-thread stack in
// shared memory (stack entries of one thread are kBlock words apart, so lanes never conflict);
// the closest-hit query culls boxes beyond its best hit.
template <bool COUNT>
__device__ __forceinline__ Hit trace_sah(const DevScene &S, float3 o, float3 d, float tmin, float tmax, bool any,
                                         uint32_t *stk, TraceCounters *cnt) {
    uint32_t *sn = stk;
    float *st = reinterpret_cast<float *>(stk + kStack * kBlock);
    Hit h;
    h.t = INFINITY;
    h.tri = 0xFFFFFFFFu;
    h.b1 = h.b2 = 0.0f;
    if (S.nnodes == 0)
        return h;
    float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float cull = tmax;
    uint32_t link = __float_as_uint(__ldg(&S.nlo[0].w));
    uint32_t count = __float_as_uint(__ldg(&S.nhi[0].w));
    int sp = 0;
    while (true) {
        if (count == 0) {
            if (!E8G_CHK(S.check, link + 1 < S.nnodes, kChkNode, link))
                break;
            float4 l0 = __ldg(&S.nlo[link]), h0 = __ldg(&S.nhi[link]);
            float4 l1 = __ldg(&S.nlo[link + 1]), h1 = __ldg(&S.nhi[link + 1]);
            if (COUNT)
                cnt->nodes += 2;
            float tn0, tn1;
            bool hit0 = slab(l0, h0, o, inv, tmin, cull, tn0);
            bool hit1 = slab(l1, h1, o, inv, tmin, cull, tn1);
            if (hit0 && hit1) {
                bool swap = tn1 < tn0;
                if (!E8G_CHK(S.check, sp < kStack, kChkStack, link))
                    break;
                sn[sp * kBlock] = swap ? link : link + 1;
                st[sp * kBlock] = swap ? tn0 : tn1;
                sp++;
                float4 nl = swap ? l1 : l0, nh = swap ? h1 : h0;
                link = __float_as_uint(nl.w);
                count = __float_as_uint(nh.w);
                continue;
            } else if (hit0 || hit1) {
                link = __float_as_uint(hit0 ? l0.w : l1.w);
                count = __float_as_uint(hit0 ? h0.w : h1.w);
                continue;
            }
        } else {
            if (!E8G_CHK(S.check, link + count <= S.ntris, kChkTri, link + count - 1))
                count = 0;
            for (uint32_t k = link; k < link + count; k++) {
                float4 a = __ldg(&S.tri[3 * k]), b = __ldg(&S.tri[3 * k + 1]), c = __ldg(&S.tri[3 * k + 2]);
                if (COUNT)
                    cnt->tris++;
                float t0, b1, b2;
                if (tri_test(o, d, a, b, c, tmin, tmax, t0, b1, b2) && t0 < h.t) {
                    h.t = t0;
                    h.tri = __float_as_uint(a.w);
                    h.b1 = b1;
                    h.b2 = b2;
                    if (any)
                        return h;
                    cull = fminf(t0, tmax);
                }
            }
        }
        // pop the next box still in front of the closest hit
        bool found = false;
        while (sp > 0) {
            sp--;
            uint32_t node = sn[sp * kBlock];
            float tn = st[sp * kBlock];
            if (tn <= cull) {
                link = __float_as_uint(__ldg(&S.nlo[node].w));
                count = __float_as_uint(__ldg(&S.nhi[node].w));
                found = true;
                break;
            }
        }
        if (!found)
            break;
    }
    return h;
}

// ---- the reference's tree, visited in the reference's order ----
// bvh_path_space_layout::intersect / has_intersect (pathspace.cpp:330-456): depth-first with an
// explicit stack, both children tested on the fixed interval and pushed left then right (so the
// right child is visited first), no ordering and no culling by the closest hit; node boxes are
// the reference's, uninflated. Triangles are met in the reference's order, so ties on shared
// edges resolve as in the reference.

__device__ __forceinline__ float ref_max(float a, float b) { return a < b ? b : a; } // std::max(a, b)
__device__ __forceinline__ float ref_min(float a, float b) { return b < a ? b : a; } // std::min(a, b)

// aabb::intersect (tensor.h:815-840)
__device__ __forceinline__ bool ref_slab(float4 lo, float4 hi, float3 o, float3 inv, float tmin, float tmax) {
    float k0 = (lo.x - o.x) * inv.x, k1 = (hi.x - o.x) * inv.x;
    if (k0 > k1) {
        tmin = ref_max(k1, tmin);
        tmax = ref_min(k0, tmax);
    } else {
        tmin = ref_max(k0, tmin);
        tmax = ref_min(k1, tmax);
    }
    if (tmin > tmax)
        return false;
    k0 = (lo.y - o.y) * inv.y;
    k1 = (hi.y - o.y) * inv.y;
    if (k0 > k1) {
        tmin = ref_max(k1, tmin);
        tmax = ref_min(k0, tmax);
    } else {
        tmin = ref_max(k0, tmin);
        tmax = ref_min(k1, tmax);
    }
    if (tmin > tmax)
        return false;
    k0 = (lo.z - o.z) * inv.z;
    k1 = (hi.z - o.z) * inv.z;
    if (k0 > k1) {
        tmin = ref_max(k1, tmin);
        tmax = ref_min(k0, tmax);
    } else {
        tmin = ref_max(k0, tmin);
        tmax = ref_min(k1, tmax);
    }
    return !(tmin > tmax);
}

template <bool COUNT>
__device__ __forceinline__ bool trace_ref(const DevScene &S, float3 o, float3 d, float tmin, float tmax, bool any,
                                          Hit &h, uint32_t *stk, TraceCounters *cnt) {
    if (S.nnodes == 0)
        return false;
    float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    int sp = 0;
    stk[0] = 0;
    sp = 1;
    while (sp > 0) {
        sp--;
        uint32_t n = stk[sp * kBlock];
        if (!E8G_CHK(S.check, n < S.nnodes, kChkNode, n))
            return false;
        uint32_t link = __float_as_uint(__ldg(&S.nlo[n].w));
        uint32_t count = __float_as_uint(__ldg(&S.nhi[n].w));
        if (!E8G_CHK(S.check, count == 0 || link + count <= S.ntris, kChkTri, link + count - 1))
            count = 0;
        if (!E8G_CHK(S.check, count > 0 || sp + 2 <= kStackWords, kChkStack, n))
            return false;
        if (count > 0) {
            for (uint32_t k = link; k < link + count; k++) {
                float4 a = __ldg(&S.tri[3 * k]), b = __ldg(&S.tri[3 * k + 1]), c = __ldg(&S.tri[3 * k + 2]);
                if (COUNT)
                    cnt->tris++;
                float t0, b1, b2;
                if (tri_test(o, d, a, b, c, tmin, tmax, t0, b1, b2)) {
                    if (any) {
                        h.t = t0;
                        h.tri = __float_as_uint(a.w);
                        return true;
                    }
                    if (t0 < h.t) {
                        h.t = t0;
                        h.tri = __float_as_uint(a.w);
                        h.b1 = b1;
                        h.b2 = b2;
                    }
                }
            }
        } else {
            uint32_t left = n + 1, right = link;
            if (COUNT)
                cnt->nodes += 2;
            if (ref_slab(__ldg(&S.nlo[left]), __ldg(&S.nhi[left]), o, inv, tmin, tmax))
                stk[(sp++) * kBlock] = left;
            if (ref_slab(__ldg(&S.nlo[right]), __ldg(&S.nhi[right]), o, inv, tmin, tmax))
                stk[(sp++) * kBlock] = right;
        }
    }
    return false;
}

// linear_path_space_layout::intersect / has_intersect (pathspace.cpp:36-114): every triangle in
// mesh order (the records of the linear layout are in global triangle order), the first of equal
// distances kept (strict <), an any-hit query returning at the first triangle it hits.
template <bool COUNT>
__device__ __forceinline__ Hit trace_linear(const DevScene &S, float3 o, float3 d, float tmin, float tmax, bool any,
                                            TraceCounters *cnt) {
    Hit h;
    h.t = INFINITY;
    h.tri = 0xFFFFFFFFu;
    h.b1 = h.b2 = 0.0f;
    for (uint32_t k = 0; k < S.ntris; k++) {
        float4 a = __ldg(&S.tri[3 * static_cast<size_t>(k)]);
        float4 b = __ldg(&S.tri[3 * static_cast<size_t>(k) + 1]);
        float4 c = __ldg(&S.tri[3 * static_cast<size_t>(k) + 2]);
        if (COUNT)
            cnt->tris++;
        float t0, b1, b2;
        if (tri_test(o, d, a, b, c, tmin, tmax, t0, b1, b2) && t0 < h.t) {
            h.t = t0;
            h.tri = __float_as_uint(a.w);
            h.b1 = b1;
            h.b2 = b2;
            if (any)
                return h;
        }
    }
    return h;
}

// One query in a given layout: closest hit (any = false) or any hit (any = true) on [tmin, tmax].
// Kernels on the hot path call this from a single site, so each holds one inlined traversal.
template <int LAYOUT, bool COUNT>
__device__ __forceinline__ Hit trace_l(const DevScene &S, float3 o, float3 d, float tmin, float tmax, bool any,
                                       uint32_t *stk, TraceCounters *cnt) {
    if (LAYOUT == 1) {
        Hit h;
        h.t = INFINITY;
        h.tri = 0xFFFFFFFFu;
        h.b1 = h.b2 = 0.0f;
        trace_ref<COUNT>(S, o, d, tmin, tmax, any, h, stk, cnt);
        return h;
    }
    if (LAYOUT == 2) {
        WideView W{S.wnodes, S.tri, S.nnodes, S.ntris, S.check};
        return wide_trace(W, o, d, tmin, tmax, any, stk, kBlock, COUNT ? &cnt->nodes : nullptr,
                          COUNT ? &cnt->tris : nullptr);
    }
    if (LAYOUT == 3)
        return trace_linear<COUNT>(S, o, d, tmin, tmax, any, cnt);
    return trace_sah<COUNT>(S, o, d, tmin, tmax, any, stk, cnt);
}

// Closest hit on [1e-4, 1000] (pathspace.cpp:335-336) in the scene's layout, chosen at run time
// (kernels off the hot path; the eight-wide traversal is called out of line).
template <bool COUNT>
__device__ __forceinline__ Hit trace_closest(const DevScene &S, float3 o, float3 d, uint32_t *stk, TraceCounters *cnt) {
    if (S.layout == 1)
        return trace_l<1, COUNT>(S, o, d, 1e-4f, 1000.0f, false, stk, cnt);
    if (S.layout == 2)
        return wide_trace_call(WideView{S.wnodes, S.tri, S.nnodes, S.ntris, S.check}, o, d, 1e-4f, 1000.0f, false, stk, kBlock,
                               COUNT ? &cnt->nodes : nullptr, COUNT ? &cnt->tris : nullptr);
    if (S.layout == 3)
        return trace_linear<COUNT>(S, o, d, 1e-4f, 1000.0f, false, cnt);
    return trace_l<0, COUNT>(S, o, d, 1e-4f, 1000.0f, false, stk, cnt);
}

// Any hit on [tmin, tmax] in the scene's layout.
template <bool COUNT>
__device__ __forceinline__ bool trace_any(const DevScene &S, float3 o, float3 d, float tmin, float tmax, uint32_t *stk,
                                          TraceCounters *cnt) {
    if (S.layout == 1)
        return trace_l<1, COUNT>(S, o, d, tmin, tmax, true, stk, cnt).tri != 0xFFFFFFFFu;
    if (S.layout == 2)
        return wide_trace_call(WideView{S.wnodes, S.tri, S.nnodes, S.ntris, S.check}, o, d, tmin, tmax, true, stk, kBlock,
                               COUNT ? &cnt->nodes : nullptr, COUNT ? &cnt->tris : nullptr)
                   .tri != 0xFFFFFFFFu;
    if (S.layout == 3)
        return trace_linear<COUNT>(S, o, d, tmin, tmax, true, cnt).tri != 0xFFFFFFFFu;
    return trace_l<0, COUNT>(S, o, d, tmin, tmax, true, stk, cnt).tri != 0xFFFFFFFFu;
}

// ---- resumable traversal (SAH layout): one node per call ----
// Lets a persistent trace kernel give a lane a new ray as soon as its ray is done, instead of
// holding the lane until the warp's slowest ray finishes.
struct TravState {
    float3 o, d, inv;
    float tmin, cull;     // closest: min(best, 1000); any: tmax
    uint32_t link, count; // current node (count == 0: interior)
    int sp;
    bool found;           // any-hit: an occluder was found
    Hit best;
};

__device__ __forceinline__ void trav_begin(const DevScene &S, TravState &T, float3 o, float3 d, float tmin, float tmax) {
    T.o = o;
    T.d = d;
    T.inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    T.tmin = tmin;
    T.cull = tmax;
    T.sp = 0;
    T.found = false;
    T.best.t = INFINITY;
    T.best.tri = 0xFFFFFFFFu;
    T.best.b1 = T.best.b2 = 0.0f;
    T.link = __float_as_uint(__ldg(&S.nlo[0].w));
    T.count = __float_as_uint(__ldg(&S.nhi[0].w));
}

// Visits one node; returns true when the ray is finished (stack empty, or any-hit found).
// Same tests, order and culling as trace_closest_sah / trace_any_sah.
template <bool ANY>
__device__ __forceinline__ bool trav_step(const DevScene &S, TravState &T, uint32_t *stk) {
    uint32_t *sn = stk;
    float *st = reinterpret_cast<float *>(stk + kStack * kBlock);
    if (T.count == 0) {
        float4 l0 = __ldg(&S.nlo[T.link]), h0 = __ldg(&S.nhi[T.link]);
        float4 l1 = __ldg(&S.nlo[T.link + 1]), h1 = __ldg(&S.nhi[T.link + 1]);
        float tn0, tn1;
        bool hit0 = slab(l0, h0, T.o, T.inv, T.tmin, T.cull, tn0);
        bool hit1 = slab(l1, h1, T.o, T.inv, T.tmin, T.cull, tn1);
        if (hit0 && hit1) {
            bool swap = tn1 < tn0;
            sn[T.sp * kBlock] = swap ? T.link : T.link + 1;
            if (!ANY)
                st[T.sp * kBlock] = swap ? tn0 : tn1;
            T.sp++;
            float4 nl = swap ? l1 : l0, nh = swap ? h1 : h0;
            T.link = __float_as_uint(nl.w);
            T.count = __float_as_uint(nh.w);
            return false;
        }
        if (hit0 || hit1) {
            T.link = __float_as_uint(hit0 ? l0.w : l1.w);
            T.count = __float_as_uint(hit0 ? h0.w : h1.w);
            return false;
        }
    } else {
        for (uint32_t k = T.link; k < T.link + T.count; k++) {
            float4 a = __ldg(&S.tri[3 * k]), b = __ldg(&S.tri[3 * k + 1]), c = __ldg(&S.tri[3 * k + 2]);
            float t0, b1, b2;
            if (ANY) {
                if (tri_test(T.o, T.d, a, b, c, T.tmin, T.cull, t0, b1, b2)) {
                    T.found = true;
                    return true;
                }
            } else if (tri_test(T.o, T.d, a, b, c, T.tmin, 1000.0f, t0, b1, b2) && t0 < T.best.t) {
                T.best.t = t0;
                T.best.tri = __float_as_uint(a.w);
                T.best.b1 = b1;
                T.best.b2 = b2;
                T.cull = fminf(t0, 1000.0f);
            }
        }
    }
    while (T.sp > 0) {
        T.sp--;
        uint32_t node = sn[T.sp * kBlock];
        if (ANY || st[T.sp * kBlock] <= T.cull) {
            T.link = __float_as_uint(__ldg(&S.nlo[node].w));
            T.count = __float_as_uint(__ldg(&S.nhi[node].w));
            return false;
        }
    }
    return true;
}

// ------------------------------------------------------------------ surfaces ----

struct Vert {
    float3 p, n;
    int32_t mesh;
    float t;
};

// Interpolated vertex and renormalised normal of a hit (pathspace.cpp:385-409).
// A vertex's position and normal from the interleaved shading copy (one sector).
__device__ __forceinline__ void shading_vertex(const DevScene &S, uint32_t i, float3 &p, float3 &n) {
    float4 a = __ldg(&S.vtx[2 * static_cast<size_t>(i)]), b = __ldg(&S.vtx[2 * static_cast<size_t>(i) + 1]);
    p = f3(a.x, a.y, a.z);
    n = f3(a.w, b.x, b.y);
}

__device__ __forceinline__ Vert make_vert(const DevScene &S, const Hit &h) {
    uint32_t tri = E8G_CHK(S.check, h.tri < S.ntris, kChkTri, h.tri) ? h.tri : 0u;
    uint4 ti = __ldg(&S.tidx[tri]);
    if (!E8G_CHK(S.check, ti.x < S.nverts && ti.y < S.nverts && ti.z < S.nverts, kChkVertex, tri))
        ti.x = ti.y = ti.z = 0;
    if (!E8G_CHK(S.check, ti.w < S.nm, kChkMesh, ti.w))
        ti.w = 0;
    float b0 = 1.0f - h.b1 - h.b2; // tensor.h:723
    float3 p0, p1, p2, n0, n1, n2;
    shading_vertex(S, ti.x, p0, n0);
    shading_vertex(S, ti.y, p1, n1);
    shading_vertex(S, ti.z, p2, n2);
    Vert v;
    v.p = add(add(scale(p0, b0), scale(p1, h.b1)), scale(p2, h.b2));
    v.n = normalize(add(add(scale(n0, b0), scale(n1, h.b1)), scale(n2, h.b2)));
    v.mesh = static_cast<int32_t>(ti.w);
    v.t = h.t;
    return v;
}

// pinhole_camera::sample (camera.cpp:38-48).
__device__ __forceinline__ void camera_ray(const DevCamera &c, uint32_t x, uint32_t y, uint32_t w, uint32_t h,
                                           float3 &o, float3 &d) {
    float sz = c.sensor;
    float vx = (__uint2float_rn(x) / __uint2float_rn(w - 1) * sz - sz / 2.0f) * c.aspect;
    float vy = (__uint2float_rn(h - 1) - __uint2float_rn(y)) / __uint2float_rn(h - 1) * sz - sz / 2.0f;
    float vz = -c.focal;
    float r[3];
#pragma unroll
    for (int i = 0; i < 3; i++)
        r[i] = c.rot[3 * i] * vx + c.rot[3 * i + 1] * vy + c.rot[3 * i + 2] * vz;
    o = f3(c.origin[0], c.origin[1], c.origin[2]);
    d = normalize(f3(r[0], r[1], r[2]));
}

// ----------------------------------------------------------------- materials ----

__device__ __forceinline__ const DevMaterial &vert_mat(const DevScene &S, int32_t mesh) {
    if (!E8G_CHK(S.check, mesh >= 0 && static_cast<uint32_t>(mesh) < S.nm, kChkMesh, mesh))
        mesh = 0;
    int32_t mi = __ldg(&S.mesh_mat[mesh]);
    if (!E8G_CHK(S.check, mi >= 0 && static_cast<uint32_t>(mi) <= S.nmat, kChkMaterial, mi)) // nmat: fail-safe
        mi = static_cast<int32_t>(S.nmat);
    return S.mats[mi];
}

// vec3_basis (tensor.h:939-943)
__device__ __forceinline__ void basis(float3 n, float3 &u, float3 &v) {
    float3 ref = fabsf(n.x) > .1f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 1.0f, 1.0f);
    u = normalize(cross(ref, n));
    v = cross(n, u);
}

// vec3_cos_hemisphere_sample (tensor.h:972-985) with the draw order the reference's calls
// produce under GCC (first draw -> e1, second -> e0).
template <class R> __device__ __forceinline__ float3 cos_hemisphere(float3 n, R &rng) {
    float e1 = rng.next();
    float e0 = rng.next();
    float3 u, v;
    basis(n, u, v);
    float z = sqrtf(e1);
    float r = sqrtf(1 - z * z);
    float phi = e0 * 2 * kPi;
    float x = r * cosf(phi);
    float y = r * sinf(phi);
    return add(add(scale(u, x), scale(v, y)), scale(n, z));
}

__device__ __forceinline__ float fresnel(float re, float im, float3 i, float3 h) { // material.cpp:10-19
    float f = 1.0f - dot(i, h);
    float f2 = f * f;
    float f4 = f2 * f2;
    float f5 = f4 * f;
    float a = (re - 1) * (re - 1) + 4 * re * f5 + im * im;
    float b = (re + 1) * (re + 1) + im * im;
    return a / b;
}
__device__ __forceinline__ float ggx_distri(float alpha2, float3 n, float3 h) { // :21-27
    float c = dot(n, h);
    float c2 = c * c;
    float tan2 = (1.0f - c2) / c2;
    float k = 1.0f + tan2 / alpha2;
    return 1.0f / (kPi * alpha2 * c2 * c2 * k * k);
}
__device__ __forceinline__ float ggx_lambda(float alpha2, float3 n, float3 w) { // :29-34
    float c = dot(n, w);
    float c2 = c * c;
    float tan2 = (1.0f - c2) / c2;
    return (-1.0f + sqrtf(1.0f + alpha2 * tan2)) / 2.0f;
}
__device__ __forceinline__ float ggx_shadow(float alpha2, float3 i, float3 o, float3 n) { // :36-39
    return 1.0f / (1.0f + ggx_lambda(alpha2, n, i) + ggx_lambda(alpha2, n, o));
}

__device__ __forceinline__ float3 eval_leaf(const DevMaterial &m, float3 n, float3 o, float3 i) {
    float3 albedo = f3(m.albedo[0], m.albedo[1], m.albedo[2]);
    if (m.type == 1) { // oren_nayar, material.cpp:134-161
        float cos_i = clamp01(dot(i, n));
        float cos_o = clamp01(dot(o, n));
        if (feq0(cos_i) || feq0(cos_o))
            return f3(0, 0, 0);
        float ca, cb;
        if (cos_i < cos_o) {
            ca = cos_i;
            cb = cos_o;
        } else {
            ca = cos_o;
            cb = cos_i;
        }
        float sa = sqrtf(1.0f - ca * ca);
        float sb = sqrtf(1.0f - cb * cb);
        float cio = ca * cb + sa * sb;
        float tan_b = sb / cos_o;
        return scale(scale(albedo, kInvPi), m.a + m.b * smax(0.0f, cio) * sa * tan_b);
    }
    if (m.type == 2) { // cook_torr, material.cpp:199-222
        float cos_o = smax(0.0f, dot(n, o));
        float cos_i = smax(0.0f, dot(n, i));
        if (feq0(cos_i) || feq0(cos_o))
            return f3(0, 0, 0);
        float3 h = add(i, o);
        if (vequals0(h))
            return f3(0, 0, 0);
        h = normalize(h);
        float f = fresnel(m.ior_re, m.ior_im, i, h);
        float d = ggx_distri(m.alpha2, n, h);
        float g = ggx_shadow(m.alpha2, i, o, n);
        float c = f * d * g / (4.0f * cos_i * cos_o);
        return scale(albedo, c);
    }
    return scale(albedo, kInvPi); // mat_fail_safe, material.cpp:64-68
}

// One out-of-line copy of a leaf material's code for kernels whose instruction footprint
// overflows the instruction cache (OUT = true in the BSDF functions below): every call site
// then shares it instead of inlining both materials' code again. Same arithmetic either way.
static __device__ __noinline__ float3 eval_leaf_call(const DevMaterial &m, float3 n, float3 o, float3 i) {
    return eval_leaf(m, n, o, i);
}

template <bool OUT = false>
__device__ __forceinline__ float3 bsdf_eval(const DevScene &S, const DevMaterial &m, float3 n, float3 o, float3 i) {
    if (m.type == 3) { // mat_mixture, material.cpp:90-93
        float3 f0 = OUT ? eval_leaf_call(S.mats[m.mix0], n, o, i) : eval_leaf(S.mats[m.mix0], n, o, i);
        float3 f1 = OUT ? eval_leaf_call(S.mats[m.mix1], n, o, i) : eval_leaf(S.mats[m.mix1], n, o, i);
        return add(scale(f0, m.ratio), scale(f1, 1 - m.ratio));
    }
    return OUT ? eval_leaf_call(m, n, o, i) : eval_leaf(m, n, o, i);
}

template <class R>
__device__ __forceinline__ float3 sample_leaf(const DevMaterial &m, R &rng, float &dens, float3 n, float3 o) {
    if (m.type == 2) { // cook_torr::sample, material.cpp:224-252
        float ms_slope = m.alpha2;
        float3 u, v;
        basis(n, u, v);
        float theta = 2.0f * kPi * rng.next();
        float t = rng.next();
        float phi = atanf(sqrtf(ms_slope * t / (1.0f - t)));
        float sin_phi = sinf(phi);
        float cos_phi = cosf(phi);
        float x = sin_phi * cosf(theta);
        float y = sin_phi * sinf(theta);
        float z = cos_phi;
        float3 h = add(add(scale(u, x), scale(v, y)), scale(n, z));
        float hdo = dot(h, o);
        float3 i = sub(scale(h, 2.0f * hdo), o);
        if (dot(i, n) < 0.0f) {
            dens = 0.0f;
            return f3(0, 0, 0);
        }
        dens = ggx_distri(ms_slope, n, h) * cos_phi / (4.0f * hdo);
        return i;
    }
    float3 i = cos_hemisphere(n, rng); // oren_nayar / fail-safe, material.cpp:70-76, :163-169
    dens = dot(i, n) / kPi;
    return i;
}

template <class R>
__device__ __noinline__ float3 sample_leaf_call(const DevMaterial &m, R &rng, float &dens, float3 n, float3 o) {
    return sample_leaf(m, rng, dens, n, o);
}

// Reference sampling (mat_mixture returns the picked lobe's density x its weight, :95-106).
template <bool OUT = false, class R>
__device__ __forceinline__ float3 bsdf_sample_ref(const DevScene &S, const DevMaterial &m, R &rng, float &dens,
                                                  float3 n, float3 o) {
    if (m.type == 3) {
        float3 i;
        if (rng.next() < m.ratio) {
            i = OUT ? sample_leaf_call(S.mats[m.mix0], rng, dens, n, o) : sample_leaf(S.mats[m.mix0], rng, dens, n, o);
            dens *= m.ratio;
        } else {
            i = OUT ? sample_leaf_call(S.mats[m.mix1], rng, dens, n, o) : sample_leaf(S.mats[m.mix1], rng, dens, n, o);
            dens *= 1 - m.ratio;
        }
        return i;
    }
    return OUT ? sample_leaf_call(m, rng, dens, n, o) : sample_leaf(m, rng, dens, n, o);
}

// Solid-angle density of direction i under the sampling above (product modes).
__device__ __forceinline__ float pdf_leaf(const DevMaterial &m, float3 n, float3 o, float3 i) {
    if (m.type == 2) {
        if (dot(i, n) < 0.0f)
            return 0.0f;
        float3 h = add(i, o);
        if (vequals0(h))
            return 0.0f;
        h = normalize(h);
        float hdo = dot(h, o);
        float ch = dot(n, h);
        if (hdo <= 0.0f || ch <= 0.0f)
            return 0.0f;
        return ggx_distri(m.alpha2, n, h) * ch / (4.0f * hdo);
    }
    float c = dot(i, n);
    return c > 0.0f ? c / kPi : 0.0f;
}
static __device__ __noinline__ float pdf_leaf_call(const DevMaterial &m, float3 n, float3 o, float3 i) {
    return pdf_leaf(m, n, o, i);
}
template <bool OUT = false>
__device__ __forceinline__ float bsdf_pdf(const DevScene &S, const DevMaterial &m, float3 n, float3 o, float3 i) {
    if (m.type == 3) {
        float p0 = OUT ? pdf_leaf_call(S.mats[m.mix0], n, o, i) : pdf_leaf(S.mats[m.mix0], n, o, i);
        float p1 = OUT ? pdf_leaf_call(S.mats[m.mix1], n, o, i) : pdf_leaf(S.mats[m.mix1], n, o, i);
        return m.ratio * p0 + (1 - m.ratio) * p1;
    }
    return OUT ? pdf_leaf_call(m, n, o, i) : pdf_leaf(m, n, o, i);
}
// Product-mode sampling: a mixture reports its true mixture density.
template <bool OUT = false, class R>
__device__ __forceinline__ float3 bsdf_sample_mis(const DevScene &S, const DevMaterial &m, R &rng, float &pdf,
                                                  float3 n, float3 o) {
    if (m.type == 3) {
        float lobe_pdf;
        float3 i;
        DevMaterial const &lobe = rng.next() < m.ratio ? S.mats[m.mix0] : S.mats[m.mix1];
        i = OUT ? sample_leaf_call(lobe, rng, lobe_pdf, n, o) : sample_leaf(lobe, rng, lobe_pdf, n, o);
        if (lobe_pdf == 0.0f) {
            pdf = 0.0f;
            return f3(0, 0, 0);
        }
        pdf = bsdf_pdf<OUT>(S, m, n, o, i);
        return i;
    }
    return OUT ? sample_leaf_call(m, rng, pdf, n, o) : sample_leaf(m, rng, pdf, n, o);
}

// -------------------------------------------------------------------- lights ----

__device__ __forceinline__ float3 light_rad(const DevScene &S, int l) { return xyz(__ldg(&S.light_rad[l])); }

__device__ __forceinline__ float3 light_radiance(const DevScene &S, int l, float3 w, float3 n) { // light.cpp:64-71
    float c = dot(n, w);
    return c > 0 ? light_rad(S, l) : f3(0, 0, 0);
}
__device__ __forceinline__ float3 light_projected(const DevScene &S, int l, float3 w, float3 n) { // :54-62
    float c = dot(n, w);
    return c > 0 ? scale(light_rad(S, l), c) : f3(0, 0, 0);
}
__device__ __forceinline__ float3 light_eval(const DevScene &S, int l, float3 i, float3 n_light,
                                             float3 n_target) { // :41-52
    float r2 = dot(i, i);
    float3 in = divs(i, sqrtf(r2));
    float cos_o = dot(n_light, in);
    float cos_i = dot(n_target, neg(in));
    if (cos_o > 0 && cos_i > 0)
        return divs(scale(scale(light_rad(S, l), cos_i), cos_o), r2);
    return f3(0, 0, 0);
}

// basic_light_sources::sample_light (lightsources.cpp:59-75)
template <class R> __device__ __forceinline__ int sample_light(const DevScene &S, R &rng, float &pmf) {
    float e = rng.next() * S.total_power;
    uint32_t lo = 0, hi = S.nl;
    while (lo < hi) {
        uint32_t mi = (lo + hi) >> 1;
        if (__ldg(&S.light_cum[mi]) < e)
            lo = mi + 1;
        else
            hi = mi;
    }
    if (lo >= S.nl)
        lo = S.nl - 1;
    pmf = __ldg(&S.light_pnorm[lo]) / S.total_power;
    return static_cast<int>(lo);
}

struct Surf {
    float3 p, n;
    float area_dens;
};

// trimesh::sample (geometry.cpp:44-66): triangle uniform by index (reference modes) or from
// the area CDF (product modes), barycentrics (1 - sqrt u, sqrt u * v).
template <class R>
__device__ __forceinline__ Surf mesh_sample(const DevScene &S, uint32_t mesh, R &rng, bool area_weighted) {
    uint32_t t0 = __ldg(&S.mesh_toff[mesh]);
    uint32_t ntris = __ldg(&S.mesh_toff[mesh + 1]) - t0;
    float q = rng.next();
    uint32_t i;
    if (!area_weighted) {
        i = __float2uint_rz(q * __uint2float_rn(ntris));
    } else {
        float e = q * __ldg(&S.mesh_area[mesh]);
        uint32_t lo = 0, hi = ntris;
        while (lo < hi) {
            uint32_t mi = (lo + hi) >> 1;
            if (__ldg(&S.tri_cum[t0 + mi]) <= e)
                lo = mi + 1;
            else
                hi = mi;
        }
        i = lo;
    }
    if (i >= ntris)
        i = ntris - 1;
    uint4 ti = __ldg(&S.tidx[t0 + i]);
    float u = rng.next();
    float v = rng.next();
    float r = sqrtf(u);
    float b0 = 1 - r;
    float b1 = r * v;
    float b2 = 1 - b0 - b1;
    float3 p0, p1, p2, n0, n1, n2;
    shading_vertex(S, ti.x, p0, n0);
    shading_vertex(S, ti.y, p1, n1);
    shading_vertex(S, ti.z, p2, n2);
    Surf s;
    s.p = add(add(scale(p0, b0), scale(p1, b1)), scale(p2, b2));
    s.n = normalize(add(add(scale(n0, b0), scale(n1, b1)), scale(n2, b2)));
    s.area_dens = 1.0f / __ldg(&S.mesh_area[mesh]);
    return s;
}

__device__ __forceinline__ float power_heuristic(float a, float b) {
    float a2 = a * a, b2 = b * b;
    return a2 / (a2 + b2);
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

} // namespace e8g
