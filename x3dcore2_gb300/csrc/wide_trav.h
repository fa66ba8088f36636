// Traversal of the eight-wide quantized BVH (layout in bvh_wide.h), written once for the device
// kernels and for the host-side checker (tests/cpp/wide_check.cpp), which runs the same code
// against brute force on the CPU.
//
// One node visit loads the 96-byte record, tests the eight child boxes against [tmin, cull],
// tests the triangles of every hit leaf slot at once, descends into the first hit interior child
// in the ray's octant order and keeps the other hit interior children as one stack entry
// (child base, interior mask, remaining hit mask). The stack therefore grows by at most one entry
// per level, and the builder keeps the tree at most kWideMaxDepth levels deep.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector_types.h>

#if defined(__CUDACC__)
#define E8G_HD __host__ __device__ __forceinline__
// Out of line: for kernels with many traversal call sites (keeps them within the instruction cache)
#define E8G_HD_CALL static __host__ __device__ __noinline__
#else
#define E8G_HD inline
#define E8G_HD_CALL inline
#endif

namespace e8g {

// Bounds checks of the debug build (E8G_CHECKS defined for the device compilation; nothing in the
// other builds). A failed check records its code and the offending index in the check word, the
// first failure winning, and the caller skips the access; the host reads the word after the call
// and reports E8G_ERR_INTERNAL with both. Nothing traps.
enum : uint32_t {
    kChkNode = 1,     // BVH node index beyond the node array
    kChkTri = 2,      // triangle record index beyond the triangle array
    kChkStack = 3,    // traversal stack full
    kChkVertex = 4,   // vertex index of a triangle beyond the vertex array
    kChkMesh = 5,     // mesh index beyond the mesh table
    kChkMaterial = 6, // material index beyond the material table
    kChkLight = 7,    // light index beyond the light table
    kChkQueue = 8,    // wavefront queue entry beyond the slot capacity
    kChkSlot = 9      // wavefront slot index beyond the slot capacity
};
#if defined(E8G_CHECKS) && defined(__CUDA_ARCH__)
__device__ __forceinline__ bool e8g_chk(unsigned long long *word, bool ok, uint32_t code, uint32_t idx) {
    if (!ok && word)
        atomicCAS(word, 0ull, (static_cast<unsigned long long>(code) << 32) | idx);
    return ok;
}
#define E8G_CHK(word, cond, code, idx) e8g::e8g_chk((word), (cond), (code), static_cast<uint32_t>(idx))
#else
#define E8G_CHK(word, cond, code, idx) true
#endif

struct Hit {
    float t;
    uint32_t tri; // triangle record position (traversal) or global triangle index; 0xFFFFFFFF = miss
    float b1, b2;
};

E8G_HD float hd_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}
E8G_HD uint32_t hd_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
E8G_HD int hd_ffs(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return __ffs(static_cast<int>(v));
#else
    return __builtin_ffs(static_cast<int>(v));
#endif
}
E8G_HD int hd_popc(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return __popc(v);
#else
    return __builtin_popcount(v);
#endif
}
E8G_HD float hd_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
E8G_HD float hd_rcp(float x) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}
// Reciprocal for the box tests only, within 1 ulp on the device (one MUFU instruction); the
// boxes are pushed out by about 1e-6 of the scene's extent, far more than a 1-ulp change of the
// slab distances, so no box that a hit lies in is culled.
E8G_HD float hd_rcp_box(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}
E8G_HD uint4 hd_ld(uint4 const *p) {
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}
E8G_HD float4 hd_ld(float4 const *p) {
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}

// ray::intersect (tensor.h:688-725) on a triangle stored as (v0, v1 - v0, v2 - v0), in the
// reference's operation order; callers compile it without FMA contraction.
E8G_HD bool hd_tri_test(float3 o, float3 d, float4 a, float4 b, float4 c, float tmin, float tmax, float &t0,
                        float &b1o, float &b2o) {
    float vax = b.x, vay = b.y, vaz = b.z; // va = v1 - v0
    float vbx = c.x, vby = c.y, vbz = c.z; // vb = v2 - v0
    float vcx = o.x - a.x, vcy = o.y - a.y, vcz = o.z - a.z;
    // e2 = d x vb
    float e2x = d.y * vbz - d.z * vby, e2y = d.z * vbx - d.x * vbz, e2z = d.x * vby - d.y * vbx;
    float det = vax * e2x + vay * e2y + vaz * e2z;
    if (det == 0.0f)
        return false;
    float inv = hd_rcp(det);
    float b1 = (vcx * e2x + vcy * e2y + vcz * e2z) * inv;
    if (b1 < 0.0f || b1 > 1.0f)
        return false;
    // e1 = vc x va
    float e1x = vcy * vaz - vcz * vay, e1y = vcz * vax - vcx * vaz, e1z = vcx * vay - vcy * vax;
    float b2 = (d.x * e1x + d.y * e1y + d.z * e1z) * inv;
    if (b2 < 0.0f || b1 + b2 > 1.0f)
        return false;
    float t = (vbx * e1x + vby * e1y + vbz * e1z) * inv;
    if (t < tmin || t > tmax)
        return false;
    t0 = t;
    b1o = b1;
    b2o = b2;
    return true;
}

struct WideView {
    uint4 const *nodes;  // 6 per node
    float4 const *tri;   // 3 per triangle record: (v0 | global id), (v1 - v0), (v2 - v0)
    uint32_t nnodes;
    uint32_t ntris;                 // triangle records (bounds checks of the debug build)
    unsigned long long *check;      // check word of the debug build, or null
};

constexpr int kWideStack = 16; // stack entries (the builder keeps the tree at most 16 levels deep);
                               // entry i takes words 2i and 2i + 1 of stk, `stride` apart

// Byte j of word w as the float 1 + q * 2^-15 (exact), placed into the mantissa with one byte
// permute: result bytes (0x00, q, 0x80, 0x3F).
E8G_HD float hd_qf(uint32_t w, uint32_t j) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | (j << 4)));
#else
    return hd_u2f(0x3F800000u | ((w >> (8u * j)) & 0xFFu) << 8);
#endif
}

// max / min of three floats (one instruction on sm_100 and later; NaN operands are dropped like
// fmaxf / fminf do).
E8G_HD float hd_max3(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}
E8G_HD float hd_min3(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fminf(fminf(a, b), c);
#endif
}

// The permutation bit s -> bit s ^ oct of an eight-bit mask.
E8G_HD uint32_t hd_xor_perm(uint32_t m, uint32_t oct) {
    uint32_t a = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    m = (oct & 1u) ? a : m;
    uint32_t b = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    m = (oct & 2u) ? b : m;
    uint32_t c = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
    return (oct & 4u) ? c : m;
}

// Resumable traversal state of one ray: wide_begin, then wide_step until it returns true. A
// persistent trace kernel can give a lane a new ray as soon as its ray is done.
struct WideTrav {
    float3 o, d;     // ray (triangle tests use d as given)
    float ix, iy, iz; // reciprocal direction of the box tests
    float tmin, cull; // any: cull stays tmax; closest: the best hit so far
    uint32_t oct;    // direction sign octant
    uint32_t node;   // the node to visit next
    int sp;          // stack entries in use
    bool any;
    Hit h;           // any: the occluder found; closest: the best hit (global triangle id)
};

E8G_HD void wide_begin(WideTrav &T, float3 o, float3 d, float tmin, float tmax, bool any) {
    T.o = o;
    T.d = d;
    // Box tests use direction components at least 1e-30 in magnitude: an exactly parallel ray
    // would turn the factored plane distance q * (step / d) + (p - o) / d into 0 * inf or
    // inf - inf. The nudged ray moves less than 1e-27 off its line over t <= 1000, and boxes are
    // inflated far beyond that, so no box a triangle hit lies in is culled; triangle tests use d.
    T.ix = hd_rcp_box(fabsf(d.x) < 1e-30f ? copysignf(1e-30f, d.x) : d.x);
    T.iy = hd_rcp_box(fabsf(d.y) < 1e-30f ? copysignf(1e-30f, d.y) : d.y);
    T.iz = hd_rcp_box(fabsf(d.z) < 1e-30f ? copysignf(1e-30f, d.z) : d.z);
    T.oct = (T.ix < 0.0f ? 1u : 0u) | (T.iy < 0.0f ? 2u : 0u) | (T.iz < 0.0f ? 4u : 0u);
    T.tmin = tmin;
    T.cull = tmax;
    T.node = 0;
    T.sp = 0;
    T.any = any;
    T.h.t = INFINITY;
    T.h.tri = 0xFFFFFFFFu;
    T.h.b1 = T.h.b2 = 0.0f;
}

// The eight child boxes of a node against [T.tmin, T.cull]: bit s set when slot s is hit. All
// eight slots are tested, also for nodes with at most four children (the callers mask the bits
// of empty slots with the node's interior and leaf masks): a warp whose lanes visit nodes of both
// sizes runs the eight-slot form anyway, and the unrolled form selects no words per half
// (measured: 5% less time in the wavefront's trace kernel than testing the second half only when
// the node has children there).
E8G_HD uint32_t wide_child_hits(WideTrav const &T, uint4 n0, uint4 n2, uint4 n3, uint4 n4) {
    const uint32_t oct = T.oct;
    // plane of byte q on axis a: p + q * step = (p - 2^15 step) + (1 + q 2^-15) * 2^15 step, so
    // t = (1 + q 2^-15) * S + O with S = 2^15 step / d and O = (p - 2^15 step - o) / d
    float gx = hd_u2f((n0.w & 0xFFu) << 23) * 32768.0f;
    float gy = hd_u2f(((n0.w >> 8) & 0xFFu) << 23) * 32768.0f;
    float gz = hd_u2f(((n0.w >> 16) & 0xFFu) << 23) * 32768.0f;
    float sx = gx * T.ix, sy = gy * T.iy, sz = gz * T.iz;
    float ox = (hd_u2f(n0.x) - gx - T.o.x) * T.ix, oy = (hd_u2f(n0.y) - gy - T.o.y) * T.iy,
          oz = (hd_u2f(n0.z) - gz - T.o.z) * T.iz;
    uint32_t hits = 0;
    // slots 0-3 then 4-7; near / far planes per axis follow the ray's direction signs
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (uint32_t half = 0; half < 2; half++) {
        uint32_t lx = half ? n2.y : n2.x, hx = half ? n3.w : n3.z;
        uint32_t ly = half ? n2.w : n2.z, hy = half ? n4.y : n4.x;
        uint32_t lz = half ? n3.y : n3.x, hz = half ? n4.w : n4.z;
        uint32_t wnx = (oct & 1u) ? hx : lx, wfx = (oct & 1u) ? lx : hx;
        uint32_t wny = (oct & 2u) ? hy : ly, wfy = (oct & 2u) ? ly : hy;
        uint32_t wnz = (oct & 4u) ? hz : lz, wfz = (oct & 4u) ? lz : hz;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (uint32_t j = 0; j < 4; j++) {
            float tnx = hd_fma(hd_qf(wnx, j), sx, ox), tfx = hd_fma(hd_qf(wfx, j), sx, ox);
            float tny = hd_fma(hd_qf(wny, j), sy, oy), tfy = hd_fma(hd_qf(wfy, j), sy, oy);
            float tnz = hd_fma(hd_qf(wnz, j), sz, oz), tfz = hd_fma(hd_qf(wfz, j), sz, oz);
            float tn = fmaxf(hd_max3(tnx, tny, tnz), T.tmin);
            float tf = fminf(hd_min3(tfx, tfy, tfz), T.cull);
            hits |= (tn <= tf ? 1u : 0u) << (4 * half + j);
        }
    }
    return hits;
}

// Moves T.node to the next node: the first hit interior child in octant order (the other hit
// interior children go on the stack as one entry), else the stack's top. Returns false when
// there is none.
E8G_HD bool wide_advance(WideTrav &T, uint32_t hits, uint32_t imask, uint32_t base, uint32_t *stk, int stride,
                         unsigned long long *check = nullptr) {
    const uint32_t oct = T.oct;
    uint32_t hit_int = hd_xor_perm(hits & imask, oct);
    if (hit_int) {
        uint32_t k = static_cast<uint32_t>(hd_ffs(hit_int) - 1);
        hit_int &= hit_int - 1u;
        uint32_t s = k ^ oct;
        if (hit_int && E8G_CHK(check, T.sp < kWideStack, kChkStack, T.node) && T.sp < kWideStack) {
            stk[2 * T.sp * stride] = base;
            stk[(2 * T.sp + 1) * stride] = imask << 8 | hit_int;
            T.sp++;
        }
        T.node = base + static_cast<uint32_t>(hd_popc(imask & ((1u << s) - 1u)));
        return true;
    }
    if (T.sp > 0) {
        uint32_t sbase = stk[2 * (T.sp - 1) * stride];
        uint32_t info = stk[(2 * (T.sp - 1) + 1) * stride];
        uint32_t m = info & 0xFFu, im = info >> 8;
        uint32_t k = static_cast<uint32_t>(hd_ffs(m) - 1);
        m &= m - 1u;
        if (m)
            stk[(2 * (T.sp - 1) + 1) * stride] = im << 8 | m;
        else
            T.sp--;
        uint32_t s = k ^ oct;
        T.node = sbase + static_cast<uint32_t>(hd_popc(im & ((1u << s) - 1u)));
        return true;
    }
    return false;
}

// The triangles of leaf slot s of a node (its words 5-7 and 20: tri_base, meta, counts).
// Returns true when an any-hit ray found its occluder.
E8G_HD bool wide_leaf_slot(WideView const &W, WideTrav &T, uint32_t s, uint32_t tri_base, uint32_t meta_lo,
                           uint32_t meta_hi, uint32_t counts, uint32_t *cnt_tris) {
    uint32_t meta = (s < 4 ? meta_lo : meta_hi) >> (8u * (s & 3u)) & 0xFFu;
    uint32_t k0 = tri_base + meta, k1 = k0 + ((counts >> (4u * s)) & 0xFu);
    if (!E8G_CHK(W.check, k1 <= W.ntris, kChkTri, k1 - 1))
        return false;
    for (uint32_t k = k0; k < k1; k++) {
        float4 a = hd_ld(W.tri + 3 * static_cast<size_t>(k));
        float4 b = hd_ld(W.tri + 3 * static_cast<size_t>(k) + 1);
        float4 c = hd_ld(W.tri + 3 * static_cast<size_t>(k) + 2);
        if (cnt_tris)
            (*cnt_tris)++;
        float t0, b1, b2;
        if (hd_tri_test(T.o, T.d, a, b, c, T.tmin, T.cull, t0, b1, b2) && t0 < T.h.t) {
            T.h.t = t0;
            T.h.tri = hd_f2u(a.w);
            T.h.b1 = b1;
            T.h.b2 = b2;
            if (T.any)
                return true;
            T.cull = t0;
        }
    }
    return false;
}

// Visits T.node: tests its eight child boxes, the triangles of every hit leaf slot, and moves
// T.node to the next node (the first hit interior child in octant order; the rest go on the
// stack as one entry). Returns true when the ray is finished (stack empty, or an any-hit found).
E8G_HD bool wide_step(WideView const &W, WideTrav &T, uint32_t *stk, int stride, uint32_t *cnt_nodes,
                      uint32_t *cnt_tris) {
    if (!E8G_CHK(W.check, T.node < W.nnodes, kChkNode, T.node))
        return true;
    uint4 const *np = W.nodes + 6 * static_cast<size_t>(T.node);
    uint4 n0 = hd_ld(np), n1 = hd_ld(np + 1), n2 = hd_ld(np + 2), n3 = hd_ld(np + 3), n4 = hd_ld(np + 4),
          n5 = hd_ld(np + 5);
    uint32_t counts = n5.x, leaves = n5.y;
    if (cnt_nodes)
        (*cnt_nodes)++;
    uint32_t hits = wide_child_hits(T, n0, n2, n3, n4);
    bool more = wide_advance(T, hits, n0.w >> 24, n1.x, stk, stride, W.check);
    uint32_t hit_leaf = hits & leaves;
    while (hit_leaf) {
        uint32_t s = static_cast<uint32_t>(hd_ffs(hit_leaf) - 1);
        hit_leaf &= hit_leaf - 1u;
        if (wide_leaf_slot(W, T, s, n1.y, n1.z, n1.w, counts, cnt_tris))
            return true;
    }
    return !more;
}

// any: returns at the first triangle with t in [tmin, tmax] (h.tri != miss). Otherwise returns
// the closest hit (h.tri = global triangle id, h.t = infinity on a miss). stk holds
// 2 * kWideStack words, `stride` apart. The counters, when given, add one per node visited and
// one per triangle tested. Each node is visited at most once, so the loop ends within nnodes
// steps.
E8G_HD Hit wide_trace(WideView W, float3 o, float3 d, float tmin, float tmax, bool any, uint32_t *stk, int stride,
                      uint32_t *cnt_nodes, uint32_t *cnt_tris) {
    WideTrav T;
    wide_begin(T, o, d, tmin, tmax, any);
    if (W.nnodes == 0)
        return T.h;
    for (uint32_t guard = 0; guard <= W.nnodes; guard++)
        if (wide_step(W, T, stk, stride, cnt_nodes, cnt_tris))
            break;
    return T.h;
}

// The same as one out-of-line function, for kernels that trace from many call sites.
E8G_HD_CALL Hit wide_trace_call(WideView W, float3 o, float3 d, float tmin, float tmax, bool any, uint32_t *stk,
                                int stride, uint32_t *cnt_nodes, uint32_t *cnt_tris) {
    return wide_trace(W, o, d, tmin, tmax, any, stk, stride, cnt_nodes, cnt_tris);
}

} // namespace e8g
