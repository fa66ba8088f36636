// Box arithmetic shared by the host builders (bvh.cpp, bvh_wide.cpp) and the device refit
// (refit.cu), so a refit of an unchanged scene writes the bytes the host build wrote.
//
// Every stored box is the exact union of the triangles below it, pushed outwards by
// |v| * 1e-6 + eps with eps = 1e-6 * (largest extent of the scene's box). The eight-wide layout
// then quantizes the pushed-out boxes of a node's children on a per-node grid.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <math.h>

#if defined(__CUDACC__)
#define E8G_BOX_HD __host__ __device__ __forceinline__
#else
#define E8G_BOX_HD inline
#endif

namespace e8g {

E8G_BOX_HD uint32_t box_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}

E8G_BOX_HD float inflate_lo(float v, float eps) { return v - (fabsf(v) * 1.0e-6f + eps); }
E8G_BOX_HD float inflate_hi(float v, float eps) { return v + (fabsf(v) * 1.0e-6f + eps); }

// eps of a scene whose exact box is [lo, hi].
E8G_BOX_HD float scene_eps(float const lo[3], float const hi[3]) {
    float diag = 0;
    for (int a = 0; a < 3; a++) {
        float d = hi[a] - lo[a];
        diag = diag < d ? d : diag;
    }
    return diag * 1.0e-6f;
}

// Smallest grid step of the quantized layout: 2^-18 of the largest coordinate the scene and the
// rays reach (far above the rounding of the slab arithmetic, so one step of outward rounding
// keeps every box conservative), and at least 2^-100.
E8G_BOX_HD double wide_step_min(float max_abs) {
    double s = static_cast<double>(max_abs) * ldexp(1.0, -18);
    double floor_step = ldexp(1.0, -100);
    return s > floor_step ? s : floor_step;
}

// Smallest e in [-126, 127] with 2^e >= want (want > 0), computed without log2 so the host and
// the device agree exactly.
E8G_BOX_HD int wide_exponent(double want) {
    int x;
    double m = frexp(want, &x); // want = m * 2^x, m in [0.5, 1)
    int e = m == 0.5 ? x - 1 : x;
    return e < -126 ? -126 : (e > 127 ? 127 : e);
}

// floor and ceil of (v - org) * inv, with inv a power of two, from the exact difference: s + err
// = v - org exactly (Knuth's TwoSum in single precision), s * inv is exact, and a float quotient
// is at least one of its ulps away from the next integer, so only an integer quotient can move,
// by the sign of err. The same result as the double-precision expression whenever v - org is
// exact in double (exponents within 29 of each other), without double arithmetic (slow on this
// GPU).
E8G_BOX_HD void wide_grid_floor_ceil(float v, float org, float inv, float &fl, float &cl) {
    float s = v - org;
    float bb = s - v;
    float err = (v - (s - bb)) + (-org - bb);
    float q = s * inv;
    fl = floorf(q);
    cl = ceilf(q);
    if (fl == q && err < 0.0f)
        fl -= 1.0f;
    if (cl == q && err > 0.0f)
        cl += 1.0f;
}

// Fills a node's grid and quantized child boxes: words[0..2] (grid origin), the exponent bytes of
// words[3] (the interior mask byte is left alone) and words[8..19]. lo/hi hold the pushed-out
// boxes of the eight slots; only slots in `present` are used.
E8G_BOX_HD void wide_quantize(float const lo[8][3], float const hi[8][3], uint32_t present, double step_min,
                          uint32_t words[24]) {
    float u_lo[3] = {INFINITY, INFINITY, INFINITY}, u_hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int s = 0; s < 8; s++) {
        if (!(present >> s & 1))
            continue;
        for (int a = 0; a < 3; a++) {
            u_lo[a] = lo[s][a] < u_lo[a] ? lo[s][a] : u_lo[a];
            u_hi[a] = u_hi[a] < hi[s][a] ? hi[s][a] : u_hi[a];
        }
    }
    // The grid starts one step below the children's union and 253 steps cover it, so no child box
    // is clamped to the grid's ends and every quantized plane lies at least one step outside the
    // (already pushed-out) child box: the slack absorbs the rounding of the traversal's plane
    // arithmetic.
    float inv_step[3]; // 2^-e: dividing by the step 2^e is this exact product
    float org[3];
    uint32_t ebytes = 0;
    for (int a = 0; a < 3; a++) {
        double ext = static_cast<double>(u_hi[a]) - static_cast<double>(u_lo[a]);
        double want = ext / 251.0;
        want = want > step_min ? want : step_min;
        int e = wide_exponent(want);
        inv_step[a] = ldexpf(1.0f, -e);
        ebytes |= static_cast<uint32_t>(e + 127) << (8 * a);
        double l = static_cast<double>(u_lo[a]) - ldexp(1.0, e);
        float f = static_cast<float>(l);
        if (static_cast<double>(f) > l)
            f = nextafterf(f, -INFINITY);
        org[a] = f;
        words[a] = box_f2u(f);
    }
    words[3] = (words[3] & 0xFF000000u) | ebytes;
    uint32_t qb[12] = {0};
    for (int s = 0; s < 8; s++) {
        if (!(present >> s & 1))
            continue;
        for (int a = 0; a < 3; a++) {
            float fl, cl, unused;
            wide_grid_floor_ceil(lo[s][a], org[a], inv_step[a], fl, unused);
            wide_grid_floor_ceil(hi[s][a], org[a], inv_step[a], unused, cl);
            float ql = fl - 1.0f, qh = cl + 1.0f;
            ql = ql < 0.0f ? 0.0f : (ql > 255.0f ? 255.0f : ql);
            qh = qh < 0.0f ? 0.0f : (qh > 255.0f ? 255.0f : qh);
            // byte s of plane a (lo) and plane 3 + a (hi); 8 bytes per plane, little endian
            qb[2 * a + (s >> 2)] |= static_cast<uint32_t>(ql) << (8 * (s & 3));
            qb[2 * (3 + a) + (s >> 2)] |= static_cast<uint32_t>(qh) << (8 * (s & 3));
        }
    }
    for (int k = 0; k < 12; k++)
        words[8 + k] = qb[k];
}

} // namespace e8g
