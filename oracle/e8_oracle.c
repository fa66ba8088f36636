/*
 * e8_oracle.c — CPU restatement of e8yescg corelib's per-pixel path integral.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the CPU stand-in for the reference
 * where the reference cannot be compiled. Never linked into the product.
 *
 * Arithmetic follows the reference operation by operation (vec ops of corelib/src/tensor.h
 * evaluate component-wise, dot products as ((0 + a0 b0) + a1 b1) + a2 b2, `k * v` as k * v_i),
 * so that with -ffp-contract=off both produce identical bits from identical draws. Citations
 * are file:line in the reference project.
 */
#define _GNU_SOURCE
#include "e8_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define PI_F ((float)M_PI) /* static_cast<float>(M_PI) throughout the reference */

/* std::min / std::max (libstdc++: min(a,b) = b < a ? b : a; max(a,b) = a < b ? b : a) */
static inline float smin(float a, float b) { return b < a ? b : a; }
static inline float smax(float a, float b) { return a < b ? b : a; }

/* ------------------------------------------------------------------ vec3 -- */
/* corelib/src/tensor.h:32-308 */

typedef struct v3 {
    float x, y, z;
} v3;

static inline v3 V(float x, float y, float z) {
    v3 r = {x, y, z};
    return r;
}
static const v3 V0 = {0.0f, 0.0f, 0.0f};
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline v3 vmul(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vscale(v3 a, float k) { return V(k * a.x, k * a.y, k * a.z); } /* :147-163 */
static inline v3 vdivs(v3 a, float k) { return V(a.x / k, a.y / k, a.z / k); }  /* :154-159 */
static inline float vdot(v3 a, v3 b) {                                          /* :165-170 */
    float v = 0.0f;
    v += a.x * b.x;
    v += a.y * b.y;
    v += a.z * b.z;
    return v;
}
static inline v3 vcross(v3 a, v3 b) { /* :204-211 */
    return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float vnorm(v3 a) { return sqrtf(vdot(a, a)); }
static inline v3 vnormalize(v3 a) { /* :225-227 */
    float k = 1.0f / vnorm(a);
    return vscale(a, k);
}
static inline float vsum(v3 a) { /* :217-223 */
    float s = a.x;
    s += a.y;
    s += a.z;
    return s;
}
static inline int feq(float a, float b) { return fabsf(a - b) <= 1e-5f; } /* :14-16 */
static inline int vequals0(v3 a) { return feq(a.x, 0.0f) && feq(a.y, 0.0f) && feq(a.z, 0.0f); }
static inline float vget(v3 a, unsigned i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline v3 vld(const float *p) { return V(p[0], p[1], p[2]); }
static inline void vst(float *p, v3 a) {
    p[0] = a.x;
    p[1] = a.y;
    p[2] = a.z;
}

/* ------------------------------------------------------------- ray / aabb -- */

typedef struct oray {
    v3 o, v, v_inv;
} oray;

static inline oray mkray(v3 o, v3 v) { /* tensor.h:686 */
    oray r;
    r.o = o;
    r.v = v;
    r.v_inv = V(1.0f / v.x, 1.0f / v.y, 1.0f / v.z);
    return r;
}

/* ray::intersect, tensor.h:688-725 */
static inline int tri_intersect(const oray *r, v3 v0, v3 v1, v3 v2, float t_min, float t_max,
                                float *b1o, float *b2o, float *t0o) {
    v3 va = vsub(v1, v0);
    v3 vb = vsub(v2, v0);
    v3 vc = vsub(r->o, v0);
    v3 e2 = vcross(r->v, vb);
    float det = vdot(va, e2);
    if (det == 0.0f)
        return 0;
    float inv = 1.0f / det;
    float b1 = vdot(vc, e2) * inv;
    if (b1 < 0.0f || b1 > 1.0f)
        return 0;
    v3 e1 = vcross(vc, va);
    float b2 = vdot(r->v, e1) * inv;
    if (b2 < 0.0f || b1 + b2 > 1.0f)
        return 0;
    float t0 = vdot(vb, e1) * inv;
    if (t0 < t_min || t0 > t_max)
        return 0;
    *b1o = b1;
    *b2o = b2;
    *t0o = t0;
    return 1;
}

typedef struct oaabb {
    v3 mn, mx;
    int empty;
} oaabb;

/* aabb() leaves min/max as vec3() = 0 and is_empty = true, tensor.h:757 */
static inline oaabb aabb_empty(void) {
    oaabb b;
    b.mn = V0;
    b.mx = V0;
    b.empty = 1;
    return b;
}
static inline oaabb aabb_make(v3 mn, v3 mx) { /* :759-761 */
    oaabb b;
    b.mn = mn;
    b.mx = mx;
    b.empty = mn.x > mx.x || mn.y > mx.y || mn.z > mx.z;
    return b;
}
/* aabb + aabb, :763-772. A non-empty box merged with an empty one takes the empty box's zero
 * corners into account, exactly as the reference does. */
static inline oaabb aabb_merge(oaabb a, oaabb rhs) {
    if (!a.empty)
        return aabb_make(V(smin(a.mn.x, rhs.mn.x), smin(a.mn.y, rhs.mn.y), smin(a.mn.z, rhs.mn.z)),
                         V(smax(a.mx.x, rhs.mx.x), smax(a.mx.y, rhs.mx.y), smax(a.mx.z, rhs.mx.z)));
    return rhs;
}
/* aabb + vec3, :774-783 */
static inline oaabb aabb_add_point(oaabb a, v3 p) {
    if (!a.empty)
        return aabb_make(V(smin(a.mn.x, p.x), smin(a.mn.y, p.y), smin(a.mn.z, p.z)),
                         V(smax(a.mx.x, p.x), smax(a.mx.y, p.y), smax(a.mx.z, p.z)));
    return aabb_make(p, p);
}
static inline float aabb_area(oaabb b) { /* :802-809 */
    if (b.empty)
        return 0.0f;
    v3 d = vsub(b.mx, b.mn);
    return 2.0f * (d.x * d.y + d.x * d.z + d.y * d.z);
}
/* aabb::intersect, :815-840 */
static inline int aabb_hit(const oaabb *b, const oray *r, float t_min, float t_max) {
    for (unsigned i = 0; i < 3; i++) {
        float k0 = (vget(b->mn, i) - vget(r->o, i)) * vget(r->v_inv, i);
        float k1 = (vget(b->mx, i) - vget(r->o, i)) * vget(r->v_inv, i);
        if (k0 > k1) {
            t_min = smax(k1, t_min);
            t_max = smin(k0, t_max);
        } else {
            t_min = smax(k0, t_min);
            t_max = smin(k1, t_max);
        }
        if (t_min > t_max)
            return 0;
    }
    return 1;
}

/* ---------------------------------------------------------------- random -- */

/* e8util::rng = std::default_random_engine (minstd_rand0: x <- 16807 x mod 2^31-1) feeding
 * uniform_real_distribution<float>(0,1); libstdc++'s generate_canonical<float> takes one engine
 * call: float(x - 1) / float(2^31 - 2) (= 2^31 after rounding), clamped below 1. tensor.h:987-1001 */
typedef struct orng {
    int kind;
    uint32_t x;           /* minstd state */
    uint32_t key[2];      /* philox */
    uint32_t ctr[3];      /* philox counter words (pixel, sample, tag) */
    uint32_t block, lane; /* philox position */
    uint32_t buf[4];
} orng;

static inline void minstd_seed(orng *r, uint32_t s) {
    r->kind = E8G_RNG_MINSTD;
    uint32_t m = 2147483647u;
    r->x = s % m;
    if (r->x == 0)
        r->x = 1;
}

static inline float minstd_draw(orng *r) {
    r->x = (uint32_t)(((uint64_t)r->x * 16807u) % 2147483647u);
    float f = (float)(r->x - 1u) / 2147483648.0f;
    if (f >= 1.0f)
        f = nextafterf(1.0f, 0.0f);
    return f;
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), own implementation. */
static inline void philox_block(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; round++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

static inline void philox_seed(orng *r, uint64_t seed, uint32_t pixel, uint32_t sample) {
    r->kind = E8G_RNG_PHILOX;
    r->key[0] = (uint32_t)seed;
    r->key[1] = (uint32_t)(seed >> 32);
    r->ctr[0] = pixel;
    r->ctr[1] = sample;
    r->ctr[2] = 0x0E8A0E8Au;
    r->block = 0;
    r->lane = 4;
}

static inline float philox_draw(orng *r) {
    if (r->lane == 4) {
        uint32_t c[4] = {r->block, r->ctr[0], r->ctr[1], r->ctr[2]};
        philox_block(c, r->key, r->buf);
        r->block++;
        r->lane = 0;
    }
    uint32_t u = r->buf[r->lane++];
    return (float)(u >> 8) * (1.0f / 16777216.0f);
}

static inline float draw(orng *r) { return r->kind == E8G_RNG_MINSTD ? minstd_draw(r) : philox_draw(r); }

static inline uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint32_t o_path_seed(uint64_t seed, uint32_t pixel, uint32_t sample) {
    uint64_t z = splitmix64(splitmix64(seed) ^ (((uint64_t)pixel << 32) | sample));
    uint32_t s = (uint32_t)(z % 2147483647ull);
    return s == 0 ? 1u : s;
}

void o_minstd_draws(uint32_t seed, uint32_t n, float *out) {
    orng r;
    minstd_seed(&r, seed);
    for (uint32_t i = 0; i < n; i++)
        out[i] = minstd_draw(&r);
}

void o_philox_draws(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t n, float *out) {
    orng r;
    philox_seed(&r, seed, pixel, sample);
    for (uint32_t i = 0; i < n; i++)
        out[i] = philox_draw(&r);
}

/* ------------------------------------------------------------------ scene -- */

typedef struct omat {
    uint32_t type;
    v3 albedo;
    float sigma, a, b;   /* oren_nayar, material.cpp:108-116 */
    float alpha2;        /* cook_torr, material.cpp:176 */
    float ior_re, ior_im;
    int32_t mix0, mix1;
    float ratio;
} omat;

typedef struct onode { /* flattened_node, pathspace.h:138-156 */
    oaabb bound;
    uint32_t num_prims;
    uint32_t split_axis;
    uint32_t next_child;
    uint32_t prim_start;
} onode;

typedef struct oprim { /* primitive, pathspace.h:86-93 (triangle kept as a global index) */
    uint32_t tri;
    uint32_t mesh;
} oprim;

struct o_scene {
    uint32_t nm, nv, nt;
    uint32_t *voff, *toff;
    int32_t *mesh_mat;
    int32_t *mesh_light;
    uint32_t *tri_mesh;
    v3 *pos, *nrm;
    uint32_t *tri; /* global vertex indices */
    float *mesh_area;  /* trimesh::update_face_cdf m_area, geometry.cpp:105-118 */
    float *tri_cum;    /* per mesh prefix area (product-mode light sampling) */
    oaabb bound;       /* if_path_space::m_bound, pathspace.cpp:17 */
    uint32_t nmat;
    omat *mats;
    omat fail_safe;
    uint32_t nl;
    e8g_light *lights;
    float *light_cum; /* basic_light_sources::m_light_cdf, lightsources.cpp:45-52 */
    float *light_pnorm;
    float total_power;
    e8g_camera cam;
    onode *bvh;
    uint32_t nnodes, nnodes_cap;
    oprim *prims;
    uint32_t max_depth, nleaves;
};

static inline v3 P(const o_scene *s, uint32_t mesh, uint32_t local) { return s->pos[s->voff[mesh] + local]; }

static void mat_init(omat *m, const e8g_material *d) {
    memset(m, 0, sizeof(*m));
    m->type = d->type;
    m->albedo = vld(d->albedo);
    if (d->type == E8G_MAT_OREN_NAYAR) {
        m->sigma = d->roughness;
        float sigma2 = m->sigma * m->sigma;
        m->a = 1 - 0.5f * sigma2 / (sigma2 + 0.33f);
        m->b = 0.45f * sigma2 / (sigma2 + 0.09f);
    } else if (d->type == E8G_MAT_COOK_TORR) {
        m->alpha2 = 2 * d->roughness * d->roughness;
        m->ior_re = d->ior_re;
        m->ior_im = d->ior_im;
    } else if (d->type == E8G_MAT_MIXTURE) {
        m->mix0 = d->mix0;
        m->mix1 = d->mix1;
        m->ratio = d->ratio;
    } else {
        m->albedo = V(0.8f, 0.8f, 0.8f); /* mat_fail_safe, material.cpp:54-55 */
    }
}

/* --------------------------------------------------------------- BVH build -- */
/* bvh_path_space_layout::commit and helpers, pathspace.cpp:121-328 */

#define BVH_MAX_PRIMS 4
#define BVH_BUCKET_COUNT 20
#define BVH_RAY_TRIANGLE_COST 8
#define BVH_RAY_BOX_COST 1

typedef struct oprimd {
    oprim p;
    oaabb bound;
    v3 centroid;
} oprimd;

typedef struct obucket {
    float cost;
    unsigned num_prims;
    oaabb bound;
} obucket;

static void sah_buckets(const oprimd *prims, unsigned start, unsigned end, unsigned axis, oaabb bound,
                        v3 range, obucket *buckets) {
    for (unsigned i = 0; i < BVH_BUCKET_COUNT; i++) {
        buckets[i].cost = 0.0f;
        buckets[i].num_prims = 0;
        buckets[i].bound = aabb_empty();
    }
    float bucket_width = vget(range, axis) / BVH_BUCKET_COUNT;
    for (unsigned i = start; i < end; i++) {
        unsigned ib = (unsigned)((vget(prims[i].centroid, axis) - vget(bound.mn, axis)) / bucket_width);
        if (ib == BVH_BUCKET_COUNT)
            ib = BVH_BUCKET_COUNT - 1;
        buckets[ib].bound = aabb_merge(buckets[ib].bound, prims[i].bound);
        buckets[ib].num_prims++;
    }
    buckets[BVH_BUCKET_COUNT - 1].cost = INFINITY;
    for (unsigned i = 0; i < BVH_BUCKET_COUNT - 1; i++) {
        oaabb first = aabb_empty(), second = aabb_empty();
        unsigned c_first = 0, c_second = 0;
        for (unsigned j = 0; j <= i; j++) {
            first = aabb_merge(first, buckets[j].bound);
            c_first += buckets[j].num_prims;
        }
        for (unsigned j = i + 1; j < BVH_BUCKET_COUNT; j++) {
            second = aabb_merge(second, buckets[j].bound);
            c_second += buckets[j].num_prims;
        }
        buckets[i].cost = BVH_RAY_BOX_COST +
                          BVH_RAY_TRIANGLE_COST * (+aabb_area(first) / aabb_area(bound) * (float)c_first +
                                                   aabb_area(second) / aabb_area(bound) * (float)c_second);
    }
}

static unsigned g_sort_axis;
static int cmp_centroid(const void *a, const void *b) {
    float ca = vget(((const oprimd *)a)->centroid, g_sort_axis);
    float cb = vget(((const oprimd *)b)->centroid, g_sort_axis);
    if (ca < cb)
        return -1;
    if (cb < ca)
        return 1;
    /* equal keys: keep input order (the reference's std::sort leaves it unspecified) */
    return (a < b) ? -1 : (a > b);
}

static void stable_sort_axis(oprimd *p, unsigned n, unsigned axis) {
    /* merge sort: deterministic order for equal centroids */
    if (n < 2)
        return;
    oprimd *tmp = (oprimd *)malloc(sizeof(oprimd) * n);
    for (unsigned width = 1; width < n; width *= 2) {
        for (unsigned lo = 0; lo < n; lo += 2 * width) {
            unsigned mid = lo + width < n ? lo + width : n;
            unsigned hi = lo + 2 * width < n ? lo + 2 * width : n;
            unsigned i = lo, j = mid, k = lo;
            while (i < mid && j < hi) {
                if (vget(p[j].centroid, axis) < vget(p[i].centroid, axis))
                    tmp[k++] = p[j++];
                else
                    tmp[k++] = p[i++];
            }
            while (i < mid)
                tmp[k++] = p[i++];
            while (j < hi)
                tmp[k++] = p[j++];
        }
        memcpy(p, tmp, sizeof(oprimd) * n);
    }
    free(tmp);
    (void)cmp_centroid;
    (void)g_sort_axis;
}

/* std::partition for bidirectional iterators (the two-pointer exchange libstdc++ uses), with
 * predicate centroid(axis) < split. Returns the partition point. */
static unsigned partition_lt(oprimd *p, unsigned first, unsigned last, unsigned axis, float split) {
    for (;;) {
        for (;;) {
            if (first == last)
                return first;
            if (vget(p[first].centroid, axis) < split)
                ++first;
            else
                break;
        }
        --last;
        for (;;) {
            if (first == last)
                return first;
            if (!(vget(p[last].centroid, axis) < split))
                --last;
            else
                break;
        }
        oprimd t = p[first];
        p[first] = p[last];
        p[last] = t;
        ++first;
    }
}

static uint32_t push_node(o_scene *s) {
    if (s->nnodes == s->nnodes_cap) {
        s->nnodes_cap = s->nnodes_cap ? s->nnodes_cap * 2 : 1024;
        s->bvh = (onode *)realloc(s->bvh, sizeof(onode) * s->nnodes_cap);
    }
    memset(&s->bvh[s->nnodes], 0, sizeof(onode));
    return s->nnodes++;
}

static oaabb bound_range(const oprimd *prims, unsigned start, unsigned end) { /* :168-175 */
    oaabb b = aabb_empty();
    for (unsigned i = start; i < end; i++)
        b = aabb_merge(b, prims[i].bound);
    return b;
}

/* bvh() :177-260 fused with flatten() :274-290 (left subtree emitted right after its parent). */
static void bvh_build(o_scene *s, oprimd *prims, unsigned nprims, unsigned start, unsigned end,
                      unsigned depth) {
    if (end - start == 0)
        return;
    if (end - start == 1) {
        uint32_t n = push_node(s);
        s->bvh[n].bound = prims[start].bound;
        s->bvh[n].num_prims = 1;
        s->bvh[n].prim_start = start;
        s->bvh[n].split_axis = 0xFF;
        s->bvh[n].next_child = 0xFFFFFFFFu;
        if (depth + 1 > s->max_depth)
            s->max_depth = depth + 1;
        s->nleaves++;
        return;
    }
    oaabb b = bound_range(prims, start, end);
    v3 range = vsub(b.mx, b.mn);
    unsigned axis;
    if (range.x > range.y && range.x > range.z)
        axis = 0;
    else if (range.y > range.z)
        axis = 1;
    else
        axis = 2;
    float cost_nonsplit = (float)((end - start) * BVH_RAY_TRIANGLE_COST);
    obucket buckets[BVH_BUCKET_COUNT];
    sah_buckets(prims, start, end, axis, b, range, buckets);
    unsigned split_antiaxis = 1; /* the reference starts from 1 while comparing against bucket 0 */
    float cost_split = buckets[0].cost;
    for (unsigned i = 1; i < BVH_BUCKET_COUNT - 1; i++) {
        if (buckets[i].cost < cost_split) {
            split_antiaxis = i;
            cost_split = buckets[i].cost;
        }
    }
    if (cost_split < cost_nonsplit || end - start > BVH_MAX_PRIMS) {
        unsigned mid;
        if ((double)depth > log2((double)nprims)) {
            stable_sort_axis(prims + start, end - start, axis);
            mid = (start + end) >> 1;
        } else {
            float split = vget(b.mn, axis) + (float)(split_antiaxis + 1) * vget(range, axis) / BVH_BUCKET_COUNT;
            mid = partition_lt(prims, start, end, axis, split);
            if (mid == start)
                mid++;
            else if (mid == end)
                mid--;
        }
        uint32_t n = push_node(s);
        bvh_build(s, prims, nprims, start, mid, depth + 1);
        s->bvh[n].bound = b;
        s->bvh[n].num_prims = 0;
        s->bvh[n].split_axis = axis;
        s->bvh[n].next_child = s->nnodes;
        s->bvh[n].prim_start = 0xFFFFFFFFu;
        bvh_build(s, prims, nprims, mid, end, depth + 1);
    } else {
        uint32_t n = push_node(s);
        s->bvh[n].bound = b;
        s->bvh[n].num_prims = end - start;
        s->bvh[n].prim_start = start;
        s->bvh[n].split_axis = 0xFF;
        s->bvh[n].next_child = 0xFFFFFFFFu;
        if (depth + 1 > s->max_depth)
            s->max_depth = depth + 1;
        s->nleaves++;
    }
}

static void commit_bvh(o_scene *s) {
    oprimd *prims = (oprimd *)malloc(sizeof(oprimd) * (s->nt ? s->nt : 1));
    for (uint32_t m = 0; m < s->nm; m++) {
        for (uint32_t t = s->toff[m]; t < s->toff[m + 1]; t++) {
            oprimd *p = &prims[t];
            p->p.tri = t;
            p->p.mesh = m;
            v3 v0 = s->pos[s->tri[3 * t]], v1 = s->pos[s->tri[3 * t + 1]], v2 = s->pos[s->tri[3 * t + 2]];
            oaabb b = aabb_empty();
            b = aabb_add_point(b, v0);
            b = aabb_add_point(b, v1);
            b = aabb_add_point(b, v2);
            p->bound = b;
            p->centroid = vdivs(vadd(b.mx, b.mn), 2.0f); /* pathspace.h:106 */
        }
    }
    s->nnodes = 0;
    s->max_depth = 0;
    s->nleaves = 0;
    bvh_build(s, prims, s->nt, 0, s->nt, 0);
    s->prims = (oprim *)malloc(sizeof(oprim) * (s->nt ? s->nt : 1));
    for (uint32_t i = 0; i < s->nt; i++)
        s->prims[i] = prims[i].p;
    free(prims);
}

void o_bvh_stats(const o_scene *s, uint32_t *num_nodes, uint32_t *max_depth, uint32_t *num_leaves) {
    *num_nodes = s->nnodes;
    *max_depth = s->max_depth;
    *num_leaves = s->nleaves;
}

o_scene *o_scene_create(const e8g_scene_desc *d) {
    o_scene *s = (o_scene *)calloc(1, sizeof(o_scene));
    s->nm = d->num_meshes;
    s->nv = d->mesh_vert_offset[d->num_meshes];
    s->nt = d->mesh_tri_offset[d->num_meshes];
    s->voff = (uint32_t *)malloc(sizeof(uint32_t) * (s->nm + 1));
    s->toff = (uint32_t *)malloc(sizeof(uint32_t) * (s->nm + 1));
    memcpy(s->voff, d->mesh_vert_offset, sizeof(uint32_t) * (s->nm + 1));
    memcpy(s->toff, d->mesh_tri_offset, sizeof(uint32_t) * (s->nm + 1));
    s->mesh_mat = (int32_t *)malloc(sizeof(int32_t) * (s->nm + 1));
    s->mesh_light = (int32_t *)malloc(sizeof(int32_t) * (s->nm + 1));
    s->mesh_area = (float *)malloc(sizeof(float) * (s->nm + 1));
    s->pos = (v3 *)malloc(sizeof(v3) * (s->nv + 1));
    s->nrm = (v3 *)malloc(sizeof(v3) * (s->nv + 1));
    s->tri = (uint32_t *)malloc(sizeof(uint32_t) * 3 * (s->nt + 1));
    s->tri_mesh = (uint32_t *)malloc(sizeof(uint32_t) * (s->nt + 1));
    s->tri_cum = (float *)malloc(sizeof(float) * (s->nt + 1));
    for (uint32_t i = 0; i < s->nv; i++) {
        s->pos[i] = vld(d->positions + 3 * i);
        s->nrm[i] = vld(d->normals + 3 * i);
    }
    s->bound = aabb_empty();
    for (uint32_t m = 0; m < s->nm; m++) {
        s->mesh_mat[m] = d->mesh_material ? d->mesh_material[m] : -1;
        s->mesh_light[m] = -1;
        for (uint32_t t = s->toff[m]; t < s->toff[m + 1]; t++) {
            for (int k = 0; k < 3; k++)
                s->tri[3 * t + k] = s->voff[m] + d->triangles[3 * t + k];
            s->tri_mesh[t] = m;
        }
        /* update_aabb, geometry.cpp:97-103 */
        if (s->voff[m + 1] > s->voff[m]) {
            oaabb mb = aabb_make(s->pos[s->voff[m]], s->pos[s->voff[m]]);
            for (uint32_t v = s->voff[m] + 1; v < s->voff[m + 1]; v++)
                mb = aabb_add_point(mb, s->pos[v]);
            s->bound = aabb_merge(s->bound, mb);
        }
        /* update_face_cdf, geometry.cpp:105-118 */
        float cum = 0;
        for (uint32_t t = s->toff[m]; t < s->toff[m + 1]; t++) {
            v3 v0 = s->pos[s->tri[3 * t]], v1 = s->pos[s->tri[3 * t + 1]], v2 = s->pos[s->tri[3 * t + 2]];
            float a = 0.5f * vnorm(vcross(vsub(v1, v0), vsub(v2, v0)));
            cum += a;
            s->tri_cum[t] = cum;
        }
        s->mesh_area[m] = cum;
    }
    s->nmat = d->num_materials;
    s->mats = (omat *)calloc(s->nmat + 1, sizeof(omat));
    for (uint32_t i = 0; i < s->nmat; i++)
        mat_init(&s->mats[i], &d->materials[i]);
    e8g_material fs;
    memset(&fs, 0, sizeof(fs));
    fs.type = E8G_MAT_FAIL_SAFE;
    mat_init(&s->fail_safe, &fs);
    /* lights: load() in order (first light of a mesh wins the lookup), commit() builds the CDF */
    s->nl = d->num_lights;
    s->lights = (e8g_light *)malloc(sizeof(e8g_light) * (s->nl + 1));
    s->light_cum = (float *)malloc(sizeof(float) * (s->nl + 1));
    s->light_pnorm = (float *)malloc(sizeof(float) * (s->nl + 1));
    s->total_power = 0;
    for (uint32_t l = 0; l < s->nl; l++) {
        s->lights[l] = d->lights[l];
        uint32_t m = d->lights[l].mesh;
        if (s->mesh_light[m] < 0)
            s->mesh_light[m] = (int32_t)l;
        /* m_power = pi * area * rad, light.cpp:20; power().norm(), lightsources.cpp:49 */
        v3 power = vscale(vld(d->lights[l].radiance), PI_F * s->mesh_area[m]);
        s->light_pnorm[l] = vnorm(power);
        s->total_power += s->light_pnorm[l];
        s->light_cum[l] = s->total_power;
    }
    s->cam = d->camera;
    commit_bvh(s);
    return s;
}

void o_scene_free(o_scene *s) {
    if (!s)
        return;
    free(s->voff);
    free(s->toff);
    free(s->mesh_mat);
    free(s->mesh_light);
    free(s->mesh_area);
    free(s->pos);
    free(s->nrm);
    free(s->tri);
    free(s->tri_mesh);
    free(s->tri_cum);
    free(s->mats);
    free(s->lights);
    free(s->light_cum);
    free(s->light_pnorm);
    free(s->bvh);
    free(s->prims);
    free(s);
}

/* ------------------------------------------------------------- traversal -- */

typedef struct overt { /* intersect_info, pathspace.h:18-31 (uv omitted: it only feeds texture
                          maps, which the material container's copies drop, material.cpp:118-120) */
    int valid;
    float t;
    v3 vertex, normal;
    int32_t mesh, tri;
    float b1, b2;
} overt;

static overt make_vert(const o_scene *s, uint32_t tri, float t, float b1, float b2) {
    /* pathspace.cpp:385-409 */
    overt h;
    float b0 = 1.0f - b1 - b2; /* tensor.h:723 */
    uint32_t i0 = s->tri[3 * tri], i1 = s->tri[3 * tri + 1], i2 = s->tri[3 * tri + 2];
    h.vertex = vadd(vadd(vscale(s->pos[i0], b0), vscale(s->pos[i1], b1)), vscale(s->pos[i2], b2));
    h.normal = vnormalize(vadd(vadd(vscale(s->nrm[i0], b0), vscale(s->nrm[i1], b1)), vscale(s->nrm[i2], b2)));
    h.valid = 1;
    h.t = t;
    h.mesh = (int32_t)s->tri_mesh[tri];
    h.tri = (int32_t)(tri - s->toff[h.mesh]);
    h.b1 = b1;
    h.b2 = b2;
    return h;
}

static overt miss_vert(void) {
    overt h;
    memset(&h, 0, sizeof(h));
    h.mesh = -1;
    h.tri = -1;
    return h;
}

typedef struct ocount {
    uint64_t nodes, tris;
} ocount;

/* bvh_path_space_layout::intersect, pathspace.cpp:330-413 */
static overt intersect_bvh(const o_scene *s, const oray *r, ocount *cnt) {
    if (s->nnodes == 0)
        return miss_vert();
    const float t_min = 1e-4f, t_max = 1000.0f;
    float t = INFINITY, hb1 = 0, hb2 = 0;
    int64_t hit = -1;
    uint32_t stack[256];
    uint32_t *heap_stack = NULL;
    uint32_t cap = 256, sp = 0;
    uint32_t *st = stack;
    st[sp++] = 0;
    while (sp) {
        uint32_t n = st[--sp];
        const onode *nd = &s->bvh[n];
        if (nd->num_prims > 0) {
            for (uint32_t i = nd->prim_start; i < nd->prim_start + nd->num_prims; i++) {
                uint32_t tri = s->prims[i].tri;
                float b1, b2, t0;
                if (cnt)
                    cnt->tris++;
                if (tri_intersect(r, s->pos[s->tri[3 * tri]], s->pos[s->tri[3 * tri + 1]],
                                  s->pos[s->tri[3 * tri + 2]], t_min, t_max, &b1, &b2, &t0) &&
                    t0 < t) {
                    t = t0;
                    hit = tri;
                    hb1 = b1;
                    hb2 = b2;
                }
            }
        } else {
            uint32_t left = n + 1, right = nd->next_child;
            if (cnt)
                cnt->nodes += 2;
            if (sp + 2 > cap) {
                uint32_t ncap = cap * 2;
                uint32_t *ns = (uint32_t *)malloc(sizeof(uint32_t) * ncap);
                memcpy(ns, st, sizeof(uint32_t) * sp);
                free(heap_stack);
                heap_stack = ns;
                st = ns;
                cap = ncap;
            }
            if (aabb_hit(&s->bvh[left].bound, r, t_min, t_max))
                st[sp++] = left;
            if (aabb_hit(&s->bvh[right].bound, r, t_min, t_max))
                st[sp++] = right;
        }
    }
    free(heap_stack);
    if (hit < 0)
        return miss_vert();
    return make_vert(s, (uint32_t)hit, t, hb1, hb2);
}

/* bvh_path_space_layout::has_intersect, pathspace.cpp:415-456 */
static int has_intersect_bvh(const o_scene *s, const oray *r, float t_min, float t_max) {
    if (s->nnodes == 0)
        return 0;
    uint32_t stack[256];
    uint32_t *heap_stack = NULL;
    uint32_t cap = 256, sp = 0;
    uint32_t *st = stack;
    st[sp++] = 0;
    int found = 0;
    while (sp && !found) {
        uint32_t n = st[--sp];
        const onode *nd = &s->bvh[n];
        if (nd->num_prims > 0) {
            for (uint32_t i = nd->prim_start; i < nd->prim_start + nd->num_prims; i++) {
                uint32_t tri = s->prims[i].tri;
                float b1, b2, t0;
                if (tri_intersect(r, s->pos[s->tri[3 * tri]], s->pos[s->tri[3 * tri + 1]],
                                  s->pos[s->tri[3 * tri + 2]], t_min, t_max, &b1, &b2, &t0)) {
                    found = 1;
                    break;
                }
            }
        } else {
            uint32_t left = n + 1, right = nd->next_child;
            if (sp + 2 > cap) {
                uint32_t ncap = cap * 2;
                uint32_t *ns = (uint32_t *)malloc(sizeof(uint32_t) * ncap);
                memcpy(ns, st, sizeof(uint32_t) * sp);
                free(heap_stack);
                heap_stack = ns;
                st = ns;
                cap = ncap;
            }
            if (aabb_hit(&s->bvh[left].bound, r, t_min, t_max))
                st[sp++] = left;
            if (aabb_hit(&s->bvh[right].bound, r, t_min, t_max))
                st[sp++] = right;
        }
    }
    free(heap_stack);
    return found;
}

/* linear_path_space_layout::intersect, pathspace.cpp:36-92 */
static overt intersect_linear(const o_scene *s, const oray *r) {
    const float t_min = 1e-4f, t_max = 1000.0f;
    float t = INFINITY, hb1 = 0, hb2 = 0;
    int64_t hit = -1;
    for (uint32_t tri = 0; tri < s->nt; tri++) {
        float b1, b2, t0;
        if (tri_intersect(r, s->pos[s->tri[3 * tri]], s->pos[s->tri[3 * tri + 1]], s->pos[s->tri[3 * tri + 2]],
                          t_min, t_max, &b1, &b2, &t0) &&
            t0 < t) {
            hb1 = b1;
            hb2 = b2;
            hit = tri;
            t = t0;
        }
    }
    if (hit < 0)
        return miss_vert();
    return make_vert(s, (uint32_t)hit, t, hb1, hb2);
}

/* linear_path_space_layout::has_intersect, pathspace.cpp:94-114 */
static int has_intersect_linear(const o_scene *s, const oray *r, float t_min, float t_max) {
    for (uint32_t tri = 0; tri < s->nt; tri++) {
        float b1, b2, t0;
        if (tri_intersect(r, s->pos[s->tri[3 * tri]], s->pos[s->tri[3 * tri + 1]], s->pos[s->tri[3 * tri + 2]],
                          t_min, t_max, &b1, &b2, &t0))
            return 1;
    }
    return 0;
}

static inline overt intersect(const o_scene *s, const oray *r) { return intersect_bvh(s, r, NULL); }
static inline int has_intersect(const o_scene *s, const oray *r, float t_min, float t_max) {
    return has_intersect_bvh(s, r, t_min, t_max);
}

static oray ray_from(const e8g_ray *r) { return mkray(vld(r->o), vld(r->d)); }

static void fill_hit(o_hit *h, const overt *v) {
    h->t = v->valid ? v->t : 0.0f;
    h->mesh = v->valid ? v->mesh : -1;
    h->tri = v->valid ? v->tri : -1;
    h->b1 = v->b1;
    h->b2 = v->b2;
    vst(h->vertex, v->vertex);
    vst(h->normal, v->normal);
}

void o_trace_closest(const o_scene *s, const e8g_ray *rays, uint32_t n, int use_bvh, o_hit *hits) {
    for (uint32_t i = 0; i < n; i++) {
        oray r = ray_from(&rays[i]);
        overt v = use_bvh ? intersect_bvh(s, &r, NULL) : intersect_linear(s, &r);
        fill_hit(&hits[i], &v);
    }
}

void o_trace_closest_counts(const o_scene *s, const e8g_ray *rays, uint32_t n, uint64_t *nodes,
                            uint64_t *tris) {
    ocount c = {0, 0};
    for (uint32_t i = 0; i < n; i++) {
        oray r = ray_from(&rays[i]);
        intersect_bvh(s, &r, &c);
    }
    *nodes = c.nodes;
    *tris = c.tris;
}

void o_trace_any(const o_scene *s, const e8g_ray *rays, const float *t_min, const float *t_max,
                 uint32_t n, int use_bvh, uint8_t *occluded) {
    for (uint32_t i = 0; i < n; i++) {
        oray r = ray_from(&rays[i]);
        occluded[i] = (uint8_t)(use_bvh ? has_intersect_bvh(s, &r, t_min[i], t_max[i])
                                        : has_intersect_linear(s, &r, t_min[i], t_max[i]));
    }
}

/* ---------------------------------------------------------------- camera -- */

/* pinhole_camera::sample, camera.cpp:38-48; m_r is the camera transform's rotation block. */
static oray camera_ray(const o_scene *s, unsigned x, unsigned y, unsigned w, unsigned h) {
    const e8g_camera *c = &s->cam;
    float sz = c->sensor_size;
    v3 v = V(((float)x / (float)(w - 1) * sz - sz / 2.0f) * c->aspect,
             ((float)(h - 1) - (float)y) / (float)(h - 1) * sz - sz / 2.0f, -c->focal_len);
    /* (m_r * v.homo(0)).trunc(): mat44 * vec4 accumulates v(i) += m(i,j) * rhs(j), j = 0..3 */
    float d[3];
    for (int i = 0; i < 3; i++) {
        float acc = 0.0f;
        acc = acc + c->rot[3 * i + 0] * v.x;
        acc = acc + c->rot[3 * i + 1] * v.y;
        acc = acc + c->rot[3 * i + 2] * v.z;
        acc = acc + 0.0f * 0.0f;
        d[i] = acc;
    }
    return mkray(vld(c->origin), vnormalize(V(d[0], d[1], d[2])));
}

void o_camera_rays(const o_scene *s, uint32_t width, uint32_t height, e8g_ray *rays) {
    for (uint32_t y = 0; y < height; y++)
        for (uint32_t x = 0; x < width; x++) {
            oray r = camera_ray(s, x, y, width, height);
            vst(rays[y * width + x].o, r.o);
            vst(rays[y * width + x].d, r.v);
        }
}

/* ------------------------------------------------------------ materials -- */

static const omat *find_mat(const o_scene *s, int32_t m) { /* materialcontainer.cpp:7-17 */
    if (m < 0 || (uint32_t)m >= s->nmat)
        return &s->fail_safe;
    return &s->mats[m];
}

static inline float clampf(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

/* vec3_basis, tensor.h:939-943 */
static inline void basis(v3 n, v3 *u, v3 *v) {
    v3 ref = fabsf(n.x) > .1f ? V(0.0f, 1.0f, 0.0f) : V(1.0f, 1.0f, 1.0f);
    *u = vnormalize(vcross(ref, n));
    *v = vcross(n, *u);
}

/* vec3_cos_hemisphere_sample, tensor.h:972-985. The reference calls it as
 * f(n, rng->draw(), rng->draw()); GCC evaluates the arguments right to left, so the FIRST draw
 * is e1 (z = sqrt(e1)) and the SECOND is e0 (phi). */
static inline v3 cos_hemisphere(v3 n, orng *rng) {
    float e1 = draw(rng);
    float e0 = draw(rng);
    v3 u, v;
    basis(n, &u, &v);
    float z = sqrtf(e1);
    float r = sqrtf(1 - z * z);
    float phi = e0 * 2 * PI_F;
    float x = r * cosf(phi);
    float y = r * sinf(phi);
    return vadd(vadd(vscale(u, x), vscale(v, y)), vscale(n, z));
}

/* material.cpp:10-39 */
static inline float fresnel(float re, float im, v3 i, v3 h) {
    float f = 1.0f - vdot(i, h);
    float f2 = f * f;
    float f4 = f2 * f2;
    float f5 = f4 * f;
    float a = (re - 1) * (re - 1) + 4 * re * f5 + im * im;
    float b = (re + 1) * (re + 1) + im * im;
    return a / b;
}
static inline float ggx_distri(float alpha2, v3 n, v3 h) {
    float c = vdot(n, h);
    float c2 = c * c;
    float tan2 = (1.0f - c2) / c2;
    float k = 1.0f + tan2 / alpha2;
    return 1.0f / (PI_F * alpha2 * c2 * c2 * k * k);
}
static inline float ggx_lambda(float alpha2, v3 n, v3 w) {
    float c = vdot(n, w);
    float c2 = c * c;
    float tan2 = (1.0f - c2) / c2;
    return (-1.0f + sqrtf(1.0f + alpha2 * tan2)) / 2.0f;
}
static inline float ggx_shadow(float alpha2, v3 i, v3 o, v3 n) {
    return 1.0f / (1.0f + ggx_lambda(alpha2, n, i) + ggx_lambda(alpha2, n, o));
}

static v3 eval_leaf(const omat *m, v3 n, v3 o, v3 i) {
    switch (m->type) {
    case E8G_MAT_OREN_NAYAR: { /* material.cpp:134-161 */
        float cos_i = clampf(vdot(i, n), 0.0f, 1.0f);
        float cos_o = clampf(vdot(o, n), 0.0f, 1.0f);
        if (feq(cos_i, 0.0f) || feq(cos_o, 0.0f))
            return V0;
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
        return vscale(vscale(m->albedo, 1.0f / PI_F), m->a + m->b * smax(0.0f, cio) * sa * tan_b);
    }
    case E8G_MAT_COOK_TORR: { /* material.cpp:199-222 */
        float cos_o = smax(0.0f, vdot(n, o));
        float cos_i = smax(0.0f, vdot(n, i));
        if (feq(cos_i, 0.0f) || feq(cos_o, 0.0f))
            return V0;
        v3 h = vadd(i, o);
        if (vequals0(h))
            return V0;
        h = vnormalize(h);
        float f = fresnel(m->ior_re, m->ior_im, i, h);
        float d = ggx_distri(m->alpha2, n, h);
        float g = ggx_shadow(m->alpha2, i, o, n);
        float c = f * d * g / (4.0f * cos_i * cos_o);
        return vscale(m->albedo, c);
    }
    default: /* mat_fail_safe, material.cpp:64-68 */
        return vscale(m->albedo, 1.0f / PI_F);
    }
}

static v3 bsdf_eval(const o_scene *s, const omat *m, v3 n, v3 o, v3 i) {
    if (m->type == E8G_MAT_MIXTURE) { /* material.cpp:90-93 */
        v3 f0 = eval_leaf(find_mat(s, m->mix0), n, o, i);
        v3 f1 = eval_leaf(find_mat(s, m->mix1), n, o, i);
        return vadd(vscale(f0, m->ratio), vscale(f1, 1 - m->ratio));
    }
    return eval_leaf(m, n, o, i);
}

static v3 sample_leaf(const omat *m, orng *rng, float *dens, v3 n, v3 o) {
    if (m->type == E8G_MAT_COOK_TORR) { /* material.cpp:224-252 */
        float ms_slope = m->alpha2;
        v3 u, v;
        basis(n, &u, &v);
        float theta = 2.0f * PI_F * draw(rng);
        float t = draw(rng);
        float phi = atanf(sqrtf(ms_slope * t / (1.0f - t)));
        float sin_phi = sinf(phi);
        float cos_phi = cosf(phi);
        float x = sin_phi * cosf(theta);
        float y = sin_phi * sinf(theta);
        float z = cos_phi;
        v3 h = vadd(vadd(vscale(u, x), vscale(v, y)), vscale(n, z));
        float h_dot_o = vdot(h, o);
        v3 i = vsub(vscale(h, 2.0f * h_dot_o), o);
        if (vdot(i, n) < 0.0f) {
            *dens = 0.0f;
            return V0;
        }
        *dens = ggx_distri(ms_slope, n, h) * cos_phi / (4.0f * h_dot_o);
        return i;
    }
    /* oren_nayar / mat_fail_safe: material.cpp:70-76, :163-169 */
    v3 i = cos_hemisphere(n, rng);
    *dens = vdot(i, n) / PI_F;
    return i;
}

static v3 bsdf_sample(const o_scene *s, const omat *m, orng *rng, float *dens, v3 n, v3 o) {
    if (m->type == E8G_MAT_MIXTURE) { /* material.cpp:95-106 */
        v3 i;
        if (draw(rng) < m->ratio) {
            i = sample_leaf(find_mat(s, m->mix0), rng, dens, n, o);
            *dens *= m->ratio;
        } else {
            i = sample_leaf(find_mat(s, m->mix1), rng, dens, n, o);
            *dens *= 1 - m->ratio;
        }
        return i;
    }
    return sample_leaf(m, rng, dens, n, o);
}

void o_bsdf_eval(const o_scene *s, int32_t m, const float n[3], const float o[3], const float i[3],
                 float f_out[3]) {
    vst(f_out, bsdf_eval(s, find_mat(s, m), vld(n), vld(o), vld(i)));
}

void o_bsdf_sample(const o_scene *s, int32_t m, uint32_t seed, const float n[3], const float o[3],
                   uint32_t count, float *dirs_out, float *pdf_out) {
    orng rng;
    minstd_seed(&rng, seed);
    for (uint32_t k = 0; k < count; k++) {
        float dens = -1;
        v3 i = bsdf_sample(s, find_mat(s, m), &rng, &dens, vld(n), vld(o));
        vst(dirs_out + 3 * k, i);
        pdf_out[k] = dens;
    }
}

/* ---------------------------------------------------------------- lights -- */

static inline v3 light_rad(const o_scene *s, int l) { return vld(s->lights[l].radiance); }

/* area_light::radiance, light.cpp:64-71 */
static inline v3 light_radiance(const o_scene *s, int l, v3 w, v3 n) {
    float c = vdot(n, w);
    return c > 0 ? light_rad(s, l) : V0;
}
/* area_light::projected_radiance, light.cpp:54-62 */
static inline v3 light_projected_radiance(const o_scene *s, int l, v3 w, v3 n) {
    float c = vdot(n, w);
    return c > 0 ? vscale(light_rad(s, l), c) : V0;
}
/* area_light::eval, light.cpp:41-52 */
static inline v3 light_eval(const o_scene *s, int l, v3 i, v3 n_light, v3 n_target) {
    float r2 = vdot(i, i);
    v3 in = vdivs(i, sqrtf(r2));
    float cos_o = vdot(n_light, in);
    float cos_i = vdot(n_target, vneg(in));
    if (cos_o > 0 && cos_i > 0)
        return vdivs(vscale(vscale(light_rad(s, l), cos_i), cos_o), r2);
    return V0;
}

/* basic_light_sources::sample_light, lightsources.cpp:59-75 */
static int sample_light(const o_scene *s, orng *rng, float *pmf) {
    float e = draw(rng) * s->total_power;
    unsigned lo = 0, hi = s->nl;
    while (lo < hi) {
        unsigned mi = (lo + hi) >> 1;
        if (s->light_cum[mi] < e)
            lo = mi + 1;
        else
            hi = mi;
    }
    if (lo >= s->nl)
        lo = s->nl - 1;
    *pmf = s->light_pnorm[lo] / s->total_power;
    return (int)lo;
}

typedef struct osurf {
    v3 p, n;
    float area_dens;
} osurf;

/* trimesh::sample, geometry.cpp:44-66 (triangle uniform by index). With area_weighted, the
 * triangle is drawn from the area CDF instead (product modes; same draw count). */
static osurf mesh_sample(const o_scene *s, uint32_t mesh, orng *rng, int area_weighted) {
    uint32_t ntris = s->toff[mesh + 1] - s->toff[mesh];
    float q = draw(rng);
    unsigned i;
    if (!area_weighted) {
        i = (unsigned)(q * (float)ntris);
    } else {
        float e = q * s->mesh_area[mesh];
        unsigned lo = 0, hi = ntris;
        const float *cum = s->tri_cum + s->toff[mesh];
        while (lo < hi) {
            unsigned mi = (lo + hi) >> 1;
            if (cum[mi] <= e)
                lo = mi + 1;
            else
                hi = mi;
        }
        i = lo;
    }
    if (i >= ntris)
        i = ntris - 1;
    uint32_t t = s->toff[mesh] + i;
    float u = draw(rng);
    float v = draw(rng);
    float r = sqrtf(u);
    float b0 = 1 - r;
    float b1 = r * v;
    float b2 = 1 - b0 - b1;
    uint32_t i0 = s->tri[3 * t], i1 = s->tri[3 * t + 1], i2 = s->tri[3 * t + 2];
    osurf o;
    o.p = vadd(vadd(vscale(s->pos[i0], b0), vscale(s->pos[i1], b1)), vscale(s->pos[i2], b2));
    o.n = vnormalize(vadd(vadd(vscale(s->nrm[i0], b0), vscale(s->nrm[i1], b1)), vscale(s->nrm[i2], b2)));
    o.area_dens = 1.0f / s->mesh_area[mesh];
    return o;
}

/* ---------------------------------------------------------- integrators -- */

typedef struct octx {
    const o_scene *s;
    const o_policy *pol;
    orng *rng;
} octx;

static inline const omat *vert_mat(const o_scene *s, const overt *v) { return find_mat(s, s->mesh_mat[v->mesh]); }
static inline int vert_light(const o_scene *s, const overt *v) { return s->mesh_light[v->mesh]; }

/* transport_illum_source, pathtracer.cpp:152-176 */
static v3 transport_illum_source(const o_scene *s, int light, v3 p_illum, v3 n_illum, const overt *tv, v3 o) {
    v3 l = vsub(tv->vertex, p_illum);
    v3 illum = light_eval(s, light, l, n_illum, tv->normal);
    if (vequals0(illum))
        return V0;
    float distance = vnorm(l);
    v3 i = vdivs(vneg(l), distance);
    oray lr = mkray(tv->vertex, i);
    if (!has_intersect(s, &lr, 1e-4f, distance - 1e-3f))
        return vmul(illum, bsdf_eval(s, vert_mat(s, tv), tv->normal, o, i));
    return V0;
}

/* transport_direct_illum + sample_light_source, pathtracer.cpp:197-242 (multi_light_samps = 1) */
static v3 transport_direct_illum(octx *c, v3 o, const overt *tv) {
    v3 rad = V0;
    float pmf;
    int light = sample_light(c->s, c->rng, &pmf);
    osurf surf = mesh_sample(c->s, c->s->lights[light].mesh, c->rng, 0);
    surf.area_dens *= pmf;
    rad = vadd(rad, vdivs(transport_illum_source(c->s, light, surf.p, surf.n, tv, o), surf.area_dens));
    return vdivs(rad, (float)1u);
}

/* unidirect_path_tracer::sample_indirect_illum, pathtracer.cpp:528-566 */
static v3 uni_rec(octx *c, v3 o, const overt *vert, unsigned depth) {
    const o_scene *s = c->s;
    if (c->pol->max_depth && depth >= c->pol->max_depth)
        return V0;
    float ps = c->pol->rr_prob;
    if (depth >= c->pol->rr_start) {
        if (draw(c->rng) >= ps)
            return V0;
    } else {
        ps = 1;
    }
    int light = vert_light(s, vert);
    v3 le = V0;
    if (light >= 0)
        le = light_radiance(s, light, o, vert->normal);
    float pdf;
    v3 i = bsdf_sample(s, vert_mat(s, vert), c->rng, &pdf, vert->normal, o);
    if (pdf == 0.0f)
        return vdivs(le, ps);
    oray r = mkray(vert->vertex, i);
    overt nv = intersect(s, &r);
    if (!nv.valid || vdot(nv.normal, vneg(i)) <= 0.0f)
        return vdivs(le, ps);
    v3 next = uni_rec(c, vneg(i), &nv, depth + 1);
    float cos_w = vdot(vert->normal, i);
    v3 ind = vdivs(vscale(vmul(next, bsdf_eval(s, vert_mat(s, vert), vert->normal, o, i)), cos_w), pdf);
    return vdivs(vadd(le, ind), ps);
}

/* unidirect_lt1_path_tracer::sample_indirect_illum, pathtracer.cpp:587-628 */
static v3 lt1_rec(octx *c, v3 o, const overt *vert, unsigned depth) {
    const o_scene *s = c->s;
    if (c->pol->max_depth && depth >= c->pol->max_depth)
        return V0;
    float ps = c->pol->rr_prob;
    if (depth >= c->pol->rr_start) {
        if (draw(c->rng) >= ps)
            return V0;
    } else {
        ps = 1;
    }
    v3 direct = transport_direct_illum(c, o, vert);
    v3 multi = V0;
    float pdf;
    do {
        v3 i = bsdf_sample(s, vert_mat(s, vert), c->rng, &pdf, vert->normal, o);
        if (pdf == 0.0f)
            break;
        oray r = mkray(vert->vertex, i);
        overt nv = intersect(s, &r);
        if (!nv.valid || vdot(nv.normal, vneg(i)) <= 0.0f)
            break;
        v3 ind = lt1_rec(c, vneg(i), &nv, depth + 1);
        float cos_w = vdot(vert->normal, i);
        multi = vadd(multi, vdivs(vscale(vmul(ind, bsdf_eval(s, vert_mat(s, vert), vert->normal, o, i)), cos_w), pdf));
    } while (0);
    return vdivs(vadd(direct, vdivs(multi, (float)1u)), ps);
}

/* ---- bidirect_lt2_path_tracer, pathtracer.cpp:655-752 ---- */

/* join_with_light_paths, pathtracer.cpp:655-699: one light sample (transport_direct_illum)
 * plus a one-vertex light path (emission sample, the light ray's hit) joined to poi; the light
 * ray's miss drops both terms (:667-668). */
static v3 lt2_join(octx *c, v3 o, const overt *poi, unsigned cam_path_len) {
    const o_scene *s = c->s;
    v3 p1 = transport_direct_illum(c, o, poi);
    float pmf;
    int light = sample_light(s, c->rng, &pmf);
    osurf em = mesh_sample(s, s->lights[light].mesh, c->rng, 0); /* area_light::sample_emssion, light.cpp:26-32 */
    v3 w = cos_hemisphere(em.n, c->rng);
    float sa_dens = vdot(em.n, w) / PI_F;
    oray lr = mkray(em.p, w);
    overt term = intersect(s, &lr);
    if (!term.valid)
        return V0;
    v3 light_illum = vdivs(light_projected_radiance(s, light, w, em.n), pmf * em.area_dens * sa_dens);
    v3 tray = vneg(w);
    v3 join = vsub(poi->vertex, term.vertex);
    float distance = vnorm(join);
    join = vdivs(join, distance);
    oray jr = mkray(term.vertex, join);
    float cos_w2 = vdot(term.normal, tray);
    float cos_wo = vdot(term.normal, join);
    float cos_wi = vdot(poi->normal, vneg(join));
    if (cos_wo > 0.0f && cos_wi > 0.0f && cos_w2 > 0.0f && !has_intersect(s, &jr, 1e-4f, distance - 1e-3f)) {
        v3 f2 = vscale(vmul(light_illum, bsdf_eval(s, vert_mat(s, &term), term.normal, join, tray)), cos_w2);
        v3 p2 = vscale(vmul(vdivs(vscale(f2, cos_wo), distance * distance),
                            bsdf_eval(s, vert_mat(s, poi), poi->normal, o, vneg(join))),
                       cos_wi);
        if (cam_path_len == 0)
            return vadd(p1, vscale(p2, 0.5f));
        return vscale(vadd(p1, p2), 0.5f);
    }
    return p1;
}

/* bidirect_lt2_path_tracer::sample_indirect_illum, pathtracer.cpp:701-729: Russian roulette
 * from mutate_depth = 1 (the policy's rr_start), no back-face test on the continuation's hit,
 * and a continuation leaving below the surface (cos_w < 0, tested after the recursion) zeroes
 * the whole vertex. */
static v3 lt2_rec(octx *c, v3 o, const overt *vert, unsigned depth) {
    const o_scene *s = c->s;
    if (c->pol->max_depth && depth >= c->pol->max_depth)
        return V0;
    float ps = c->pol->rr_prob;
    if (depth >= c->pol->rr_start) {
        if (draw(c->rng) >= ps)
            return V0;
    } else {
        ps = 1;
    }
    v3 bidirect = lt2_join(c, o, vert, depth);
    float pdf;
    v3 i = bsdf_sample(s, vert_mat(s, vert), c->rng, &pdf, vert->normal, o);
    oray r = mkray(vert->vertex, i);
    overt nv = intersect(s, &r);
    v3 rr = V0;
    if (nv.valid) {
        v3 ind = lt2_rec(c, vneg(i), &nv, depth + 1);
        float cos_w = vdot(vert->normal, i);
        if (cos_w < 0.0f)
            return V0;
        rr = vdivs(vscale(vmul(ind, bsdf_eval(s, vert_mat(s, vert), vert->normal, o, i)), cos_w), pdf);
    }
    return vdivs(vadd(bidirect, rr), ps);
}

/* ---- bidirectional (bidirect_mis_path_tracer), pathtracer.cpp:12-137, :247-452, :754-803 ---- */

typedef struct opathlet {
    v3 v;        /* towards_prev */
    float dens;
    overt vert;
    int light;
} opathlet;

static unsigned sample_path_rec(octx *c, opathlet *path, unsigned depth, unsigned max_depth) {
    const o_scene *s = c->s;
    while (depth != max_depth) {
        float w_dens;
        const opathlet *prev = &path[depth - 1];
        v3 i = bsdf_sample(s, vert_mat(s, &prev->vert), c->rng, &w_dens, prev->vert.normal, prev->v);
        if (feq(w_dens, 0.0f))
            return depth;
        oray r = mkray(prev->vert.vertex, i);
        overt nv = intersect(s, &r);
        if (nv.valid && vdot(nv.normal, vneg(i)) > 0) {
            path[depth].v = vneg(i);
            path[depth].vert = nv;
            path[depth].light = -1;
            path[depth].dens = w_dens;
            depth++;
        } else {
            return depth;
        }
    }
    return depth;
}

/* projected_brdf / projected_adjoint_brdf, pathtracer.cpp:54-68 */
static v3 projected_brdf(const o_scene *s, const opathlet *cur, const opathlet *next) {
    v3 towards = vneg(next->v);
    float cos_w = vdot(cur->vert.normal, towards);
    return vscale(bsdf_eval(s, vert_mat(s, &cur->vert), cur->vert.normal, towards, cur->v), cos_w);
}
static v3 projected_adjoint_brdf(const o_scene *s, const opathlet *cur, const opathlet *next) {
    v3 towards = vneg(next->v);
    float cos_w = vdot(cur->vert.normal, towards);
    return vscale(bsdf_eval(s, vert_mat(s, &cur->vert), cur->vert.normal, cur->v, towards), cos_w);
}

static v3 bdpt_connect(const o_scene *s, const opathlet *cam, unsigned clen, const opathlet *lp,
                       unsigned llen, const osurf *em, int light) {
    if (clen == 0)
        return V0;
    v3 cam_pre[64], light_pre[64];
    /* light_transport_info, :259-282 */
    v3 tr = V(1.0f, 1.0f, 1.0f);
    cam_pre[0] = tr;
    for (unsigned k = 0; k + 1 < clen; k++) {
        tr = vmul(tr, vdivs(projected_adjoint_brdf(s, &cam[k], &cam[k + 1]), cam[k + 1].dens));
        cam_pre[k + 1] = tr;
    }
    tr = V(1.0f, 1.0f, 1.0f);
    light_pre[0] = tr;
    for (unsigned k = 0; k + 1 < llen; k++) {
        tr = vmul(tr, vdivs(projected_brdf(s, &lp[k], &lp[k + 1]), lp[k + 1].dens));
        light_pre[k + 1] = tr;
    }
    v3 rad = V0;
    for (unsigned plen = 1; plen <= clen + llen + 1; plen++) {
        unsigned cam_plen = plen - 1 < clen ? plen - 1 : clen; /* std::min(plen - 1, max_cam_path_len) */
        unsigned light_plen = plen - 1 - cam_plen;
        v3 psum = V0;
        float wsum = 0.0f;
        float cw = 1.0f;
        while ((int)cam_plen >= 0 && light_plen <= llen) {
            if (light_plen == 0 && cam_plen == 0) {
                if (cam[0].light >= 0) {
                    v3 pr = light_radiance(s, cam[0].light, cam[0].v, cam[0].vert.normal);
                    psum = vadd(psum, vscale(pr, cw));
                }
                wsum += cw;
            } else if (light_plen == 0) {
                const opathlet *cj = &cam[cam_plen - 1];
                v3 ti = vdivs(transport_illum_source(s, light, em->p, em->n, &cj->vert, cj->v), em->area_dens);
                v3 pr = vdivs(vmul(ti, cam_pre[cam_plen - 1]), cam[0].dens);
                psum = vadd(psum, vscale(pr, cw));
                wsum += cw;
            } else if (cam_plen == 0) {
                ;
            } else {
                const opathlet *lj = &lp[light_plen - 1];
                const opathlet *cj = &cam[cam_plen - 1];
                v3 join = vsub(cj->vert.vertex, lj->vert.vertex);
                float jd = vnorm(join);
                join = vdivs(join, jd);
                oray jr = mkray(lj->vert.vertex, join);
                float cos_wo = vdot(lj->vert.normal, join);
                float cos_wi = vdot(cj->vert.normal, vneg(join));
                if (cos_wo > 0.0f && cos_wi > 0.0f && !has_intersect(s, &jr, 1e-3f, jd - 1e-3f)) {
                    v3 le = vdivs(light_projected_radiance(s, light, vneg(lp[0].v), em->n), lp[0].dens * em->area_dens);
                    v3 lsi = vmul(le, light_pre[light_plen - 1]);
                    float to_area = cos_wi * cos_wo / (jd * jd);
                    v3 ljw = bsdf_eval(s, vert_mat(s, &lj->vert), lj->vert.normal, join, lj->v);
                    v3 cjw = bsdf_eval(s, vert_mat(s, &cj->vert), cj->vert.normal, cj->v, vneg(join));
                    v3 ti = vscale(vmul(vmul(lsi, ljw), cjw), to_area);
                    v3 csr = vdivs(vmul(ti, cam_pre[cam_plen - 1]), cam[0].dens);
                    psum = vadd(psum, vscale(csr, cw));
                }
                wsum += cw;
            }
            light_plen++;
            cam_plen--;
        }
        if (wsum > 0)
            rad = vadd(rad, vdivs(psum, wsum));
    }
    return rad;
}

static v3 bdpt_path(octx *c, const oray *cam_ray, const overt *first, int first_light) {
    const o_scene *s = c->s;
    unsigned maxlen = c->pol->bdpt_max_len;
    if (maxlen > 64)
        maxlen = 64;
    opathlet cam[64], lp[64];
    unsigned clen = 0;
    if (first->valid && maxlen != 0) {
        cam[0].v = vneg(cam_ray->v);
        cam[0].vert = *first;
        cam[0].light = first_light;
        cam[0].dens = 1.0f;
        clen = sample_path_rec(c, cam, 1, maxlen);
    }
    /* sample_illum_source, :754-767 + area_light::sample_emssion, light.cpp:26-32 */
    float pmf;
    int light = sample_light(s, c->rng, &pmf);
    osurf em = mesh_sample(s, s->lights[light].mesh, c->rng, 0);
    v3 w = cos_hemisphere(em.n, c->rng);
    float sa_dens = vdot(em.n, w) / PI_F;
    em.area_dens *= pmf;
    oray r0 = mkray(em.p, w);
    unsigned llen = 0;
    overt v0 = intersect(s, &r0);
    if (v0.valid && !(vdot(v0.normal, vneg(r0.v)) <= 0.0f) && maxlen != 0) {
        lp[0].v = vneg(r0.v);
        lp[0].vert = v0;
        lp[0].light = -1;
        lp[0].dens = sa_dens;
        llen = sample_path_rec(c, lp, 1, maxlen);
    }
    return bdpt_connect(s, cam, clen, lp, llen, &em, light);
}

/* ---- product mode: NEE + BSDF sampling with power-heuristic MIS (new; not in the reference) ---- */

/* density of sampling direction i at a vertex (solid angle), consistent with bsdf_sample */
static float pdf_leaf(const omat *m, v3 n, v3 o, v3 i) {
    if (m->type == E8G_MAT_COOK_TORR) {
        if (vdot(i, n) < 0.0f)
            return 0.0f;
        v3 h = vadd(i, o);
        if (vequals0(h))
            return 0.0f;
        h = vnormalize(h);
        float hdo = vdot(h, o);
        float cos_h = vdot(n, h);
        if (hdo <= 0.0f || cos_h <= 0.0f)
            return 0.0f;
        return ggx_distri(m->alpha2, n, h) * cos_h / (4.0f * hdo);
    }
    float c = vdot(i, n);
    return c > 0.0f ? c / PI_F : 0.0f;
}
static float bsdf_pdf(const o_scene *s, const omat *m, v3 n, v3 o, v3 i) {
    if (m->type == E8G_MAT_MIXTURE)
        return m->ratio * pdf_leaf(find_mat(s, m->mix0), n, o, i) +
               (1 - m->ratio) * pdf_leaf(find_mat(s, m->mix1), n, o, i);
    return pdf_leaf(m, n, o, i);
}
static v3 bsdf_sample_mis(const o_scene *s, const omat *m, orng *rng, float *pdf, v3 n, v3 o) {
    if (m->type == E8G_MAT_MIXTURE) {
        float dummy;
        v3 i;
        if (draw(rng) < m->ratio)
            i = sample_leaf(find_mat(s, m->mix0), rng, &dummy, n, o);
        else
            i = sample_leaf(find_mat(s, m->mix1), rng, &dummy, n, o);
        if (dummy == 0.0f) {
            *pdf = 0.0f;
            return V0;
        }
        *pdf = bsdf_pdf(s, m, n, o, i);
        return i;
    }
    return sample_leaf(m, rng, pdf, n, o);
}

static inline float power_w(float a, float b) {
    float a2 = a * a, b2 = b * b;
    return a2 / (a2 + b2);
}

static v3 mis_path(octx *c, const oray *cam_ray, const overt *first, int first_light) {
    const o_scene *s = c->s;
    const o_policy *pol = c->pol;
    if (!first->valid)
        return V0;
    v3 L = V0;
    if (first_light >= 0)
        L = vadd(L, light_radiance(s, first_light, vneg(cam_ray->v), first->normal));
    v3 beta = V(1.0f, 1.0f, 1.0f);
    overt vert = *first;
    v3 o = vneg(cam_ray->v);
    for (unsigned depth = 0;; depth++) {
        if (pol->max_depth && depth >= pol->max_depth)
            break;
        if (depth >= pol->rr_start) {
            if (draw(c->rng) >= pol->rr_prob)
                break;
            beta = vdivs(beta, pol->rr_prob);
        }
        const omat *m = vert_mat(s, &vert);
        /* next-event estimation */
        float pmf;
        int light = sample_light(s, c->rng, &pmf);
        uint32_t lmesh = s->lights[light].mesh;
        osurf ls = mesh_sample(s, lmesh, c->rng, 1);
        v3 l = vsub(vert.vertex, ls.p);
        float r2 = vdot(l, l);
        float dist = sqrtf(r2);
        v3 ln = vdivs(l, dist);
        float cos_l = vdot(ls.n, ln);
        v3 wi = vneg(ln);
        float cos_x = vdot(vert.normal, wi);
        if (cos_l > 0.0f && cos_x > 0.0f) {
            v3 f = bsdf_eval(s, m, vert.normal, o, wi);
            if (!vequals0(f)) {
                float p_l = pmf * ls.area_dens * r2 / cos_l;
                float p_b = bsdf_pdf(s, m, vert.normal, o, wi);
                oray sr = mkray(vert.vertex, wi);
                if (!has_intersect(s, &sr, 1e-4f, dist - 1e-3f)) {
                    float w = power_w(p_l, p_b);
                    v3 contrib = vscale(vmul(vmul(beta, f), light_rad(s, light)), cos_x * w / p_l);
                    L = vadd(L, contrib);
                }
            }
        }
        /* BSDF continuation */
        float pdf;
        v3 i = bsdf_sample_mis(s, m, c->rng, &pdf, vert.normal, o);
        if (!(pdf > 0.0f))
            break;
        float cos_w = vdot(vert.normal, i);
        if (cos_w <= 0.0f)
            break;
        v3 f = bsdf_eval(s, m, vert.normal, o, i);
        beta = vmul(beta, vscale(f, cos_w / pdf));
        oray r = mkray(vert.vertex, i);
        overt nv = intersect(s, &r);
        if (!nv.valid || vdot(nv.normal, vneg(i)) <= 0.0f)
            break;
        int hl = vert_light(s, &nv);
        if (hl >= 0) {
            float cos_l2 = vdot(nv.normal, vneg(i));
            float pl = s->light_pnorm[hl] / s->total_power;
            float p_l = pl * (1.0f / s->mesh_area[s->lights[hl].mesh]) * (nv.t * nv.t) / cos_l2;
            float w = power_w(pdf, p_l);
            L = vadd(L, vscale(vmul(beta, light_rad(s, hl)), w));
        }
        vert = nv;
        o = vneg(i);
    }
    return L;
}

/* ---- product mode: bidirectional with power-heuristic MIS (new; not in the reference) ----
 * Camera subpath from the cached first hit, light subpath from an area-weighted emission
 * sample with a cosine direction, every (s light, t camera) connection with t >= 1, weighted by
 * the power heuristic over all strategies that could produce the same path. Densities are kept
 * in area measure per vertex: fwd (from the predecessor in its own subpath) and rev (from the
 * successor); the connection updates the four densities it changes (Veach's recurrence). */

typedef struct obv {
    v3 p, n;
    int32_t mesh;
    v3 beta;
    float fwd, rev;
} obv;

static inline float to_area(float pdf_w, v3 from, v3 to, v3 n_to) {
    v3 d = vsub(to, from);
    float d2 = vdot(d, d);
    if (d2 <= 0.0f)
        return 0.0f;
    float c = fabsf(vdot(n_to, d)) / sqrtf(d2);
    return pdf_w * c / d2;
}

/* BSDF density at vertex v of going out along `wi` given the other direction `wo` */
static inline float vpdf(const o_scene *s, const obv *v, v3 wo, v3 wi) {
    return bsdf_pdf(s, find_mat(s, s->mesh_mat[v->mesh]), v->n, wo, wi);
}

static unsigned bdp_walk(octx *c, obv *path, unsigned len, unsigned max_len, v3 wo) {
    const o_scene *s = c->s;
    while (len < max_len) {
        obv *cur = &path[len - 1];
        const omat *m = find_mat(s, s->mesh_mat[cur->mesh]);
        float pdf;
        v3 i = bsdf_sample_mis(s, m, c->rng, &pdf, cur->n, wo);
        if (!(pdf > 0.0f))
            break;
        float cw = vdot(cur->n, i);
        if (cw <= 0.0f)
            break;
        v3 f = bsdf_eval(s, m, cur->n, wo, i);
        oray r = mkray(cur->p, i);
        overt nv = intersect(s, &r);
        if (!nv.valid || vdot(nv.normal, vneg(i)) <= 0.0f)
            break;
        obv *nx = &path[len];
        nx->p = nv.vertex;
        nx->n = nv.normal;
        nx->mesh = nv.mesh;
        nx->beta = vmul(cur->beta, vscale(f, cw / pdf));
        nx->fwd = to_area(pdf, cur->p, nx->p, nx->n);
        nx->rev = 0.0f;
        /* density of sampling cur from nx (reverse direction) */
        float prev_w = vpdf(s, cur, i, wo);
        if (len >= 2)
            cur[-1].rev = to_area(prev_w, cur->p, cur[-1].p, cur[-1].n);
        wo = vneg(i);
        len++;
    }
    return len;
}

static v3 bdpt_power_path(octx *c, const oray *cam_ray, const overt *first) {
    const o_scene *s = c->s;
    unsigned maxlen = c->pol->bdpt_max_len;
    if (maxlen > 16)
        maxlen = 16;
    obv cam[16], lp[16];
    unsigned clen = 0, llen = 0;
    v3 o0 = vneg(cam_ray->v);
    if (first->valid && maxlen) {
        cam[0].p = first->vertex;
        cam[0].n = first->normal;
        cam[0].mesh = first->mesh;
        cam[0].beta = V(1, 1, 1);
        cam[0].fwd = 1.0f;
        cam[0].rev = 0.0f;
        clen = bdp_walk(c, cam, 1, maxlen, o0);
    }
    /* emission sample: light (CDF), area-weighted point, cosine direction */
    float pmf;
    int light = sample_light(s, c->rng, &pmf);
    osurf em = mesh_sample(s, s->lights[light].mesh, c->rng, 1);
    v3 w = cos_hemisphere(em.n, c->rng);
    float pdf_w = vdot(em.n, w) / PI_F;
    if (maxlen) {
        lp[0].p = em.p;
        lp[0].n = em.n;
        lp[0].mesh = (int32_t)s->lights[light].mesh;
        lp[0].fwd = pmf * em.area_dens;
        lp[0].rev = 0.0f;
        lp[0].beta = V(1.0f / lp[0].fwd, 1.0f / lp[0].fwd, 1.0f / lp[0].fwd);
        llen = 1;
        if (pdf_w > 0.0f && maxlen > 1) {
            oray r0 = mkray(em.p, w);
            overt v0 = intersect(s, &r0);
            if (v0.valid && vdot(v0.normal, vneg(w)) > 0.0f) {
                lp[1].p = v0.vertex;
                lp[1].n = v0.normal;
                lp[1].mesh = v0.mesh;
                /* beta_1 = Le cos / (pmf pA pdf_w) */
                lp[1].beta = vscale(light_rad(s, light), vdot(em.n, w) / (pdf_w * lp[0].fwd));
                lp[1].fwd = to_area(pdf_w, em.p, lp[1].p, lp[1].n);
                lp[1].rev = 0.0f;
                llen = bdp_walk(c, lp, 2, maxlen, vneg(w));
            }
        }
    }
    if (clen == 0)
        return V0;
    v3 L = V0;
    for (unsigned t = 1; t <= clen; t++) {
        for (unsigned sl = 0; sl <= llen; sl++) {
            obv *cv = &cam[t - 1];
            v3 wo_c = t >= 2 ? vnormalize(vsub(cam[t - 2].p, cv->p)) : o0;
            v3 contrib = V0;
            /* densities the connection changes (restored after) */
            float save_c_rev = cv->rev, save_c2_rev = t >= 2 ? cam[t - 2].rev : 0.0f;
            float save_l_rev = sl >= 1 ? lp[sl - 1].rev : 0.0f, save_l2_rev = sl >= 2 ? lp[sl - 2].rev : 0.0f;
            if (sl == 0) {
                int hl = s->mesh_light[cv->mesh];
                if (hl < 0)
                    continue;
                v3 le = light_radiance(s, hl, wo_c, cv->n);
                if (vequals0(le))
                    continue;
                contrib = vmul(cv->beta, le);
                float pl = s->light_pnorm[hl] / s->total_power;
                cv->rev = pl * (1.0f / s->mesh_area[s->lights[hl].mesh]);
                if (t >= 2) {
                    float ew = fmaxf(vdot(cv->n, wo_c), 0.0f) / PI_F;
                    cam[t - 2].rev = to_area(ew, cv->p, cam[t - 2].p, cam[t - 2].n);
                }
            } else {
                obv *lv = &lp[sl - 1];
                v3 d = vsub(lv->p, cv->p);
                float d2 = vdot(d, d);
                if (d2 <= 0.0f)
                    continue;
                float dist = sqrtf(d2);
                v3 dir = vdivs(d, dist); /* from camera vertex to light vertex */
                float cos_c = vdot(cv->n, dir);
                float cos_l = vdot(lv->n, vneg(dir));
                if (cos_c <= 0.0f || cos_l <= 0.0f)
                    continue;
                const omat *mc = find_mat(s, s->mesh_mat[cv->mesh]);
                v3 fc = bsdf_eval(s, mc, cv->n, wo_c, dir);
                if (vequals0(fc))
                    continue;
                v3 fl;
                v3 wo_l = V0;
                if (sl == 1) {
                    fl = light_radiance(s, light, vneg(dir), lv->n);
                } else {
                    wo_l = vnormalize(vsub(lp[sl - 2].p, lv->p));
                    fl = bsdf_eval(s, find_mat(s, s->mesh_mat[lv->mesh]), lv->n, vneg(dir), wo_l);
                }
                if (vequals0(fl))
                    continue;
                oray sr = mkray(cv->p, dir);
                if (has_intersect(s, &sr, 1e-4f, dist - 1e-3f))
                    continue;
                float G = cos_c * cos_l / d2;
                contrib = vscale(vmul(vmul(vmul(cv->beta, fc), fl), lv->beta), G);
                /* reverse densities of the connection */
                float pc = vpdf(s, cv, wo_c, dir);       /* camera vertex generating the light vertex */
                lv->rev = to_area(pc, cv->p, lv->p, lv->n);
                if (sl == 1)
                    cv->rev = to_area(cos_l / PI_F, lv->p, cv->p, cv->n);
                else
                    cv->rev = to_area(vpdf(s, lv, wo_l, vneg(dir)), lv->p, cv->p, cv->n);
                if (t >= 2)
                    cam[t - 2].rev = to_area(vpdf(s, cv, dir, wo_c), cv->p, cam[t - 2].p, cam[t - 2].n);
                if (sl >= 2)
                    lp[sl - 2].rev = to_area(vpdf(s, lv, vneg(dir), wo_l), lv->p, lp[sl - 2].p, lp[sl - 2].n);
            }
            /* power-heuristic weight over strategies producing this path */
            /* strategies whose subpaths would exceed the cap are impossible: stop there */
            /* single precision: a ratio product whose square overflows gives weight 0, where */
            /* double precision would give a weight below 1e-38 */
            float sum = 0.0f, ri = 1.0f;
            for (int i = (int)t - 1; i >= 1; i--) {
                if (sl + t - (unsigned)i > maxlen)
                    break;
                ri *= (cam[i].fwd > 0.0f) ? cam[i].rev / cam[i].fwd : 0.0f;
                sum += ri * ri;
            }
            ri = 1.0f;
            for (int i = (int)sl - 1; i >= 0; i--) {
                if (t + sl - (unsigned)i > maxlen)
                    break;
                ri *= (lp[i].fwd > 0.0f) ? lp[i].rev / lp[i].fwd : 0.0f;
                sum += ri * ri;
            }
            float wgt = 1.0f / (1.0f + sum);
            L = vadd(L, vscale(contrib, wgt));
            cv->rev = save_c_rev;
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

/* ---------------------------------------------------------- path driver -- */

typedef struct ofirst {
    overt hit;
    int light;
    oray ray;
} ofirst;

/* compute_first_hit, pathtracer.cpp:456-472 */
static ofirst first_hit(const o_scene *s, unsigned x, unsigned y, unsigned w, unsigned h) {
    ofirst f;
    f.ray = camera_ray(s, x, y, w, h);
    f.hit = intersect(s, &f.ray);
    f.light = -1;
    if (vdot(f.hit.normal, vneg(f.ray.v)) <= 0) {
        f.hit = miss_vert();
    } else if (f.hit.valid) {
        f.light = vert_light(s, &f.hit);
    }
    return f;
}

static v3 path_radiance(const o_scene *s, uint32_t mode, const o_policy *pol, orng *rng, const ofirst *f) {
    octx c = {s, pol, rng};
    switch (mode) {
    case E8G_MODE_REF_UNI: /* unidirect_path_tracer::sample, :568-585 */
        if (!f->hit.valid)
            return V0;
        return uni_rec(&c, vneg(f->ray.v), &f->hit, 0);
    case E8G_MODE_REF_LT1: { /* unidirect_lt1_path_tracer::sample, :630-653 */
        if (!f->hit.valid)
            return V0;
        v3 p = lt1_rec(&c, vneg(f->ray.v), &f->hit, 0);
        if (f->light >= 0)
            return vadd(p, light_radiance(s, f->light, vneg(f->ray.v), f->hit.normal));
        return p;
    }
    case E8G_MODE_REF_DIRECT: { /* direct_path_tracer::sample, :508-526 */
        if (!f->hit.valid)
            return V0;
        v3 r = transport_direct_illum(&c, vneg(f->ray.v), &f->hit);
        if (f->light >= 0)
            r = vadd(r, light_projected_radiance(s, f->light, vneg(f->ray.v), f->hit.normal));
        return r;
    }
    case E8G_MODE_REF_BDPT:
        return bdpt_path(&c, &f->ray, &f->hit, f->light);
    case E8G_MODE_REF_LT2: { /* bidirect_lt2_path_tracer::sample, :731-752 */
        if (!f->hit.valid)
            return V0;
        v3 p = lt2_rec(&c, vneg(f->ray.v), &f->hit, 0);
        if (f->light >= 0)
            return vadd(p, light_projected_radiance(s, f->light, vneg(f->ray.v), f->hit.normal));
        return p;
    }
    case E8G_MODE_MIS:
        return mis_path(&c, &f->ray, &f->hit, f->light);
    case E8G_MODE_BDPT_POWER:
        return bdpt_power_path(&c, &f->ray, &f->hit);
    case E8G_MODE_NORMAL: /* normal_tracer, :492-506 */
        if (!f->hit.valid)
            return V0;
        return vdivs(vadd(f->hit.normal, V(1.0f, 1.0f, 1.0f)), 2.0f);
    case E8G_MODE_POSITION: { /* position_tracer, :474-490 */
        if (!f->hit.valid)
            return V0;
        v3 range = vsub(s->bound.mx, s->bound.mn);
        v3 p = vsub(f->hit.vertex, s->bound.mn);
        return V(p.x / range.x, p.y / range.y, p.z / range.z);
    }
    default:
        return V0;
    }
}

typedef struct ojob {
    const o_scene *s;
    uint32_t mode, rng_kind;
    uint64_t seed;
    const o_policy *pol;
    uint32_t w, h;
    /* paths */
    const uint32_t *pixel, *seeds;
    uint32_t n;
    float *rgb;
    /* image */
    uint32_t spp, offset, x0, y0, x1, y1;
    float *rgba;
    /* work distribution */
    uint32_t next;
    pthread_mutex_t mu;
} ojob;

static uint32_t take(ojob *j, uint32_t chunk, uint32_t limit) {
    pthread_mutex_lock(&j->mu);
    uint32_t v = j->next;
    j->next = v + chunk < limit ? v + chunk : limit;
    pthread_mutex_unlock(&j->mu);
    return v;
}

static void *paths_worker(void *p) {
    ojob *j = (ojob *)p;
    for (;;) {
        uint32_t k0 = take(j, 64, j->n);
        if (k0 >= j->n)
            break;
        uint32_t k1 = k0 + 64 < j->n ? k0 + 64 : j->n;
        for (uint32_t k = k0; k < k1; k++) {
            uint32_t px = j->pixel[k];
            ofirst f = first_hit(j->s, px % j->w, px / j->w, j->w, j->h);
            orng rng;
            if (j->rng_kind == E8G_RNG_MINSTD)
                minstd_seed(&rng, j->seeds[k]);
            else
                philox_seed(&rng, j->seed, px, j->seeds[k]);
            v3 L = path_radiance(j->s, j->mode, j->pol, &rng, &f);
            vst(j->rgb + 3 * k, L);
        }
    }
    return NULL;
}

static void run_threads(void *(*fn)(void *), ojob *j, int num_threads) {
    if (num_threads <= 1) {
        fn(j);
        return;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)num_threads);
    for (int i = 0; i < num_threads; i++)
        pthread_create(&th[i], NULL, fn, j);
    for (int i = 0; i < num_threads; i++)
        pthread_join(th[i], NULL);
    free(th);
}

void o_render_paths(const o_scene *s, uint32_t mode, uint32_t rng_kind, uint64_t seed,
                    const o_policy *pol, uint32_t width, uint32_t height, const uint32_t *pixel,
                    const uint32_t *seeds, uint32_t n, float *rgb_out, int num_threads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.s = s;
    j.mode = mode;
    j.rng_kind = rng_kind;
    j.seed = seed;
    j.pol = pol;
    j.w = width;
    j.h = height;
    j.pixel = pixel;
    j.seeds = seeds;
    j.n = n;
    j.rgb = rgb_out;
    pthread_mutex_init(&j.mu, NULL);
    run_threads(paths_worker, &j, num_threads);
    pthread_mutex_destroy(&j.mu);
}

static void *image_worker(void *p) {
    ojob *j = (ojob *)p;
    uint32_t cw = j->x1 - j->x0, ch = j->y1 - j->y0;
    uint32_t npix = cw * ch;
    for (;;) {
        uint32_t k0 = take(j, 16, npix);
        if (k0 >= npix)
            break;
        uint32_t k1 = k0 + 16 < npix ? k0 + 16 : npix;
        for (uint32_t k = k0; k < k1; k++) {
            uint32_t x = j->x0 + k % cw, y = j->y0 + k / cw;
            uint32_t px = y * j->w + x;
            ofirst f = first_hit(j->s, x, y, j->w, j->h);
            v3 acc = V0;
            for (uint32_t sidx = 0; sidx < j->spp; sidx++) {
                orng rng;
                uint32_t sample = j->offset + sidx;
                if (j->rng_kind == E8G_RNG_MINSTD)
                    minstd_seed(&rng, o_path_seed(j->seed, px, sample));
                else
                    philox_seed(&rng, j->seed, px, sample);
                acc = vadd(acc, path_radiance(j->s, j->mode, j->pol, &rng, &f));
            }
            float inv = 1.0f / (float)j->spp;
            float *o = j->rgba + 4 * (size_t)k;
            o[0] = acc.x * inv;
            o[1] = acc.y * inv;
            o[2] = acc.z * inv;
            o[3] = 1.0f;
        }
    }
    return NULL;
}

void o_render(const o_scene *s, uint32_t mode, uint32_t rng_kind, uint64_t seed,
              const o_policy *pol, uint32_t width, uint32_t height, uint32_t spp,
              uint32_t sample_offset, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
              float *rgba_out, int num_threads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.s = s;
    j.mode = mode;
    j.rng_kind = rng_kind;
    j.seed = seed;
    j.pol = pol;
    j.w = width;
    j.h = height;
    j.spp = spp;
    j.offset = sample_offset;
    j.x0 = x0;
    j.y0 = y0;
    j.x1 = x1;
    j.y1 = y1;
    j.rgba = rgba_out;
    pthread_mutex_init(&j.mu, NULL);
    run_threads(image_worker, &j, num_threads);
    pthread_mutex_destroy(&j.mu);
}

/* pt_image_renderer::sampling_task::run, the firefly clamp (renderer.cpp:46-83) applied to one
 * sample image est (w*h rgb): an interior pixel whose squared norm (vec::norm2, tensor.h:213)
 * exceeds each of its 8 neighbours' by more than FireFlyMinDiff = 1.5 (renderer.h:118) has every
 * channel capped (vec::at_most, tensor.h:284-289) at the neighbours' mean squared norm plus 1.5.
 * Border pixels pass unchanged. The result is added to acc (w*h rgb). */
static float sqn(const float *v) {
    float r = 0.0f;
    r += v[0] * v[0];
    r += v[1] * v[1];
    r += v[2] * v[2];
    return r;
}

void o_firefly_add(const float *est, uint32_t w, uint32_t h, float *acc) {
    const float diff = 1.5f;
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) {
            size_t k = (size_t)y * w + x;
            const float *e = est + 3 * k;
            float *a = acc + 3 * k;
            if (x > 0 && x < w - 1 && y > 0 && y < h - 1) {
                float r00 = sqn(est + 3 * (k - w - 1)), r10 = sqn(est + 3 * (k - w)), r20 = sqn(est + 3 * (k - w + 1));
                float r01 = sqn(est + 3 * (k - 1)), r11 = sqn(e), r21 = sqn(est + 3 * (k + 1));
                float r02 = sqn(est + 3 * (k + w - 1)), r12 = sqn(est + 3 * (k + w)), r22 = sqn(est + 3 * (k + w + 1));
                int ff = (r11 - r00) > diff && (r11 - r10) > diff && (r11 - r20) > diff && (r11 - r01) > diff &&
                         (r11 - r21) > diff && (r11 - r02) > diff && (r11 - r12) > diff && (r11 - r22) > diff;
                if (ff) {
                    float cap = 1.0f / 8.0f * (r00 + r10 + r20 + r01 + r21 + r02 + r12 + r22) + diff;
                    for (int i = 0; i < 3; i++)
                        a[i] += cap < e[i] ? cap : e[i];
                    continue;
                }
            }
            for (int i = 0; i < 3; i++)
                a[i] += e[i];
        }
}

/* pt_image_renderer::render (renderer.cpp:106-166) with a single sampling task: the task's
 * stream is std::minstd_rand0 seeded task_seed (i*1361+33 for task i, renderer.cpp:102); each of
 * the spp samples runs the integrator over every pixel in row-major order drawing from that one
 * stream (for example unidirect_lt1_path_tracer::sample, pathtracer.cpp:630-653), passes the
 * sample image through the firefly clamp when asked (renderer.cpp:46-83), and adds it to the
 * task's estimate. The compositor receives (estimate, 1) and scales it by 1/spp, so alpha is
 * 1/spp, as in the reference. */
void o_render_task(const o_scene *s, uint32_t mode, const o_policy *pol, uint32_t w, uint32_t h, uint32_t spp,
                   int firefly, uint32_t task_seed, float *rgba_out) {
    size_t npix = (size_t)w * h;
    ofirst *f = (ofirst *)malloc(sizeof(ofirst) * npix);
    float *est = (float *)malloc(sizeof(float) * 3 * npix);
    float *acc = (float *)calloc(3 * npix, sizeof(float));
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++)
            f[(size_t)y * w + x] = first_hit(s, x, y, w, h);
    orng rng;
    memset(&rng, 0, sizeof(rng));
    minstd_seed(&rng, task_seed);
    for (uint32_t k = 0; k < spp; k++) {
        for (size_t i = 0; i < npix; i++) {
            v3 L = path_radiance(s, mode, pol, &rng, &f[i]);
            est[3 * i] = L.x;
            est[3 * i + 1] = L.y;
            est[3 * i + 2] = L.z;
        }
        if (firefly)
            o_firefly_add(est, w, h, acc);
        else
            for (size_t i = 0; i < 3 * npix; i++)
                acc[i] += est[i];
    }
    float scale = 1.0f / (float)spp;
    for (size_t i = 0; i < npix; i++) {
        for (int c = 0; c < 3; c++)
            rgba_out[4 * i + c] = (0.0f + acc[3 * i + c]) * scale;
        rgba_out[4 * i + 3] = (0.0f + 1.0f) * scale;
    }
    free(f);
    free(est);
    free(acc);
}

/* ---- compositors, compositor.cpp:29-98 ---- */

/* if_compositor::pixel_of (compositor.cpp:29-38): CLAMP to [0, 1], pow 1/2.2, * 255 truncated;
 * alpha * 255 truncated without a clamp. */
static unsigned char comp_channel(float c) {
    float x = c < 0.0f ? 0.0f : (c > 1.0f ? 1.0f : c);
    return (unsigned char)(powf(x, 1.0f / 2.2f) * 255.0f);
}

/* vec == 0.0f with the reference's epsilon: every component within 1e-5 (tensor.h:14-16, :123-128) */
static int comp_is_zero(const float *c) {
    for (int k = 0; k < 4; k++)
        if (!(fabsf(c[k] - 0.0f) <= 1e-5f))
            return 0;
    return 1;
}

/* aces_compositor::exposure (compositor.cpp:87-98): exp of the mean log(luminance + 1e-3) over
 * the pixels that are not all-zero, summed in float in pixel order. */
static float comp_exposure(const float *rgba, size_t npix) {
    unsigned n = 0;
    float sum = 0;
    for (size_t i = 0; i < npix; i++) {
        const float *c = rgba + 4 * i;
        if (!comp_is_zero(c)) {
            float lum = c[0] * 0.299f + c[1] * 0.587f + c[2] * 0.114f; /* luminance, :83-85 */
            sum += logf(lum + 1e-3f);
            n++;
        }
    }
    sum /= n;
    return expf(sum);
}

void o_composite(const float *rgba, uint32_t w, uint32_t h, uint32_t tonemap, int auto_exposure, float exposure,
                 unsigned char *out) {
    size_t npix = (size_t)w * h;
    float e = exposure;
    if (tonemap == E8G_TONEMAP_ACES && auto_exposure)
        e = comp_exposure(rgba, npix);
    for (size_t i = 0; i < npix; i++) {
        const float *c = rgba + 4 * i;
        float v[4];
        if (tonemap == E8G_TONEMAP_ACES) { /* aces_tonemap, :71-81 */
            const float A = 2.51f, B = 0.03f, C = 2.43f, D = 0.59f, E = 0.14f;
            for (int k = 0; k < 3; k++) {
                float x = c[k] * e;
                v[k] = x * (x * A + B) / (x * (x * C + D) + E);
            }
            v[3] = c[3];
        } else { /* clamp_compositor::commit, :47-53: at_least(0).at_most(1) */
            for (int k = 0; k < 4; k++) {
                float x = 0.0f > c[k] ? 0.0f : c[k]; /* at_least, tensor.h:277-282 */
                v[k] = 1.0f < x ? 1.0f : x;          /* at_most, tensor.h:284-289 */
            }
        }
        for (int k = 0; k < 3; k++)
            out[4 * i + k] = comp_channel(v[k]);
        out[4 * i + 3] = (unsigned char)(v[3] * 255.0f);
    }
}

/* ------------------------------------------------- FP64 adjoint reference -- */
/* Double-precision restatement of the product estimator (mis_path above) and of the path-replay
 * gradient the GPU computes: same draws and discrete decisions (light, triangle, Russian
 * roulette, hits), contributions and derivatives carried in double. Not in the reference: it is
 * the checker of the GPU adjoint. */

typedef struct dv3 {
    double x, y, z;
} dv3;
static inline dv3 D3(double x, double y, double z) {
    dv3 r = {x, y, z};
    return r;
}
static inline dv3 dfrom(v3 a) { return D3(a.x, a.y, a.z); }
static inline v3 dto(dv3 a) { return V((float)a.x, (float)a.y, (float)a.z); }
static inline dv3 dadd(dv3 a, dv3 b) { return D3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline dv3 dsub(dv3 a, dv3 b) { return D3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline dv3 dmul(dv3 a, dv3 b) { return D3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline dv3 dscale(dv3 a, double k) { return D3(a.x * k, a.y * k, a.z * k); }
static inline double ddot(dv3 a, dv3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline dv3 dcross(dv3 a, dv3 b) { return D3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline dv3 dnorm(dv3 a) { return dscale(a, 1.0 / sqrt(ddot(a, a))); }

static void dbasis(dv3 n, dv3 *u, dv3 *v) {
    dv3 ref = fabs(n.x) > .1 ? D3(0, 1, 0) : D3(1, 1, 1);
    *u = dnorm(dcross(ref, n));
    *v = dcross(n, *u);
}

static double d_ggx(double a2, dv3 n, dv3 h) {
    double c = ddot(n, h), c2 = c * c, t2 = (1 - c2) / c2, k = 1 + t2 / a2;
    return 1.0 / (M_PI * a2 * c2 * c2 * k * k);
}
static double d_lambda(double a2, dv3 n, dv3 w) {
    double c = ddot(n, w), c2 = c * c, t2 = (1 - c2) / c2;
    return (-1 + sqrt(1 + a2 * t2)) / 2;
}

/* f (per channel) of a leaf material; *g receives d ln f / d r for cook_torr */
static dv3 d_eval_leaf(const omat *m, dv3 n, dv3 o, dv3 i, double *dlog_dr) {
    *dlog_dr = 0;
    dv3 alb = dfrom(m->albedo);
    if (m->type == E8G_MAT_OREN_NAYAR) {
        double ci = ddot(i, n), co = ddot(o, n);
        ci = ci < 0 ? 0 : (ci > 1 ? 1 : ci);
        co = co < 0 ? 0 : (co > 1 ? 1 : co);
        if (ci <= 1e-5 || co <= 1e-5)
            return D3(0, 0, 0);
        double ca = ci < co ? ci : co, cb = ci < co ? co : ci;
        double sa = sqrt(1 - ca * ca), sb = sqrt(1 - cb * cb);
        double cio = ca * cb + sa * sb;
        return dscale(alb, (m->a + m->b * (cio > 0 ? cio : 0) * sa * (sb / co)) / M_PI);
    }
    if (m->type == E8G_MAT_COOK_TORR) {
        double co = ddot(n, o), ci = ddot(n, i);
        if (ci <= 1e-5 || co <= 1e-5)
            return D3(0, 0, 0);
        dv3 h = dadd(i, o);
        if (fabs(h.x) <= 1e-5 && fabs(h.y) <= 1e-5 && fabs(h.z) <= 1e-5)
            return D3(0, 0, 0);
        h = dnorm(h);
        double a2 = (double)m->alpha2;
        double fl = 1 - ddot(i, h), f5 = fl * fl * fl * fl * fl;
        double re = m->ior_re, im = m->ior_im;
        double F = ((re - 1) * (re - 1) + 4 * re * f5 + im * im) / ((re + 1) * (re + 1) + im * im);
        double D = d_ggx(a2, n, h);
        double li = d_lambda(a2, n, i), lo = d_lambda(a2, n, o);
        double G = 1 / (1 + li + lo);
        double c = ddot(n, h), c2 = c * c, t2 = (1 - c2) / c2, k = 1 + t2 / a2;
        double dlnD = -1 / a2 + 2 * t2 / (a2 * a2 * k);
        double ti = (1 - ci * ci) / (ci * ci), to = (1 - co * co) / (co * co);
        double dli = ti / (4 * sqrt(1 + a2 * ti)), dlo = to / (4 * sqrt(1 + a2 * to));
        double dlnG = -(dli + dlo) / (1 + li + lo);
        double r = sqrt(a2 / 2);
        *dlog_dr = (dlnD + dlnG) * 4 * r;
        return dscale(alb, F * D * G / (4 * ci * co));
    }
    return dscale(alb, 1.0 / M_PI);
}

static double d_pdf_leaf(const omat *m, dv3 n, dv3 o, dv3 i) {
    if (m->type == E8G_MAT_COOK_TORR) {
        if (ddot(i, n) < 0)
            return 0;
        dv3 h = dnorm(dadd(i, o));
        double hdo = ddot(h, o), ch = ddot(n, h);
        if (hdo <= 0 || ch <= 0)
            return 0;
        return d_ggx((double)m->alpha2, n, h) * ch / (4 * hdo);
    }
    double c = ddot(i, n);
    return c > 0 ? c / M_PI : 0;
}

static void d_grad(const o_scene *s, int32_t mesh, dv3 C, double dlr, const float w[3], double *da, double *dr) {
    int32_t mi = s->mesh_mat[mesh];
    if (mi < 0 || (uint32_t)mi >= s->nmat)
        return;
    const omat *m = &s->mats[mi];
    if (m->type != E8G_MAT_OREN_NAYAR && m->type != E8G_MAT_COOK_TORR)
        return;
    double c[3] = {C.x, C.y, C.z};
    double alb[3] = {m->albedo.x, m->albedo.y, m->albedo.z};
    for (int k = 0; k < 3; k++)
        if (alb[k] > 0)
            da[3 * mi + k] += w[k] * c[k] / alb[k];
    if (m->type == E8G_MAT_COOK_TORR)
        dr[mi] += (w[0] * c[0] + w[1] * c[1] + w[2] * c[2]) * dlr;
}

static dv3 d_replay(const o_scene *s, uint64_t seed, const o_policy *pol, const ofirst *f, uint32_t pixel,
                    uint32_t sample, int grad, dv3 Ltot, const float w[3], double *da, double *dr) {
    orng rng;
    philox_seed(&rng, seed, pixel, sample);
    dv3 L = D3(0, 0, 0);
    if (f->light >= 0) {
        v3 le = light_radiance(s, f->light, vneg(f->ray.v), f->hit.normal);
        L = dfrom(le);
    }
    dv3 beta = D3(1, 1, 1);
    dv3 p = dfrom(f->hit.vertex), n = dfrom(f->hit.normal), o = dscale(dfrom(f->ray.v), -1);
    int32_t mesh = f->hit.mesh;
    for (unsigned depth = 0;; depth++) {
        if (pol->max_depth && depth >= pol->max_depth)
            break;
        if (depth >= pol->rr_start) {
            if (draw(&rng) >= pol->rr_prob)
                break;
            beta = dscale(beta, 1.0 / pol->rr_prob);
        }
        const omat *m = find_mat(s, s->mesh_mat[mesh]);
        /* light sample (float draws, double geometry) */
        float pmf;
        int light = sample_light(s, &rng, &pmf);
        uint32_t lm = s->lights[light].mesh;
        uint32_t ntris = s->toff[lm + 1] - s->toff[lm];
        float q = draw(&rng);
        float e = q * s->mesh_area[lm];
        unsigned lo = 0, hi = ntris;
        const float *cum = s->tri_cum + s->toff[lm];
        while (lo < hi) {
            unsigned mi = (lo + hi) >> 1;
            if (cum[mi] <= e)
                lo = mi + 1;
            else
                hi = mi;
        }
        if (lo >= ntris)
            lo = ntris - 1;
        uint32_t t = s->toff[lm] + lo;
        double u = draw(&rng), vv = draw(&rng);
        double r = sqrt(u), b0 = 1 - r, b1 = r * vv, b2 = 1 - b0 - b1;
        uint32_t i0 = s->tri[3 * t], i1 = s->tri[3 * t + 1], i2 = s->tri[3 * t + 2];
        dv3 lp = dadd(dadd(dscale(dfrom(s->pos[i0]), b0), dscale(dfrom(s->pos[i1]), b1)), dscale(dfrom(s->pos[i2]), b2));
        dv3 lnrm = dnorm(dadd(dadd(dscale(dfrom(s->nrm[i0]), b0), dscale(dfrom(s->nrm[i1]), b1)), dscale(dfrom(s->nrm[i2]), b2)));
        dv3 l = dsub(p, lp);
        double r2 = ddot(l, l), dist = sqrt(r2);
        dv3 ln = dscale(l, 1 / dist);
        double cos_l = ddot(lnrm, ln);
        dv3 wi = dscale(ln, -1);
        double cos_x = ddot(n, wi);
        if (cos_l > 0 && cos_x > 0) {
            double dlr;
            dv3 fv = d_eval_leaf(m, n, o, wi, &dlr);
            if (!(fabs(fv.x) <= 1e-5 && fabs(fv.y) <= 1e-5 && fabs(fv.z) <= 1e-5)) {
                double p_l = pmf * (1.0 / s->mesh_area[lm]) * r2 / cos_l;
                double p_b = d_pdf_leaf(m, n, o, wi);
                oray sr = mkray(dto(p), dto(wi));
                if (!has_intersect(s, &sr, 1e-4f, (float)dist - 1e-3f)) {
                    double wgt = p_l * p_l / (p_l * p_l + p_b * p_b);
                    dv3 c = dscale(dmul(dmul(beta, fv), dfrom(light_rad(s, light))), cos_x * wgt / p_l);
                    L = dadd(L, c);
                    if (grad)
                        d_grad(s, mesh, c, dlr, w, da, dr);
                }
            }
        }
        /* BSDF sample (draw order of sample_leaf) */
        dv3 i;
        double pdf;
        if (m->type == E8G_MAT_COOK_TORR) {
            dv3 uu, vb;
            dbasis(n, &uu, &vb);
            double theta = 2.0 * M_PI * draw(&rng);
            double tt = draw(&rng);
            double phi = atan(sqrt((double)m->alpha2 * tt / (1 - tt)));
            dv3 h = dadd(dadd(dscale(uu, sin(phi) * cos(theta)), dscale(vb, sin(phi) * sin(theta))), dscale(n, cos(phi)));
            double hdo = ddot(h, o);
            i = dsub(dscale(h, 2 * hdo), o);
            if (ddot(i, n) < 0)
                break;
            pdf = d_ggx((double)m->alpha2, n, h) * cos(phi) / (4 * hdo);
        } else if (m->type == E8G_MAT_MIXTURE) {
            break; /* mixtures are not part of the gradient check scenes */
        } else {
            double e1 = draw(&rng), e0 = draw(&rng);
            dv3 uu, vb;
            dbasis(n, &uu, &vb);
            double z = sqrt(e1), rr = sqrt(1 - z * z), ph = e0 * 2 * M_PI;
            i = dadd(dadd(dscale(uu, rr * cos(ph)), dscale(vb, rr * sin(ph))), dscale(n, z));
            pdf = ddot(i, n) / M_PI;
        }
        if (!(pdf > 0))
            break;
        double cw = ddot(n, i);
        if (cw <= 0)
            break;
        double dlr;
        dv3 fv = d_eval_leaf(m, n, o, i, &dlr);
        if (grad)
            d_grad(s, mesh, dsub(Ltot, L), dlr, w, da, dr);
        beta = dmul(beta, dscale(fv, cw / pdf));
        oray rr_ = mkray(dto(p), dto(i));
        overt nv = intersect(s, &rr_);
        if (!nv.valid)
            break;
        dv3 nn = dfrom(nv.normal);
        if (ddot(nn, dscale(i, -1)) <= 0)
            break;
        int hl = vert_light(s, &nv);
        if (hl >= 0) {
            double cos_l2 = ddot(nn, dscale(i, -1));
            double pl = (double)s->light_pnorm[hl] / s->total_power;
            double t2 = (double)nv.t * nv.t;
            double p_l = pl * (1.0 / s->mesh_area[s->lights[hl].mesh]) * t2 / cos_l2;
            double wgt = pdf * pdf / (pdf * pdf + p_l * p_l);
            L = dadd(L, dscale(dmul(beta, dfrom(light_rad(s, hl))), wgt));
        }
        p = dfrom(nv.vertex);
        n = nn;
        mesh = nv.mesh;
        o = dscale(i, -1);
    }
    return L;
}

void o_path_gradient_f64(const o_scene *s, uint64_t seed, const o_policy *pol, uint32_t width,
                         uint32_t height, uint32_t pixel, uint32_t sample, const float w[3],
                         double *d_albedo, double *d_roughness, double rgb_out[3]) {
    ofirst f = first_hit(s, pixel % width, pixel / width, width, height);
    rgb_out[0] = rgb_out[1] = rgb_out[2] = 0.0;
    if (!f.hit.valid)
        return;
    dv3 Ltot = d_replay(s, seed, pol, &f, pixel, sample, 0, D3(0, 0, 0), w, d_albedo, d_roughness);
    d_replay(s, seed, pol, &f, pixel, sample, 1, Ltot, w, d_albedo, d_roughness);
    rgb_out[0] = Ltot.x;
    rgb_out[1] = Ltot.y;
    rgb_out[2] = Ltot.z;
}

/* The same gradient summed over a whole image: every pixel's spp paths (samples 0 .. spp - 1),
 * each weighted by dl[pixel] / spp (float, as the device weights them). Pixels are handed out in
 * chunks to num_threads threads; each sums into its own arrays, merged at the end. */
typedef struct ograd_job {
    const o_scene *s;
    uint64_t seed;
    const o_policy *pol;
    uint32_t w, h, spp;
    const float *dl;
    double *da, *dr;
    uint32_t next;
    pthread_mutex_t mu;
} ograd_job;

static void *grad_worker(void *p) {
    ograd_job *j = (ograd_job *)p;
    uint32_t nm = j->s->nmat, npix = j->w * j->h;
    double *da = (double *)calloc((size_t)nm * 4 + 4, sizeof(double));
    double *dr = da + 3 * (size_t)nm + 2;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        uint32_t k0 = j->next;
        j->next = k0 + 16 < npix ? k0 + 16 : npix;
        pthread_mutex_unlock(&j->mu);
        if (k0 >= npix)
            break;
        uint32_t k1 = k0 + 16 < npix ? k0 + 16 : npix;
        for (uint32_t px = k0; px < k1; px++) {
            float wgt[3];
            for (int c = 0; c < 3; c++)
                wgt[c] = j->dl[3 * (size_t)px + c] / (float)j->spp;
            double rgb[3];
            for (uint32_t smp = 0; smp < j->spp; smp++)
                o_path_gradient_f64(j->s, j->seed, j->pol, j->w, j->h, px, smp, wgt, da, dr, rgb);
        }
    }
    pthread_mutex_lock(&j->mu);
    for (uint32_t i = 0; i < 3 * nm; i++)
        j->da[i] += da[i];
    for (uint32_t i = 0; i < nm; i++)
        j->dr[i] += dr[i];
    pthread_mutex_unlock(&j->mu);
    free(da);
    return NULL;
}

void o_image_gradient_f64(const o_scene *s, uint64_t seed, const o_policy *pol, uint32_t width,
                          uint32_t height, uint32_t spp, const float *dl, double *d_albedo,
                          double *d_roughness, int num_threads) {
    ograd_job j;
    memset(&j, 0, sizeof(j));
    j.s = s;
    j.seed = seed;
    j.pol = pol;
    j.w = width;
    j.h = height;
    j.spp = spp;
    j.dl = dl;
    j.da = d_albedo;
    j.dr = d_roughness;
    memset(d_albedo, 0, sizeof(double) * 3 * s->nmat);
    memset(d_roughness, 0, sizeof(double) * s->nmat);
    pthread_mutex_init(&j.mu, NULL);
    if (num_threads <= 1) {
        grad_worker(&j);
    } else {
        pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)num_threads);
        for (int i = 0; i < num_threads; i++)
            pthread_create(&th[i], NULL, grad_worker, &j);
        for (int i = 0; i < num_threads; i++)
            pthread_join(th[i], NULL);
        free(th);
    }
    pthread_mutex_destroy(&j.mu);
}

/* ------------------------------------------------------------- transform -- */
/* trimesh::transform, geometry.cpp:76-87, on mat<4,4> of tensor.h. */

/* mat::det(next_row, curr_col, removed_col), tensor.h:451-473: Laplace expansion along column
 * `col` (1-based) over the rows left in the linked list next[] (1-based, 5 ends it), the next
 * column skipping `removed`. */
static float mat4_minor(const float a[4][4], unsigned next[5], unsigned col, unsigned removed) {
    unsigned row = next[0];
    if (next[row] == 5)
        return a[row - 1][col - 1];
    float d = 0.0f;
    unsigned i = 0, prev = 0;
    while (row != 5) {
        next[prev] = next[row];
        float m = mat4_minor(a, next, col + 1 == removed ? col + 2 : col + 1, removed);
        next[prev] = row;
        float x = a[row - 1][col - 1];
        d += (i & 1 ? -x : x) * m;
        prev = row;
        row = next[row];
        i++;
    }
    return d;
}

/* mat::operator^(-1) (tensor.h:511-540) through adjugate (:483-504) and det(adj) (:475-481),
 * transposed (operator~, :551-559). */
static int mat4_normal_matrix(const float a[4][4], float out[4][4]) {
    unsigned next[5] = {1, 2, 3, 4, 5};
    float adj[4][4];
    for (unsigned j = 1; j <= 4; j++)
        for (unsigned i = 1; i <= 4; i++) {
            next[i - 1] = i + 1;
            float m = mat4_minor(a, next, j == 1 ? 2 : 1, j);
            next[i - 1] = i;
            adj[j - 1][i - 1] = ((i + j) & 1) ? -m : m;
        }
    float d = 0;
    for (unsigned i = 0; i < 4; i++)
        d += a[i][0] * adj[0][i];
    if (fabsf(d - 0.0f) <= 1e-5f)
        return 0;
    float k = 1.0f / d;
    for (unsigned i = 0; i < 4; i++)
        for (unsigned j = 0; j < 4; j++)
            out[j][i] = k * adj[i][j];
    return 1;
}

/* (m * (x, y, z, w)).cart(): mat * vec (tensor.h:425-433) then vec::cart (:261-268). */
static void mat4_apply_cart(const float a[4][4], const float *x, float w, float *out) {
    float h[4] = {x[0], x[1], x[2], w}, v[4] = {0, 0, 0, 0};
    for (unsigned j = 0; j < 4; j++)
        for (unsigned i = 0; i < 4; i++)
            v[i] = v[i] + a[i][j] * h[j];
    float inv_w = 1.0f / v[3];
    for (unsigned i = 0; i < 3; i++)
        out[i] = inv_w * v[i];
}

int o_transform_mesh(const float m[16], const float *pos, const float *nrm, uint32_t n, float *pos_out,
                     float *nrm_out) {
    float a[4][4], nm[4][4];
    for (unsigned i = 0; i < 4; i++)
        for (unsigned j = 0; j < 4; j++)
            a[i][j] = m[4 * i + j];
    if (!mat4_normal_matrix(a, nm))
        return 0;
    for (uint32_t v = 0; v < n; v++)
        mat4_apply_cart(a, &pos[3 * (size_t)v], 1.0f, &pos_out[3 * (size_t)v]);
    for (uint32_t v = 0; v < n; v++)
        mat4_apply_cart(nm, &nrm[3 * (size_t)v], 1.0f, &nrm_out[3 * (size_t)v]);
    return 1;
}
