// The reference's own BVH, rebuilt in the GPU node arrays: bvh_path_space_layout::commit and its
// helpers (corelib/src/pathspace.cpp:121-328) restated step for step — 20 buckets on the largest
// axis, cost 1 + 8 (SA_L/SA n_L + SA_R/SA n_R), the bucket-0 / split_antiaxis = 1 start of the
// minimum search (:209-216), median split with std::sort past depth log2 N (:223-230),
// std::partition otherwise (:233-245), and aabb's union with an empty box taking the empty box's
// zero corners (tensor.h:757, :763-772). std::sort and std::partition are the same library calls
// the reference makes, so the tree, its depth-first layout (left child = n + 1, right child =
// next_child, :274-290) and therefore the order in which traversal meets triangles are the
// reference's. Used when hit identities must match the reference bit for bit, ties included.
#include "bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace e8g {
namespace {

struct rbox { // e8util::aabb
    float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    bool empty = true;
};

inline float rmin(float a, float b) { return b < a ? b : a; } // std::min
inline float rmax(float a, float b) { return a < b ? b : a; } // std::max

inline rbox make_box(float const *mn, float const *mx) {
    rbox b;
    for (int i = 0; i < 3; i++) {
        b.mn[i] = mn[i];
        b.mx[i] = mx[i];
    }
    b.empty = mn[0] > mx[0] || mn[1] > mx[1] || mn[2] > mx[2];
    return b;
}
inline rbox merge(rbox const &a, rbox const &r) {
    if (a.empty)
        return r;
    float mn[3], mx[3];
    for (int i = 0; i < 3; i++) {
        mn[i] = rmin(a.mn[i], r.mn[i]);
        mx[i] = rmax(a.mx[i], r.mx[i]);
    }
    return make_box(mn, mx);
}
inline rbox add_point(rbox const &a, float const *p) {
    if (a.empty)
        return make_box(p, p);
    float mn[3], mx[3];
    for (int i = 0; i < 3; i++) {
        mn[i] = rmin(a.mn[i], p[i]);
        mx[i] = rmax(a.mx[i], p[i]);
    }
    return make_box(mn, mx);
}
inline float area(rbox const &b) {
    if (b.empty)
        return 0.0f;
    float d0 = b.mx[0] - b.mn[0], d1 = b.mx[1] - b.mn[1], d2 = b.mx[2] - b.mn[2];
    return 2.0f * (d0 * d1 + d0 * d2 + d1 * d2);
}

struct prim { // primitive_details
    uint32_t tri;
    rbox bound;
    float centroid[3];
};

struct bucket {
    float cost = 0.0f;
    unsigned num_prims = 0;
    rbox bound;
};

struct ref_builder {
    std::vector<prim> prims;
    flat_bvh *out;
    uint32_t max_depth = 0;

    uint32_t push(rbox const &b, uint32_t link, uint32_t count) {
        uint32_t n = out->num_nodes++;
        out->lo.resize(4 * static_cast<size_t>(out->num_nodes));
        out->hi.resize(4 * static_cast<size_t>(out->num_nodes));
        set(n, b, link, count);
        return n;
    }
    void set(uint32_t n, rbox const &b, uint32_t link, uint32_t count) {
        float *lo = &out->lo[4 * static_cast<size_t>(n)];
        float *hi = &out->hi[4 * static_cast<size_t>(n)];
        for (int i = 0; i < 3; i++) {
            lo[i] = b.mn[i];
            hi[i] = b.mx[i];
        }
        std::memcpy(&lo[3], &link, 4);
        std::memcpy(&hi[3], &count, 4);
    }

    void leaf(rbox const &b, unsigned start, unsigned count, unsigned depth) {
        push(b, start, count);
        out->num_leaves++;
        max_depth = std::max(max_depth, depth + 1);
    }

    void build(unsigned start, unsigned end, unsigned depth) {
        if (end - start == 0)
            return;
        if (end - start == 1) {
            leaf(prims[start].bound, start, 1, depth);
            return;
        }
        rbox b;
        for (unsigned i = start; i < end; i++)
            b = merge(b, prims[i].bound);
        float range[3] = {b.mx[0] - b.mn[0], b.mx[1] - b.mn[1], b.mx[2] - b.mn[2]};
        unsigned axis;
        if (range[0] > range[1] && range[0] > range[2])
            axis = 0;
        else if (range[1] > range[2])
            axis = 1;
        else
            axis = 2;
        float cost_nonsplit = static_cast<float>((end - start) * 8u);
        bucket buckets[20];
        float width = range[axis] / 20;
        for (unsigned i = start; i < end; i++) {
            // a node whose primitives all sit at one point has width 0: the reference divides 0 by
            // 0 and converts the NaN to an index (undefined behaviour); here they go to bucket 0
            float q = width > 0 ? (prims[i].centroid[axis] - b.mn[axis]) / width : 0.0f;
            unsigned ib = q >= 19.0f ? 19u : static_cast<unsigned>(q);
            buckets[ib].bound = merge(buckets[ib].bound, prims[i].bound);
            buckets[ib].num_prims++;
        }
        buckets[19].cost = INFINITY;
        for (unsigned i = 0; i < 19; i++) {
            rbox first, second;
            unsigned cf = 0, cs = 0;
            for (unsigned j = 0; j <= i; j++) {
                first = merge(first, buckets[j].bound);
                cf += buckets[j].num_prims;
            }
            for (unsigned j = i + 1; j < 20; j++) {
                second = merge(second, buckets[j].bound);
                cs += buckets[j].num_prims;
            }
            buckets[i].cost = 1 + 8 * (+area(first) / area(b) * static_cast<float>(cf) +
                                       area(second) / area(b) * static_cast<float>(cs));
        }
        unsigned split_antiaxis = 1;
        float cost_split = buckets[0].cost;
        for (unsigned i = 1; i < 19; i++) {
            if (buckets[i].cost < cost_split) {
                split_antiaxis = i;
                cost_split = buckets[i].cost;
            }
        }
        if (cost_split < cost_nonsplit || end - start > 4) {
            unsigned mid;
            if (depth > std::log2(prims.size())) {
                std::sort(prims.begin() + start, prims.begin() + end,
                          [axis](prim const &a, prim const &c) { return a.centroid[axis] < c.centroid[axis]; });
                mid = (start + end) >> 1;
            } else {
                float split = b.mn[axis] + (split_antiaxis + 1) * range[axis] / 20;
                auto it = std::partition(prims.begin() + start, prims.begin() + end,
                                         [axis, split](prim const &a) { return a.centroid[axis] < split; });
                mid = static_cast<unsigned>(it - prims.begin());
                if (mid == start)
                    mid++;
                else if (mid == end)
                    mid--;
            }
            uint32_t n = push(b, 0, 0);
            build(start, mid, depth + 1);
            set(n, b, out->num_nodes, 0); // next_child: the right subtree starts here
            build(mid, end, depth + 1);
        } else {
            leaf(b, start, end - start, depth);
        }
    }
};

} // namespace

flat_bvh build_bvh_reference(float const *pos, uint32_t const *tris, uint32_t num_tris) {
    flat_bvh out;
    if (num_tris == 0)
        return out;
    ref_builder rb;
    rb.out = &out;
    rb.prims.resize(num_tris);
    for (uint32_t t = 0; t < num_tris; t++) {
        prim &p = rb.prims[t];
        p.tri = t;
        rbox b;
        for (int k = 0; k < 3; k++)
            b = add_point(b, &pos[3 * static_cast<size_t>(tris[3 * static_cast<size_t>(t) + k])]);
        p.bound = b;
        for (int i = 0; i < 3; i++)
            p.centroid[i] = (b.mx[i] + b.mn[i]) / 2.0f;
    }
    out.lo.reserve(8 * static_cast<size_t>(num_tris));
    out.hi.reserve(8 * static_cast<size_t>(num_tris));
    rb.build(0, num_tris, 0);
    out.tri_order.resize(num_tris);
    for (uint32_t i = 0; i < num_tris; i++)
        out.tri_order[i] = rb.prims[i].tri;
    out.max_depth = rb.max_depth;
    return out;
}

} // namespace e8g
