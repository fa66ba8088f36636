// Binned-SAH BVH builder (host). The reference's cost model (pathspace.cpp:121-260: box cost +
// triangle cost x area-weighted counts, leaf size cap), with its constants as options, but bins
// over all three axes of the centroid bounds, builds large subtrees on several threads, caps the
// depth at kMaxTreeDepth and writes the GPU layout directly.
#include "bvh.h"
#include "bvh_boxes.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <future>
#include <thread>

namespace e8g {
namespace {

struct box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(box const &b) {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow(float const *p) {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    float area() const {
        float d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
        if (d0 < 0 || d1 < 0 || d2 < 0)
            return 0.0f;
        return 2.0f * (d0 * d1 + d0 * d2 + d1 * d2);
    }
};

struct tmp_node {
    box b;
    int32_t child[2] = {-1, -1};
    uint32_t start = 0, count = 0;
    uint32_t depth = 0;
};

struct builder {
    bvh_build_opts o;
    std::vector<box> pb;           // per-triangle bounds
    std::vector<float> pc;         // per-triangle centroid, 3 floats
    std::vector<uint32_t> ids;     // permutation being partitioned
    std::vector<tmp_node> nodes;
    std::atomic<uint32_t> next{0};
    std::atomic<uint32_t> max_depth{0};
    uint32_t parallel_cutoff = 1u << 15;

    uint32_t alloc() { return next.fetch_add(1); }

    void make_leaf(uint32_t n, uint32_t start, uint32_t end, uint32_t depth) {
        nodes[n].start = start;
        nodes[n].count = end - start;
        uint32_t d = depth + 1, cur = max_depth.load();
        while (d > cur && !max_depth.compare_exchange_weak(cur, d)) {
        }
    }

    void build(uint32_t n, uint32_t start, uint32_t end, uint32_t depth) {
        tmp_node &nd = nodes[n];
        nd.depth = depth;
        box b, cb;
        for (uint32_t i = start; i < end; i++) {
            b.grow(pb[ids[i]]);
            cb.grow(&pc[3 * ids[i]]);
        }
        nd.b = b;
        uint32_t count = end - start;
        if (count == 1 || depth + 1 >= kMaxTreeDepth) {
            make_leaf(n, start, end, depth);
            return;
        }
        // SAH over binned centroids, all three axes.
        const uint32_t nb = std::max<uint32_t>(2, std::min<uint32_t>(o.num_bins, 64));
        float best_cost = INFINITY;
        int best_axis = -1;
        uint32_t best_bin = 0;
        float parent_area = b.area();
        for (int a = 0; a < 3; a++) {
            float ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0))
                continue;
            box bins[64];
            uint32_t cnt[64] = {0};
            float k = nb / ext;
            for (uint32_t i = start; i < end; i++) {
                uint32_t id = ids[i];
                uint32_t bi = std::min<uint32_t>(nb - 1, static_cast<uint32_t>((pc[3 * id + a] - cb.lo[a]) * k));
                bins[bi].grow(pb[id]);
                cnt[bi]++;
            }
            float right_area[64];
            uint32_t right_cnt[64];
            box acc;
            uint32_t c = 0;
            for (int i = static_cast<int>(nb) - 1; i > 0; i--) {
                acc.grow(bins[i]);
                c += cnt[i];
                right_area[i] = acc.area();
                right_cnt[i] = c;
            }
            box lacc;
            uint32_t lc = 0;
            for (uint32_t i = 0; i + 1 < nb; i++) {
                lacc.grow(bins[i]);
                lc += cnt[i];
                if (lc == 0 || right_cnt[i + 1] == 0)
                    continue;
                float cost = o.node_cost + o.tri_cost * (lacc.area() * lc + right_area[i + 1] * right_cnt[i + 1]) /
                                               std::max(parent_area, 1e-30f);
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = a;
                    best_bin = i + 1;
                }
            }
        }
        float leaf_cost = o.tri_cost * count;
        if (count <= o.max_leaf_prims && (best_axis < 0 || best_cost >= leaf_cost)) {
            make_leaf(n, start, end, depth);
            return;
        }
        uint32_t mid;
        if (best_axis < 0) {
            mid = start + count / 2; // all centroids coincide: split by index
        } else {
            int a = best_axis;
            float k = nb / (cb.hi[a] - cb.lo[a]);
            float lo = cb.lo[a];
            auto it = std::partition(ids.begin() + start, ids.begin() + end, [&](uint32_t id) {
                return std::min<uint32_t>(nb - 1, static_cast<uint32_t>((pc[3 * id + a] - lo) * k)) < best_bin;
            });
            mid = static_cast<uint32_t>(it - ids.begin());
            if (mid == start || mid == end)
                mid = start + count / 2;
        }
        uint32_t l = alloc(), r = alloc();
        nodes[n].child[0] = static_cast<int32_t>(l);
        nodes[n].child[1] = static_cast<int32_t>(r);
        if (count > parallel_cutoff) {
            auto fut = std::async(std::launch::async, [this, l, start, mid, depth] { build(l, start, mid, depth + 1); });
            build(r, mid, end, depth + 1);
            fut.get();
        } else {
            build(l, start, mid, depth + 1);
            build(r, mid, end, depth + 1);
        }
    }
};

} // namespace

flat_bvh build_bvh(float const *pos, uint32_t const *tris, uint32_t num_tris, bvh_build_opts const &o) {
    flat_bvh out;
    if (num_tris == 0)
        return out;
    builder b;
    b.o = o;
    b.o.tri_cost = effective_tri_cost(o);
    b.pb.resize(num_tris);
    b.pc.resize(3 * static_cast<size_t>(num_tris));
    b.ids.resize(num_tris);
    box scene;
    for (uint32_t t = 0; t < num_tris; t++) {
        box tb;
        for (int k = 0; k < 3; k++)
            tb.grow(&pos[3 * static_cast<size_t>(tris[3 * static_cast<size_t>(t) + k])]);
        b.pb[t] = tb;
        for (int a = 0; a < 3; a++)
            b.pc[3 * static_cast<size_t>(t) + a] = 0.5f * (tb.lo[a] + tb.hi[a]);
        b.ids[t] = t;
        scene.grow(tb);
    }
    b.nodes.resize(2 * static_cast<size_t>(num_tris) + 1);
    uint32_t root = b.alloc();
    b.build(root, 0, num_tris, 0);
    uint32_t n_tmp = b.next.load();

    // Flatten depth first; the two children of an interior node take adjacent slots.
    out.lo.assign(4 * static_cast<size_t>(n_tmp), 0.0f);
    out.hi.assign(4 * static_cast<size_t>(n_tmp), 0.0f);
    float eps = scene_eps(scene.lo, scene.hi);
    out.eps = eps;
    uint32_t next_slot = 1;
    uint64_t leaf_depth_sum = 0;
    struct item {
        uint32_t tmp, slot;
    };
    std::vector<item> stack{{root, 0}};
    while (!stack.empty()) {
        item it = stack.back();
        stack.pop_back();
        tmp_node const &t = b.nodes[it.tmp];
        float *lo = &out.lo[4 * static_cast<size_t>(it.slot)];
        float *hi = &out.hi[4 * static_cast<size_t>(it.slot)];
        for (int a = 0; a < 3; a++) {
            lo[a] = inflate_lo(t.b.lo[a], eps);
            hi[a] = inflate_hi(t.b.hi[a], eps);
        }
        uint32_t link, count;
        if (t.child[0] < 0) {
            link = t.start;
            count = t.count;
            out.num_leaves++;
            leaf_depth_sum += t.depth;
        } else {
            link = next_slot;
            count = 0;
            next_slot += 2;
            stack.push_back({static_cast<uint32_t>(t.child[1]), link + 1});
            stack.push_back({static_cast<uint32_t>(t.child[0]), link});
        }
        std::memcpy(&lo[3], &link, 4);
        std::memcpy(&hi[3], &count, 4);
    }
    out.num_nodes = next_slot;
    out.lo.resize(4 * static_cast<size_t>(out.num_nodes));
    out.hi.resize(4 * static_cast<size_t>(out.num_nodes));
    out.tri_order = std::move(b.ids);
    out.max_depth = b.max_depth.load();
    out.avg_leaf_depth = out.num_leaves ? static_cast<double>(leaf_depth_sum) / out.num_leaves : 0.0;
    return out;
}

} // namespace e8g
