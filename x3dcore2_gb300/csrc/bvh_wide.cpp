// Collapse of the binary SAH tree into the eight-wide quantized layout described in bvh_wide.h.
//
// Each wide node starts from one binary subtree and repeatedly opens the child with the largest
// surface area until eight children are collected or none can be opened (greedy collapse).
// Binary leaves become leaf slots; a leaf with more than kWideMaxLeaf triangles is split by
// position into halves with their own boxes. Wide nodes are laid out breadth first so that each
// node's interior children are contiguous.
#include "bvh_wide.h"
#include "bvh_boxes.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>

namespace e8g {
namespace {

struct wbox {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(wbox const &b) {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    float area() const {
        float d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
        if (!(d0 >= 0) || !(d1 >= 0) || !(d2 >= 0))
            return 0.0f;
        return 2.0f * (d0 * d1 + d0 * d2 + d1 * d2);
    }
};

// A subtree to place in a slot: a binary node, or a range of triangle positions (a leaf).
struct item {
    wbox b;
    int32_t bn = -1;          // binary node index (interior), or -1 for a triangle range
    uint32_t start = 0, count = 0;
};

struct collapser {
    flat_bvh const &b;
    float const *pos;
    uint32_t const *tris;
    float eps;

    uint32_t link(uint32_t n) const {
        uint32_t v;
        std::memcpy(&v, &b.lo[4 * static_cast<size_t>(n) + 3], 4);
        return v;
    }
    uint32_t count(uint32_t n) const {
        uint32_t v;
        std::memcpy(&v, &b.hi[4 * static_cast<size_t>(n) + 3], 4);
        return v;
    }
    item of_node(uint32_t n) const {
        item it;
        for (int a = 0; a < 3; a++) {
            it.b.lo[a] = b.lo[4 * static_cast<size_t>(n) + a];
            it.b.hi[a] = b.hi[4 * static_cast<size_t>(n) + a];
        }
        if (count(n) == 0) {
            it.bn = static_cast<int32_t>(n);
        } else {
            it.start = link(n);
            it.count = count(n);
        }
        return it;
    }
    // Box of a triangle range, inflated like the binary tree's boxes.
    item of_range(uint32_t start, uint32_t n) const {
        item it;
        it.start = start;
        it.count = n;
        for (uint32_t k = start; k < start + n; k++) {
            uint32_t t = b.tri_order[k];
            for (int v = 0; v < 3; v++) {
                float const *p = &pos[3 * static_cast<size_t>(tris[3 * static_cast<size_t>(t) + v])];
                for (int a = 0; a < 3; a++) {
                    it.b.lo[a] = std::min(it.b.lo[a], p[a]);
                    it.b.hi[a] = std::max(it.b.hi[a], p[a]);
                }
            }
        }
        for (int a = 0; a < 3; a++) {
            it.b.lo[a] = inflate_lo(it.b.lo[a], eps);
            it.b.hi[a] = inflate_hi(it.b.hi[a], eps);
        }
        return it;
    }
    static bool openable(item const &it) { return it.bn >= 0 || it.count > kWideMaxLeaf; }
    void open(item const &it, item out[2]) const {
        if (it.bn >= 0) {
            uint32_t l = link(static_cast<uint32_t>(it.bn));
            out[0] = of_node(l);
            out[1] = of_node(l + 1);
        } else {
            uint32_t h = it.count / 2;
            out[0] = of_range(it.start, h);
            out[1] = of_range(it.start + h, it.count - h);
        }
    }
};

} // namespace

wide_bvh collapse_wide(flat_bvh const &b, float const *pos, uint32_t const *tris, float max_abs) {
    wide_bvh w;
    if (b.num_nodes == 0)
        return w;
    // split leaves get boxes pushed out like the binary tree's, so every slot box is the exact
    // union of its triangles pushed out by the same eps (what the device refit recomputes)
    collapser cl{b, pos, tris, b.eps};
    double step_min = wide_step_min(max_abs);

    struct job {
        item it;
        uint32_t node, depth;
    };
    std::deque<job> q;
    q.push_back({cl.of_node(0), 0, 1});
    w.num_nodes = 1;
    w.nodes.assign(kWideWords, 0u);
    w.tri_order.reserve(b.tri_order.size());
    while (!q.empty()) {
        job jb = q.front();
        q.pop_front();
        if (jb.depth > w.level_start.size()) // the queue is breadth first: a level's nodes are contiguous
            w.level_start.push_back(jb.node);
        w.max_depth = std::max(w.max_depth, jb.depth);
        // collect up to eight children
        item ch[8];
        int n = 0;
        if (collapser::openable(jb.it)) {
            cl.open(jb.it, ch);
            n = 2;
            while (n < 8) {
                int best = -1;
                float best_area = -1.0f;
                for (int i = 0; i < n; i++)
                    if (collapser::openable(ch[i]) && ch[i].b.area() > best_area) {
                        best = i;
                        best_area = ch[i].b.area();
                    }
                if (best < 0)
                    break;
                item two[2];
                cl.open(ch[best], two);
                ch[best] = two[0];
                ch[n++] = two[1];
            }
        } else {
            ch[0] = jb.it; // a root that is a small leaf
            n = 1;
        }
        // slot assignment: child i goes to slot s with the smallest projection of its centre
        // offset onto octant s's direction, greedily over all (child, slot) pairs; a node with
        // at most four children uses slots 0-3 only (ordered by the x and y signs), so the
        // traversal tests one half of the slots
        wbox u;
        for (int i = 0; i < n; i++)
            u.grow(ch[i].b);
        int slot_of[8], child_in[8];
        for (int i = 0; i < 8; i++)
            slot_of[i] = child_in[i] = -1;
        float cost[8][8];
        for (int i = 0; i < n; i++)
            for (int s = 0; s < 8; s++) {
                float c = 0;
                for (int a = 0; a < 3; a++) {
                    float off = 0.5f * (ch[i].b.lo[a] + ch[i].b.hi[a]) - 0.5f * (u.lo[a] + u.hi[a]);
                    c += (s >> a & 1) ? -off : off;
                }
                cost[i][s] = c;
            }
        for (int k = 0; k < n; k++) {
            int bi = -1, bs = -1;
            float bc = INFINITY;
            for (int i = 0; i < n; i++) {
                if (slot_of[i] >= 0)
                    continue;
                for (int s = 0; s < (n <= 4 ? 4 : 8); s++)
                    if (child_in[s] < 0 && (bi < 0 || cost[i][s] < bc)) {
                        bi = i;
                        bs = s;
                        bc = cost[i][s];
                    }
            }
            slot_of[bi] = bs;
            child_in[bs] = bi;
        }
        // quantization grid and child boxes
        uint32_t words[kWideWords] = {0};
        float slo[8][3] = {{0}}, shi[8][3] = {{0}};
        uint32_t present = 0;
        for (int s = 0; s < 8; s++) {
            if (child_in[s] < 0)
                continue;
            present |= 1u << s;
            for (int a = 0; a < 3; a++) {
                slo[s][a] = ch[child_in[s]].b.lo[a];
                shi[s][a] = ch[child_in[s]].b.hi[a];
            }
        }
        wide_quantize(slo, shi, present, step_min, words);
        uint32_t imask = 0, n_int = 0;
        for (int s = 0; s < 8; s++)
            if (child_in[s] >= 0 && collapser::openable(ch[child_in[s]]))
                imask |= 1u << s, n_int++;
        uint32_t child_base = w.num_nodes;
        w.num_nodes += n_int;
        w.nodes.resize(static_cast<size_t>(w.num_nodes) * kWideWords, 0u);
        uint32_t tri_base = static_cast<uint32_t>(w.tri_order.size());
        words[3] |= imask << 24;
        words[4] = child_base;
        words[5] = tri_base;
        uint8_t meta[8] = {0};
        uint32_t counts = 0, rank = 0, leaves = 0;
        for (int s = 0; s < 8; s++) {
            int i = child_in[s];
            if (i < 0)
                continue;
            item const &c = ch[i];
            if (imask >> s & 1) {
                q.push_back({c, child_base + rank, jb.depth + 1});
                rank++;
            } else {
                meta[s] = static_cast<uint8_t>(w.tri_order.size() - tri_base);
                counts |= c.count << (4 * s);
                leaves |= 1u << s;
                for (uint32_t k = c.start; k < c.start + c.count; k++)
                    w.tri_order.push_back(b.tri_order[k]);
                w.num_leaves++;
            }
        }
        std::memcpy(&words[6], meta, 8);
        words[20] = counts;
        words[21] = leaves;
        std::memcpy(&w.nodes[static_cast<size_t>(jb.node) * kWideWords], words, sizeof(words));
    }
    w.level_start.push_back(w.num_nodes);
    w.ok = w.max_depth <= kWideMaxDepth;
    return w;
}

} // namespace e8g
